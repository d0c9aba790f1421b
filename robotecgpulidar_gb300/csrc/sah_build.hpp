// Host builds of binary BVH topologies by the surface area heuristic (SAH): a full sweep for the
// TLAS over the instances' world boxes (tens to thousands of boxes, microseconds to milliseconds; it
// places instances as large as the scene, a terrain, next to the root, where a Morton-ordered LBVH
// buries them in a subtree whose box then covers everything), and a binned SAH for mesh BLASes
// (25 % fewer node visits per ray than the Morton LBVH on the 1M-triangle scene, at the same cost as
// the full sweep). The wide collapse then runs unchanged on either.
//
// Output format = the LBVH's (bvh_core.hpp CollapseInputs): n - 1 binary nodes with boxes, children
// >= 0 internal, < 0 ~sorted position; per internal node the range of sorted positions; sortedIds maps
// a sorted position to the instance index. The wide collapse then runs unchanged.
#pragma once

#include <algorithm>
#include <numeric>
#include <vector>

#include "bvh_core.hpp"

namespace rgl {

struct SahTree
{
	std::vector<BinNode> bin;
	std::vector<int32_t> rangeFirst, rangeLast;
	std::vector<int32_t> sortedIds;
};

inline SahTree buildSahTree(const std::vector<Box>& boxes)
{
	const int n = (int) boxes.size();
	SahTree t;
	t.sortedIds.resize(n);
	std::iota(t.sortedIds.begin(), t.sortedIds.end(), 0);
	if (n < 2) {
		return t;
	}
	t.bin.resize(n - 1);
	t.rangeFirst.resize(n - 1);
	t.rangeLast.resize(n - 1);
	std::vector<float> cen[3];
	for (int a = 0; a < 3; ++a) {
		cen[a].resize(n);
	}
	for (int i = 0; i < n; ++i) {
		cen[0][i] = 0.5f * (boxes[i].lox + boxes[i].hix);
		cen[1][i] = 0.5f * (boxes[i].loy + boxes[i].hiy);
		cen[2][i] = 0.5f * (boxes[i].loz + boxes[i].hiz);
	}
	int nextNode = 0;
	std::vector<int> ids = t.sortedIds;
	std::vector<float> rightArea(n);
	// Node `node` covers sorted positions [lo, hi); returns the child reference of that range.
	struct Item
	{
		int lo, hi, node;
	};
	std::vector<Item> stack;
	stack.push_back({0, n, nextNode++});
	while (!stack.empty()) {
		const Item it = stack.back();
		stack.pop_back();
		const int cnt = it.hi - it.lo;
		int bestAxis = 0, bestSplit = it.lo + cnt / 2;
		float bestCost = INFINITY;
		std::vector<int> sorted[3];
		for (int a = 0; a < 3; ++a) {
			sorted[a].assign(ids.begin() + it.lo, ids.begin() + it.hi);
			std::stable_sort(sorted[a].begin(), sorted[a].end(), [&](int x, int y) { return cen[a][x] < cen[a][y]; });
			Box acc = emptyBox();
			for (int k = cnt - 1; k >= 1; --k) {
				acc = unite(acc, boxes[sorted[a][k]]);
				rightArea[k] = halfArea(acc);
			}
			acc = emptyBox();
			for (int k = 1; k < cnt; ++k) {
				acc = unite(acc, boxes[sorted[a][k - 1]]);
				const float cost = halfArea(acc) * (float) k + rightArea[k] * (float) (cnt - k);
				if (cost < bestCost) {
					bestCost = cost;
					bestAxis = a;
					bestSplit = it.lo + k;
				}
			}
		}
		std::copy(sorted[bestAxis].begin(), sorted[bestAxis].end(), ids.begin() + it.lo);
		BinNode& b = t.bin[it.node];
		Box u = emptyBox();
		for (int k = it.lo; k < it.hi; ++k) {
			u = unite(u, boxes[ids[k]]);
		}
		b.lox = u.lox;
		b.loy = u.loy;
		b.loz = u.loz;
		b.hix = u.hix;
		b.hiy = u.hiy;
		b.hiz = u.hiz;
		t.rangeFirst[it.node] = it.lo;
		t.rangeLast[it.node] = it.hi - 1;
		const int ranges[2][2] = {{it.lo, bestSplit}, {bestSplit, it.hi}};
		int32_t child[2];
		for (int c = 0; c < 2; ++c) {
			if (ranges[c][1] - ranges[c][0] == 1) {
				child[c] = ~ranges[c][0];
			} else {
				child[c] = nextNode;
				stack.push_back({ranges[c][0], ranges[c][1], nextNode++});
			}
		}
		b.left = child[0];
		b.right = child[1];
	}
	t.sortedIds = ids;
	return t;
}

// Binned SAH (after Wald, "On fast construction of SAH-based bounding volume hierarchies", 2007):
// at every node the centroids are binned into `bins` equal slices per axis and the split with the
// lowest area x count cost among the bin boundaries is taken; nodes whose centroids coincide are split
// at the middle of the range. O(n log n); used for BLASes, whose primitive counts reach millions.
// Output format as buildSahTree.
inline SahTree buildBinnedSahTree(const std::vector<Box>& boxes, int bins = 32)
{
	const int n = (int) boxes.size();
	SahTree t;
	t.sortedIds.resize(n);
	std::iota(t.sortedIds.begin(), t.sortedIds.end(), 0);
	if (n < 2) {
		return t;
	}
	t.bin.resize(n - 1);
	t.rangeFirst.resize(n - 1);
	t.rangeLast.resize(n - 1);
	std::vector<float> cen(3 * (size_t) n);
	for (int i = 0; i < n; ++i) {
		cen[3 * i] = 0.5f * (boxes[i].lox + boxes[i].hix);
		cen[3 * i + 1] = 0.5f * (boxes[i].loy + boxes[i].hiy);
		cen[3 * i + 2] = 0.5f * (boxes[i].loz + boxes[i].hiz);
	}
	std::vector<int>& ids = t.sortedIds;
	std::vector<Box> binBox(bins), rightBox(bins);
	std::vector<int> binCount(bins), rightCount(bins);
	struct Item
	{
		int lo, hi, node;
	};
	std::vector<Item> stack;
	stack.push_back({0, n, 0});
	int nextNode = 1;
	while (!stack.empty()) {
		const Item it = stack.back();
		stack.pop_back();
		Box u = emptyBox();
		float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
		for (int k = it.lo; k < it.hi; ++k) {
			u = unite(u, boxes[ids[k]]);
			for (int a = 0; a < 3; ++a) {
				cmin[a] = std::min(cmin[a], cen[3 * ids[k] + a]);
				cmax[a] = std::max(cmax[a], cen[3 * ids[k] + a]);
			}
		}
		int bestAxis = -1, bestBin = 0;
		float bestCost = INFINITY;
		for (int a = 0; a < 3; ++a) {
			const float ext = cmax[a] - cmin[a];
			if (!(ext > 0.0f)) {
				continue;
			}
			const float scale = (float) bins / ext;
			std::fill(binBox.begin(), binBox.end(), emptyBox());
			std::fill(binCount.begin(), binCount.end(), 0);
			for (int k = it.lo; k < it.hi; ++k) {
				const int b = std::min(bins - 1, (int) ((cen[3 * ids[k] + a] - cmin[a]) * scale));
				binBox[b] = unite(binBox[b], boxes[ids[k]]);
				++binCount[b];
			}
			Box acc = emptyBox();
			int cnt = 0;
			for (int b = bins - 1; b >= 1; --b) {
				acc = unite(acc, binBox[b]);
				cnt += binCount[b];
				rightBox[b] = acc;
				rightCount[b] = cnt;
			}
			acc = emptyBox();
			cnt = 0;
			for (int b = 1; b < bins; ++b) { // split between bins b-1 and b
				acc = unite(acc, binBox[b - 1]);
				cnt += binCount[b - 1];
				if (cnt == 0 || rightCount[b] == 0) {
					continue;
				}
				const float cost = halfArea(acc) * (float) cnt + halfArea(rightBox[b]) * (float) rightCount[b];
				if (cost < bestCost) {
					bestCost = cost;
					bestAxis = a;
					bestBin = b;
				}
			}
		}
		int mid = (it.lo + it.hi) / 2;
		if (bestAxis >= 0) {
			const float ext = cmax[bestAxis] - cmin[bestAxis], scale = (float) bins / ext;
			const float lo0 = cmin[bestAxis];
			const int a = bestAxis, split = bestBin;
			auto* first = ids.data() + it.lo;
			auto* pivot = std::stable_partition(first, ids.data() + it.hi, [&](int id) {
				return std::min(bins - 1, (int) ((cen[3 * id + a] - lo0) * scale)) < split;
			});
			const int m = (int) (pivot - ids.data());
			if (m > it.lo && m < it.hi) {
				mid = m;
			}
		}
		BinNode& bn = t.bin[it.node];
		bn.lox = u.lox;
		bn.loy = u.loy;
		bn.loz = u.loz;
		bn.hix = u.hix;
		bn.hiy = u.hiy;
		bn.hiz = u.hiz;
		t.rangeFirst[it.node] = it.lo;
		t.rangeLast[it.node] = it.hi - 1;
		const int ranges[2][2] = {{it.lo, mid}, {mid, it.hi}};
		int32_t child[2];
		for (int c = 0; c < 2; ++c) {
			if (ranges[c][1] - ranges[c][0] == 1) {
				child[c] = ~ranges[c][0];
			} else {
				child[c] = nextNode;
				stack.push_back({ranges[c][0], ranges[c][1], nextNode++});
			}
		}
		bn.left = child[0];
		bn.right = child[1];
	}
	return t;
}

} // namespace rgl
