// Host build of the TLAS topology over the instances' world boxes by a full sweep SAH (surface area
// heuristic). Instances are few (tens to thousands), so an O(n log^2 n) build on the host takes
// microseconds to milliseconds, and it places instances as large as the scene (a terrain) next to the
// root, where a Morton-ordered LBVH buries them in a subtree whose box then covers everything.
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

} // namespace rgl
