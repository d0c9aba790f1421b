// On-device BVH construction: per-mesh BLAS (8-wide, quantised) and per-scene TLAS (binary) with a
// refit path for pose updates. The per-item logic lives in bvh_core.hpp.
//
// Replaces the OptiX acceleration-structure builds of reference src/scene/GASBuilder.hpp:31-100 and
// src/scene/Scene.cpp:131-190 (where any pose change triggers a full IAS rebuild plus a stream sync).
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "bvh_core.hpp"
#include "kernels.hpp"
#include "sah_build.hpp"

namespace rgl {

namespace {

#define RGL_CUDA_OK(expr)                                                                                                      \
	do {                                                                                                                       \
		cudaError_t e_ = (expr);                                                                                               \
		if (e_ != cudaSuccess) {                                                                                               \
			throw std::runtime_error(std::string("CUDA error in BVH build: ") + cudaGetErrorString(e_) + " at " #expr);        \
		}                                                                                                                      \
	} while (0)

__device__ __forceinline__ uint32_t orderedBits(float f)
{
	uint32_t u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float orderedFloat(uint32_t u)
{
	uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#if defined(__CUDA_ARCH__)
	return __uint_as_float(v);
#else
	float f;
	__builtin_memcpy(&f, &v, 4);
	return f;
#endif
}

// Triangle boxes, centroids and the centroid bounds (6 ordered uints: min xyz, max xyz).
__global__ void kTriBounds(const float* __restrict__ v, const int32_t* __restrict__ idx, int nTris, float4* lo, float4* hi,
                           uint32_t* cbounds)
{
	__shared__ uint32_t sh[6];
	if (threadIdx.x < 6) {
		sh[threadIdx.x] = threadIdx.x < 3 ? 0xffffffffu : 0u;
	}
	__syncthreads();
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t < nTris) {
		const float* a = v + 3 * (size_t) idx[3 * t];
		const float* b = v + 3 * (size_t) idx[3 * t + 1];
		const float* c = v + 3 * (size_t) idx[3 * t + 2];
		float4 l = make_float4(fminf(fminf(a[0], b[0]), c[0]), fminf(fminf(a[1], b[1]), c[1]), fminf(fminf(a[2], b[2]), c[2]), 0.f);
		float4 h = make_float4(fmaxf(fmaxf(a[0], b[0]), c[0]), fmaxf(fmaxf(a[1], b[1]), c[1]), fmaxf(fmaxf(a[2], b[2]), c[2]), 0.f);
		lo[t] = l;
		hi[t] = h;
		float cx = 0.5f * (l.x + h.x), cy = 0.5f * (l.y + h.y), cz = 0.5f * (l.z + h.z);
		atomicMin(&sh[0], orderedBits(cx));
		atomicMin(&sh[1], orderedBits(cy));
		atomicMin(&sh[2], orderedBits(cz));
		atomicMax(&sh[3], orderedBits(cx));
		atomicMax(&sh[4], orderedBits(cy));
		atomicMax(&sh[5], orderedBits(cz));
	}
	__syncthreads();
	if (threadIdx.x < 3) {
		atomicMin(&cbounds[threadIdx.x], sh[threadIdx.x]);
	} else if (threadIdx.x < 6) {
		atomicMax(&cbounds[threadIdx.x], sh[threadIdx.x]);
	}
}

__global__ void kMorton(const float4* __restrict__ lo, const float4* __restrict__ hi, int n, const uint32_t* cbounds,
                        uint32_t* codes, uint32_t* ids)
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= n) {
		return;
	}
	Box cb{orderedFloat(cbounds[0]), orderedFloat(cbounds[1]), orderedFloat(cbounds[2]),
	       orderedFloat(cbounds[3]), orderedFloat(cbounds[4]), orderedFloat(cbounds[5])};
	float4 l = lo[t], h = hi[t];
	codes[t] = morton30(0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z), cb);
	ids[t] = (uint32_t) t;
}

__global__ void kLbvh(const uint32_t* __restrict__ codes, int n, BinNode* bin, int32_t* rangeFirst, int32_t* rangeLast,
                      int32_t* parentInt, int32_t* parentLeaf)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n - 1) {
		return;
	}
	int32_t l, r, f, la;
	lbvhInternal(i, codes, n, l, r, f, la);
	if (l >= 0) {
		parentInt[l] = i;
	} else {
		parentLeaf[~l] = i;
	}
	if (r >= 0) {
		parentInt[r] = i;
	} else {
		parentLeaf[~r] = i;
	}
	bin[i].left = l;
	bin[i].right = r;
	if (rangeFirst) {
		rangeFirst[i] = f;
		rangeLast[i] = la;
	}
	if (i == 0) {
		parentInt[0] = -1;
	}
}

__device__ __forceinline__ Box loadBoxCg(const BinNode* n)
{
	const float4* p = reinterpret_cast<const float4*>(n);
	float4 a = __ldcg(p), b = __ldcg(p + 1);
	return Box{a.x, a.y, a.z, b.x, b.y, b.z};
}

// Bottom-up bounds: the second child to arrive at a node unites both children and moves up.
// Leaf boxes: lo/hi[ids[k]] for sorted position k.
__global__ void kBottomUp(int n, const uint32_t* __restrict__ ids, const float4* __restrict__ lo, const float4* __restrict__ hi,
                          BinNode* bin, const int32_t* __restrict__ parentInt, const int32_t* __restrict__ parentLeaf,
                          uint32_t* visits)
{
	int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= n) {
		return;
	}
	int node = parentLeaf[k];
	while (node >= 0) {
		__threadfence();
		if (atomicAdd(&visits[node], 1u) == 0u) {
			return;
		}
		int32_t c[2] = {bin[node].left, bin[node].right};
		Box bx[2];
		for (int q = 0; q < 2; ++q) {
			if (c[q] >= 0) {
				bx[q] = loadBoxCg(&bin[c[q]]);
			} else {
				int li = (int) ids[~c[q]];
				float4 l = lo[li], h = hi[li];
				bx[q] = Box{l.x, l.y, l.z, h.x, h.y, h.z};
			}
		}
		Box u = unite(bx[0], bx[1]);
		float4* p = reinterpret_cast<float4*>(&bin[node]);
		__stcg(p, make_float4(u.lox, u.loy, u.loz, __int_as_float(c[0])));
		__stcg(p + 1, make_float4(u.hix, u.hiy, u.hiz, __int_as_float(c[1])));
		node = parentInt[node];
	}
}

__global__ void kCollapse(const int2* __restrict__ qIn, const uint32_t* __restrict__ qInCount, CollapseInputs in,
                          CollapseOutputs out)
{
	uint32_t cnt = *qInCount;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
		int2 it = qIn[i];
		collapseItem(it.x, (uint32_t) it.y, in, out);
	}
}

inline int blocks(int n, int b) { return (n + b - 1) / b; }

template<class T>
T* mallocAsync(size_t count, cudaStream_t s)
{
	void* p = nullptr;
	RGL_CUDA_OK(cudaMallocAsync(&p, sizeof(T) * (count ? count : 1), s));
	return static_cast<T*>(p);
}

} // namespace

namespace {

struct WideBuildResult
{
	uint32_t nodeCount;
	Box bounds;
};

// Wide BVH over n primitive boxes lo/hi (device) whose centroid bounds are in cb (6 ordered uints),
// all written on stream s: the binary topology (binned SAH when `sah`, else Morton codes, onesweep
// sort, LBVH and bottom-up bounds), then the collapse into 8-wide nodes, one launch per depth. Leaf
// records are triangles (dV/dI given) or primitive indices (dV null). With levelStarts, it receives the
// first node index of every depth and the node count (the collapse allocates the nodes of depth L + 1
// while it writes depth L, so the counter before each launch starts the next depth). Frees lo, hi, cb
// and its temporaries and synchronises s (a one-off build).
WideBuildResult buildWide(float4* lo, float4* hi, uint32_t* cb, int n, const float* dV, const int32_t* dI, int leafMax,
                          WideNode* outNodes, TriRecord* outLeaves, Box* outBoxes, cudaStream_t s, bool sah,
                          std::vector<int32_t>* levelStarts = nullptr)
{
	uint32_t* codes = mallocAsync<uint32_t>(n, s);
	uint32_t* ids = mallocAsync<uint32_t>(n, s);
	void* sortScratch = mallocAsync<uint8_t>(sortPairsScratchBytes(n, 30), s);
	BinNode* bin = mallocAsync<BinNode>(n, s);
	int32_t* rf = mallocAsync<int32_t>(n, s);
	int32_t* rl = mallocAsync<int32_t>(n, s);
	int32_t* pi = mallocAsync<int32_t>(n, s);
	int32_t* pl = mallocAsync<int32_t>(n, s);
	uint32_t* visits = mallocAsync<uint32_t>(n, s);
	int2* q0 = mallocAsync<int2>(n, s);
	int2* q1 = mallocAsync<int2>(n, s);
	// counters: [0] wide, [1] leaf records, [2] q0 count, [3] q1 count, [4] error
	uint32_t* ctr = mallocAsync<uint32_t>(8, s);
	RGL_CUDA_OK(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * n, s));
	RGL_CUDA_OK(cudaMemsetAsync(ctr, 0, sizeof(uint32_t) * 8, s));
	int32_t* err = reinterpret_cast<int32_t*>(ctr + 4);

	if (sah) {
		buildSahTopologyDevice(lo, hi, n, bin, rf, rl, ids, s);
	} else {
		kMorton<<<blocks(n, 256), 256, 0, s>>>(lo, hi, n, cb, codes, ids);
		countLaunch();
		sortPairs(codes, ids, n, 30, sortScratch, err, s);
		if (n > 1) {
			kLbvh<<<blocks(n - 1, 256), 256, 0, s>>>(codes, n, bin, rf, rl, pi, pl);
			countLaunch();
			kBottomUp<<<blocks(n, 256), 256, 0, s>>>(n, ids, lo, hi, bin, pi, pl, visits);
			countLaunch();
		}
	}
	int2 root = make_int2(n == 1 ? ~0 : 0, 0);
	uint32_t one[2] = {1u, 0u};
	RGL_CUDA_OK(cudaMemcpyAsync(q0, &root, sizeof(int2), cudaMemcpyHostToDevice, s));
	RGL_CUDA_OK(cudaMemcpyAsync(ctr, one, sizeof(uint32_t), cudaMemcpyHostToDevice, s));     // wide counter = 1 (root)
	RGL_CUDA_OK(cudaMemcpyAsync(ctr + 2, one, sizeof(uint32_t), cudaMemcpyHostToDevice, s)); // q0 count = 1
	CollapseInputs ci{bin, rf, rl, reinterpret_cast<const int32_t*>(ids), lo, hi, dV, dI, leafMax};
	int2* qa = q0;
	int2* qb = q1;
	uint32_t* ca = ctr + 2;
	uint32_t* cbn = ctr + 3;
	// A wide level descends at least one binary level. The LBVH's binary depth is below 64 (30-bit keys
	// with index tie-break); an SAH tree may be deeper, so the queue is checked after every 16 levels
	// (empty launches exit immediately).
	const int grid = 152 * 4;
	uint32_t pending = 1;
	uint32_t* snap = levelStarts ? mallocAsync<uint32_t>(16, s) : nullptr; // node counter before each launch of a round
	uint32_t hostSnap[16];
	if (levelStarts) {
		levelStarts->assign(1, 0);
	}
	for (int round = 0; pending != 0; ++round) {
		for (int level = 0; level < 16; ++level) {
			if (snap) {
				RGL_CUDA_OK(cudaMemcpyAsync(snap + level, ctr, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
			}
			RGL_CUDA_OK(cudaMemsetAsync(cbn, 0, sizeof(uint32_t), s));
			CollapseOutputs co{outNodes, outLeaves, ctr, ctr + 1, qb, cbn, outBoxes};
			kCollapse<<<grid, 128, 0, s>>>(qa, ca, ci, co);
			countLaunch();
			int2* tq = qa;
			qa = qb;
			qb = tq;
			uint32_t* tc = ca;
			ca = cbn;
			cbn = tc;
		}
		RGL_CUDA_OK(cudaMemcpyAsync(&pending, ca, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
		if (snap) {
			RGL_CUDA_OK(cudaMemcpyAsync(hostSnap, snap, sizeof(hostSnap), cudaMemcpyDeviceToHost, s));
		}
		RGL_CUDA_OK(cudaStreamSynchronize(s));
		if (levelStarts) {
			levelStarts->insert(levelStarts->end(), hostSnap, hostSnap + 16);
		}
		if (round > (n >> 4) + 4) {
			throw std::runtime_error("BVH build: wide collapse does not terminate");
		}
	}
	uint32_t hostCtr[8];
	RGL_CUDA_OK(cudaMemcpyAsync(hostCtr, ctr, sizeof(hostCtr), cudaMemcpyDeviceToHost, s));
	BinNode rootBox{};
	float4 leafLo{}, leafHi{};
	if (n > 1) {
		RGL_CUDA_OK(cudaMemcpyAsync(&rootBox, bin, sizeof(BinNode), cudaMemcpyDeviceToHost, s));
	} else {
		RGL_CUDA_OK(cudaMemcpyAsync(&leafLo, lo, sizeof(float4), cudaMemcpyDeviceToHost, s));
		RGL_CUDA_OK(cudaMemcpyAsync(&leafHi, hi, sizeof(float4), cudaMemcpyDeviceToHost, s));
	}
	void* temps[] = {lo, hi, cb, codes, ids, sortScratch, bin, rf, rl, pi, pl, visits, q0, q1, ctr};
	for (void* p : temps) {
		RGL_CUDA_OK(cudaFreeAsync(p, s));
	}
	if (snap) {
		RGL_CUDA_OK(cudaFreeAsync(snap, s));
	}
	RGL_CUDA_OK(cudaStreamSynchronize(s));
	if (hostCtr[4] != 0) {
		throw std::runtime_error("BVH build: radix sort look-back did not complete");
	}
	if (hostCtr[1] != (uint32_t) n || hostCtr[0] > (uint32_t) n || hostCtr[ca - ctr] != 0) {
		throw std::runtime_error("BVH build: collapse produced an inconsistent tree (leaf records " + std::to_string(hostCtr[1]) +
		                         ", nodes " + std::to_string(hostCtr[0]) + ")");
	}
	WideBuildResult r;
	r.nodeCount = hostCtr[0];
	r.bounds = n > 1 ? Box{rootBox.lox, rootBox.loy, rootBox.loz, rootBox.hix, rootBox.hiy, rootBox.hiz}
	                 : Box{leafLo.x, leafLo.y, leafLo.z, leafHi.x, leafHi.y, leafHi.z};
	return r;
}

} // namespace

void buildBlas(const float* dVertices, int nVertices, const int32_t* dIndices, int nTris, BlasBuild& out, cudaStream_t s, bool sah)
{
	(void) nVertices;
	if (nTris <= 0) {
		throw std::invalid_argument("mesh without triangles");
	}
	const int T = nTris;
	float4* lo = mallocAsync<float4>(T, s);
	float4* hi = mallocAsync<float4>(T, s);
	uint32_t* cb = mallocAsync<uint32_t>(8, s);
	// A rebuild (an animated entity) reuses the previous storage when it is large enough.
	if (out.nodes == nullptr || out.nodeCapacity < (uint32_t) T) {
		if (out.nodes != nullptr) {
			freeBlas(out);
		}
		RGL_CUDA_OK(cudaMalloc(&out.nodes, sizeof(WideNode) * (size_t) T));
		RGL_CUDA_OK(cudaMalloc(&out.tris, sizeof(TriRecord) * (size_t) T));
		out.nodeCapacity = (uint32_t) T;
	}
	out.triCount = T;
	uint32_t cbInit[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
	RGL_CUDA_OK(cudaMemcpyAsync(cb, cbInit, sizeof(cbInit), cudaMemcpyHostToDevice, s));
	kTriBounds<<<blocks(T, 256), 256, 0, s>>>(dVertices, dIndices, T, lo, hi, cb);
	countLaunch();
	const WideBuildResult r = buildWide(lo, hi, cb, T, dVertices, dIndices, kLeafMaxTris, out.nodes, out.tris, nullptr, s, sah);
	out.nodeCount = r.nodeCount;
	out.bounds[0] = r.bounds.lox;
	out.bounds[1] = r.bounds.loy;
	out.bounds[2] = r.bounds.loz;
	out.bounds[3] = r.bounds.hix;
	out.bounds[4] = r.bounds.hiy;
	out.bounds[5] = r.bounds.hiz;
}

void buildBlasHost(const float* hVertices, int nVertices, const int32_t* hIndices, int nTris, BlasBuild& out)
{
	(void) nVertices;
	if (nTris <= 0) {
		throw std::invalid_argument("mesh without triangles");
	}
	const int T = nTris;
	std::vector<Box> boxes(T);
	std::vector<float4> lo(T), hi(T);
	for (int t = 0; t < T; ++t) {
		const float* a = hVertices + 3 * hIndices[3 * t];
		const float* b = hVertices + 3 * hIndices[3 * t + 1];
		const float* c = hVertices + 3 * hIndices[3 * t + 2];
		Box bx{std::min(a[0], std::min(b[0], c[0])), std::min(a[1], std::min(b[1], c[1])), std::min(a[2], std::min(b[2], c[2])),
		       std::max(a[0], std::max(b[0], c[0])), std::max(a[1], std::max(b[1], c[1])), std::max(a[2], std::max(b[2], c[2]))};
		boxes[t] = bx;
		lo[t] = make_float4(bx.lox, bx.loy, bx.loz, 0.0f);
		hi[t] = make_float4(bx.hix, bx.hiy, bx.hiz, 0.0f);
	}
	const SahTree tree = buildBinnedSahTree(boxes);
	std::vector<WideNode> wide(T);
	std::vector<TriRecord> tris(T);
	uint32_t wideCounter = 1, triCounter = 0;
	std::vector<int2> qa(T), qb(T);
	uint32_t qaCount = 1, qbCount = 0;
	qa[0] = make_int2(T == 1 ? ~0 : 0, 0);
	CollapseInputs in{tree.bin.data(), tree.rangeFirst.data(), tree.rangeLast.data(), tree.sortedIds.data(), lo.data(), hi.data(),
	                  hVertices, hIndices, kLeafMaxTris};
	while (qaCount > 0) {
		qbCount = 0;
		CollapseOutputs o{wide.data(), tris.data(), &wideCounter, &triCounter, qb.data(), &qbCount, nullptr};
		for (uint32_t i = 0; i < qaCount; ++i) {
			collapseItem(qa[i].x, (uint32_t) qa[i].y, in, o);
		}
		std::swap(qa, qb);
		qaCount = qbCount;
	}
	if (triCounter != (uint32_t) T || wideCounter > (uint32_t) T) {
		throw std::runtime_error("BLAS build: collapse produced an inconsistent tree");
	}
	if (out.nodes == nullptr || out.nodeCapacity < (uint32_t) T) {
		if (out.nodes != nullptr) {
			freeBlas(out);
		}
		RGL_CUDA_OK(cudaMalloc(&out.nodes, sizeof(WideNode) * (size_t) T));
		RGL_CUDA_OK(cudaMalloc(&out.tris, sizeof(TriRecord) * (size_t) T));
		out.nodeCapacity = (uint32_t) T;
	}
	RGL_CUDA_OK(cudaMemcpy(out.nodes, wide.data(), sizeof(WideNode) * wideCounter, cudaMemcpyHostToDevice));
	RGL_CUDA_OK(cudaMemcpy(out.tris, tris.data(), sizeof(TriRecord) * (size_t) T, cudaMemcpyHostToDevice));
	out.nodeCount = wideCounter;
	out.triCount = T;
	const Box root = T == 1 ? boxes[0] : Box{tree.bin[0].lox, tree.bin[0].loy, tree.bin[0].loz, tree.bin[0].hix, tree.bin[0].hiy, tree.bin[0].hiz};
	out.bounds[0] = root.lox;
	out.bounds[1] = root.loy;
	out.bounds[2] = root.loz;
	out.bounds[3] = root.hix;
	out.bounds[4] = root.hiy;
	out.bounds[5] = root.hiz;
}

void freeBlas(BlasBuild& b)
{
	cudaFree(b.nodes);
	cudaFree(b.tris);
	b.nodes = nullptr;
	b.tris = nullptr;
}

namespace {

// TLAS refit after pose changes, one block: depth by depth from the leaves up, every wide node takes
// the union of its children's boxes (child nodes' stored boxes, instances' world boxes) and
// re-quantises its children in a new frame with the builder's arithmetic. Topology and slots stay.
__global__ void __launch_bounds__(256) kRefitTlas(WideNode* nodes, const TriRecord* __restrict__ leaves, Box* boxes,
                                                  const InstanceRec* __restrict__ inst, const int32_t* __restrict__ levelStarts,
                                                  const int32_t* __restrict__ nLevelsWord)
{
	const int nLevels = *nLevelsWord;
	for (int L = nLevels - 1; L >= 0; --L) {
		const int a = levelStarts[L], b = levelStarts[L + 1];
		for (int i = a + (int) threadIdx.x; i < b; i += blockDim.x) {
			WideNode w = nodes[i];
			Box cbx[kWideArity];
			uint32_t present = 0;
			Box nb = emptyBox();
			for (int k = 0; k < kWideArity; ++k) {
				const bool internal = (w.imask >> k) & 1u;
				if (!internal && w.meta[k] == 0) {
					continue;
				}
				if (internal) {
					cbx[k] = boxes[w.childBase + (uint32_t) __popc(w.imask & ((1u << k) - 1u))];
				} else {
					const InstanceRec& r = inst[leaves[w.triBase + (w.meta[k] & 31u)].primId];
					cbx[k] = Box{r.lox, r.loy, r.loz, r.hix, r.hiy, r.hiz};
				}
				present |= 1u << k;
				nb = unite(nb, cbx[k]);
			}
			setWideFrame(w, nb);
			for (int k = 0; k < kWideArity; ++k) {
				if ((present >> k) & 1u) {
					quantizeChild(w, k, cbx[k]);
				} else {
					clearChild(w, k);
				}
			}
			nodes[i] = w;
			boxes[i] = nb;
		}
		__syncthreads();
	}
}

// World boxes of the instances (their records' padded boxes) as the builder's primitive boxes.
__global__ void kTlasBoxes(const InstanceRec* __restrict__ inst, int n, float4* lo, float4* hi)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) {
		const InstanceRec& r = inst[i];
		lo[i] = make_float4(r.lox, r.loy, r.loz, 0.0f);
		hi[i] = make_float4(r.hix, r.hiy, r.hiz, 0.0f);
	}
}

// Shared-memory layout of the one-block collapse over n primitives (16-byte aligned parts): primitive
// boxes lo[n] | hi[n] | binary nodes[n - 1] | two queues[n] | sorted ids[n] | ranges first[n - 1],
// last[n - 1] | counters[4].
struct SmallCollapseLayout
{
	size_t lo, hi, bin, q0, q1, ids, rf, rl, ctr, bytes;
};
__host__ __device__ SmallCollapseLayout smallCollapseLayout(int n)
{
	auto up = [](size_t b) { return (b + 15) & ~size_t{15}; };
	const size_t m = (size_t) (n > 1 ? n - 1 : 1);
	SmallCollapseLayout L;
	L.lo = 0;
	L.hi = L.lo + up(sizeof(float4) * (size_t) n);
	L.bin = L.hi + up(sizeof(float4) * (size_t) n);
	L.q0 = L.bin + up(sizeof(BinNode) * m);
	L.q1 = L.q0 + up(sizeof(int2) * (size_t) n);
	L.ids = L.q1 + up(sizeof(int2) * (size_t) n);
	L.rf = L.ids + up(sizeof(int32_t) * (size_t) n);
	L.rl = L.rf + up(sizeof(int32_t) * m);
	L.ctr = L.rl + up(sizeof(int32_t) * m);
	L.bytes = L.ctr + 16;
	return L;
}

// The wide collapse of a small binary tree by one block, depth by depth until its queue is empty. The
// tree, the primitive boxes, the queues and the counters live in shared memory, so each depth costs
// shared-memory latency, not a chain of global loads. Records the first node of every depth and the
// number of depths (the collapse allocates depth L + 1 while it writes depth L).
__global__ void __launch_bounds__(256) kCollapseSmall(CollapseInputs gin, WideNode* wide, TriRecord* leaves, Box* boxes,
                                                      int32_t* levelStarts, int32_t* nLevels, int n)
{
	extern __shared__ __align__(16) uint8_t smem[];
	const SmallCollapseLayout L = smallCollapseLayout(n);
	float4* lo = reinterpret_cast<float4*>(smem + L.lo);
	float4* hi = reinterpret_cast<float4*>(smem + L.hi);
	BinNode* bin = reinterpret_cast<BinNode*>(smem + L.bin);
	int2* qa = reinterpret_cast<int2*>(smem + L.q0);
	int2* qb = reinterpret_cast<int2*>(smem + L.q1);
	int32_t* ids = reinterpret_cast<int32_t*>(smem + L.ids);
	int32_t* rf = reinterpret_cast<int32_t*>(smem + L.rf);
	int32_t* rl = reinterpret_cast<int32_t*>(smem + L.rl);
	uint32_t* counters = reinterpret_cast<uint32_t*>(smem + L.ctr);
	for (int i = threadIdx.x; i < n; i += blockDim.x) {
		lo[i] = gin.triLo[i];
		hi[i] = gin.triHi[i];
		ids[i] = gin.sortedIds[i];
	}
	for (int i = threadIdx.x; i < n - 1; i += blockDim.x) {
		bin[i] = gin.bin[i];
		rf[i] = gin.rangeFirst[i];
		rl[i] = gin.rangeLast[i];
	}
	if (threadIdx.x == 0) {
		counters[0] = 1u; // wide nodes (the root)
		counters[1] = 0u; // leaf records
		counters[2] = 1u; // items in qa
		counters[3] = 0u;
		qa[0] = make_int2(n == 1 ? ~0 : 0, 0);
		levelStarts[0] = 0;
	}
	const CollapseInputs in{bin, rf, rl, ids, lo, hi, nullptr, nullptr, gin.leafMax};
	uint32_t* ca = counters + 2;
	uint32_t* cb = counters + 3;
	int level = 0;
	for (;; ++level) {
		__syncthreads();
		const uint32_t cnt = *(volatile uint32_t*) ca;
		__syncthreads();
		if (threadIdx.x == 0) {
			levelStarts[level + 1] = (int32_t) *(volatile uint32_t*) counters;
			*cb = 0u;
		}
		__syncthreads();
		if (cnt == 0u || level > n + 1) {
			break;
		}
		const CollapseOutputs out{wide, leaves, counters, counters + 1, qb, cb, boxes};
		for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
			const int2 it = qa[i];
			collapseItem(it.x, (uint32_t) it.y, in, out);
		}
		int2* tq = qa;
		qa = qb;
		qb = tq;
		uint32_t* tc = ca;
		ca = cb;
		cb = tc;
	}
	if (threadIdx.x == 0) {
		*nLevels = level;
	}
}

} // namespace

// The TLAS is a wide BVH over the instances' world boxes, one instance per leaf child, built on the
// device like a mesh BLAS (binned SAH topology, then the wide collapse with one instance per leaf).
// The node range of every depth (contiguous: the collapse allocates nodes depth by depth) drives the
// refit kernel.
namespace {

void allocTlas(TlasBuild& t, int n)
{
	if (n <= t.capacity) {
		return;
	}
	freeTlas(t);
	t.capacity = n;
	RGL_CUDA_OK(cudaMalloc(&t.nodes, sizeof(WideNode) * (size_t) n));
	RGL_CUDA_OK(cudaMalloc(&t.leaves, sizeof(TriRecord) * (size_t) n));
	RGL_CUDA_OK(cudaMalloc(&t.boxes, sizeof(Box) * (size_t) n));
	t.levelCapacity = n + 2;
	RGL_CUDA_OK(cudaMalloc(&t.levelStarts, sizeof(int32_t) * (size_t) t.levelCapacity));
	RGL_CUDA_OK(cudaMalloc(&t.nLevels, sizeof(int32_t)));
	if (n <= kSahSmallMax) {
		RGL_CUDA_OK(cudaMalloc(&t.lo, sizeof(float4) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.hi, sizeof(float4) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.sahScratch, sahSmallScratchBytes(n)));
		RGL_CUDA_OK(cudaMalloc(&t.bin, sizeof(BinNode) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.rangeFirst, sizeof(int32_t) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.rangeLast, sizeof(int32_t) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.sortedIds, sizeof(uint32_t) * (size_t) n));
		// Shared memory of the one-block collapse for up to n instances (set outside any capture).
		RGL_CUDA_OK(cudaFuncSetAttribute(kCollapseSmall, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smallCollapseLayout(n).bytes));
	}
}

// The rebuild of up to kSahSmallMax instances from their device records: four launches, no host
// interaction, so a captured frame can hold it.
void rebuildTlas(const InstanceRec* dInst, TlasBuild& t, cudaStream_t s)
{
	const int n = t.nInstances;
	kTlasBoxes<<<blocks(n, 128), 128, 0, s>>>(dInst, n, t.lo, t.hi);
	countLaunch();
	enqueueSahTopologySmall(t.lo, t.hi, n, t.sahScratch, t.bin, t.rangeFirst, t.rangeLast, t.sortedIds, s);
	const CollapseInputs ci{t.bin, t.rangeFirst, t.rangeLast, reinterpret_cast<const int32_t*>(t.sortedIds), t.lo, t.hi, nullptr, nullptr, 1};
	kCollapseSmall<<<1, 256, smallCollapseLayout(n).bytes, s>>>(ci, t.nodes, t.leaves, reinterpret_cast<Box*>(t.boxes), t.levelStarts,
	                                                            t.nLevels, n);
	countLaunch();
}

} // namespace

void buildTlas(const InstanceRec* hInst, const InstanceRec* dInst, int n, TlasBuild& t, cudaStream_t s)
{
	if (n > 0) {
		allocTlas(t, n);
	}
	t.nInstances = n;
	t.nodeCount = 0;
	if (n <= 0) {
		return;
	}
	if (n <= kSahSmallMax) {
		rebuildTlas(dInst, t, s);
		return;
	}
	std::vector<float4> hLo(n), hHi(n);
	for (int i = 0; i < n; ++i) {
		const InstanceRec& r = hInst[i];
		hLo[i] = make_float4(r.lox, r.loy, r.loz, 0.0f);
		hHi[i] = make_float4(r.hix, r.hiy, r.hiz, 0.0f);
	}
	float4* lo = mallocAsync<float4>(n, s);
	float4* hi = mallocAsync<float4>(n, s);
	uint32_t* cb = mallocAsync<uint32_t>(8, s); // centroid bounds: read by the Morton path only
	// Pageable sources: each copy is staged before the call returns.
	RGL_CUDA_OK(cudaMemcpyAsync(lo, hLo.data(), sizeof(float4) * (size_t) n, cudaMemcpyHostToDevice, s));
	RGL_CUDA_OK(cudaMemcpyAsync(hi, hHi.data(), sizeof(float4) * (size_t) n, cudaMemcpyHostToDevice, s));
	std::vector<int32_t> starts;
	const WideBuildResult r = buildWide(lo, hi, cb, n, nullptr, nullptr, 1, t.nodes, t.leaves, reinterpret_cast<Box*>(t.boxes), s,
	                                    true, &starts);
	t.nodeCount = r.nodeCount;
	// Depths past the deepest node hold no nodes (their starts equal the node count): dropped.
	int levels = (int) starts.size() - 1;
	while (levels > 1 && starts[(size_t) levels - 1] == (int32_t) r.nodeCount) {
		--levels;
	}
	if (starts.back() != (int32_t) r.nodeCount || starts[(size_t) levels] != (int32_t) r.nodeCount || levels + 1 > t.levelCapacity) {
		throw std::runtime_error("TLAS build: depth ranges do not cover the nodes");
	}
	RGL_CUDA_OK(cudaMemcpyAsync(t.levelStarts, starts.data(), sizeof(int32_t) * (size_t) (levels + 1), cudaMemcpyHostToDevice, s));
	RGL_CUDA_OK(cudaMemcpyAsync(t.nLevels, &levels, sizeof(int32_t), cudaMemcpyHostToDevice, s));
	RGL_CUDA_OK(cudaStreamSynchronize(s));
}

void updateTlas(const InstanceRec* dInst, TlasBuild& t, cudaStream_t s)
{
	if (t.nInstances <= 0) {
		return;
	}
	if (t.nInstances <= kSahSmallMax) {
		rebuildTlas(dInst, t, s);
	} else {
		refitTlas(dInst, t, s);
	}
}

void refitTlas(const InstanceRec* dInst, TlasBuild& t, cudaStream_t s)
{
	if (t.nInstances <= 0) {
		return;
	}
	kRefitTlas<<<1, 256, 0, s>>>(t.nodes, t.leaves, reinterpret_cast<Box*>(t.boxes), dInst, t.levelStarts, t.nLevels);
	countLaunch();
}

void freeTlas(TlasBuild& t)
{
	void* ptrs[] = {t.nodes, t.leaves, t.boxes, t.levelStarts, t.nLevels, t.lo, t.hi, t.sahScratch, t.bin, t.rangeFirst,
	                t.rangeLast, t.sortedIds};
	for (void* p : ptrs) {
		cudaFree(p);
	}
	t = TlasBuild{};
}

} // namespace rgl
