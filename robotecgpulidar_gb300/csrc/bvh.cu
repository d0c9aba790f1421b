// On-device BVH construction: per-mesh BLAS (8-wide, quantised) and per-scene TLAS (binary) with a
// refit path for pose updates. The per-item logic lives in bvh_core.hpp.
//
// Replaces the OptiX acceleration-structure builds of reference src/scene/GASBuilder.hpp:31-100 and
// src/scene/Scene.cpp:131-190 (where any pose change triggers a full IAS rebuild plus a stream sync).
#include <cuda_runtime.h>
#include <stdexcept>
#include <string>

#include "bvh_core.hpp"
#include "kernels.hpp"

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
                      int32_t* parentInt, int32_t* parentLeaf, const uint32_t* __restrict__ remapIds)
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
	if (remapIds) { // TLAS: leaves reference instance indices
		if (l < 0) {
			l = ~(int32_t) remapIds[~l];
		}
		if (r < 0) {
			r = ~(int32_t) remapIds[~r];
		}
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
// Leaf boxes: lo/hi[ids[k]] for sorted position k; a leaf child ~c indexes lo/hi directly when
// `leafChildIsId` (TLAS, remapped) or through ids[] otherwise (BLAS).
__global__ void kBottomUp(int n, const uint32_t* __restrict__ ids, const float4* __restrict__ lo, const float4* __restrict__ hi,
                          BinNode* bin, const int32_t* __restrict__ parentInt, const int32_t* __restrict__ parentLeaf,
                          uint32_t* visits, int leafChildIsId)
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
				int li = leafChildIsId ? ~c[q] : (int) ids[~c[q]];
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

__global__ void kInstBoxes(const InstanceRec* __restrict__ inst, int n, float4* lo, float4* hi)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) {
		const InstanceRec& r = inst[i];
		lo[i] = make_float4(r.lox, r.loy, r.loz, 0.f);
		hi[i] = make_float4(r.hix, r.hiy, r.hiz, 0.f);
	}
}

__global__ void kCentroidBounds(const float4* __restrict__ lo, const float4* __restrict__ hi, int n, uint32_t* cbounds)
{
	int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t < n) {
		float4 l = lo[t], h = hi[t];
		float c[3] = {0.5f * (l.x + h.x), 0.5f * (l.y + h.y), 0.5f * (l.z + h.z)};
		for (int a = 0; a < 3; ++a) {
			atomicMin(&cbounds[a], orderedBits(c[a]));
			atomicMax(&cbounds[3 + a], orderedBits(c[a]));
		}
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

void buildBlas(const float* dVertices, int nVertices, const int32_t* dIndices, int nTris, BlasBuild& out, cudaStream_t s)
{
	(void) nVertices;
	if (nTris <= 0) {
		throw std::invalid_argument("mesh without triangles");
	}
	const int T = nTris;
	float4* lo = mallocAsync<float4>(T, s);
	float4* hi = mallocAsync<float4>(T, s);
	uint32_t* cb = mallocAsync<uint32_t>(8, s);
	uint32_t* codes = mallocAsync<uint32_t>(T, s);
	uint32_t* ids = mallocAsync<uint32_t>(T, s);
	void* sortScratch = mallocAsync<uint8_t>(sortPairsScratchBytes(T, 30), s);
	BinNode* bin = mallocAsync<BinNode>(T, s);
	int32_t* rf = mallocAsync<int32_t>(T, s);
	int32_t* rl = mallocAsync<int32_t>(T, s);
	int32_t* pi = mallocAsync<int32_t>(T, s);
	int32_t* pl = mallocAsync<int32_t>(T, s);
	uint32_t* visits = mallocAsync<uint32_t>(T, s);
	int2* q0 = mallocAsync<int2>(T, s);
	int2* q1 = mallocAsync<int2>(T, s);
	// counters: [0] wide, [1] tri, [2] q0 count, [3] q1 count, [4] error
	uint32_t* ctr = mallocAsync<uint32_t>(8, s);

	out.nodeCapacity = (uint32_t) T;
	out.triCount = T;
	RGL_CUDA_OK(cudaMalloc(&out.nodes, sizeof(WideNode) * (size_t) T));
	RGL_CUDA_OK(cudaMalloc(&out.tris, sizeof(TriRecord) * (size_t) T));

	uint32_t cbInit[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
	RGL_CUDA_OK(cudaMemcpyAsync(cb, cbInit, sizeof(cbInit), cudaMemcpyHostToDevice, s));
	RGL_CUDA_OK(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * T, s));
	RGL_CUDA_OK(cudaMemsetAsync(ctr, 0, sizeof(uint32_t) * 8, s));
	int32_t* err = reinterpret_cast<int32_t*>(ctr + 4);

	kTriBounds<<<blocks(T, 256), 256, 0, s>>>(dVertices, dIndices, T, lo, hi, cb);
	countLaunch();
	kMorton<<<blocks(T, 256), 256, 0, s>>>(lo, hi, T, cb, codes, ids);
	countLaunch();
	sortPairs(codes, ids, T, 30, sortScratch, err, s);
	if (T > 1) {
		kLbvh<<<blocks(T - 1, 256), 256, 0, s>>>(codes, T, bin, rf, rl, pi, pl, nullptr);
		countLaunch();
		kBottomUp<<<blocks(T, 256), 256, 0, s>>>(T, ids, lo, hi, bin, pi, pl, visits, 0);
		countLaunch();
	}
	int2 root = make_int2(T == 1 ? ~0 : 0, 0);
	uint32_t one[2] = {1u, 0u};
	RGL_CUDA_OK(cudaMemcpyAsync(q0, &root, sizeof(int2), cudaMemcpyHostToDevice, s));
	RGL_CUDA_OK(cudaMemcpyAsync(ctr, one, sizeof(uint32_t), cudaMemcpyHostToDevice, s));     // wide counter = 1 (root)
	RGL_CUDA_OK(cudaMemcpyAsync(ctr + 2, one, sizeof(uint32_t), cudaMemcpyHostToDevice, s)); // q0 count = 1
	CollapseInputs ci{bin, rf, rl, reinterpret_cast<const int32_t*>(ids), lo, hi, dVertices, dIndices};
	int2* qa = q0;
	int2* qb = q1;
	uint32_t* ca = ctr + 2;
	uint32_t* cbn = ctr + 3;
	// A wide level descends at least one binary level; binary depth is below 64 for 30-bit keys with
	// index tie-break, so 64 launches always drain the queue (empty launches exit immediately).
	const int grid = 152 * 4;
	for (int level = 0; level < 64; ++level) {
		RGL_CUDA_OK(cudaMemsetAsync(cbn, 0, sizeof(uint32_t), s));
		CollapseOutputs co{out.nodes, out.tris, ctr, ctr + 1, qb, cbn};
		kCollapse<<<grid, 128, 0, s>>>(qa, ca, ci, co);
		countLaunch();
		int2* tq = qa;
		qa = qb;
		qb = tq;
		uint32_t* tc = ca;
		ca = cbn;
		cbn = tc;
	}
	uint32_t hostCtr[8];
	RGL_CUDA_OK(cudaMemcpyAsync(hostCtr, ctr, sizeof(hostCtr), cudaMemcpyDeviceToHost, s));
	BinNode rootBox{};
	float4 leafLo{}, leafHi{};
	if (T > 1) {
		RGL_CUDA_OK(cudaMemcpyAsync(&rootBox, bin, sizeof(BinNode), cudaMemcpyDeviceToHost, s));
	} else {
		RGL_CUDA_OK(cudaMemcpyAsync(&leafLo, lo, sizeof(float4), cudaMemcpyDeviceToHost, s));
		RGL_CUDA_OK(cudaMemcpyAsync(&leafHi, hi, sizeof(float4), cudaMemcpyDeviceToHost, s));
	}
	void* temps[] = {lo, hi, cb, codes, ids, sortScratch, bin, rf, rl, pi, pl, visits, q0, q1, ctr};
	for (void* p : temps) {
		RGL_CUDA_OK(cudaFreeAsync(p, s));
	}
	RGL_CUDA_OK(cudaStreamSynchronize(s));
	if (hostCtr[4] != 0) {
		throw std::runtime_error("BVH build: radix sort look-back did not complete");
	}
	if (hostCtr[1] != (uint32_t) T || hostCtr[0] > (uint32_t) T || hostCtr[ca - ctr] != 0) {
		throw std::runtime_error("BVH build: collapse produced an inconsistent tree (tris " + std::to_string(hostCtr[1]) +
		                         ", nodes " + std::to_string(hostCtr[0]) + ")");
	}
	out.nodeCount = hostCtr[0];
	if (T > 1) {
		out.bounds[0] = rootBox.lox;
		out.bounds[1] = rootBox.loy;
		out.bounds[2] = rootBox.loz;
		out.bounds[3] = rootBox.hix;
		out.bounds[4] = rootBox.hiy;
		out.bounds[5] = rootBox.hiz;
	} else {
		out.bounds[0] = leafLo.x;
		out.bounds[1] = leafLo.y;
		out.bounds[2] = leafLo.z;
		out.bounds[3] = leafHi.x;
		out.bounds[4] = leafHi.y;
		out.bounds[5] = leafHi.z;
	}
}

void freeBlas(BlasBuild& b)
{
	cudaFree(b.nodes);
	cudaFree(b.tris);
	b.nodes = nullptr;
	b.tris = nullptr;
}

namespace {
struct TlasTemps
{
	float4* lo;
	float4* hi;
	uint32_t* codes;
	uint32_t* ids;
	uint32_t* cbounds;
};
TlasTemps tlasTemps(TlasBuild& t)
{
	uint8_t* p = static_cast<uint8_t*>(t.scratch);
	int n = t.capacity;
	TlasTemps r;
	r.lo = reinterpret_cast<float4*>(p);
	r.hi = r.lo + n;
	r.codes = reinterpret_cast<uint32_t*>(r.hi + n);
	r.ids = r.codes + n;
	r.cbounds = r.ids + n;
	return r;
}
} // namespace

void buildTlas(const InstanceRec* dInst, int n, TlasBuild& t, int32_t* dError, cudaStream_t s)
{
	t.nInstances = n;
	if (n <= 1) {
		return;
	}
	if (n > t.capacity) {
		freeTlas(t);
		t.capacity = n;
		size_t sortBytes = sortPairsScratchBytes(n, 30);
		t.scratchBytes = sizeof(float4) * 2 * (size_t) n + sizeof(uint32_t) * (2 * (size_t) n + 8) + sortBytes;
		RGL_CUDA_OK(cudaMalloc(&t.nodes, sizeof(BinNode) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.parents, sizeof(int32_t) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.leafParents, sizeof(int32_t) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.visits, sizeof(uint32_t) * (size_t) n));
		RGL_CUDA_OK(cudaMalloc(&t.scratch, t.scratchBytes));
		t.nInstances = n;
	}
	TlasTemps tt = tlasTemps(t);
	void* sortScratch = reinterpret_cast<uint8_t*>(tt.cbounds + 8);
	kInstBoxes<<<blocks(n, 128), 128, 0, s>>>(dInst, n, tt.lo, tt.hi);
	countLaunch();
	uint32_t cbInit[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
	RGL_CUDA_OK(cudaMemcpyAsync(tt.cbounds, cbInit, sizeof(cbInit), cudaMemcpyHostToDevice, s));
	kCentroidBounds<<<blocks(n, 128), 128, 0, s>>>(tt.lo, tt.hi, n, tt.cbounds);
	countLaunch();
	kMorton<<<blocks(n, 128), 128, 0, s>>>(tt.lo, tt.hi, n, tt.cbounds, tt.codes, tt.ids);
	countLaunch();
	sortPairs(tt.codes, tt.ids, n, 30, sortScratch, dError, s);
	kLbvh<<<blocks(n - 1, 128), 128, 0, s>>>(tt.codes, n, t.nodes, nullptr, nullptr, t.parents, t.leafParents, tt.ids);
	countLaunch();
	refitTlas(dInst, t, s);
}

void refitTlas(const InstanceRec* dInst, TlasBuild& t, cudaStream_t s)
{
	int n = t.nInstances;
	if (n <= 1) {
		return;
	}
	TlasTemps tt = tlasTemps(t);
	kInstBoxes<<<blocks(n, 128), 128, 0, s>>>(dInst, n, tt.lo, tt.hi);
	countLaunch();
	RGL_CUDA_OK(cudaMemsetAsync(t.visits, 0, sizeof(uint32_t) * (size_t) (n - 1), s));
	kBottomUp<<<blocks(n, 128), 128, 0, s>>>(n, tt.ids, tt.lo, tt.hi, t.nodes, t.parents, t.leafParents, t.visits, 1);
	countLaunch();
}

void freeTlas(TlasBuild& t)
{
	cudaFree(t.nodes);
	cudaFree(t.parents);
	cudaFree(t.leafParents);
	cudaFree(t.visits);
	cudaFree(t.scratch);
	t = TlasBuild{};
}

} // namespace rgl
