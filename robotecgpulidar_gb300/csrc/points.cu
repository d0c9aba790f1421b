// Point-pipeline kernels: ray/point transforms, Gaussian noise, compaction and formatting.
//
// Reference counterparts: kTransformRays / kTransformPoints (src/gpu/nodeKernels.cu:45-56),
// kAddGaussianNoise* (src/gpu/gaussianNoiseKernels.cu:20-66), gpuFindCompaction + kApplyCompaction
// (nodeKernels.cu:58-68,424-436: a Thrust scan, a blocking count read-back and one scatter launch per
// field), kFormatSoaToAos / kFormatAosToSoa (nodeKernels.cu:25-43: byte-wise memcpy per field).
// Here compaction is one decoupled-look-back pass over all fields with the count left on the device,
// and formatting writes the packed output word by word (coalesced 4-byte stores).
#include <cuda_runtime.h>

#include <algorithm>

#include "common.hpp"
#include "kernels.hpp"
#include "philox.hpp"

namespace rgl {

namespace {
// One warp per parameter block: 4-byte words, then any tail bytes (pinned and device allocations
// are at least 256-byte aligned).
__global__ void kGatherParams(const ParamCopy* __restrict__ table, int n)
{
	const int warp = (int) ((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = (int) (threadIdx.x & 31);
	if (warp >= n) {
		return;
	}
	const ParamCopy c = table[warp];
	const uint32_t words = c.bytes >> 2;
	const uint32_t* src = static_cast<const uint32_t*>(c.src);
	uint32_t* dst = static_cast<uint32_t*>(c.dst);
	for (uint32_t i = lane; i < words; i += 32) {
		dst[i] = src[i];
	}
	for (uint32_t i = (words << 2) + lane; i < c.bytes; i += 32) {
		static_cast<uint8_t*>(c.dst)[i] = static_cast<const uint8_t*>(c.src)[i];
	}
}
} // namespace

cudaError_t addParamGatherNode(cudaGraph_t graph, const ParamCopy* dTable, int n)
{
	if (n <= 0) {
		return cudaSuccess;
	}
	size_t nRoots = 0;
	cudaError_t e = cudaGraphGetRootNodes(graph, nullptr, &nRoots);
	std::vector<cudaGraphNode_t> roots(nRoots);
	if (e == cudaSuccess && nRoots > 0) {
		e = cudaGraphGetRootNodes(graph, roots.data(), &nRoots);
	}
	if (e != cudaSuccess) {
		return e;
	}
	constexpr int kBlock = 128;
	void* args[] = {(void*) &dTable, (void*) &n};
	cudaKernelNodeParams p = {};
	p.func = reinterpret_cast<void*>(&kGatherParams);
	p.gridDim = dim3((unsigned) ((n * 32 + kBlock - 1) / kBlock));
	p.blockDim = dim3(kBlock);
	p.sharedMemBytes = 0;
	p.kernelParams = args;
	cudaGraphNode_t gather = nullptr;
	e = cudaGraphAddKernelNode(&gather, graph, nullptr, 0, &p);
	for (size_t i = 0; i < nRoots && e == cudaSuccess; ++i) {
		e = cudaGraphAddDependencies(graph, &gather, &roots[i], nullptr, 1);
	}
	if (e == cudaSuccess) {
		countLaunch();
	}
	return e;
}

namespace {

constexpr int kBlock = 256;

inline int blocks(long n, int b) { return (int) ((n + b - 1) / b); }

__device__ __forceinline__ int countOf(int cap, const int32_t* dCount) { return dCount ? *dCount : cap; }

__device__ __forceinline__ Vec3 loadXyz(const float* p, int i) { return v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void storeXyz(float* p, int i, Vec3 v)
{
	p[3 * i] = v.x;
	p[3 * i + 1] = v.y;
	p[3 * i + 2] = v.z;
}

__device__ __forceinline__ Mat34 loadMat(const Mat34* p)
{
	const float4* q = reinterpret_cast<const float4*>(p);
	float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
	return Mat34{{{a.x, a.y, a.z, a.w}, {b.x, b.y, b.z, b.w}, {c.x, c.y, c.z, c.w}}};
}
__device__ __forceinline__ void storeMat(Mat34* p, const Mat34& m)
{
	float4* q = reinterpret_cast<float4*>(p);
	q[0] = make_float4(m.m[0][0], m.m[0][1], m.m[0][2], m.m[0][3]);
	q[1] = make_float4(m.m[1][0], m.m[1][1], m.m[1][2], m.m[1][3]);
	q[2] = make_float4(m.m[2][0], m.m[2][1], m.m[2][2], m.m[2][3]);
}

// Transforms and noise parameters are read from device memory: the host stages them before every
// run and the (possibly captured and replayed) run copies them in, so new poses, seeds and frames
// need no new launch.
__global__ void kTransformRays(const Mat34* __restrict__ in, Mat34* __restrict__ out, int n, const Mat34* __restrict__ dTf)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) {
		storeMat(out + i, mul(loadMat(dTf), loadMat(in + i)));
	}
}

__global__ void kTransformPoints(const float* __restrict__ in, float* __restrict__ out, int cap, const int32_t* dCount,
                                 const Mat34* __restrict__ dTf)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < countOf(cap, dCount)) {
		storeXyz(out, i, loadMat(dTf).point(loadXyz(in, i)));
	}
}

// Block-wide copy of the staged noise parameters.
__device__ __forceinline__ void loadNoise(NoiseParams& sp, const NoiseParams* __restrict__ dNp)
{
	constexpr int words = sizeof(NoiseParams) / 4;
	static_assert(sizeof(NoiseParams) % 4 == 0, "NoiseParams must be a whole number of words");
	for (int w = threadIdx.x; w < words; w += blockDim.x) {
		reinterpret_cast<uint32_t*>(&sp)[w] = __ldg(reinterpret_cast<const uint32_t*>(dNp) + w);
	}
	__syncthreads();
}

__device__ __forceinline__ float noiseNormal(const NoiseParams& np, int i)
{
	return standardNormal(np.seedLo, np.seedHi, np.kind, (uint32_t) i, np.frameLo, np.frameHi);
}

__device__ __forceinline__ Mat34 axisRotation(int axis, float angle)
{
	float s, c;
	sincosf(angle, &s, &c);
	return rotationAxis(axis, c, s);
}

__global__ void kNoiseAngularRay(const Mat34* __restrict__ in, Mat34* __restrict__ out, int n, const NoiseParams* __restrict__ dNp)
{
	__shared__ NoiseParams np;
	loadNoise(np, dNp);
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) {
		float angle = np.mean + noiseNormal(np, i) * np.stDev;
		Mat34 r = mul(np.lookAtInv, mul(axisRotation(np.axis, angle), mul(np.lookAt, loadMat(in + i))));
		storeMat(out + i, r);
	}
}

// Per-point arithmetic of the point noise nodes, shared by their kernels and by the compaction that
// absorbs them (the same expressions, so both paths give the same bits).
__device__ __forceinline__ Vec3 angularHitpoint(const NoiseParams& np, int i, Vec3 p, float* distOut)
{
	float angle = np.mean + noiseNormal(np, i) * np.stDev;
	Vec3 q = axisRotation(np.axis, angle).point(np.lookAt.point(p));
	if (distOut) {
		*distOut = length(q);
	}
	return np.lookAtInv.point(q);
}

__device__ __forceinline__ Vec3 distanceNoise(const NoiseParams& np, int i, Vec3 p, float& d)
{
	float sigma = d * np.stDevRise + np.stDev; // stDev holds the base deviation for distance noise
	float e = np.mean + noiseNormal(np, i) * sigma;
	Vec3 pl = np.lookAt.point(p);
	Vec3 moved = pl + normalized(pl) * e;
	d = d + e;
	return np.lookAtInv.point(moved);
}

__global__ void kNoiseAngularHitpoint(const float* __restrict__ inXyz, float* __restrict__ outXyz, float* __restrict__ outDist,
                                      int cap, const int32_t* dCount, const NoiseParams* __restrict__ dNp)
{
	__shared__ NoiseParams np;
	loadNoise(np, dNp);
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < countOf(cap, dCount)) {
		storeXyz(outXyz, i, angularHitpoint(np, i, loadXyz(inXyz, i), outDist ? outDist + i : nullptr));
	}
}

__global__ void kNoiseDistance(const float* __restrict__ inXyz, const float* __restrict__ inDist, float* __restrict__ outXyz,
                               float* __restrict__ outDist, int cap, const int32_t* dCount, const NoiseParams* __restrict__ dNp)
{
	__shared__ NoiseParams np;
	loadNoise(np, dNp);
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < countOf(cap, dCount)) {
		float d = inDist[i];
		storeXyz(outXyz, i, distanceNoise(np, i, loadXyz(inXyz, i), d));
		outDist[i] = d;
	}
}

// ---------------------------------------------------------------- compaction

constexpr int kCompactItems = 4;
constexpr int kCompactTile = kBlock * kCompactItems;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr int kSpinLimit = 1 << 24;

__device__ __forceinline__ void copyElem(const uint8_t* src, uint8_t* dst, int size)
{
	switch (size) {
		case 4: *reinterpret_cast<uint32_t*>(dst) = *reinterpret_cast<const uint32_t*>(src); break;
		case 12: {
			const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
			uint32_t* d = reinterpret_cast<uint32_t*>(dst);
			d[0] = s[0];
			d[1] = s[1];
			d[2] = s[2];
			break;
		}
		case 1: *dst = *src; break;
		case 2: *reinterpret_cast<uint16_t*>(dst) = *reinterpret_cast<const uint16_t*>(src); break;
		case 8: *reinterpret_cast<uint2*>(dst) = *reinterpret_cast<const uint2*>(src); break;
		default:
			for (int b = 0; b < size; ++b) {
				dst[b] = src[b];
			}
	}
}

// One pass: per-tile flag counts, decoupled look-back for the tile offset, scatter of every field.
// scratch: [0] tile ticket, [1..tiles] tile status words, [tiles + 1] finished tiles; zero before the
// first launch, and the last tile to finish zeroes it again for the next one.
// Parameters of the absorbed point operations, copied into shared memory once per block.
constexpr int kOpParamWords = (int) (sizeof(NoiseParams) / 4);
static_assert(sizeof(NoiseParams) % 16 == 0 && sizeof(Mat34) <= sizeof(NoiseParams), "point-op parameter slot");

__global__ void __launch_bounds__(kBlock) kCompact(const int32_t* __restrict__ flags, int cap, const int32_t* dInCount,
                                                   const __grid_constant__ FieldCopies fc, const __grid_constant__ PointOps ops,
                                                   int32_t* dOutCount, uint32_t* scratch,
                                                   int32_t* errorFlag, int32_t* hostCount)
{
	__shared__ uint32_t warpSums[kBlock / 32];
	__shared__ uint32_t tileBase, tileKept;
	__shared__ int tileShared;
	__shared__ uint16_t keptLocal[kCompactTile]; // tile-local indices of the kept points, in order
	__shared__ __align__(16) uint32_t opParams[kMaxPointOps][kOpParamWords];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	__shared__ uint32_t lbBallot[kBlock / 32], lbSum[kBlock / 32];
	__shared__ int lbFail;
	if (tid == 0) {
		tileShared = (int) atomicAdd(scratch, 1u);
		lbFail = 0;
	}
	for (int k = 0; k < ops.count; ++k) {
		const int words = ops.op[k].kind == kOpTransform ? (int) (sizeof(Mat34) / 4) : kOpParamWords;
		for (int w = tid; w < words; w += kBlock) {
			opParams[k][w] = __ldg(static_cast<const uint32_t*>(ops.op[k].params) + w);
		}
	}
	__syncthreads();
	const int tile = tileShared;
	const int n = dInCount ? *dInCount : cap;
	const int first = tile * kCompactTile + tid * kCompactItems;
	int keep[kCompactItems];
	int cnt = 0;
	if (first + kCompactItems <= n && (reinterpret_cast<uintptr_t>(flags + first) & 15u) == 0) {
		// one 16-byte load of the thread's four flags
		const int4 f4 = __ldg(reinterpret_cast<const int4*>(flags + first));
		keep[0] = f4.x != 0;
		keep[1] = f4.y != 0;
		keep[2] = f4.z != 0;
		keep[3] = f4.w != 0;
		cnt = keep[0] + keep[1] + keep[2] + keep[3];
	} else {
#pragma unroll
		for (int k = 0; k < kCompactItems; ++k) {
			int i = first + k;
			keep[k] = (i < n) && flags[i] != 0;
			cnt += keep[k];
		}
	}
	// block exclusive scan of cnt
	int incl = cnt;
#pragma unroll
	for (int off = 1; off < 32; off <<= 1) {
		int v = __shfl_up_sync(0xffffffffu, incl, off);
		if (lane >= off) {
			incl += v;
		}
	}
	if (lane == 31) {
		warpSums[warp] = (uint32_t) incl;
	}
	__syncthreads();
	if (tid == 0) {
		// Per-warp offsets and the tile total, then the tile's status word: its aggregate (tile 0: its
		// inclusive prefix), published before the look-back so successors never wait on a look-back.
		uint32_t run = 0;
		for (int w = 0; w < kBlock / 32; ++w) {
			const uint32_t v = warpSums[w];
			warpSums[w] = run;
			run += v;
		}
		atomicExch(&scratch[1 + tile], (tile == 0 ? kFlagInc : kFlagAgg) | run);
		tileKept = run;
	}
	// Decoupled look-back by the whole block: each step reads the status words of the kBlock
	// predecessors before the window's end (one per thread, spinning until it is published) and sums
	// them up to the nearest inclusive prefix. With every tile of a one-wave grid resident at once,
	// a window reaches back kBlock tiles per L2 round trip instead of 32.
	uint32_t prefix = 0;
	for (int k = tile - 1; tile > 0; k -= kBlock) {
		const int idx = k - tid;
		uint32_t st = kFlagInc; // before tile 0: an inclusive prefix of 0
		if (idx >= 0) {
			const volatile uint32_t* p = scratch + 1 + idx;
			int spins = 0;
			st = *p;
			while ((st & ~kValueMask) == 0u && ++spins < kSpinLimit) {
				st = *p;
			}
			if ((st & ~kValueMask) == 0u) {
				lbFail = 1; // never expected: the predecessor holds an earlier ticket and is running
				st = kFlagInc;
			}
		}
		const unsigned inc = __ballot_sync(0xffffffffu, (st & ~kValueMask) == kFlagInc);
		if (lane == 0) {
			lbBallot[warp] = inc;
		}
		__syncthreads();
		int stop = kBlock - 1; // lowest thread holding an inclusive prefix, if any
		bool found = false;
		for (int w = kBlock / 32 - 1; w >= 0; --w) {
			const unsigned bw = lbBallot[w];
			stop = bw ? w * 32 + __ffs((int) bw) - 1 : stop;
			found = found || bw != 0u;
		}
		uint32_t v = tid <= stop ? (st & kValueMask) : 0u;
#pragma unroll
		for (int off = 16; off > 0; off >>= 1) {
			v += __shfl_xor_sync(0xffffffffu, v, off);
		}
		if (lane == 0) {
			lbSum[warp] = v;
		}
		__syncthreads();
		for (int w = 0; w < kBlock / 32; ++w) {
			prefix += lbSum[w];
		}
		__syncthreads(); // lbBallot and lbSum are rewritten by the next step
		if (found) {
			break;
		}
	}
	if (tid == 0) {
		if (lbFail) {
			*(volatile int32_t*) errorFlag = 1; // an error slot in mapped host memory (or a device word)
		}
		const uint32_t run = tileKept;
		if (tile > 0) {
			atomicExch(&scratch[1 + tile], kFlagInc | (prefix + run));
		}
		tileBase = prefix;
		const int tiles = (cap + kCompactTile - 1) / kCompactTile;
		if (tile == tiles - 1) {
			*dOutCount = (int32_t) (prefix + run);
			if (hostCount) {
				*(volatile int32_t*) hostCount = (int32_t) (prefix + run);
			}
		}
	}
	__syncthreads();
	// The tile's kept points in order, then one kept point per thread: consecutive threads write
	// consecutive output positions, and the point operations run with every lane busy.
	uint32_t local = warpSums[warp] + (uint32_t) (incl - cnt);
#pragma unroll
	for (int k = 0; k < kCompactItems; ++k) {
		if (keep[k]) {
			keptLocal[local++] = (uint16_t) (tid * kCompactItems + k);
		}
	}
	__syncthreads();
	const uint32_t kept = tileKept;
	// Kept points c = tid + j * kBlock (at most kCompactItems per thread). Each field's source values of
	// all the thread's points are loaded before the first store: the compiler cannot move a load past a
	// store to a pointer that may alias it, so a point-at-a-time loop would serialise the loads.
	int src[kCompactItems];
#pragma unroll
	for (int j = 0; j < kCompactItems; ++j) {
		const uint32_t c = (uint32_t) (tid + j * kBlock);
		src[j] = c < kept ? tile * kCompactTile + keptLocal[c] : -1;
	}
	for (int f = 0; f < fc.count; ++f) {
		if (f == ops.xyzField || f == ops.distField) {
			continue;
		}
		const int sz = fc.f[f].size;
		const uint8_t* s = static_cast<const uint8_t*>(fc.f[f].src);
		uint8_t* d = static_cast<uint8_t*>(fc.f[f].dst);
		if (sz == 4) {
			uint32_t v[kCompactItems];
#pragma unroll
			for (int j = 0; j < kCompactItems; ++j) {
				v[j] = src[j] >= 0 ? reinterpret_cast<const uint32_t*>(s)[src[j]] : 0u;
			}
#pragma unroll
			for (int j = 0; j < kCompactItems; ++j) {
				if (src[j] >= 0) {
					reinterpret_cast<uint32_t*>(d)[tileBase + tid + j * kBlock] = v[j];
				}
			}
		} else {
#pragma unroll
			for (int j = 0; j < kCompactItems; ++j) {
				if (src[j] >= 0) {
					copyElem(s + (size_t) src[j] * sz, d + (size_t) (tileBase + tid + j * kBlock) * sz, sz);
				}
			}
		}
	}
	if (ops.xyzField >= 0 || ops.distField >= 0) {
		// XYZ and distance of the chain's source, through the absorbed operations in order.
		Vec3 p[kCompactItems];
		float dd[kCompactItems];
#pragma unroll
		for (int j = 0; j < kCompactItems; ++j) {
			p[j] = (src[j] >= 0 && ops.srcXyz) ? loadXyz(ops.srcXyz, src[j]) : v3(0.0f, 0.0f, 0.0f);
			dd[j] = (src[j] >= 0 && ops.srcDist) ? ops.srcDist[src[j]] : 0.0f;
		}
#pragma unroll
		for (int j = 0; j < kCompactItems; ++j) {
			if (src[j] < 0) {
				continue;
			}
			const int i = src[j];
			const uint32_t pos = tileBase + (uint32_t) (tid + j * kBlock);
			Vec3 q = p[j];
			float d = dd[j];
			for (int o = 0; o < ops.count; ++o) {
				const uint32_t* prm = opParams[o];
				if (ops.op[o].kind == kOpTransform) {
					q = reinterpret_cast<const Mat34*>(prm)->point(q);
				} else if (ops.op[o].kind == kOpNoiseAngularHitpoint) {
					q = angularHitpoint(*reinterpret_cast<const NoiseParams*>(prm), i, q, ops.op[o].withDistance ? &d : nullptr);
				} else {
					q = distanceNoise(*reinterpret_cast<const NoiseParams*>(prm), i, q, d);
				}
			}
			if (ops.xyzField >= 0) {
				storeXyz(static_cast<float*>(fc.f[ops.xyzField].dst), (int) pos, q);
			}
			if (ops.distField >= 0) {
				static_cast<float*>(fc.f[ops.distField].dst)[pos] = d;
			}
		}
	}
	// Re-arm the scratch for the next launch once every tile has finished its look-back.
	__shared__ bool lastTile;
	__syncthreads();
	const int tiles = (cap + kCompactTile - 1) / kCompactTile;
	if (tid == 0) {
		__threadfence();
		lastTile = atomicAdd(&scratch[1 + tiles], 1u) == (uint32_t) (tiles - 1);
	}
	__syncthreads();
	if (lastTile) {
		for (int k = tid; k < tiles + 2; k += kBlock) {
			scratch[k] = 0u;
		}
	}
}

// ---------------------------------------------------------------- format

struct WordMap
{
	int8_t field[64];  // field index of output word k, -1 = padding
	int8_t word[64];   // word index inside that field
};

// Word-aligned layouts: one thread per output 32-bit word, coalesced stores.
// The point of word w is w / pointWords; `magic` = ceil(2^32 / pointWords) turns that into one
// multiply-high, exact for w < 2^26 (pointWords <= 64), and is 0 for larger launches.
__global__ void kFormatWords(const __grid_constant__ FieldCopies fc, const __grid_constant__ WordMap wm, int pointWords, uint32_t magic,
                             int cap, const int32_t* dCount, uint32_t* __restrict__ out)
{
	long w = (long) blockIdx.x * blockDim.x + threadIdx.x;
	long n = countOf(cap, dCount);
	if (w >= n * pointWords) {
		return;
	}
	int i = magic != 0 ? (int) __umulhi((uint32_t) w, magic) : (int) (w / pointWords);
	int k = (int) (w - (long) i * pointWords);
	int f = wm.field[k];
	uint32_t v = 0;
	if (f >= 0) {
		const int fw = fc.f[f].size >> 2;
		v = static_cast<const uint32_t*>(fc.f[f].src)[(size_t) i * fw + wm.word[k]];
	}
	out[w] = v;
}

// Any layout: one thread per point, byte copies (padding bytes zeroed).
__global__ void kFormatBytes(const __grid_constant__ FieldCopies fc, int pointSize, int cap, const int32_t* dCount, uint8_t* __restrict__ out)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= countOf(cap, dCount)) {
		return;
	}
	for (int f = 0; f < fc.count; ++f) {
		const int sz = fc.f[f].size;
		uint8_t* d = out + (size_t) i * pointSize + fc.f[f].offset;
		const uint8_t* s = static_cast<const uint8_t*>(fc.f[f].src);
		for (int b = 0; b < sz; ++b) {
			d[b] = s ? s[(size_t) i * sz + b] : 0;
		}
	}
}

__global__ void kAosToSoa(const uint8_t* __restrict__ in, int pointSize, int n, const __grid_constant__ FieldCopies fc)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) {
		return;
	}
	for (int f = 0; f < fc.count; ++f) {
		if (fc.f[f].dst == nullptr) {
			continue;
		}
		const int sz = fc.f[f].size;
		const uint8_t* s = in + (size_t) i * pointSize + fc.f[f].offset;
		uint8_t* d = static_cast<uint8_t*>(fc.f[f].dst) + (size_t) i * sz;
		for (int b = 0; b < sz; ++b) {
			d[b] = s[b];
		}
	}
}

// Point clouds concatenated: blockIdx.y is the input, blockIdx.x a tile of its points. Every block
// finds its input's offset by summing the counts before it (inputs are few); the copy moves whole
// 4-byte words when the element size allows (all but 1- and 2-byte fields).
constexpr int kMergeTile = 2048;

struct MergeTableView
{
	const MergeInput* in;
	const void* const* src;
	const FieldCopy* fld;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t{15}; }

__host__ __device__ inline MergeTableView mergeView(const void* table, int nIn, int nF)
{
	const uint8_t* b = static_cast<const uint8_t*>(table);
	const size_t offSrc = align16(sizeof(MergeInput) * (size_t) nIn);
	const size_t offFld = offSrc + align16(sizeof(void*) * (size_t) nIn * (size_t) nF);
	return {reinterpret_cast<const MergeInput*>(b), reinterpret_cast<const void* const*>(b + offSrc),
	        reinterpret_cast<const FieldCopy*>(b + offFld)};
}

__device__ __forceinline__ int mergeCount(const MergeInput& m) { return m.count ? *m.count : m.staticCount; }

template<class W>
__device__ __forceinline__ void copyRange(const void* src, void* dst, long srcFirst, long dstFirst, long n)
{
	const W* s = static_cast<const W*>(src) + srcFirst;
	W* d = static_cast<W*>(dst) + dstFirst;
	for (long k = threadIdx.x; k < n; k += blockDim.x) {
		d[k] = s[k];
	}
}

__global__ void __launch_bounds__(kBlock) kMergePoints(const void* table, int nIn, int nF, const int32_t* dBase, int32_t* dOutCount)
{
	const MergeTableView t = mergeView(table, nIn, nF);
	const int i = blockIdx.y;
	__shared__ long long sOffset;
	__shared__ int sCount;
	if (threadIdx.x < 32) {
		const int lane = threadIdx.x;
		const bool total = dOutCount != nullptr && i == 0 && blockIdx.x == 0;
		const int upTo = total ? nIn : i;
		long long before = 0, all = 0;
		for (int j = lane; j < upTo; j += 32) {
			const long long c = mergeCount(t.in[j]);
			all += c;
			before += j < i ? c : 0;
		}
		for (int o = 16; o > 0; o >>= 1) {
			before += __shfl_down_sync(0xffffffffu, before, o);
			all += __shfl_down_sync(0xffffffffu, all, o);
		}
		if (lane == 0) {
			const long long base = dBase ? *dBase : 0;
			sOffset = base + before;
			sCount = mergeCount(t.in[i]);
			if (total) {
				*dOutCount = (int32_t) (base + all);
			}
		}
	}
	__syncthreads();
	const long first = (long) blockIdx.x * kMergeTile;
	const long last = min((long) sCount, first + kMergeTile);
	if (first >= last) {
		return;
	}
	for (int f = 0; f < nF; ++f) {
		const int sz = t.fld[f].size;
		const void* src = t.src[(size_t) i * nF + f];
		void* dst = t.fld[f].dst;
		if (sz % 4 == 0) {
			const int w = sz / 4;
			copyRange<uint32_t>(src, dst, first * w, (sOffset + first) * w, (last - first) * w);
		} else if (sz % 2 == 0) {
			const int w = sz / 2;
			copyRange<uint16_t>(src, dst, first * w, (sOffset + first) * w, (last - first) * w);
		} else {
			copyRange<uint8_t>(src, dst, first * sz, (sOffset + first) * sz, (last - first) * sz);
		}
	}
}

__global__ void kAddCount(int32_t* acc, const int32_t* add, int32_t addStatic) { *acc += add ? *add : addStatic; }

__global__ void kGroundFlags(const float* __restrict__ normals, int cap, const int32_t* dCount, Vec3 up, float threshold,
                             int32_t* __restrict__ out)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= countOf(cap, dCount)) {
		return;
	}
	const Vec3 n = loadXyz(normals, i);
	out[i] = acosf(fabsf(dot(n, up))) > threshold ? 1 : 0;
}

} // namespace

size_t mergeTableBytes(int nInputs, int nFields)
{
	return align16(sizeof(MergeInput) * (size_t) nInputs) + align16(sizeof(void*) * (size_t) nInputs * (size_t) nFields) +
	       sizeof(FieldCopy) * (size_t) nFields;
}

void fillMergeTable(void* table, const std::vector<MergeInput>& inputs, const std::vector<const void*>& src,
                    const std::vector<FieldCopy>& fields)
{
	const int nIn = (int) inputs.size(), nF = (int) fields.size();
	const MergeTableView v = mergeView(table, nIn, nF);
	std::copy(inputs.begin(), inputs.end(), const_cast<MergeInput*>(v.in));
	std::copy(src.begin(), src.end(), const_cast<const void**>(v.src));
	std::copy(fields.begin(), fields.end(), const_cast<FieldCopy*>(v.fld));
}

void launchMergePoints(const void* dTable, int nInputs, int nFields, int maxCount, const int32_t* dBase, int32_t* dOutCount,
                       cudaStream_t s)
{
	if (nInputs <= 0) {
		return;
	}
	const dim3 grid((unsigned) std::max(1, blocks(maxCount, kMergeTile)), (unsigned) nInputs);
	kMergePoints<<<grid, kBlock, 0, s>>>(dTable, nInputs, nFields, dBase, dOutCount);
	countLaunch();
}

void launchGroundFlags(const float* normals, int cap, const int32_t* dCount, Vec3 up, float threshold, int32_t* out, cudaStream_t s)
{
	if (cap > 0) {
		kGroundFlags<<<blocks(cap, kBlock), kBlock, 0, s>>>(normals, cap, dCount, up, threshold, out);
		countLaunch();
	}
}

void launchAddCount(int32_t* dAcc, const int32_t* dAdd, int32_t addStatic, cudaStream_t s)
{
	kAddCount<<<1, 1, 0, s>>>(dAcc, dAdd, addStatic);
	countLaunch();
}

void launchTransformRays(const Mat34* in, Mat34* out, int n, const Mat34* dTf, cudaStream_t s)
{
	if (n > 0) {
		kTransformRays<<<blocks(n, kBlock), kBlock, 0, s>>>(in, out, n, dTf);
		countLaunch();
	}
}

void launchTransformPoints(const float* in, float* out, int cap, const int32_t* dCount, const Mat34* dTf, cudaStream_t s)
{
	if (cap > 0) {
		kTransformPoints<<<blocks(cap, kBlock), kBlock, 0, s>>>(in, out, cap, dCount, dTf);
		countLaunch();
	}
}

void launchNoiseAngularRay(const Mat34* in, Mat34* out, int n, const NoiseParams* np, cudaStream_t s)
{
	if (n > 0) {
		kNoiseAngularRay<<<blocks(n, kBlock), kBlock, 0, s>>>(in, out, n, np);
		countLaunch();
	}
}

void launchNoiseAngularHitpoint(const float* inXyz, float* outXyz, float* outDist, int cap, const int32_t* dCount,
                                const NoiseParams* np, cudaStream_t s)
{
	if (cap > 0) {
		kNoiseAngularHitpoint<<<blocks(cap, kBlock), kBlock, 0, s>>>(inXyz, outXyz, outDist, cap, dCount, np);
		countLaunch();
	}
}

void launchNoiseDistance(const float* inXyz, const float* inDist, float* outXyz, float* outDist, int cap, const int32_t* dCount,
                         const NoiseParams* np, cudaStream_t s)
{
	if (cap > 0) {
		kNoiseDistance<<<blocks(cap, kBlock), kBlock, 0, s>>>(inXyz, inDist, outXyz, outDist, cap, dCount, np);
		countLaunch();
	}
}

size_t compactScratchBytes(int cap) { return sizeof(uint32_t) * (size_t) (2 + (cap + kCompactTile - 1) / kCompactTile); }

void launchCompact(const int32_t* flags, int cap, const int32_t* dInCount, const FieldCopies& fields, const PointOps* ops,
                   int32_t* dOutCount, void* scratch, int32_t* dError, cudaStream_t s, int32_t* hostCount)
{
	PointOps po{};
	if (ops != nullptr) {
		po = *ops;
	} else {
		po.xyzField = -1;
		po.distField = -1;
	}
	if (cap <= 0) {
		cudaMemsetAsync(dOutCount, 0, sizeof(int32_t), s);
		if (hostCount) {
			cudaMemsetAsync(hostCount, 0, sizeof(int32_t), s);
		}
		return;
	}
	int tiles = (cap + kCompactTile - 1) / kCompactTile;
	kCompact<<<tiles, kBlock, 0, s>>>(flags, cap, dInCount, fields, po, dOutCount, static_cast<uint32_t*>(scratch), dError, hostCount);
	countLaunch();
}

void launchFormat(const FieldCopies& fields, int pointSize, int cap, const int32_t* dCount, uint8_t* out, cudaStream_t s)
{
	if (cap <= 0 || pointSize <= 0) {
		return;
	}
	bool words = (pointSize % 4 == 0) && pointSize / 4 <= 64;
	for (int f = 0; f < fields.count && words; ++f) {
		words = (fields.f[f].size % 4 == 0) && (fields.f[f].offset % 4 == 0);
	}
	if (words) {
		WordMap wm;
		for (int k = 0; k < 64; ++k) {
			wm.field[k] = -1;
			wm.word[k] = 0;
		}
		for (int f = 0; f < fields.count; ++f) {
			if (fields.f[f].src == nullptr) {
				continue;
			}
			for (int k = 0; k < fields.f[f].size / 4; ++k) {
				wm.field[fields.f[f].offset / 4 + k] = (int8_t) f;
				wm.word[fields.f[f].offset / 4 + k] = (int8_t) k;
			}
		}
		int pw = pointSize / 4;
		long total = (long) cap * pw;
		const uint32_t magic = total < (1l << 26) ? (uint32_t) (((1ull << 32) + (uint64_t) pw - 1) / (uint64_t) pw) : 0u;
		kFormatWords<<<blocks(total, kBlock), kBlock, 0, s>>>(fields, wm, pw, magic, cap, dCount, reinterpret_cast<uint32_t*>(out));
	} else {
		kFormatBytes<<<blocks(cap, kBlock), kBlock, 0, s>>>(fields, pointSize, cap, dCount, out);
	}
	countLaunch();
}

void launchAosToSoa(const uint8_t* in, int pointSize, int n, const FieldCopies& fields, cudaStream_t s)
{
	if (n > 0) {
		kAosToSoa<<<blocks(n, kBlock), kBlock, 0, s>>>(in, pointSize, n, fields);
		countLaunch();
	}
}

} // namespace rgl
