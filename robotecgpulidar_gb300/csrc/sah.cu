// On-device binned SAH topology for mesh BLASes: the binary tree of the host builder
// (sah_build.hpp buildBinnedSahTree), computed on the GPU with the same float arithmetic, so the
// device tree equals the host tree node for node and the sorted primitive order equals the host's.
//
// Replaces OptiX's GAS build of reference src/scene/GASBuilder.hpp:31-100 (optixAccelBuild), which
// runs on the device; the wide collapse and quantisation that follow are bvh_core.hpp's.
//
// Algorithm (after Wald 2007, binned SAH, 32 bins per axis; parallel top-down):
//  * ranges of more than kBigTask primitives are split level by level, each by many blocks: a bounds
//    pass (node box and centroid bounds), a binning pass (per-bin boxes and counts, shared-memory
//    atomics flushed to the range's global bins), one warp per range evaluating the 3 x 31 split
//    candidates, and a stable partition (per-chunk counts, then a scatter that ranks each chunk's
//    elements with a block scan);
//  * ranges of 2..kBigTask primitives are built to the leaves by one block each, in shared memory:
//    ranges above kSmallTask split with block-wide passes, smaller ones by one warp each, which keeps
//    its elements in registers and partitions them with ballots.
// Exactness: boxes and centroid bounds are min/max (order free); the centroid, the bin index, the
// half areas and the split costs use the host's expressions with round-to-nearest intrinsics and no
// FMA contraction; among equal costs the first candidate in (axis, bin) order wins, as in the host's
// strict comparison; partitions are stable; a range whose centroids all coincide splits in the
// middle. Node numbering differs from the host's (atomics instead of a depth-first counter); the
// collapse does not depend on it.
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "bvh_core.hpp"
#include "kernels.hpp"

namespace rgl {

namespace {

#define RGL_SAH_OK(expr)                                                                                                       \
	do {                                                                                                                       \
		cudaError_t e_ = (expr);                                                                                               \
		if (e_ != cudaSuccess) {                                                                                               \
			throw std::runtime_error(std::string("CUDA error in SAH build: ") + cudaGetErrorString(e_) + " at " #expr);        \
		}                                                                                                                      \
	} while (0)

constexpr int kBins = 32;
constexpr int kBinWords = 7;                    // lo xyz, hi xyz (ordered bits), count
constexpr int kTaskBinWords = 3 * kBins * kBinWords;
constexpr int kBigTask = 2048;                  // larger ranges split in the level loop
constexpr int kChunk = 2048;                    // elements per block in the level loop
constexpr int kThreads = 256;
constexpr int kItems = kChunk / kThreads;       // 8 elements per thread
constexpr int kSmallTask = 32;                  // ranges up to this size: one warp
constexpr int kWarps = kThreads / 32;
constexpr uint32_t kEmptyLo = 0xffffffffu;      // identity of min over ordered bits
constexpr uint32_t kEmptyHi = 0u;               // identity of max
constexpr float kInf = __builtin_huge_valf();

struct SahTask
{
	int32_t lo, hi, node, pad; // sorted positions [lo, hi), binary node index
};

struct SahSplit
{
	int32_t axis, bin, nLeft, pad; // axis -1: split in the middle
};

// Control words: [0] node counter, [1] next-level task count, [2] block task count, [3] chunks of the
// current level, [4] error: a partition or stack index outside its range (never expected: the counts
// and the partition use the same bin function), the offending write is skipped.
enum { kCtrNodes = 0, kCtrNext = 1, kCtrBlock = 2, kCtrChunks = 3, kCtrError = 4, kCtrWords = 8 };

__device__ __forceinline__ uint32_t ordered(float f)
{
	const uint32_t u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }

// The host's expressions (sah_build.hpp), without contraction.
__device__ __forceinline__ float halfAreaOf(float lx, float ly, float lz, float hx, float hy, float hz)
{
	const float dx = __fsub_rn(hx, lx), dy = __fsub_rn(hy, ly), dz = __fsub_rn(hz, lz);
	return __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx));
}
__device__ __forceinline__ int binOf(float c, float cmin, float scale)
{
	const int b = (int) __fmul_rn(__fsub_rn(c, cmin), scale); // >= 0 for finite input; clamped for any
	return b < 0 ? 0 : (b < kBins - 1 ? b : kBins - 1);
}
__device__ __forceinline__ float comp3(const float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// Node box and centroid bounds of a range, 12 ordered words: box lo xyz, box hi xyz, centroid lo
// xyz, centroid hi xyz.
struct Bounds12
{
	uint32_t w[12];
	__device__ __forceinline__ void clear()
	{
#pragma unroll
		for (int k = 0; k < 12; ++k) {
			w[k] = (k < 3 || (k >= 6 && k < 9)) ? kEmptyLo : kEmptyHi;
		}
	}
	__device__ __forceinline__ void add(const float4& l, const float4& h, const float4& c)
	{
		w[0] = min(w[0], ordered(l.x));
		w[1] = min(w[1], ordered(l.y));
		w[2] = min(w[2], ordered(l.z));
		w[3] = max(w[3], ordered(h.x));
		w[4] = max(w[4], ordered(h.y));
		w[5] = max(w[5], ordered(h.z));
		w[6] = min(w[6], ordered(c.x));
		w[7] = min(w[7], ordered(c.y));
		w[8] = min(w[8], ordered(c.z));
		w[9] = max(w[9], ordered(c.x));
		w[10] = max(w[10], ordered(c.y));
		w[11] = max(w[11], ordered(c.z));
	}
	__device__ __forceinline__ void warpReduce()
	{
#pragma unroll
		for (int k = 0; k < 12; ++k) {
			const bool isMin = k < 3 || (k >= 6 && k < 9);
			w[k] = isMin ? __reduce_min_sync(0xffffffffu, w[k]) : __reduce_max_sync(0xffffffffu, w[k]);
		}
	}
};
__device__ __forceinline__ bool isMinWord(int k) { return k < 3 || (k >= 6 && k < 9); }

// Binning frame of one axis: valid when the centroids spread along it (the host's ext > 0).
struct AxisFrame
{
	float cmin, scale;
	bool valid;
};
__device__ __forceinline__ AxisFrame axisFrame(const uint32_t* b12, int a)
{
	AxisFrame f;
	f.cmin = unordered(b12[6 + a]);
	const float ext = __fsub_rn(unordered(b12[9 + a]), f.cmin);
	f.valid = ext > 0.0f;
	f.scale = f.valid ? __fdiv_rn((float) kBins, ext) : 0.0f;
	return f;
}

// Best split of a range from its bins (3 x 32 x 7 words, any address space) and bounds, by one warp:
// the candidate between bins b-1 and b of axis a costs halfArea(left) * nLeft + halfArea(right) * nRight;
// candidates with an empty side are skipped; the lowest cost wins, the first in (axis, b) order among
// equal costs. Returns axis -1 when no axis has spread centroids.
__device__ SahSplit warpBestSplit(const uint32_t* bins, const uint32_t* b12, int lane)
{
	float bestCost = kInf;
	int bestKey = 1 << 30, bestLeft = 0;
	for (int a = 0; a < 3; ++a) {
		const AxisFrame f = axisFrame(b12, a);
		if (!f.valid) {
			continue;
		}
		const uint32_t* bb = bins + (a * kBins + lane) * kBinWords;
		uint32_t v[kBinWords];
#pragma unroll
		for (int k = 0; k < kBinWords; ++k) {
			v[k] = bb[k];
		}
		// inclusive prefix (bins 0..lane) and suffix (bins lane..31)
		uint32_t p[kBinWords], q[kBinWords];
#pragma unroll
		for (int k = 0; k < kBinWords; ++k) {
			p[k] = v[k];
			q[k] = v[k];
		}
#pragma unroll
		for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
			for (int k = 0; k < kBinWords; ++k) {
				const uint32_t up = __shfl_up_sync(0xffffffffu, p[k], off);
				const uint32_t dn = __shfl_down_sync(0xffffffffu, q[k], off);
				if (lane >= off) {
					p[k] = k < 3 ? min(p[k], up) : (k < 6 ? max(p[k], up) : p[k] + up);
				}
				if (lane + off < 32) {
					q[k] = k < 3 ? min(q[k], dn) : (k < 6 ? max(q[k], dn) : q[k] + dn);
				}
			}
		}
		// left side of candidate `lane` = prefix of lane - 1
		uint32_t l[kBinWords];
#pragma unroll
		for (int k = 0; k < kBinWords; ++k) {
			l[k] = __shfl_up_sync(0xffffffffu, p[k], 1);
		}
		const uint32_t lc = l[6], rc = q[6];
		if (lane >= 1 && lc != 0u && rc != 0u) {
			const float ha = halfAreaOf(unordered(l[0]), unordered(l[1]), unordered(l[2]), unordered(l[3]), unordered(l[4]), unordered(l[5]));
			const float hb = halfAreaOf(unordered(q[0]), unordered(q[1]), unordered(q[2]), unordered(q[3]), unordered(q[4]), unordered(q[5]));
			const float cost = __fadd_rn(__fmul_rn(ha, (float) lc), __fmul_rn(hb, (float) rc));
			if (cost < bestCost) {
				bestCost = cost;
				bestKey = a * kBins + lane;
				bestLeft = (int) lc;
			}
		}
	}
	// warp argmin over (cost, key)
#pragma unroll
	for (int off = 16; off >= 1; off >>= 1) {
		const float oc = __shfl_xor_sync(0xffffffffu, bestCost, off);
		const int ok = __shfl_xor_sync(0xffffffffu, bestKey, off);
		const int ol = __shfl_xor_sync(0xffffffffu, bestLeft, off);
		if (oc < bestCost || (oc == bestCost && ok < bestKey)) {
			bestCost = oc;
			bestKey = ok;
			bestLeft = ol;
		}
	}
	SahSplit s;
	if (bestKey >= (1 << 30)) {
		s.axis = -1;
		s.bin = 0;
		s.nLeft = 0;
	} else {
		s.axis = bestKey / kBins;
		s.bin = bestKey % kBins;
		s.nLeft = bestLeft;
	}
	s.pad = 0;
	return s;
}

// Writes binary node `node` over sorted positions [lo, hi) split at lo + nLeft, allocates its
// children's node indices and returns them (a leaf child is ~position).
__device__ __forceinline__ void emitNode(int node, int lo, int hi, int nLeft, const uint32_t* b12, BinNode* bin, int32_t* rangeFirst,
                                         int32_t* rangeLast, uint32_t* ctr, int32_t& left, int32_t& right)
{
	const int mid = lo + nLeft;
	left = (mid - lo == 1) ? ~lo : (int32_t) atomicAdd(&ctr[kCtrNodes], 1u);
	right = (hi - mid == 1) ? ~mid : (int32_t) atomicAdd(&ctr[kCtrNodes], 1u);
	BinNode bn;
	bn.lox = unordered(b12[0]);
	bn.loy = unordered(b12[1]);
	bn.loz = unordered(b12[2]);
	bn.hix = unordered(b12[3]);
	bn.hiy = unordered(b12[4]);
	bn.hiz = unordered(b12[5]);
	bn.left = left;
	bn.right = right;
	bin[node] = bn;
	rangeFirst[node] = lo;
	rangeLast[node] = hi - 1;
}

// ------------------------------------------------------------------ level loop (ranges > kBigTask)

__global__ void kSahInit(const float4* __restrict__ lo, const float4* __restrict__ hi, int n, float4* __restrict__ cen,
                         uint32_t* __restrict__ idsA, uint32_t* __restrict__ sorted)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) {
		const float4 l = lo[i], h = hi[i];
		cen[i] = make_float4(__fmul_rn(0.5f, __fadd_rn(l.x, h.x)), __fmul_rn(0.5f, __fadd_rn(l.y, h.y)), __fmul_rn(0.5f, __fadd_rn(l.z, h.z)),
		                     0.0f);
		idsA[i] = (uint32_t) i;
		sorted[i] = (uint32_t) i;
	}
}

// Chunk prefix sums of the level's ranges and their bounds cleared (one block).
__global__ void kSahLevelPrep(const SahTask* __restrict__ tasks, int nTasks, int32_t* chunkBase, uint32_t* bounds, uint32_t* ctr)
{
	__shared__ int32_t sWarp[32];
	__shared__ int32_t sCarry;
	if (threadIdx.x == 0) {
		sCarry = 0;
	}
	for (int i = threadIdx.x; i < nTasks * 12; i += blockDim.x) {
		bounds[i] = isMinWord(i % 12) ? kEmptyLo : kEmptyHi;
	}
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int base = 0; base < nTasks; base += blockDim.x) {
		const int t = base + (int) threadIdx.x;
		const int v = t < nTasks ? (tasks[t].hi - tasks[t].lo + kChunk - 1) / kChunk : 0;
		int incl = v;
		for (int off = 1; off < 32; off <<= 1) {
			const int u = __shfl_up_sync(0xffffffffu, incl, off);
			if (lane >= off) {
				incl += u;
			}
		}
		if (lane == 31) {
			sWarp[warp] = incl;
		}
		__syncthreads();
		if (warp == 0) {
			const int nw = blockDim.x / 32;
			int w = lane < nw ? sWarp[lane] : 0;
			for (int off = 1; off < 32; off <<= 1) {
				const int u = __shfl_up_sync(0xffffffffu, w, off);
				if (lane >= off) {
					w += u;
				}
			}
			if (lane < nw) {
				sWarp[lane] = w; // inclusive over warps
			}
		}
		__syncthreads();
		const int warpBase = warp > 0 ? sWarp[warp - 1] : 0;
		if (t < nTasks) {
			chunkBase[t] = sCarry + warpBase + incl - v;
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			sCarry += sWarp[blockDim.x / 32 - 1];
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		chunkBase[nTasks] = sCarry;
		ctr[kCtrChunks] = (uint32_t) sCarry;
	}
}

// Range of chunk c: the task whose chunk prefix covers it.
__device__ __forceinline__ bool chunkRange(const int32_t* chunkBase, int nTasks, const SahTask* tasks, int c, int& t, int& start, int& end,
                                           int& first)
{
	if (c >= chunkBase[nTasks]) {
		return false;
	}
	int lo = 0, hi = nTasks; // chunkBase[lo] <= c < chunkBase[hi]
	while (hi - lo > 1) {
		const int mid = (lo + hi) >> 1;
		if (chunkBase[mid] <= c) {
			lo = mid;
		} else {
			hi = mid;
		}
	}
	t = lo;
	first = chunkBase[lo];
	start = tasks[lo].lo + (c - first) * kChunk;
	end = min(tasks[lo].hi, start + kChunk);
	return true;
}

__device__ __forceinline__ void blockReduceBounds(Bounds12& b, uint32_t (*sRed)[12], uint32_t* out)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	b.warpReduce();
	if (lane == 0) {
#pragma unroll
		for (int k = 0; k < 12; ++k) {
			sRed[warp][k] = b.w[k];
		}
	}
	__syncthreads();
	if (threadIdx.x < 12) {
		const int k = threadIdx.x;
		uint32_t v = sRed[0][k];
		for (int w = 1; w < kWarps; ++w) {
			v = isMinWord(k) ? min(v, sRed[w][k]) : max(v, sRed[w][k]);
		}
		if (isMinWord(k)) {
			atomicMin(&out[k], v);
		} else {
			atomicMax(&out[k], v);
		}
	}
}

__global__ void __launch_bounds__(kThreads) kSahBounds(const SahTask* __restrict__ tasks, int nTasks, const int32_t* __restrict__ chunkBase,
                                                       const uint32_t* __restrict__ ids, const float4* __restrict__ lo,
                                                       const float4* __restrict__ hi, const float4* __restrict__ cen, uint32_t* bounds,
                                                       uint32_t* bins)
{
	__shared__ uint32_t sRed[kWarps][12];
	int t, start, end, first;
	if (!chunkRange(chunkBase, nTasks, tasks, blockIdx.x, t, start, end, first)) {
		return;
	}
	if ((int) blockIdx.x == first) { // the range's first chunk clears its bins for the binning pass
		uint32_t* tb = bins + (size_t) t * kTaskBinWords;
		for (int k = threadIdx.x; k < kTaskBinWords; k += blockDim.x) {
			const int w = k % kBinWords;
			tb[k] = w < 3 ? kEmptyLo : (w < 6 ? kEmptyHi : 0u);
		}
	}
	Bounds12 b;
	b.clear();
	for (int i = start + (int) threadIdx.x; i < end; i += blockDim.x) {
		const uint32_t id = ids[i];
		b.add(lo[id], hi[id], cen[id]);
	}
	blockReduceBounds(b, sRed, bounds + (size_t) t * 12);
}

__global__ void __launch_bounds__(kThreads) kSahBins(const SahTask* __restrict__ tasks, int nTasks, const int32_t* __restrict__ chunkBase,
                                                     const uint32_t* __restrict__ ids, const float4* __restrict__ lo,
                                                     const float4* __restrict__ hi, const float4* __restrict__ cen,
                                                     const uint32_t* __restrict__ bounds, uint32_t* bins)
{
	__shared__ uint32_t sb[kTaskBinWords];
	int t, start, end, first;
	if (!chunkRange(chunkBase, nTasks, tasks, blockIdx.x, t, start, end, first)) {
		return;
	}
	for (int k = threadIdx.x; k < kTaskBinWords; k += blockDim.x) {
		const int w = k % kBinWords;
		sb[k] = w < 3 ? kEmptyLo : (w < 6 ? kEmptyHi : 0u);
	}
	const uint32_t* b12 = bounds + (size_t) t * 12;
	AxisFrame fr[3];
#pragma unroll
	for (int a = 0; a < 3; ++a) {
		fr[a] = axisFrame(b12, a);
	}
	__syncthreads();
	for (int i = start + (int) threadIdx.x; i < end; i += blockDim.x) {
		const uint32_t id = ids[i];
		const float4 l = lo[id], h = hi[id], c = cen[id];
#pragma unroll
		for (int a = 0; a < 3; ++a) {
			if (!fr[a].valid) {
				continue;
			}
			uint32_t* bb = sb + (a * kBins + binOf(comp3(c, a), fr[a].cmin, fr[a].scale)) * kBinWords;
			atomicMin(&bb[0], ordered(l.x));
			atomicMin(&bb[1], ordered(l.y));
			atomicMin(&bb[2], ordered(l.z));
			atomicMax(&bb[3], ordered(h.x));
			atomicMax(&bb[4], ordered(h.y));
			atomicMax(&bb[5], ordered(h.z));
			atomicAdd(&bb[6], 1u);
		}
	}
	__syncthreads();
	uint32_t* tb = bins + (size_t) t * kTaskBinWords;
	for (int k = threadIdx.x; k < 3 * kBins; k += blockDim.x) {
		const uint32_t* bb = sb + k * kBinWords;
		if (bb[6] == 0u) {
			continue;
		}
		uint32_t* g = tb + k * kBinWords;
		atomicMin(&g[0], bb[0]);
		atomicMin(&g[1], bb[1]);
		atomicMin(&g[2], bb[2]);
		atomicMax(&g[3], bb[3]);
		atomicMax(&g[4], bb[4]);
		atomicMax(&g[5], bb[5]);
		atomicAdd(&g[6], bb[6]);
	}
}

// One warp per range: the split, the node, its children (next level, block phase or leaves).
__global__ void kSahSplit(const SahTask* __restrict__ tasks, int nTasks, const uint32_t* __restrict__ bounds,
                          const uint32_t* __restrict__ bins, SahSplit* splits, BinNode* bin, int32_t* rangeFirst, int32_t* rangeLast,
                          SahTask* next, SahTask* blockTasks, uint32_t* ctr)
{
	const int w = (int) ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
	const int lane = threadIdx.x & 31;
	if (w >= nTasks) {
		return;
	}
	const SahTask tk = tasks[w];
	const uint32_t* b12 = bounds + (size_t) w * 12;
	SahSplit s = warpBestSplit(bins + (size_t) w * kTaskBinWords, b12, lane);
	if (s.axis < 0) {
		s.nLeft = (tk.lo + tk.hi) / 2 - tk.lo;
	}
	if (lane == 0) {
		splits[w] = s;
		int32_t left, right;
		emitNode(tk.node, tk.lo, tk.hi, s.nLeft, b12, bin, rangeFirst, rangeLast, ctr, left, right);
		const int mid = tk.lo + s.nLeft;
		const int cl[2] = {left, right};
		const int r0[2] = {tk.lo, mid}, r1[2] = {mid, tk.hi};
		for (int c = 0; c < 2; ++c) {
			const int cnt = r1[c] - r0[c];
			if (cnt < 2) {
				continue;
			}
			const SahTask child{r0[c], r1[c], cl[c], 0};
			if (cnt > kBigTask) {
				next[atomicAdd(&ctr[kCtrNext], 1u)] = child;
			} else {
				blockTasks[atomicAdd(&ctr[kCtrBlock], 1u)] = child;
			}
		}
	}
}

__device__ __forceinline__ bool goesLeft(uint32_t id, int pos, const SahTask& tk, const SahSplit& s, const AxisFrame& f,
                                         const float4* __restrict__ cen)
{
	if (s.axis < 0) {
		return pos < tk.lo + s.nLeft;
	}
	return binOf(comp3(cen[id], s.axis), f.cmin, f.scale) < s.bin;
}

__global__ void __launch_bounds__(kThreads) kSahPartCount(const SahTask* __restrict__ tasks, int nTasks,
                                                          const int32_t* __restrict__ chunkBase, const uint32_t* __restrict__ ids,
                                                          const float4* __restrict__ cen, const uint32_t* __restrict__ bounds,
                                                          const SahSplit* __restrict__ splits, int32_t* chunkLeft)
{
	__shared__ int sW[kWarps];
	int t, start, end, first;
	if (!chunkRange(chunkBase, nTasks, tasks, blockIdx.x, t, start, end, first)) {
		return;
	}
	const SahTask tk = tasks[t];
	const SahSplit s = splits[t];
	const AxisFrame f = s.axis >= 0 ? axisFrame(bounds + (size_t) t * 12, s.axis) : AxisFrame{0.0f, 0.0f, false};
	int cnt = 0;
	for (int i = start + (int) threadIdx.x; i < end; i += blockDim.x) {
		cnt += goesLeft(ids[i], i, tk, s, f, cen) ? 1 : 0;
	}
	cnt = __reduce_add_sync(0xffffffffu, cnt);
	if ((threadIdx.x & 31) == 0) {
		sW[threadIdx.x >> 5] = cnt;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		int sum = 0;
		for (int w = 0; w < kWarps; ++w) {
			sum += sW[w];
		}
		chunkLeft[blockIdx.x] = sum;
	}
}

// Block-wide exclusive scan of one int per thread; returns the prefix and the block total.
__device__ __forceinline__ int blockExclusiveScan(int v, int* sW, int& total)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int incl = v;
#pragma unroll
	for (int off = 1; off < 32; off <<= 1) {
		const int u = __shfl_up_sync(0xffffffffu, incl, off);
		if (lane >= off) {
			incl += u;
		}
	}
	if (lane == 31) {
		sW[warp] = incl;
	}
	__syncthreads();
	int before = 0;
	total = 0;
	for (int w = 0; w < kWarps; ++w) {
		const int x = sW[w];
		before += w < warp ? x : 0;
		total += x;
	}
	__syncthreads();
	return before + incl - v;
}

__global__ void __launch_bounds__(kThreads) kSahPartScatter(const SahTask* __restrict__ tasks, int nTasks,
                                                            const int32_t* __restrict__ chunkBase, const uint32_t* __restrict__ ids,
                                                            const float4* __restrict__ cen, const uint32_t* __restrict__ bounds,
                                                            const SahSplit* __restrict__ splits, const int32_t* __restrict__ chunkLeft,
                                                            uint32_t* __restrict__ idsOut, uint32_t* __restrict__ sorted, uint32_t* ctr)
{
	__shared__ int sW[kWarps];
	int t, start, end, first;
	if (!chunkRange(chunkBase, nTasks, tasks, blockIdx.x, t, start, end, first)) {
		return;
	}
	const SahTask tk = tasks[t];
	const SahSplit s = splits[t];
	const AxisFrame f = s.axis >= 0 ? axisFrame(bounds + (size_t) t * 12, s.axis) : AxisFrame{0.0f, 0.0f, false};
	// left elements of the range's earlier chunks
	int before = 0;
	for (int c = first + (int) threadIdx.x; c < (int) blockIdx.x; c += blockDim.x) {
		before += chunkLeft[c];
	}
	int dummy;
	before = __reduce_add_sync(0xffffffffu, before);
	if ((threadIdx.x & 31) == 0) {
		sW[threadIdx.x >> 5] = before;
	}
	__syncthreads();
	int leftBefore = 0;
	for (int w = 0; w < kWarps; ++w) {
		leftBefore += sW[w];
	}
	__syncthreads();
	// this thread's run of kItems consecutive elements
	const int p0 = start + (int) threadIdx.x * kItems;
	uint32_t id[kItems];
	bool fl[kItems];
	int mine = 0;
#pragma unroll
	for (int k = 0; k < kItems; ++k) {
		const int p = p0 + k;
		fl[k] = false;
		id[k] = 0;
		if (p < end) {
			id[k] = ids[p];
			fl[k] = goesLeft(id[k], p, tk, s, f, cen);
			mine += fl[k] ? 1 : 0;
		}
	}
	int rank = leftBefore + blockExclusiveScan(mine, sW, dummy);
#pragma unroll
	for (int k = 0; k < kItems; ++k) {
		const int p = p0 + k;
		if (p < end) {
			// left: lo + (left elements before p); right: lo + nLeft + (right elements before p)
			const int dst = fl[k] ? tk.lo + rank : tk.lo + s.nLeft + (p - tk.lo - rank);
			rank += fl[k] ? 1 : 0;
			if (dst < tk.lo || dst >= tk.hi) {
				atomicExch(&ctr[kCtrError], 1u);
				continue;
			}
			idsOut[dst] = id[k];
			sorted[dst] = id[k];
		}
	}
}

// ------------------------------------------------------------------ block phase (ranges 2..kBigTask)

// A range of up to 32 elements built to its leaves by one warp. Lane j holds the element at relative
// position j of the range; `sx` is the warp's 32-int exchange area, `st` its 16-entry range stack.
__device__ void warpBuild(int a, int cnt, int node, int base, uint32_t* sIds, const float4* __restrict__ gLo,
                          const float4* __restrict__ gHi, const float4* __restrict__ gCen, int* sx, int4* st, BinNode* bin,
                          int32_t* rangeFirst, int32_t* rangeLast, uint32_t* ctr)
{
	const int lane = threadIdx.x & 31;
	const bool has = lane < cnt;
	uint32_t id = has ? sIds[a + lane] : 0u;
	float4 l = has ? gLo[id] : make_float4(0, 0, 0, 0);
	float4 h = has ? gHi[id] : make_float4(0, 0, 0, 0);
	float4 c = has ? gCen[id] : make_float4(0, 0, 0, 0);
	int top = 0;
	if (lane == 0) {
		st[0] = make_int4(0, cnt, node, 0);
	}
	top = 1;
	__syncwarp();
	while (top > 0) {
		const int4 tk = st[top - 1];
		__syncwarp();
		--top;
		const int x = tk.x, y = tk.y, nd = tk.z;
		const bool in = lane >= x && lane < y;
		Bounds12 b;
		b.clear();
		if (in) {
			b.add(l, h, c);
		}
		b.warpReduce();
		AxisFrame fr[3];
		int myBin[3];
#pragma unroll
		for (int ax = 0; ax < 3; ++ax) {
			fr[ax] = axisFrame(b.w, ax);
			myBin[ax] = fr[ax].valid ? binOf(comp3(c, ax), fr[ax].cmin, fr[ax].scale) : 0;
		}
		// Candidate split `lane` (between bins lane-1 and lane) of each axis: left = elements with a
		// smaller bin.
		uint32_t L[3][6], R[3][6];
		int lc[3] = {0, 0, 0}, rc[3] = {0, 0, 0};
#pragma unroll
		for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
			for (int k = 0; k < 6; ++k) {
				L[ax][k] = R[ax][k] = k < 3 ? kEmptyLo : kEmptyHi;
			}
		}
		for (int j = x; j < y; ++j) {
			const uint32_t w0 = __shfl_sync(0xffffffffu, ordered(l.x), j), w1 = __shfl_sync(0xffffffffu, ordered(l.y), j),
			               w2 = __shfl_sync(0xffffffffu, ordered(l.z), j), w3 = __shfl_sync(0xffffffffu, ordered(h.x), j),
			               w4 = __shfl_sync(0xffffffffu, ordered(h.y), j), w5 = __shfl_sync(0xffffffffu, ordered(h.z), j);
#pragma unroll
			for (int ax = 0; ax < 3; ++ax) {
				const int bj = __shfl_sync(0xffffffffu, myBin[ax], j);
				const bool left = bj < lane;
				uint32_t* D = left ? L[ax] : R[ax];
				D[0] = min(D[0], w0);
				D[1] = min(D[1], w1);
				D[2] = min(D[2], w2);
				D[3] = max(D[3], w3);
				D[4] = max(D[4], w4);
				D[5] = max(D[5], w5);
				lc[ax] += left ? 1 : 0;
				rc[ax] += left ? 0 : 1;
			}
		}
		float bestCost = kInf;
		int bestKey = 1 << 30, bestLeft = 0;
#pragma unroll
		for (int ax = 0; ax < 3; ++ax) {
			if (fr[ax].valid && lane >= 1 && lc[ax] > 0 && rc[ax] > 0) {
				const float ha = halfAreaOf(unordered(L[ax][0]), unordered(L[ax][1]), unordered(L[ax][2]), unordered(L[ax][3]),
				                            unordered(L[ax][4]), unordered(L[ax][5]));
				const float hb = halfAreaOf(unordered(R[ax][0]), unordered(R[ax][1]), unordered(R[ax][2]), unordered(R[ax][3]),
				                            unordered(R[ax][4]), unordered(R[ax][5]));
				const float cost = __fadd_rn(__fmul_rn(ha, (float) lc[ax]), __fmul_rn(hb, (float) rc[ax]));
				if (cost < bestCost) {
					bestCost = cost;
					bestKey = ax * kBins + lane;
					bestLeft = lc[ax];
				}
			}
		}
#pragma unroll
		for (int off = 16; off >= 1; off >>= 1) {
			const float oc = __shfl_xor_sync(0xffffffffu, bestCost, off);
			const int ok = __shfl_xor_sync(0xffffffffu, bestKey, off);
			const int ol = __shfl_xor_sync(0xffffffffu, bestLeft, off);
			if (oc < bestCost || (oc == bestCost && ok < bestKey)) {
				bestCost = oc;
				bestKey = ok;
				bestLeft = ol;
			}
		}
		const bool mid = bestKey >= (1 << 30);
		const int axis = mid ? -1 : bestKey / kBins, split = mid ? 0 : bestKey % kBins;
		const int nLeft = mid ? (x + y) / 2 - x : bestLeft;
		// stable partition of lanes [x, y)
		const bool goLeft = in && (mid ? lane < x + nLeft : myBin[axis] < split);
		const uint32_t ballot = __ballot_sync(0xffffffffu, goLeft);
		const int leftRank = __popc(ballot & ((1u << lane) - 1u));
		int dst = !in ? lane : (goLeft ? x + leftRank : x + nLeft + (lane - x - leftRank));
		if (dst < 0 || dst >= 32) {
			atomicExch(&ctr[kCtrError], 1u);
			dst = lane;
		}
		sx[dst] = lane;
		__syncwarp();
		const int src = sx[lane];
		__syncwarp();
		id = __shfl_sync(0xffffffffu, id, src);
		l = make_float4(__shfl_sync(0xffffffffu, l.x, src), __shfl_sync(0xffffffffu, l.y, src), __shfl_sync(0xffffffffu, l.z, src), 0.0f);
		h = make_float4(__shfl_sync(0xffffffffu, h.x, src), __shfl_sync(0xffffffffu, h.y, src), __shfl_sync(0xffffffffu, h.z, src), 0.0f);
		c = make_float4(__shfl_sync(0xffffffffu, c.x, src), __shfl_sync(0xffffffffu, c.y, src), __shfl_sync(0xffffffffu, c.z, src), 0.0f);
		const int pushes = (y - (x + nLeft) >= 2 ? 1 : 0) + (nLeft >= 2 ? 1 : 0);
		if (lane == 0) {
			const int g0 = base + a; // global sorted position of relative position 0
			int32_t left, right;
			emitNode(nd, g0 + x, g0 + y, nLeft, b.w, bin, rangeFirst, rangeLast, ctr, left, right);
			if (top + pushes > 16) {
				atomicExch(&ctr[kCtrError], 1u);
			} else {
				if (y - (x + nLeft) >= 2) {
					st[top] = make_int4(x + nLeft, y, right, 0);
				}
				if (nLeft >= 2) {
					st[top + ((y - (x + nLeft) >= 2) ? 1 : 0)] = make_int4(x, x + nLeft, left, 0);
				}
			}
		}
		top = top + pushes > 16 ? top : top + pushes;
		__syncwarp();
	}
	if (has) {
		sIds[a + lane] = id;
	}
}

struct BlockShared
{
	uint32_t ids[kBigTask];
	uint32_t tmp[kBigTask];
	uint32_t bins[kTaskBinWords];
	uint32_t red[kWarps][12];
	uint32_t bounds[12];
	int scan[kWarps];
	int4 stack[64];          // pending ranges above kSmallTask: disjoint, so at most kBigTask / 33
	int4 small[kBigTask / 2]; // ranges of 2..kSmallTask elements, built by warps at the end
	int4 warpStack[kWarps][16];
	int warpX[kWarps][32];
	int top, nSmall;
	int have; // the range popped for this iteration exists (written by thread 0, read by all)
	int4 cur;
	SahSplit split;
};

__global__ void __launch_bounds__(kThreads) kSahBlock(const SahTask* __restrict__ tasks, const float4* __restrict__ gLo,
                                                      const float4* __restrict__ gHi, const float4* __restrict__ gCen,
                                                      uint32_t* __restrict__ sorted, BinNode* bin, int32_t* rangeFirst,
                                                      int32_t* rangeLast, uint32_t* ctr)
{
	__shared__ BlockShared S;
	const SahTask task = tasks[blockIdx.x];
	const int base = task.lo, cnt = task.hi - task.lo;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
		S.ids[i] = sorted[base + i];
	}
	if (threadIdx.x == 0) {
		S.top = 0;
		S.nSmall = 0;
		if (cnt > kSmallTask) {
			S.stack[S.top++] = make_int4(0, cnt, task.node, 0);
		} else {
			S.small[S.nSmall++] = make_int4(0, cnt, task.node, 0);
		}
	}
	__syncthreads();
	for (;;) {
		// Thread 0 pops; every thread decides from the same popped flag after the barrier, which thread 0
		// rewrites only after the body's barriers (a loop test on S.top itself would race with the pop).
		if (threadIdx.x == 0) {
			S.have = S.top > 0 ? 1 : 0;
			if (S.have) {
				S.cur = S.stack[--S.top];
			}
		}
		__syncthreads();
		if (!S.have) {
			break;
		}
		const int a = S.cur.x, b = S.cur.y, node = S.cur.z;
		// bounds
		Bounds12 bd;
		bd.clear();
		for (int i = a + (int) threadIdx.x; i < b; i += blockDim.x) {
			const uint32_t id = S.ids[i];
			bd.add(gLo[id], gHi[id], gCen[id]);
		}
		bd.warpReduce();
		if (lane == 0) {
#pragma unroll
			for (int k = 0; k < 12; ++k) {
				S.red[warp][k] = bd.w[k];
			}
		}
		for (int k = threadIdx.x; k < kTaskBinWords; k += blockDim.x) {
			const int w = k % kBinWords;
			S.bins[k] = w < 3 ? kEmptyLo : (w < 6 ? kEmptyHi : 0u);
		}
		__syncthreads();
		if (threadIdx.x < 12) {
			const int k = threadIdx.x;
			uint32_t v = S.red[0][k];
			for (int w = 1; w < kWarps; ++w) {
				v = isMinWord(k) ? min(v, S.red[w][k]) : max(v, S.red[w][k]);
			}
			S.bounds[k] = v;
		}
		__syncthreads();
		// bins
		AxisFrame fr[3];
#pragma unroll
		for (int ax = 0; ax < 3; ++ax) {
			fr[ax] = axisFrame(S.bounds, ax);
		}
		for (int i = a + (int) threadIdx.x; i < b; i += blockDim.x) {
			const uint32_t id = S.ids[i];
			const float4 l = gLo[id], h = gHi[id], c = gCen[id];
#pragma unroll
			for (int ax = 0; ax < 3; ++ax) {
				if (!fr[ax].valid) {
					continue;
				}
				uint32_t* bb = S.bins + (ax * kBins + binOf(comp3(c, ax), fr[ax].cmin, fr[ax].scale)) * kBinWords;
				atomicMin(&bb[0], ordered(l.x));
				atomicMin(&bb[1], ordered(l.y));
				atomicMin(&bb[2], ordered(l.z));
				atomicMax(&bb[3], ordered(h.x));
				atomicMax(&bb[4], ordered(h.y));
				atomicMax(&bb[5], ordered(h.z));
				atomicAdd(&bb[6], 1u);
			}
		}
		__syncthreads();
		if (warp == 0) {
			SahSplit s = warpBestSplit(S.bins, S.bounds, lane);
			if (s.axis < 0) {
				s.nLeft = (a + b) / 2 - a;
			}
			if (lane == 0) {
				S.split = s;
			}
		}
		__syncthreads();
		const SahSplit s = S.split;
		// stable partition of [a, b): runs of consecutive elements per thread
		const int len = b - a;
		const int per = (len + kThreads - 1) / kThreads;
		const int p0 = a + (int) threadIdx.x * per;
		const int p1 = min(b, p0 + per);
		const AxisFrame f = s.axis >= 0 ? fr[s.axis] : AxisFrame{0.0f, 0.0f, false};
		int mine = 0;
		for (int p = p0; p < p1; ++p) {
			const bool gl = s.axis < 0 ? p < a + s.nLeft : binOf(comp3(gCen[S.ids[p]], s.axis), f.cmin, f.scale) < s.bin;
			mine += gl ? 1 : 0;
		}
		int total;
		int rank = blockExclusiveScan(mine, S.scan, total);
		for (int p = p0; p < p1; ++p) {
			const uint32_t id = S.ids[p];
			const bool gl = s.axis < 0 ? p < a + s.nLeft : binOf(comp3(gCen[id], s.axis), f.cmin, f.scale) < s.bin;
			const int dst = gl ? a + rank : a + s.nLeft + (p - a - rank);
			rank += gl ? 1 : 0;
			if (dst < a || dst >= b) {
				atomicExch(&ctr[kCtrError], 1u);
				continue;
			}
			S.tmp[dst] = id;
		}
		__syncthreads();
		for (int i = a + (int) threadIdx.x; i < b; i += blockDim.x) {
			S.ids[i] = S.tmp[i];
		}
		if (threadIdx.x == 0) {
			int32_t left, right;
			emitNode(node, base + a, base + b, s.nLeft, S.bounds, bin, rangeFirst, rangeLast, ctr, left, right);
			const int mid = a + s.nLeft;
			const int r0[2] = {a, mid}, r1[2] = {mid, b};
			const int cl[2] = {left, right};
			for (int q = 0; q < 2; ++q) {
				const int n = r1[q] - r0[q];
				if (n > kSmallTask && S.top < 64) {
					S.stack[S.top++] = make_int4(r0[q], r1[q], cl[q], 0);
				} else if (n >= 2 && n <= kSmallTask && S.nSmall < kBigTask / 2) {
					S.small[S.nSmall++] = make_int4(r0[q], r1[q], cl[q], 0);
				} else if (n >= 2) {
					atomicExch(&ctr[kCtrError], 1u);
				}
			}
		}
		__syncthreads();
	}
	// ranges of up to 32 elements, one warp each
	for (int k = warp; k < S.nSmall; k += kWarps) {
		const int4 t = S.small[k];
		warpBuild(t.x, t.y - t.x, t.z, base, S.ids, gLo, gHi, gCen, S.warpX[warp], S.warpStack[warp], bin, rangeFirst, rangeLast, ctr);
	}
	__syncthreads();
	for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
		sorted[base + i] = S.ids[i];
	}
}

inline int blocksFor(int n, int b) { return (n + b - 1) / b; }

template<class T>
T* sahAlloc(size_t count, cudaStream_t s)
{
	void* p = nullptr;
	RGL_SAH_OK(cudaMallocAsync(&p, sizeof(T) * (count ? count : 1), s));
	return static_cast<T*>(p);
}

} // namespace

void buildSahTopologyDevice(const float4* lo, const float4* hi, int n, BinNode* bin, int32_t* rangeFirst, int32_t* rangeLast,
                            uint32_t* sortedIds, cudaStream_t s)
{
	if (n <= 0) {
		return;
	}
	float4* cen = sahAlloc<float4>(n, s);
	uint32_t* idsA = sahAlloc<uint32_t>(n, s);
	uint32_t* idsB = sahAlloc<uint32_t>(n, s);
	kSahInit<<<blocksFor(n, 256), 256, 0, s>>>(lo, hi, n, cen, idsA, sortedIds);
	countLaunch();
	if (n < 2) {
		RGL_SAH_OK(cudaFreeAsync(cen, s));
		RGL_SAH_OK(cudaFreeAsync(idsA, s));
		RGL_SAH_OK(cudaFreeAsync(idsB, s));
		return;
	}
	const int maxBig = n / (kBigTask + 1) + 1;         // disjoint ranges above kBigTask
	const int maxBlock = n / 2 + 1;                     // disjoint ranges of at least 2
	SahTask* cur = sahAlloc<SahTask>(maxBig, s);
	SahTask* nxt = sahAlloc<SahTask>(maxBig, s);
	SahTask* blockTasks = sahAlloc<SahTask>(maxBlock, s);
	SahSplit* splits = sahAlloc<SahSplit>(maxBig, s);
	uint32_t* bounds = sahAlloc<uint32_t>((size_t) maxBig * 12, s);
	uint32_t* bins = sahAlloc<uint32_t>((size_t) maxBig * kTaskBinWords, s);
	const int maxChunks = n / kChunk + maxBig + 1;
	int32_t* chunkBase = sahAlloc<int32_t>(maxBig + 1, s);
	int32_t* chunkLeft = sahAlloc<int32_t>(maxChunks, s);
	uint32_t* ctr = sahAlloc<uint32_t>(kCtrWords, s);
	uint32_t* hostCtr = nullptr;
	RGL_SAH_OK(cudaMallocHost(&hostCtr, sizeof(uint32_t) * kCtrWords));

	uint32_t init[kCtrWords] = {1u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
	const SahTask root{0, n, 0, 0};
	int nCur = 0;
	if (n > kBigTask) {
		RGL_SAH_OK(cudaMemcpyAsync(cur, &root, sizeof(root), cudaMemcpyHostToDevice, s));
		nCur = 1;
	} else {
		RGL_SAH_OK(cudaMemcpyAsync(blockTasks, &root, sizeof(root), cudaMemcpyHostToDevice, s));
		init[kCtrBlock] = 1u;
	}
	RGL_SAH_OK(cudaMemcpyAsync(ctr, init, sizeof(init), cudaMemcpyHostToDevice, s));
	uint32_t* idsCur = idsA;
	uint32_t* idsNext = idsB;
	while (nCur > 0) {
		kSahLevelPrep<<<1, 1024, 0, s>>>(cur, nCur, chunkBase, bounds, ctr);
		const int grid = n / kChunk + nCur + 1; // bound on the level's chunks; blocks past them return
		kSahBounds<<<grid, kThreads, 0, s>>>(cur, nCur, chunkBase, idsCur, lo, hi, cen, bounds, bins);
		kSahBins<<<grid, kThreads, 0, s>>>(cur, nCur, chunkBase, idsCur, lo, hi, cen, bounds, bins);
		RGL_SAH_OK(cudaMemsetAsync(ctr + kCtrNext, 0, sizeof(uint32_t), s));
		kSahSplit<<<blocksFor(nCur * 32, 128), 128, 0, s>>>(cur, nCur, bounds, bins, splits, bin, rangeFirst, rangeLast, nxt, blockTasks,
		                                                   ctr);
		kSahPartCount<<<grid, kThreads, 0, s>>>(cur, nCur, chunkBase, idsCur, cen, bounds, splits, chunkLeft);
		kSahPartScatter<<<grid, kThreads, 0, s>>>(cur, nCur, chunkBase, idsCur, cen, bounds, splits, chunkLeft, idsNext, sortedIds, ctr);
		countLaunch(6);
		RGL_SAH_OK(cudaMemcpyAsync(hostCtr, ctr, sizeof(uint32_t) * kCtrWords, cudaMemcpyDeviceToHost, s));
		RGL_SAH_OK(cudaStreamSynchronize(s));
		nCur = (int) hostCtr[kCtrNext];
		std::swap(cur, nxt);
		std::swap(idsCur, idsNext);
	}
	RGL_SAH_OK(cudaMemcpyAsync(hostCtr, ctr, sizeof(uint32_t) * kCtrWords, cudaMemcpyDeviceToHost, s));
	RGL_SAH_OK(cudaStreamSynchronize(s));
	const int nBlock = (int) hostCtr[kCtrBlock];
	if (nBlock > 0) {
		kSahBlock<<<nBlock, kThreads, 0, s>>>(blockTasks, lo, hi, cen, sortedIds, bin, rangeFirst, rangeLast, ctr);
		countLaunch();
	}
	RGL_SAH_OK(cudaMemcpyAsync(hostCtr, ctr, sizeof(uint32_t) * kCtrWords, cudaMemcpyDeviceToHost, s));
	void* temps[] = {cen, idsA, idsB, cur, nxt, blockTasks, splits, bounds, bins, chunkBase, chunkLeft, ctr};
	for (void* p : temps) {
		RGL_SAH_OK(cudaFreeAsync(p, s));
	}
	RGL_SAH_OK(cudaStreamSynchronize(s));
	const uint32_t nodes = hostCtr[kCtrNodes], error = hostCtr[kCtrError];
	RGL_SAH_OK(cudaFreeHost(hostCtr));
	if (error != 0) {
		throw std::runtime_error("SAH build: a partition or range stack index left its range");
	}
	if (nodes != (uint32_t) (n - 1)) {
		throw std::runtime_error("SAH build: " + std::to_string(nodes) + " binary nodes for " + std::to_string(n) + " primitives");
	}
}

namespace {
static_assert(kBigTask == kSahSmallMax, "one block builds ranges up to kSahSmallMax primitives");

// Root task and control words of a one-block build.
__global__ void kSahSmallRoot(SahTask* task, uint32_t* ctr, int n)
{
	if (threadIdx.x < kCtrWords) {
		ctr[threadIdx.x] = (threadIdx.x == kCtrNodes || threadIdx.x == kCtrBlock) ? 1u : 0u;
	}
	if (threadIdx.x == 0) {
		task[0] = SahTask{0, n, 0, 0};
	}
}

struct SmallScratch
{
	float4* cen;
	uint32_t* ids;
	SahTask* task;
	uint32_t* ctr;
};
SmallScratch carveSmall(void* scratch, int n)
{
	uint8_t* p = static_cast<uint8_t*>(scratch);
	auto take = [&](size_t bytes) {
		uint8_t* q = p;
		p += (bytes + 255) & ~size_t{255};
		return q;
	};
	SmallScratch s;
	s.cen = reinterpret_cast<float4*>(take(sizeof(float4) * (size_t) n));
	s.ids = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (size_t) n));
	s.task = reinterpret_cast<SahTask*>(take(sizeof(SahTask)));
	s.ctr = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * kCtrWords));
	return s;
}
} // namespace

size_t sahSmallScratchBytes(int n)
{
	auto up = [](size_t b) { return (b + 255) & ~size_t{255}; };
	return up(sizeof(float4) * (size_t) n) + up(sizeof(uint32_t) * (size_t) n) + up(sizeof(SahTask)) + up(sizeof(uint32_t) * kCtrWords);
}

void enqueueSahTopologySmall(const float4* lo, const float4* hi, int n, void* scratch, BinNode* bin, int32_t* rangeFirst,
                             int32_t* rangeLast, uint32_t* sortedIds, cudaStream_t s)
{
	if (n <= 0 || n > kSahSmallMax) {
		throw std::runtime_error("SAH build: one-block topology takes 1.." + std::to_string(kSahSmallMax) + " primitives");
	}
	const SmallScratch sc = carveSmall(scratch, n);
	kSahInit<<<blocksFor(n, 256), 256, 0, s>>>(lo, hi, n, sc.cen, sc.ids, sortedIds);
	countLaunch();
	if (n >= 2) {
		kSahSmallRoot<<<1, 32, 0, s>>>(sc.task, sc.ctr, n);
		kSahBlock<<<1, kThreads, 0, s>>>(sc.task, lo, hi, sc.cen, sortedIds, bin, rangeFirst, rangeLast, sc.ctr);
		countLaunch(2);
	}
}

} // namespace rgl
