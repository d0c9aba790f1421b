// Segmented stream compaction for served batches: the points of many requests (segments), each with
// int32 is-hit flags and XYZ / distance / entity-id fields, compacted into per-request outputs in
// three launches for the whole batch:
//   kSegCount    one block per 1024-point tile: number of kept points in the tile;
//   kSegScan     one block per segment: exclusive scan of its tile counts, and the segment's total;
//   kSegScatter  one block per tile: in-tile ranks from warp ballots gather the kept points into shared
//                memory, then the block writes the tile's contiguous output ranges word by word.
// The outputs are usually pinned host memory mapped for the device (the server's result arena), which
// the GPU writes across the host link: there, stores from consecutive lanes to consecutive words (full
// 128-byte lines) run several times faster than each kept point storing its own 12- and 4-byte
// pieces at scattered offsets.
// Order is preserved, so each segment's output equals a compaction of that segment alone (reference
// CompactByFieldPointsNode semantics, src/graph/CompactByFieldPointsNode.cpp:33-105: keep points
// whose flag is non-zero, in order). HBM-bound: flags are read twice, fields once, kept points
// written once.
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "kernels.hpp"

namespace rgl {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = kSegTile / kThreads;

__device__ __forceinline__ int findSegment(const int32_t* sBase, int nSeg, int t)
{
	int lo = 0, hi = nSeg;
	while (hi - lo > 1) {
		const int mid = (lo + hi) >> 1;
		if (sBase[mid] <= t) {
			lo = mid;
		} else {
			hi = mid;
		}
	}
	return lo;
}

__device__ __forceinline__ void stageBases(int32_t* sBase, const int32_t* tileBase, int nSeg)
{
	for (int i = threadIdx.x; i <= nSeg; i += blockDim.x) {
		sBase[i] = tileBase[i];
	}
	__syncthreads();
}

__global__ void __launch_bounds__(kThreads) kSegCount(const SegCompactJob* __restrict__ segs, const int32_t* __restrict__ tileBase,
                                                      int nSeg, uint32_t* __restrict__ tileCounts)
{
	extern __shared__ int32_t sBase[];
	__shared__ uint32_t warpSums[kThreads / 32];
	stageBases(sBase, tileBase, nSeg);
	const int t = blockIdx.x;
	const int j = findSegment(sBase, nSeg, t);
	const SegCompactJob& sg = segs[j];
	const int start = (t - sBase[j]) * kSegTile;
	uint32_t c = 0;
#pragma unroll
	for (int k = 0; k < kItems; ++k) {
		const int p = start + k * kThreads + threadIdx.x;
		c += (p < sg.nPoints && __ldg(sg.flags + p) != 0) ? 1u : 0u;
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		c += __shfl_down_sync(0xffffffffu, c, o);
	}
	if ((threadIdx.x & 31) == 0) {
		warpSums[threadIdx.x >> 5] = c;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t s = 0;
		for (int w = 0; w < kThreads / 32; ++w) {
			s += warpSums[w];
		}
		tileCounts[t] = s;
	}
}

__global__ void __launch_bounds__(1024) kSegScan(const int32_t* __restrict__ tileBase, const uint32_t* __restrict__ tileCounts,
                                                 uint32_t* __restrict__ tileOffsets, int32_t* __restrict__ counts)
{
	__shared__ uint32_t warpSums[32];
	__shared__ uint32_t carry;
	const int j = blockIdx.x;
	const int first = tileBase[j];
	const int nt = tileBase[j + 1] - first;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if (threadIdx.x == 0) {
		carry = 0;
	}
	__syncthreads();
	for (int c = 0; c < nt; c += 1024) {
		const int i = c + threadIdx.x;
		const uint32_t v = i < nt ? tileCounts[first + i] : 0u;
		uint32_t incl = v;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
			incl += lane >= o ? y : 0u;
		}
		if (lane == 31) {
			warpSums[warp] = incl;
		}
		__syncthreads();
		if (warp == 0) {
			uint32_t w = warpSums[lane];
			uint32_t wi = w;
#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
				wi += lane >= o ? y : 0u;
			}
			warpSums[lane] = wi - w; // exclusive prefix of warp totals
		}
		__syncthreads();
		const uint32_t base = carry;
		if (i < nt) {
			tileOffsets[first + i] = base + warpSums[warp] + incl - v;
		}
		__syncthreads();
		if (threadIdx.x == 1023) {
			carry = base + warpSums[warp] + incl;
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) {
		counts[j] = (int32_t) carry;
	}
}

__global__ void __launch_bounds__(kThreads) kSegScatter(const SegCompactJob* __restrict__ segs, const int32_t* __restrict__ tileBase,
                                                        int nSeg, const uint32_t* __restrict__ tileOffsets, const int32_t* __restrict__ counts)
{
	extern __shared__ int32_t sBase[];
	__shared__ uint32_t warpCounts[kThreads / 32];
	__shared__ float sXyz[3 * kSegTile];
	__shared__ float sDist[kSegTile];
	__shared__ int32_t sEnt[kSegTile];
	stageBases(sBase, tileBase, nSeg);
	const int t = blockIdx.x;
	const int j = findSegment(sBase, nSeg, t);
	const SegCompactJob& sg = segs[j];
	const int start = (t - sBase[j]) * kSegTile;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	// The tile's kept points, in order, into shared memory.
	uint32_t kept = 0;
	for (int k = 0; k < kItems; ++k) {
		const int p = start + k * kThreads + threadIdx.x;
		const bool keep = p < sg.nPoints && __ldg(sg.flags + p) != 0;
		const uint32_t ballot = __ballot_sync(0xffffffffu, keep);
		if (lane == 0) {
			warpCounts[warp] = __popc(ballot);
		}
		__syncthreads();
		uint32_t before = 0, total = 0;
		for (int w = 0; w < kThreads / 32; ++w) {
			const uint32_t cw = warpCounts[w];
			before += w < warp ? cw : 0u;
			total += cw;
		}
		if (keep) {
			const uint32_t r = kept + before + __popc(ballot & ((1u << lane) - 1u));
			sXyz[3 * r] = __ldg(sg.xyz + 3 * p);
			sXyz[3 * r + 1] = __ldg(sg.xyz + 3 * p + 1);
			sXyz[3 * r + 2] = __ldg(sg.xyz + 3 * p + 2);
			sDist[r] = __ldg(sg.dist + p);
			sEnt[r] = __ldg(sg.ent + p);
		}
		kept += total;
		__syncthreads();
	}
	// Contiguous output ranges of the tile, one word per thread and step.
	const uint32_t base = tileOffsets[t];
	float* ox = sg.outXyz + 3 * (size_t) base;
	for (uint32_t w = threadIdx.x; w < 3 * kept; w += kThreads) {
		ox[w] = sXyz[w];
	}
	float* od = (sg.packed ? sg.outXyz + 3 * (size_t) counts[j] : sg.outDist) + base;
	int32_t* oe = (sg.packed ? reinterpret_cast<int32_t*>(sg.outXyz + 4 * (size_t) counts[j]) : sg.outEnt) + base;
	for (uint32_t w = threadIdx.x; w < kept; w += kThreads) {
		od[w] = sDist[w];
		oe[w] = sEnt[w];
	}
}

__global__ void kPublishWords(const int32_t* __restrict__ src, volatile int32_t* dst, int n)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		dst[i] = src[i];
	}
}

void check(cudaError_t e, const char* what)
{
	if (e != cudaSuccess) {
		throw std::runtime_error(std::string("CUDA error in segmented compaction: ") + cudaGetErrorString(e) + " at " + what);
	}
}

} // namespace

void launchPublishWords(const int32_t* src, int32_t* dstMappedHost, int n, cudaStream_t s)
{
	if (n <= 0) {
		return;
	}
	kPublishWords<<<1, 256, 0, s>>>(src, dstMappedHost, n);
	countLaunch();
	check(cudaGetLastError(), "publish");
}

void launchSegCompact(const SegCompactJob* dSegs, const int32_t* dTileBase, int nSeg, int totalTiles, uint32_t* dTileCounts,
                      uint32_t* dTileOffsets, int32_t* dCounts, cudaStream_t s)
{
	if (nSeg <= 0) {
		return;
	}
	const size_t smem = sizeof(int32_t) * (size_t) (nSeg + 1);
	if (totalTiles > 0) {
		kSegCount<<<totalTiles, kThreads, smem, s>>>(dSegs, dTileBase, nSeg, dTileCounts);
		countLaunch();
	}
	kSegScan<<<nSeg, 1024, 0, s>>>(dTileBase, dTileCounts, dTileOffsets, dCounts);
	countLaunch();
	if (totalTiles > 0) {
		kSegScatter<<<totalTiles, kThreads, smem, s>>>(dSegs, dTileBase, nSeg, dTileOffsets, dCounts);
		countLaunch();
	}
	check(cudaGetLastError(), "launch");
}

} // namespace rgl
