// Onesweep LSD radix sort of (uint32 key, uint32 value) pairs for the BVH builder.
//
// Algorithm: Adinets and Merrill, "Onesweep: A Faster Least Significant Digit Radix Sort for GPUs"
// (2022). One upfront histogram kernel counts all digit passes at once; each 8-bit pass is then a
// single kernel: tiles take ids in launch order from an atomic ticket, rank their keys stably with
// warp match-any, publish per-digit tile counts and resolve their global offsets with a decoupled
// look-back over the preceding tiles. Every look-back spin has an iteration limit after which the
// kernel raises the error flag instead of waiting further.
#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.hpp"

namespace rgl {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr int kSpinLimit = 1 << 24;

__global__ void kHistogram(const uint32_t* __restrict__ keys, int n, int passes, uint32_t* __restrict__ hist)
{
	__shared__ uint32_t sh[4][256];
	for (int i = threadIdx.x; i < 4 * 256; i += blockDim.x) {
		sh[i / 256][i % 256] = 0;
	}
	__syncthreads();
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		uint32_t k = keys[i];
		for (int p = 0; p < passes; ++p) {
			atomicAdd(&sh[p][(k >> (8 * p)) & 255u], 1u);
		}
	}
	__syncthreads();
	for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
		uint32_t v = sh[i / 256][i % 256];
		if (v) {
			atomicAdd(&hist[i], v);
		}
	}
}

// In-place exclusive scan of each pass's 256 digit counts (one block of 256 threads).
__global__ void kScanHistogram(uint32_t* hist, int passes)
{
	__shared__ uint32_t s[256];
	for (int p = 0; p < passes; ++p) {
		uint32_t v = hist[p * 256 + threadIdx.x];
		s[threadIdx.x] = v;
		__syncthreads();
		for (int off = 1; off < 256; off <<= 1) {
			uint32_t t = threadIdx.x >= off ? s[threadIdx.x - off] : 0u;
			__syncthreads();
			s[threadIdx.x] += t;
			__syncthreads();
		}
		hist[p * 256 + threadIdx.x] = s[threadIdx.x] - v;
		__syncthreads();
	}
}

__global__ void __launch_bounds__(kThreads) kOnesweep(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                      uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int n, int shift,
                                                      const uint32_t* __restrict__ digitOffsets, uint32_t* tileStatus,
                                                      uint32_t* tileTicket, int32_t* errorFlag)
{
	__shared__ uint32_t warpHist[kWarps][257];
	__shared__ uint32_t digitBase[256];
	__shared__ int tileShared;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	if (tid == 0) {
		tileShared = (int) atomicAdd(tileTicket, 1u);
	}
	for (int i = tid; i < kWarps * 257; i += kThreads) {
		(&warpHist[0][0])[i] = 0;
	}
	__syncthreads();
	const int tile = tileShared;
	const long base = (long) tile * kTile + (long) warp * (kItems * 32);

	uint32_t key[kItems], val[kItems], rank[kItems];
	int dig[kItems];
	const uint32_t ltMask = (1u << lane) - 1u;
#pragma unroll
	for (int r = 0; r < kItems; ++r) {
		long idx = base + r * 32 + lane;
		bool valid = idx < n;
		key[r] = valid ? kin[idx] : 0u;
		val[r] = valid ? vin[idx] : 0u;
		int d = valid ? (int) ((key[r] >> shift) & 255u) : 256;
		dig[r] = d;
		uint32_t peers = __match_any_sync(0xffffffffu, d);
		int leader = __ffs(peers) - 1;
		uint32_t before = warpHist[warp][d];
		__syncwarp();
		rank[r] = before + __popc(peers & ltMask);
		if (lane == leader) {
			warpHist[warp][d] = before + __popc(peers);
		}
		__syncwarp();
	}
	__syncthreads();

	// Per digit: exclusive offsets across warps, tile total, decoupled look-back.
	{
		const int d = tid;
		uint32_t run = 0;
		for (int w = 0; w < kWarps; ++w) {
			uint32_t c = warpHist[w][d];
			warpHist[w][d] = run;
			run += c;
		}
		uint32_t* status = tileStatus + (size_t) tile * 256 + d;
		uint32_t prefix = 0;
		if (tile == 0) {
			atomicExch(status, kFlagInc | run);
		} else {
			atomicExch(status, kFlagAgg | run);
			int k = tile - 1;
			int spins = 0;
			while (k >= 0) {
				uint32_t s = *((volatile uint32_t*) (tileStatus + (size_t) k * 256 + d));
				uint32_t flag = s & ~kValueMask;
				if (flag == 0u) {
					if (++spins > kSpinLimit) {
						*(volatile int32_t*) errorFlag = 1;
						break;
					}
					continue;
				}
				prefix += s & kValueMask;
				if (flag == kFlagInc) {
					break;
				}
				--k;
			}
			atomicExch(status, kFlagInc | (prefix + run));
		}
		digitBase[d] = digitOffsets[d] + prefix;
	}
	__syncthreads();

#pragma unroll
	for (int r = 0; r < kItems; ++r) {
		int d = dig[r];
		if (d < 256) {
			uint32_t pos = digitBase[d] + warpHist[warp][d] + rank[r];
			kout[pos] = key[r];
			vout[pos] = val[r];
		}
	}
}

} // namespace

size_t sortPairsScratchBytes(int n, int keyBits)
{
	int passes = (keyBits + 7) / 8;
	int tiles = (n + kTile - 1) / kTile;
	return sizeof(uint32_t) * (size_t) (passes * 256 + passes + (size_t) passes * tiles * 256 + 2 * (size_t) n);
}

// Sorts keys/values in place (ascending, stable). `scratch` must hold sortPairsScratchBytes(n, keyBits).
void sortPairs(uint32_t* keys, uint32_t* values, int n, int keyBits, void* scratch, int32_t* errorFlag, cudaStream_t stream)
{
	if (n <= 1) {
		return;
	}
	int passes = (keyBits + 7) / 8;
	int tiles = (n + kTile - 1) / kTile;
	uint32_t* hist = static_cast<uint32_t*>(scratch);
	uint32_t* tickets = hist + passes * 256;
	uint32_t* status = tickets + passes;
	uint32_t* k2 = status + (size_t) passes * tiles * 256;
	uint32_t* v2 = k2 + n;
	size_t zeroBytes = sizeof(uint32_t) * (size_t) (passes * 256 + passes + (size_t) passes * tiles * 256);
	cudaMemsetAsync(hist, 0, zeroBytes, stream);
	int hb = (n + 1023) / 1024;
	hb = hb > 1024 ? 1024 : hb;
	kHistogram<<<hb, 256, 0, stream>>>(keys, n, passes, hist);
	countLaunch();
	kScanHistogram<<<1, 256, 0, stream>>>(hist, passes);
	countLaunch();
	uint32_t *ki = keys, *vi = values, *ko = k2, *vo = v2;
	for (int p = 0; p < passes; ++p) {
		kOnesweep<<<tiles, kThreads, 0, stream>>>(ki, vi, ko, vo, n, 8 * p, hist + p * 256, status + (size_t) p * tiles * 256,
		                                          tickets + p, errorFlag);
		countLaunch();
		uint32_t* t = ki;
		ki = ko;
		ko = t;
		t = vi;
		vi = vo;
		vo = t;
	}
	if (ki != keys) {
		cudaMemcpyAsync(keys, ki, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream);
		cudaMemcpyAsync(values, vi, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream);
	}
}

} // namespace rgl
