// Compaction that allocates nothing, behind rgl_gb300_compact_by_flags_noalloc
// (include/rgl/api/extensions/gb300.h).
//
// Some callers cannot allocate device memory when they need to compact points: engines that hand
// the library only pre-allocated buffers from their own pool, real-time loops that must never enter
// the CUDA allocator (cudaMalloc/cudaFree can synchronise the device and take unbounded time), and
// processes whose device memory is reserved up front. The graph API's compaction draws its
// decoupled look-back scratch from a buffer it allocates on first use; this variant keeps that
// scratch in a file-scope __device__ array of fixed size instead, so a call touches only the
// caller's inputs and outputs plus that array.
//
// Rules for callers:
//  * at most kNoAllocMaxPoints = 2^24 (16,777,216) elements per call; more are rejected;
//  * the scratch array is 65,548 bytes and stays resident on every device that loads the library,
//    until the process exits;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress, with that
//    device current); make that first call before starting any stream capture on that device;
//  * under CUDA's lazy module loading (the default) the first call on a device also makes the driver
//    load this module, allocating device memory for its code and the array; callers that must not
//    allocate at run time make one warm-up call at initialisation, after which calls allocate nothing;
//  * all calls share the array and clear the words they use at the start of each call; calls whose
//    work overlaps on the GPU (other streams, other host threads) race on it, so serialise them;
//  * the call waits for its own work on the given stream before it returns.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

#include "common.hpp"
#include "kernels.hpp"

namespace rgl {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 4;
constexpr int kTile = kThreads * kItems;
constexpr int kMaxTiles = kNoAllocMaxPoints / kTile;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1u;
constexpr int kSpinLimit = 1 << 24;
// Scratch words: [0] error flag, [1] kept count, [2] tile ticket, [3 ..] per-tile look-back status.
constexpr int kScratchWords = 3 + kMaxTiles;

static __device__ __align__(256) uint32_t noAllocScratch[kScratchWords];

__device__ __forceinline__ void copyBytes(const uint8_t* src, uint8_t* dst, int size)
{
	if (size % 4 == 0 && ((uintptr_t) src % 4) == 0 && ((uintptr_t) dst % 4) == 0) {
		for (int w = 0; w < size / 4; ++w) {
			reinterpret_cast<uint32_t*>(dst)[w] = reinterpret_cast<const uint32_t*>(src)[w];
		}
	} else {
		for (int b = 0; b < size; ++b) {
			dst[b] = src[b];
		}
	}
}

// Stable single-pass compaction of one field: keeps element i when flags[i] != 0.
__global__ void __launch_bounds__(kThreads) kCompactNoAlloc(const int32_t* __restrict__ flags, int n,
                                                            const uint8_t* __restrict__ src, int elemSize,
                                                            uint8_t* __restrict__ dst, uint32_t* scratch)
{
	__shared__ uint32_t warpSums[kThreads / 32];
	__shared__ uint32_t tileBase;
	__shared__ int tileShared;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	if (tid == 0) {
		tileShared = (int) atomicAdd(&scratch[2], 1u);
	}
	__syncthreads();
	const int tile = tileShared;
	const int first = tile * kTile + tid * kItems;
	int keep[kItems];
	int cnt = 0;
#pragma unroll
	for (int k = 0; k < kItems; ++k) {
		const int i = first + k;
		keep[k] = (i < n) && flags[i] != 0;
		cnt += keep[k];
	}
	int incl = cnt;
#pragma unroll
	for (int off = 1; off < 32; off <<= 1) {
		const int v = __shfl_up_sync(0xffffffffu, incl, off);
		if (lane >= off) {
			incl += v;
		}
	}
	if (lane == 31) {
		warpSums[warp] = (uint32_t) incl;
	}
	__syncthreads();
	if (tid == 0) {
		uint32_t run = 0;
		for (int w = 0; w < kThreads / 32; ++w) {
			const uint32_t v = warpSums[w];
			warpSums[w] = run;
			run += v;
		}
		uint32_t* status = scratch + 3;
		uint32_t prefix = 0;
		if (tile == 0) {
			atomicExch(&status[0], kFlagInc | run);
		} else {
			atomicExch(&status[tile], kFlagAgg | run);
			int k = tile - 1, spins = 0;
			while (k >= 0) {
				const uint32_t s = *((volatile uint32_t*) &status[k]);
				const uint32_t fl = s & ~kValueMask;
				if (fl == 0u) {
					if (++spins > kSpinLimit) {
						atomicExch(&scratch[0], 1u);
						break;
					}
					continue;
				}
				prefix += s & kValueMask;
				if (fl == kFlagInc) {
					break;
				}
				--k;
			}
			atomicExch(&status[tile], kFlagInc | (prefix + run));
		}
		tileBase = prefix;
		if (tile == (int) gridDim.x - 1) {
			scratch[1] = prefix + run;
		}
	}
	__syncthreads();
	uint32_t pos = tileBase + warpSums[warp] + (uint32_t) (incl - cnt);
#pragma unroll
	for (int k = 0; k < kItems; ++k) {
		if (keep[k]) {
			copyBytes(src + (size_t) (first + k) * elemSize, dst + (size_t) pos * elemSize, elemSize);
			++pos;
		}
	}
}

std::mutex setupMutex;
constexpr int kMaxDevices = 64;
uint32_t* scratchByDevice[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device.
uint32_t* scratchOnCurrentDevice()
{
	int dev = 0;
	RGL_CHECK_CUDA(cudaGetDevice(&dev));
	if (dev < 0 || dev >= kMaxDevices) {
		throw std::runtime_error(format("device ordinal %d is beyond the %d devices this entry point supports", dev, kMaxDevices));
	}
	std::lock_guard<std::mutex> lock(setupMutex);
	if (scratchByDevice[dev] == nullptr) {
		void* ptr = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&ptr, noAllocScratch);
		if (e != cudaSuccess) {
			throw std::runtime_error(format("cudaGetSymbolAddress of the compaction scratch failed: %s", cudaGetErrorString(e)));
		}
		scratchByDevice[dev] = static_cast<uint32_t*>(ptr);
	}
	return scratchByDevice[dev];
}

} // namespace

int32_t compactNoAlloc(const int32_t* flags, const void* src, int32_t count, int32_t elementSize, void* dst, cudaStream_t stream)
{
	if (count < 0 || count > kNoAllocMaxPoints) {
		throw InvalidAPIArgument(format("rgl_gb300_compact_by_flags_noalloc: count %d outside [0, %d] (the fixed scratch "
		                                "holds look-back state for at most %d elements)",
		                                (int) count, kNoAllocMaxPoints, kNoAllocMaxPoints));
	}
	if (elementSize <= 0 || elementSize > 256) {
		throw InvalidAPIArgument(format("rgl_gb300_compact_by_flags_noalloc: element size %d outside [1, 256]", (int) elementSize));
	}
	if (count == 0) {
		return 0;
	}
	if (flags == nullptr || src == nullptr || dst == nullptr) {
		throw InvalidAPIArgument("rgl_gb300_compact_by_flags_noalloc: flags, src and dst must be device pointers");
	}
	uint32_t* scratch = scratchOnCurrentDevice();
	const int tiles = (count + kTile - 1) / kTile;
	RGL_CHECK_CUDA(cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * (size_t) (3 + tiles), stream));
	kCompactNoAlloc<<<tiles, kThreads, 0, stream>>>(flags, count, static_cast<const uint8_t*>(src), elementSize,
	                                                static_cast<uint8_t*>(dst), scratch);
	RGL_CHECK_CUDA(cudaGetLastError());
	countLaunch();
	uint32_t head[2] = {0, 0};
	RGL_CHECK_CUDA(cudaMemcpyAsync(head, scratch, sizeof(head), cudaMemcpyDeviceToHost, stream));
	RGL_CHECK_CUDA(cudaStreamSynchronize(stream));
	if (head[0] != 0) {
		throw std::runtime_error("rgl_gb300_compact_by_flags_noalloc: decoupled look-back did not complete");
	}
	return (int32_t) head[1];
}

} // namespace rgl
