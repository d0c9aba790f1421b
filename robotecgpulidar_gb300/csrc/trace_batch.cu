// Batched multi-sensor traversal: one persistent launch casts the beams of many sensors (each an RGL
// raytrace node with its own rays, ranges, sub-ray pattern, return mode, non-hit distances and output
// buffers) through one device-resident scene.
//
// The reference runs one OptiX launch per raytrace node (src/graph/RaytraceNode.cpp:68-146); its
// per-beam work (src/gpu/optixPrograms.cu:46-216, src/gpu/nodeKernels.cu:334-422) is kept exactly,
// through the device functions shared with the single-sensor kernel (trace_kernel.cuh), so every
// sensor's output equals what its own graph run would write.
//
// Each job names its own scene, so one launch may cover sensors of several resident scenes.
//
// Scheduling: the beams of sensor j form tasks of one warp's worth of work (32 / G beams with the
// lane-group packing, 32 beams with the serial packing). A persistent grid of
// (SM count x resident blocks) blocks fetches `chunk` tasks at a time from one global counter; a
// warp maps a task to its sensor by binary search over the task prefix sums staged in shared memory.
// Sensors of uneven size therefore share the GPU without a tail per sensor.
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>

#include "trace_batch_kernel.cuh"

#define RGL_BATCH_CUDA_OK(expr)                                                                                                \
	do {                                                                                                                       \
		cudaError_t e_ = (expr);                                                                                               \
		if (e_ != cudaSuccess) {                                                                                               \
			throw std::runtime_error(std::string("CUDA error in batched traversal: ") + cudaGetErrorString(e_) + " at " #expr); \
		}                                                                                                                      \
	} while (0)

namespace rgl {

namespace {

using namespace tracedev;

// 10-bit spread for 3D Morton codes and 16-bit spread for 2D ones.
__device__ __forceinline__ uint32_t spread3(uint32_t v)
{
	v &= 0x3ffu;
	v = (v | (v << 16)) & 0x030000ffu;
	v = (v | (v << 8)) & 0x0300f00fu;
	v = (v | (v << 4)) & 0x030c30c3u;
	v = (v | (v << 2)) & 0x09249249u;
	return v;
}
__device__ __forceinline__ uint32_t spread2(uint32_t v)
{
	v &= 0xffffu;
	v = (v | (v << 8)) & 0x00ff00ffu;
	v = (v | (v << 4)) & 0x0f0f0f0fu;
	v = (v | (v << 2)) & 0x33333333u;
	v = (v | (v << 1)) & 0x55555555u;
	return v;
}

__device__ __forceinline__ uint32_t quant(float x, uint32_t levels)
{
	const float c = fminf(fmaxf(x, 0.0f), 1.0f);
	return min((uint32_t) (c * (float) levels), levels - 1u);
}

// Key = job index in bits 22..31, a 22-bit direction code below. Octahedral: the world direction
// folded onto the octahedron, 11 bits per coordinate, interleaved. Morton: the point 5 % of the world
// diagonal along the ray, 7 bits per axis over the world box, interleaved.
__global__ void kBeamKeys(const Mat34* __restrict__ rays, Mat34 tf, int hasTf, int n, uint32_t jobIndex, int order, float3 lo, float3 inv,
                          float probe, uint32_t* __restrict__ keys, uint32_t* __restrict__ values)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) {
		return;
	}
	Mat34 r = loadMat(rays + i);
	if (hasTf) {
		r = mul(tf, r); // a sensor transform folded into the traversal: key the world rays
	}
	const Vec3 o = r.rayOrigin();
	const Vec3 d = normalized(r.rayDir());
	uint32_t code = 0;
	if (order == kOrderOctahedral) {
		const float l1 = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
		float u = l1 > 0.0f ? d.x / l1 : 0.0f;
		float v = l1 > 0.0f ? d.y / l1 : 0.0f;
		if (d.z < 0.0f) {
			const float fu = (1.0f - fabsf(v)) * (u >= 0.0f ? 1.0f : -1.0f);
			const float fv = (1.0f - fabsf(u)) * (v >= 0.0f ? 1.0f : -1.0f);
			u = fu;
			v = fv;
		}
		code = (spread2(quant(u * 0.5f + 0.5f, 2048u)) << 1) | spread2(quant(v * 0.5f + 0.5f, 2048u));
	} else if (order == kOrderElevation) {
		// Rows of a scan: the sine of the elevation above the world xy plane in the high 11 bits, a
		// pseudo-angle of the azimuth (monotonic in atan2(y, x), in (-2, 2]) in the low 11 bits.
		const float l1 = fabsf(d.x) + fabsf(d.y);
		const float pa = l1 > 0.0f ? 1.0f - d.x / l1 : 0.0f;
		const float az = d.y < 0.0f ? -pa : pa;
		code = (quant(d.z * 0.5f + 0.5f, 2048u) << 11) | quant(az * 0.25f + 0.5f, 2048u);
	} else {
		const float px = (o.x + d.x * probe - lo.x) * inv.x;
		const float py = (o.y + d.y * probe - lo.y) * inv.y;
		const float pz = (o.z + d.z * probe - lo.z) * inv.z;
		code = (spread3(quant(px, 128u)) << 2) | (spread3(quant(py, 128u)) << 1) | spread3(quant(pz, 128u));
	}
	keys[i] = (jobIndex << 22) | (code & 0x3fffffu);
	values[i] = (uint32_t) i;
}

template<int MODE, bool SHADING>
const void* batchKernel(int regs)
{
	if (regs <= 64) {
		return reinterpret_cast<const void*>(&kTraceBatch<MODE, SHADING, 64>);
	}
	if (regs <= 80) {
		return reinterpret_cast<const void*>(&kTraceBatch<MODE, SHADING, 80>);
	}
	return regs <= 96 ? reinterpret_cast<const void*>(&kTraceBatch<MODE, SHADING, 96>)
	                  : reinterpret_cast<const void*>(&kTraceBatch<MODE, SHADING, 128>);
}

int residentBlocks(const void* fn, int block, size_t smem)
{
	static std::mutex m;
	static std::map<std::tuple<const void*, int, size_t>, int> cache;
	static std::map<const void*, bool> optedIn;
	std::lock_guard<std::mutex> g(m);
	auto key = std::make_tuple(fn, block, smem);
	auto it = cache.find(key);
	if (it != cache.end()) {
		return it->second;
	}
	if (!optedIn[fn]) {
		// Opt in once to the largest launch of this kernel (256-thread stack + the largest job
		// table), so no later launch, whatever its shape, exceeds the limit.
		const int most = (int) (sizeof(uint2) * kSmemStack * 256 + sizeof(int32_t) * (kMaxBatchJobs + 2));
		RGL_BATCH_CUDA_OK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, most));
		optedIn[fn] = true;
	}
	int n = 0;
	RGL_BATCH_CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, block, smem));
	n = n < 1 ? 1 : n;
	cache[key] = n;
	return n;
}

int smCount()
{
	static int n = [] {
		int dev = 0, v = 0;
		RGL_BATCH_CUDA_OK(cudaGetDevice(&dev));
		RGL_BATCH_CUDA_OK(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
		return v;
	}();
	return n;
}

} // namespace

int batchBeamsPerTask(int packing, int nSamples)
{
	if (packing == kPackSerial) {
		return 32;
	}
	const int G = nSamples < 32 ? nSamples : 32;
	return 32 / G;
}

namespace {
struct LaunchShape
{
	const void* fn;
	size_t smem;
	int grid;
};

LaunchShape batchLaunchShape(int nJobs, int maxSamples, bool shading, const BatchSchedule& s)
{
	// Sensor count (<= kMaxBatchJobs) and block size (64, 128 or 256) are checked by the caller.
	const int block = s.block;
	const int mode = s.packing == kPackSerial ? 2 : (maxSamples > 32 ? 1 : 0);
	const void* fn = nullptr;
	switch (mode * 2 + (shading ? 1 : 0)) {
		case 0: fn = batchKernel<0, false>(s.regs); break;
		case 1: fn = batchKernel<0, true>(s.regs); break;
		case 2: fn = batchKernel<1, false>(s.regs); break;
		case 3: fn = batchKernel<1, true>(s.regs); break;
		case 4: fn = batchKernel<2, false>(s.regs); break;
		default: fn = batchKernel<2, true>(s.regs); break;
	}
	const size_t smem = sizeof(uint2) * kSmemStack * block + sizeof(int32_t) * ((nJobs + 2) & ~1);
	return LaunchShape{fn, smem, smCount() * residentBlocks(fn, block, smem)};
}
} // namespace

bool isTraceBatchKernel(const void* fn)
{
	for (int regs : {64, 80, 96, 128}) {
		for (const void* k : {batchKernel<0, false>(regs), batchKernel<0, true>(regs), batchKernel<1, false>(regs), batchKernel<1, true>(regs),
		                      batchKernel<2, false>(regs), batchKernel<2, true>(regs)}) {
			if (k == fn) {
				return true;
			}
		}
	}
	return false;
}

void prepareTraceBatch(int nJobs, int maxSamples, bool shading, const BatchSchedule& s)
{
	if (nJobs > 0) {
		(void) batchLaunchShape(nJobs, maxSamples, shading, s);
	}
}

void launchTraceBatch(const BatchJob* dJobs, const int32_t* dTaskBase, int nJobs, int maxSamples, bool shading, const BatchSchedule& s,
                      uint32_t* dCounter, cudaStream_t stream, bool overlapPrevious)
{
	if (nJobs <= 0) {
		return;
	}
	const LaunchShape ls = batchLaunchShape(nJobs, maxSamples, shading, s);
	int chunk = s.chunk < 1 ? 1 : s.chunk;
	void* args[] = {(void*) &dJobs, (void*) &dTaskBase, (void*) &nJobs, (void*) &dCounter, (void*) &chunk};
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(ls.grid);
	cfg.blockDim = dim3(s.block);
	cfg.dynamicSmemBytes = ls.smem;
	cfg.stream = stream;
	cudaLaunchAttribute attr[1] = {};
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = attr;
	cfg.numAttrs = overlapPrevious ? 1 : 0;
	RGL_BATCH_CUDA_OK(cudaLaunchKernelExC(&cfg, ls.fn, args));
	countLaunch();
}

void launchBeamKeys(const Mat34* rays, const Mat34* transform, int n, uint32_t jobIndex, int order, const float* worldLo, const float* worldHi, uint32_t* keys,
                    uint32_t* values, cudaStream_t stream)
{
	if (n <= 0) {
		return;
	}
	float3 lo = make_float3(worldLo[0], worldLo[1], worldLo[2]);
	const float ex = fmaxf(worldHi[0] - worldLo[0], 1e-3f), ey = fmaxf(worldHi[1] - worldLo[1], 1e-3f), ez = fmaxf(worldHi[2] - worldLo[2], 1e-3f);
	const float probe = 0.05f * sqrtf(ex * ex + ey * ey + ez * ez);
	// The probe point may leave the world box by up to `probe`: widen the box by that much.
	lo.x -= probe;
	lo.y -= probe;
	lo.z -= probe;
	const float3 inv = make_float3(1.0f / (ex + 2 * probe), 1.0f / (ey + 2 * probe), 1.0f / (ez + 2 * probe));
	const Mat34 tf = transform ? *transform : Mat34::identity();
	kBeamKeys<<<(n + 255) / 256, 256, 0, stream>>>(rays, tf, transform ? 1 : 0, n, jobIndex, order, lo, inv, probe, keys, values);
	countLaunch();
}

} // namespace rgl
