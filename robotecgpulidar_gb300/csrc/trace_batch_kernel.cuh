// Device side of the persistent batch traversal: the task functions of the two packings (a beam's
// sub-rays on adjacent lanes, or one lane per beam) and the kernel template. Included by
// trace_batch.cu, which instantiates the kernels.
#pragma once

#include "trace_kernel.cuh"

namespace rgl {
namespace {

using namespace tracedev;

__device__ __forceinline__ void loadRay(const BatchJob* __restrict__ job, uint32_t beam, Mat34& ray, float& minRange, float& maxRange)
{
	ray = loadMat(job->p.rays + beam);
	if (job->hasRayTransform) {
		Mat34 tf;
#pragma unroll
		for (int r = 0; r < 3; ++r) {
#pragma unroll
			for (int c = 0; c < 4; ++c) {
				tf.m[r][c] = job->rayTransform.m[r][c];
			}
		}
		ray = mul(tf, ray);
	}
	if (job->p.ranges) {
		const float* rg = job->p.ranges + 2 * (job->p.nRanges == 1 ? 0u : beam);
		minRange = rg[0];
		maxRange = rg[1];
	} else {
		minRange = job->inlineRange[0];
		maxRange = job->inlineRange[1];
	}
}

template<int ROUNDS, bool SHADING>
__device__ __forceinline__ void laneGroupTask(const BatchJob* __restrict__ job, int task, const SceneView& sc, DevStack& st, int lane)
{
	const int G = job->groupSize;
	const int nSamples = job->p.nSamples;
	const int beamsPerTask = 32 / G;
	const int g = lane / G;
	const int sub = lane - g * G;
	const int local = task * beamsPerTask + g;
	const bool valid = g < beamsPerTask && local < job->p.nRays;
	uint32_t beam = 0;
	Mat34 ray = Mat34::identity();
	float minRange = 0.0f, maxRange = 0.0f;
	if (valid) {
		beam = job->order ? __ldg(job->order + local) : (uint32_t) local;
		loadRay(job, beam, ray, minRange, maxRange);
	}
	// A masked ray is not cast: all its samples are far non-hits (reference optixPrograms.cu:55-58).
	const bool cast = valid && !(job->p.rayMask && job->p.rayMask[beam] == 0);
	SampleVal sv[ROUNDS];
#pragma unroll
	for (int r = 0; r < ROUNDS; ++r) {
		const int s = sub + r * G;
		if (valid && !cast && s < nSamples) {
			sv[r] = emptySample();
			sv[r].dist = job->p.farNonHitDistance;
		} else if (valid && s < nSamples) {
			const Mat34 traced = SHADING ? distortRay(job->p, beam, ray) : ray;
			const Mat34 sr = (s == 0) ? traced : mul(traced, loadMat(job->samples + s));
			sv[r] = traceSample<SHADING>(job->p.nearNonHitDistance, job->p.farNonHitDistance, job->p.defaultIntensity, sc, sr, minRange,
			                             maxRange, st, s);
		} else {
			sv[r] = emptySample();
		}
	}
	const bool leader = valid && sub == 0;
	const int groupLane0 = (g < beamsPerTask) ? g * G : lane;
	ReturnReducer red;
	red.init(job->p.farNonHitDistance);
	reduceGroup<ROUNDS, SHADING>(sv, nSamples, G, groupLane0, leader, red);
	if (leader) {
		writeReturns<SHADING>(job->p, sc, job->samples, beam, ray, red);
	}
}

template<bool SHADING>
__device__ __forceinline__ void serialTask(const BatchJob* __restrict__ job, int task, const SceneView& sc, DevStack& st, int lane)
{
	const int local = task * 32 + lane;
	if (local >= job->p.nRays) {
		return;
	}
	const uint32_t beam = job->order ? __ldg(job->order + local) : (uint32_t) local;
	Mat34 ray;
	float minRange, maxRange;
	loadRay(job, beam, ray, minRange, maxRange);
	ReturnReducer red;
	red.init(job->p.farNonHitDistance);
	const int nSamples = job->p.nSamples;
	const Mat34 traced = SHADING ? distortRay(job->p, beam, ray) : ray;
	const bool cast = !(job->p.rayMask && job->p.rayMask[beam] == 0);
	for (int s = 0; s < nSamples; ++s) {
		SampleVal v = emptySample();
		v.dist = job->p.farNonHitDistance;
		if (cast) {
			const Mat34 sr = (s == 0) ? traced : mul(traced, loadMat(job->samples + s));
			v = traceSample<SHADING>(job->p.nearNonHitDistance, job->p.farNonHitDistance, job->p.defaultIntensity, sc, sr, minRange,
			                         maxRange, st, s);
		}
		red.add(s, v.hit, toSelected(v));
	}
	writeReturns<SHADING>(job->p, sc, job->samples, beam, ray, red);
}

// MODE 0: lane groups, one round; MODE 1: lane groups, two rounds (more than 32 samples); MODE 2: serial.
// REGS caps registers per thread: 64, 80 and 96 keep eight, six and five 128-thread blocks resident
// per SM (more warps to hide latency, possibly with spills); 128 avoids spills in the variants that
// hold more state. The tuner picks.
template<int MODE, bool SHADING, int REGS>
__global__ void __maxnreg__(REGS) kTraceBatch(const BatchJob* __restrict__ jobs, const int32_t* __restrict__ taskBase, int nJobs,
                                              uint32_t* counter, int chunk)
{
	// Dynamic shared memory: stack columns | task bases.
	extern __shared__ uint2 dyn[];
	int32_t* sBase = reinterpret_cast<int32_t*>(dyn + kSmemStack * blockDim.x);
	for (int i = threadIdx.x; i <= nJobs; i += blockDim.x) {
		sBase[i] = taskBase[i];
	}
	__syncthreads();
	const int total = sBase[nJobs];
	const int lane = threadIdx.x & 31;

	uint2 spill[kLocalStack];
	DevStack st;
	st.sm = dyn + threadIdx.x;
	st.spill = spill;
	st.stride = blockDim.x;
	st.sp = 0;
	st.overflow = false;

	for (;;) {
		uint32_t t0 = 0;
		if (lane == 0) {
			t0 = atomicAdd(counter, (uint32_t) chunk);
		}
		t0 = __shfl_sync(0xffffffffu, t0, 0);
		if (t0 >= (uint32_t) total) {
			break;
		}
		const int tEnd = min((int) t0 + chunk, total);
		for (int t = (int) t0; t < tEnd; ++t) {
			int lo = 0, hi = nJobs;
			while (hi - lo > 1) {
				const int mid = (lo + hi) >> 1;
				if (sBase[mid] <= t) {
					lo = mid;
				} else {
					hi = mid;
				}
			}
			const BatchJob* job = jobs + lo;
			const SceneView sc = *job->p.scene;
			if (MODE == 2) {
				serialTask<SHADING>(job, t - sBase[lo], sc, st, lane);
			} else {
				laneGroupTask<MODE + 1, SHADING>(job, t - sBase[lo], sc, st, lane);
			}
			if (st.overflow) {
				if (job->p.errorFlag) {
					*(volatile int32_t*) job->p.errorFlag = 1; // an error slot in mapped host memory
				}
				st.overflow = false;
				st.sp = 0;
			}
		}
	}
	// Every task is handed out: a traversal launched after this one with programmatic stream
	// serialization may start its blocks as this grid's blocks exit (the first warp of each block to
	// get here triggers for the block). The next launch reads nothing this one writes.
	asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
	// Launched that way itself, a launch ends only after the launch before it has completed: later work
	// on the stream, which waits for this launch, then also follows every earlier one, and each
	// launch's counter block is re-armed before the stream reaches the next launch that uses it. A
	// launch without a programmatic predecessor passes this at once.
	asm volatile("griddepcontrol.wait;" ::: "memory");
	// The last block to finish re-arms both counters for the next launch, so no launch needs a memset
	// first: every block has left the task loop when it counts itself finished.
	__syncthreads();
	if (threadIdx.x == 0) {
		__threadfence();
		if (atomicAdd(counter + 1, 1u) == gridDim.x - 1) {
			atomicExch(counter, 0u);
			atomicExch(counter + 1, 0u);
		}
	}
}

} // namespace
} // namespace rgl
