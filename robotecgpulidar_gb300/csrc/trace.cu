// Lidar traversal kernel: per beam, casts the primary ray and its beam-divergence sub-rays through the
// two-level BVH, and reduces the samples to the requested returns in registers, writing RGL's
// per-point fields directly.
//
// Replaces reference src/gpu/optixPrograms.cu:46-216 (raygen + closest-hit + miss, which store 58
// samples per beam in a scratch buffer) and src/gpu/nodeKernels.cu:334-422 (kReduceDivergentBeams,
// which re-reads that buffer). The return-selection rules, including the reference's quirks, are kept:
//  * the first hit sample (in sample order) seeds first/second/last/strongest/second-strongest;
//  * a closer sample makes the old first the second; a sample strictly between first and second
//    becomes second (which, with second seeded equal to first, never happens - kept as is);
//  * last = strictly farther; strongest/second-strongest by strict intensity comparisons;
//  * a beam without hits reports sample 0's non-hit distance for every return.
#include <cuda_runtime.h>

#include "kernels.hpp"
#include "trace_core.hpp"

namespace rgl {

namespace {

constexpr int kBlock = 128;
constexpr int kSmemStack = 16;  // entries per thread in shared memory
constexpr int kLocalStack = 48; // overflow entries per thread in local memory

struct DevStack
{
	uint2* sm; // column of this thread: sm[k * kBlock]
	int sp;
	bool overflow;
	uint2 local[kLocalStack];

	__device__ void push(int32_t i, float t)
	{
		uint2 e = make_uint2((uint32_t) i, __float_as_uint(t));
		if (sp < kSmemStack) {
			sm[sp * kBlock] = e;
		} else if (sp < kSmemStack + kLocalStack) {
			local[sp - kSmemStack] = e;
		} else {
			overflow = true;
			return;
		}
		++sp;
	}
	__device__ void pop(int32_t& i, float& t)
	{
		--sp;
		uint2 e = sp < kSmemStack ? sm[sp * kBlock] : local[sp - kSmemStack];
		i = (int32_t) e.x;
		t = __uint_as_float(e.y);
	}
	__device__ int size() const { return sp; }
};

struct DevLoader
{
	__device__ WideNode node(const WideNode* base, int32_t i) const
	{
		const uint4* p = reinterpret_cast<const uint4*>(base + i);
		WideNode n;
		uint4* q = reinterpret_cast<uint4*>(&n);
		q[0] = __ldg(p);
		q[1] = __ldg(p + 1);
		q[2] = __ldg(p + 2);
		q[3] = __ldg(p + 3);
		q[4] = __ldg(p + 4);
		return n;
	}
	__device__ TriRecord tri(const TriRecord* base, int32_t i) const
	{
		const float4* p = reinterpret_cast<const float4*>(base + i);
		TriRecord t;
		float4* q = reinterpret_cast<float4*>(&t);
		q[0] = __ldg(p);
		q[1] = __ldg(p + 1);
		q[2] = __ldg(p + 2);
		return t;
	}
	__device__ const InstanceRec& instance(const InstanceRec* base, int32_t i) const { return base[i]; }
	__device__ BinNode bin(const BinNode* base, int32_t i) const
	{
		const float4* p = reinterpret_cast<const float4*>(base + i);
		BinNode n;
		float4* q = reinterpret_cast<float4*>(&n);
		q[0] = __ldg(p);
		q[1] = __ldg(p + 1);
		return n;
	}
};

struct Sample
{
	float dist;
	float intensity;
	int32_t entity;
	float nx, ny, nz;
	float cosInc;
};

__device__ __forceinline__ Mat34 loadMat(const Mat34* p)
{
	const float4* q = reinterpret_cast<const float4*>(p);
	float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
	return Mat34{{{a.x, a.y, a.z, a.w}, {b.x, b.y, b.z, b.w}, {c.x, c.y, c.z, c.w}}};
}

__global__ void __launch_bounds__(kBlock) kTrace(TraceParams p, const Mat34* __restrict__ table)
{
	extern __shared__ uint2 stackMem[];
	__shared__ Mat34 sTable[kMaxBeamSamples];
	for (int i = threadIdx.x; i < p.nSamples * 12; i += kBlock) {
		reinterpret_cast<float*>(sTable)[i] = reinterpret_cast<const float*>(table)[i];
	}
	__syncthreads();
	const int beam = blockIdx.x * kBlock + threadIdx.x;
	if (beam >= p.nRays) {
		return;
	}
	const SceneView sc = *p.scene;
	const Mat34 ray = (p.rays != nullptr) ? loadMat(p.rays + beam) : Mat34::identity();
	const float* rg = p.ranges + 2 * (p.nRanges == 1 ? 0 : beam);
	const float minRange = rg[0], maxRange = rg[1];
	const bool wantShading = p.needIntensity != 0 || (p.out.normal != nullptr) || (p.out.incidentAngle != nullptr);

	DevStack st;
	st.sm = stackMem + threadIdx.x;
	st.sp = 0;
	st.overflow = false;
	DevLoader ld;

	bool haveFirst = false;
	float nonHitDist = p.farNonHitDistance;
	Sample first{}, second{}, last{}, strongest{}, secondStrongest{};

	for (int s = 0; s < p.nSamples; ++s) {
		const Mat34 sr = (s == 0) ? ray : mul(ray, sTable[s]);
		const Vec3 o = sr.rayOrigin();
		const Vec3 d = sr.rayDir();
		HitRec h = traceClosest(sc, o, d, maxRange, st, ld);
		Sample cur;
		bool hit = false;
		if (h.inst >= 0) {
			float dist = fmul(h.t, length(d));
			if (dist < minRange) {
				if (s == 0) {
					nonHitDist = p.nearNonHitDistance;
				}
			} else {
				hit = true;
				const InstanceRec& inst = sc.instances[h.inst];
				cur.dist = dist;
				cur.entity = inst.entityId;
				cur.intensity = 0.0f;
				cur.nx = cur.ny = cur.nz = 0.0f;
				cur.cosInc = 0.0f;
				if (wantShading) {
					TriRecord tr = ld.tri(inst.tris, h.tri);
					Vec3 wa = inst.objectToWorld.point(v3(tr.v0x, tr.v0y, tr.v0z));
					Vec3 wb = inst.objectToWorld.point(v3(tr.v1x, tr.v1y, tr.v1z));
					Vec3 wc = inst.objectToWorld.point(v3(tr.v2x, tr.v2y, tr.v2z));
					Vec3 n = normalized(cross(wb - wa, wc - wa));
					float c = fabsf(dot(n, d));
					cur.nx = n.x;
					cur.ny = n.y;
					cur.nz = n.z;
					cur.cosInc = c;
					cur.intensity = fmul(p.defaultIntensity, c);
				}
			}
		} else if (s == 0) {
			nonHitDist = p.farNonHitDistance;
		}
		if (!hit) {
			continue;
		}
		if (!haveFirst) {
			first = second = last = strongest = secondStrongest = cur;
			haveFirst = true;
			continue;
		}
		if (cur.dist < first.dist) {
			second = first;
			first = cur;
		} else if (first.dist < cur.dist && cur.dist < second.dist) {
			second = cur;
		}
		if (cur.dist > last.dist) {
			last = cur;
		}
		if (cur.intensity > strongest.intensity) {
			secondStrongest = strongest;
			strongest = cur;
		} else if (strongest.intensity > cur.intensity && cur.intensity > secondStrongest.intensity) {
			secondStrongest = cur;
		}
	}
	if (st.overflow && p.errorFlag) {
		atomicExch(p.errorFlag, 1);
	}

	const Vec3 org = ray.rayOrigin();
	const Vec3 dn = normalized(ray.rayDir());
	const TraceOutputs& out = p.out;
	for (int r = 0; r < p.returnCount; ++r) {
		const size_t pi = (size_t) beam * p.returnCount + r;
		const uint32_t type = (((uint32_t) p.returnMode) >> (8 * r)) & 0xffu;
		if (out.rayIdx) {
			out.rayIdx[pi] = (uint32_t) beam;
		}
		if (!haveFirst) {
			Vec3 disp = dn * nonHitDist;
			disp.x = isnan(disp.x) ? 0.0f : disp.x;
			disp.y = isnan(disp.y) ? 0.0f : disp.y;
			disp.z = isnan(disp.z) ? 0.0f : disp.z;
			if (out.xyz) {
				Vec3 q = org + disp;
				out.xyz[3 * pi] = q.x;
				out.xyz[3 * pi + 1] = q.y;
				out.xyz[3 * pi + 2] = q.z;
			}
			if (out.distance) out.distance[pi] = nonHitDist;
			if (out.isHit) out.isHit[pi] = 0;
			if (out.entityId) out.entityId[pi] = 0;
			if (out.returnType) out.returnType[pi] = (uint8_t) type;
			if (out.intensityF32) out.intensityF32[pi] = 0.0f;
			if (out.intensityU8) out.intensityU8[pi] = 0;
			if (out.normal) {
				out.normal[3 * pi] = __int_as_float(0x7fc00000);
				out.normal[3 * pi + 1] = __int_as_float(0x7fc00000);
				out.normal[3 * pi + 2] = __int_as_float(0x7fc00000);
			}
			if (out.incidentAngle) out.incidentAngle[pi] = __int_as_float(0x7fc00000);
			if (out.laserRetro) out.laserRetro[pi] = 0.0f;
			continue;
		}
		const Sample* sel = nullptr;
		if (type == 4u) sel = &first;
		else if (type == 3u) sel = &second;
		else if (type == 2u) sel = &last;
		else if (type == 1u) sel = &strongest;
		else if (type == 5u) sel = &secondStrongest;
		if (sel == nullptr) {
			continue;
		}
		if (out.xyz) {
			Vec3 q = org + dn * sel->dist;
			out.xyz[3 * pi] = q.x;
			out.xyz[3 * pi + 1] = q.y;
			out.xyz[3 * pi + 2] = q.z;
		}
		if (out.distance) out.distance[pi] = sel->dist;
		if (out.isHit) out.isHit[pi] = 1;
		if (out.entityId) out.entityId[pi] = sel->entity;
		if (out.returnType) out.returnType[pi] = (uint8_t) type;
		if (out.intensityF32) out.intensityF32[pi] = sel->intensity;
		if (out.intensityU8) out.intensityU8[pi] = sel->intensity < 255.0f ? (uint8_t) roundf(sel->intensity) : (uint8_t) 255;
		if (out.normal) {
			out.normal[3 * pi] = sel->nx;
			out.normal[3 * pi + 1] = sel->ny;
			out.normal[3 * pi + 2] = sel->nz;
		}
		if (out.incidentAngle) out.incidentAngle[pi] = acosf(sel->cosInc);
		if (out.laserRetro) out.laserRetro[pi] = 0.0f;
	}
}

} // namespace

void launchTrace(const TraceParams& p, const Mat34* dSampleTable, cudaStream_t stream)
{
	if (p.nRays <= 0) {
		return;
	}
	int grid = (p.nRays + kBlock - 1) / kBlock;
	size_t smem = sizeof(uint2) * kSmemStack * kBlock;
	kTrace<<<grid, kBlock, smem, stream>>>(p, dSampleTable);
	countLaunch();
}

} // namespace rgl
