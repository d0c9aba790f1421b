// Device pieces of the persistent traversal kernel (trace_batch.cu): the traversal stack, the
// loaders, one traced sample, the in-order return selection and the per-point field writes.
//
// Return selection restates reference src/gpu/nodeKernels.cu:334-422 (kReduceDivergentBeams) with
// its quirks:
//  * the first hit sample (in sample order) seeds first/second/last/strongest/second-strongest;
//  * a closer sample makes the old first the second; a sample strictly between first and second
//    becomes second (with second seeded equal to first this never fires - kept as is);
//  * last = strictly farther; strongest/second-strongest by strict intensity comparisons;
//  * a beam without hits reports sample 0's non-hit distance (near below min range, far on a miss).
// Field writes restate nodeKernels.cu:103-207 (saveReturnAsHit / saveReturnAsNonHit).
#pragma once

#include <cuda_runtime.h>

#include "kernels.hpp"
#include "trace_core.hpp"

namespace rgl {
namespace tracedev {

constexpr int kSmemStack = 24;  // entries per thread in shared memory
constexpr int kLocalStack = 40; // overflow entries per thread in local memory

// Traversal stack: the first kSmemStack entries in this thread's shared-memory column (stride =
// threads per block), the rest in a local-memory array the kernel declares. Overflow past both is
// flagged, never written. The struct holds only scalars and pointers, so its fields live in
// registers; an array member indexed at run time would put the whole struct, the stack pointer
// included, in local memory.
struct DevStack
{
	uint2* sm;
	uint2* spill; // kLocalStack entries
	int stride;
	int sp;
	bool overflow;

	__device__ __forceinline__ void push(uint32_t a, uint32_t b)
	{
		const uint2 e = make_uint2(a, b);
		if (sp < kSmemStack) {
			sm[sp * stride] = e;
		} else if (sp < kSmemStack + kLocalStack) {
			spill[sp - kSmemStack] = e;
		} else {
			overflow = true;
			return;
		}
		++sp;
	}
	__device__ __forceinline__ void pop(uint32_t& a, uint32_t& b)
	{
		--sp;
		const uint2 e = sp < kSmemStack ? sm[sp * stride] : spill[sp - kSmemStack];
		a = e.x;
		b = e.y;
	}
	__device__ __forceinline__ int size() const { return sp; }
};

struct DevLoader
{
	__device__ __forceinline__ void nodeWords(const WideNode* base, uint32_t i, uint4& w0, uint4& w1, uint4& w2, uint4& w3,
	                                          uint4& w4) const
	{
		const uint4* p = reinterpret_cast<const uint4*>(base + i);
		w0 = __ldg(p);
		w1 = __ldg(p + 1);
		w2 = __ldg(p + 2);
		w3 = __ldg(p + 3);
		w4 = __ldg(p + 4);
	}
	__device__ __forceinline__ TriRecord tri(const TriRecord* base, int32_t i) const
	{
		const float4* p = reinterpret_cast<const float4*>(base + i);
		const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
		TriRecord t;
		t.v0x = a.x;
		t.v0y = a.y;
		t.v0z = a.z;
		t.primId = __float_as_int(a.w);
		t.v1x = b.x;
		t.v1y = b.y;
		t.v1z = b.z;
		t.pad1 = 0;
		t.v2x = c.x;
		t.v2y = c.y;
		t.v2z = c.z;
		t.pad2 = 0;
		return t;
	}
	__device__ __forceinline__ const InstanceRec& instance(const InstanceRec* base, int32_t i) const { return base[i]; }
	// primId of a leaf record (a TLAS leaf's instance index).
	__device__ __forceinline__ int32_t leafPrim(const TriRecord* base, int32_t i) const { return __ldg(&base[i].primId); }
};

// One traced sample. For non-hits `dist` holds the non-hit distance (near or far).
struct SampleVal
{
	uint32_t hit;
	float dist;
	float intensity;
	int32_t inst; // hit: instance index | sample index << 24 (entity id, laser retro, velocity read when written)
	float nx, ny, nz, cosInc;
	int32_t tri;  // SHADING: the hit's triangle record (velocity of animated meshes)
};

struct Selected
{
	float dist;
	float intensity;
	int32_t inst;
	float nx, ny, nz, cosInc;
	int32_t tri;
};

__device__ __forceinline__ SampleVal emptySample() { return SampleVal{0u, 0.0f, 0.0f, 0, 0.0f, 0.0f, 0.0f, 0.0f, -1}; }

__device__ __forceinline__ Mat34 loadMat(const Mat34* p)
{
	const float4* q = reinterpret_cast<const float4*>(p);
	float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
	return Mat34{{{a.x, a.y, a.z, a.w}, {b.x, b.y, b.z, b.w}, {c.x, c.y, c.z, c.w}}};
}

// Closest hit of sample ray `sr` (reference optixPrograms.cu:89-136): distance = t * |dir| (the
// reference's FP64 norm of the object-space offset equals this within the stated tolerance), the
// min-range rule turns a closer hit into the near non-hit without continuing, a miss gives the far
// non-hit distance. With SHADING the world normal, |cos| of the incidence and intensity are added.
constexpr int kSampleShift = 24; // instance indices stay below 1 << 24
constexpr int32_t kInstMask = (1 << kSampleShift) - 1;

// Barycentric weights (of b and of c) of point p in triangle (a, b, c), from areas; 0 for a degenerate
// triangle.
__device__ __forceinline__ void barycentric(Vec3 p, Vec3 a, Vec3 b, Vec3 c, float& u, float& w)
{
	const Vec3 n = cross(b - a, c - a);
	const float nn = dot(n, n);
	u = nn > 0.0f ? dot(cross(p - a, c - a), n) / nn : 0.0f;
	w = nn > 0.0f ? dot(cross(b - a, p - a), n) / nn : 0.0f;
}

// Intensity texel at a hit (reference optixPrograms.cu:151-166): the texture coordinates of the hit
// triangle's vertices interpolated at the hit's barycentric coordinates, point-sampled with wrap.
__device__ __noinline__ float texturedIntensity(const InstanceRec& inst, const TriRecord& tr, Vec3 hitObject)
{
	float u, w;
	barycentric(hitObject, v3(tr.v0x, tr.v0y, tr.v0z), v3(tr.v1x, tr.v1y, tr.v1z), v3(tr.v2x, tr.v2y, tr.v2z), u, w);
	const int32_t* idx = inst.indices + 3 * tr.primId;
	const float* ta = inst.texCoords + 2 * idx[0];
	const float* tb = inst.texCoords + 2 * idx[1];
	const float* tc = inst.texCoords + 2 * idx[2];
	const float wa = fsub(fsub(1.0f, u), w);
	const float tu = fadd(fadd(fmul(wa, ta[0]), fmul(u, tb[0])), fmul(w, tc[0]));
	const float tv = fadd(fadd(fmul(wa, ta[1]), fmul(u, tb[1])), fmul(w, tc[1]));
	return (float) tex2D<unsigned char>((cudaTextureObject_t) inst.intensityTexture, tu, tv);
}

template<bool SHADING>
__device__ __forceinline__ SampleVal sampleFromHit(float nearNonHit, float farNonHit, float defaultIntensity, const SceneView& sc,
                                                   const HitRec& h, Vec3 o, Vec3 d, float minRange, int sample)
{
	DevLoader ld;
	SampleVal v = emptySample();
	v.dist = farNonHit;
	if (h.inst >= 0) {
		const float dist = fmul(h.t, length(d));
		if (dist < minRange) {
			v.dist = nearNonHit;
		} else {
			const InstanceRec& inst = sc.instances[h.inst];
			v.hit = 1;
			v.dist = dist;
			v.inst = h.inst | (sample << kSampleShift);
			if (SHADING) {
				const TriRecord tr = ld.tri(inst.tris, h.tri);
				const Vec3 wa = inst.objectToWorld.point(v3(tr.v0x, tr.v0y, tr.v0z));
				const Vec3 wb = inst.objectToWorld.point(v3(tr.v1x, tr.v1y, tr.v1z));
				const Vec3 wc = inst.objectToWorld.point(v3(tr.v2x, tr.v2y, tr.v2z));
				const Vec3 n = normalized(cross(wb - wa, wc - wa));
				const float c = fabsf(dot(n, d));
				v.nx = n.x;
				v.ny = n.y;
				v.nz = n.z;
				v.cosInc = c;
				float base = defaultIntensity;
				if (inst.intensityTexture != 0) {
					base = texturedIntensity(inst, tr, worldToInstance(inst, o + d * h.t));
				}
				v.intensity = fmul(base, c);
				v.tri = h.tri;
			}
		}
	}
	return v;
}

template<bool SHADING>
__device__ __forceinline__ SampleVal traceSample(float nearNonHit, float farNonHit, float defaultIntensity, const SceneView& sc,
                                                 const Mat34& sr, float minRange, float maxRange, DevStack& st, int sample)
{
	DevLoader ld;
	const Vec3 d = sr.rayDir();
	const HitRec h = traceClosest(sc, sr.rayOrigin(), d, maxRange, st, ld);
	return sampleFromHit<SHADING>(nearNonHit, farNonHit, defaultIntensity, sc, h, sr.rayOrigin(), d, minRange, sample);
}

__device__ __forceinline__ Selected toSelected(const SampleVal& v)
{
	return Selected{v.dist, v.intensity, v.inst, v.nx, v.ny, v.nz, v.cosInc, v.tri};
}

// In-order selection over a beam's samples; add() must see samples 0, 1, 2, ... in order.
struct ReturnReducer
{
	bool haveFirst;
	float nonHitDist;
	Selected first, second, last, strongest, secondStrongest;

	__device__ __forceinline__ void init(float farNonHit)
	{
		haveFirst = false;
		nonHitDist = farNonHit;
		first = second = last = strongest = secondStrongest = Selected{0.0f, 0.0f, 0, 0.0f, 0.0f, 0.0f, 0.0f, -1};
	}
	__device__ __forceinline__ void add(int s, uint32_t hit, const Selected& cur)
	{
		if (s == 0 && !hit) {
			nonHitDist = cur.dist;
		}
		if (!hit) {
			return;
		}
		if (!haveFirst) {
			first = second = last = strongest = secondStrongest = cur;
			haveFirst = true;
			return;
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
};

// Azimuth and elevation of a sensor-frame ray pose, for rays generated in a left-handed frame with the
// rotation applied in ZXY order, Y up and Z forward (reference Mat3x4f.hpp:146-175).
__device__ __forceinline__ float rayElevation(const Mat34& m)
{
	const float v = m.m[1][2];
	return v < 1.0f ? (v > -1.0f ? asinf(v) : -1.57079632679489661923f) : 1.57079632679489661923f;
}
__device__ __forceinline__ float rayAzimuth(const Mat34& m)
{
	const float v = m.m[2][1];
	return (v < 1.0f && v > -1.0f) ? atan2f(-m.m[2][0], m.m[2][2]) : 0.0f;
}

// The pose a beam is cast from: under velocity distortion the sensor-frame ray is moved by the sensor's
// motion during the ray's time offset (reference optixPrograms.cu:60-70: translation offset * linear
// velocity, rotation offset * angular velocity in degrees, both per millisecond), else the ray itself.
// Kept out of line (like hitVelocities) so the traversal's register allocation does not pay for it.
__device__ __noinline__ Mat34 distortRayOutOfLine(const TraceParams& p, uint32_t beam, const Mat34& ray)
{
	const float off = p.timeOffsetsMs[beam];
	const float toDeg = (float) (180.0 / 3.14159265358979323846);
	const Vec3 lv = p.sensorLinearVelocity, av = p.sensorAngularVelocity;
	const Vec3 t = v3(fmul(fmul(off, lv.x), 0.001f), fmul(fmul(off, lv.y), 0.001f), fmul(fmul(off, lv.z), 0.001f));
	const Vec3 r = v3(fmul(fmul(off, fmul(av.x, toDeg)), 0.001f), fmul(fmul(off, fmul(av.y, toDeg)), 0.001f),
	                  fmul(fmul(off, fmul(av.z, toDeg)), 0.001f));
	return mul(p.sensorToWorld, mul(translationRotationDeg(t, r), mul(p.worldToSensor, ray)));
}

__device__ __forceinline__ Mat34 distortRay(const TraceParams& p, uint32_t beam, const Mat34& ray)
{
	return (p.distortion && p.timeOffsetsMs != nullptr) ? distortRayOutOfLine(p, beam, ray) : ray;
}

// Velocities of a hit (reference optixPrograms.cu:169-212): the hit point of the selected sample
// (sample pose `sr`, distance `dist`), its instance's pose one scene time step earlier, the sensor's
// velocities. Absolute velocity is the displacement since the previous pose over the time step;
// relative velocity is that velocity in the sensor frame minus the sensor's linear velocity and the
// rotation of the hit point about the sensor; radial speed is its component along the sensor-to-hit
// direction. NaN when the scene has no time step.
__device__ __noinline__ void hitVelocities(const TraceParams& p, const InstanceRec& inst, const Mat34& sr, float dist, int32_t tri,
                                            Vec3& absV, Vec3& relV, float& radial)
{
	const float nan = __int_as_float(0x7fc00000);
	absV = relV = v3(nan, nan, nan);
	radial = nan;
	if (!(p.sceneDeltaTime > 0.0f)) {
		return;
	}
	// The hit point in the instance's frame, and back in the world with the current pose, so an instance
	// whose previous pose equals the current one moves by exactly zero.
	const Vec3 d = sr.rayDir();
	const Vec3 hitObject = worldToInstance(inst, sr.rayOrigin() + d * (dist / length(d)));
	const Vec3 hitWorld = inst.objectToWorld.point(hitObject);
	Vec3 disp = v3(0.0f, 0.0f, 0.0f);
	if (inst.hasPrev) {
		disp = hitWorld - inst.prevObjectToWorld.point(hitObject);
	}
	if (inst.vertexDisplacement != nullptr && tri >= 0) {
		// Animated mesh: the triangle's vertex displacements since the previous step, rotated into the
		// world and interpolated at the hit's barycentric coordinates (reference optixPrograms.cu:185-195).
		const TriRecord& tr = inst.tris[tri];
		float u, w; // weights of vertices 1 and 2
		barycentric(hitObject, v3(tr.v0x, tr.v0y, tr.v0z), v3(tr.v1x, tr.v1y, tr.v1z), v3(tr.v2x, tr.v2y, tr.v2z), u, w);
		const int32_t* idx = inst.indices + 3 * tr.primId;
		auto vdisp = [&](int k) {
			const float* q = inst.vertexDisplacement + 3 * idx[k];
			return inst.objectToWorld.vector(v3(q[0], q[1], q[2]));
		};
		disp = disp + vdisp(0) * fsub(fsub(1.0f, u), w) + vdisp(1) * u + vdisp(2) * w;
	}
	absV = v3(disp.x / p.sceneDeltaTime, disp.y / p.sceneDeltaTime, disp.z / p.sceneDeltaTime);
	const Vec3 absInSensor = p.worldToSensorRotation.vector(absV);
	const Vec3 hitInSensor = p.worldToSensor.point(hitWorld);
	relV = (absInSensor - p.sensorLinearVelocity) + (v3(0.0f, 0.0f, 0.0f) - cross(p.sensorAngularVelocity, hitInSensor));
	radial = dot(normalized(hitInSensor), relV);
}

// Writes beam `beam`'s returns at points beam * returnCount + r. `ray` is the primary ray pose as
// given (XYZ and the beam fields use it; velocities use the pose the samples were cast from,
// distortRay). Velocities, like shading, exist only in the SHADING variants of the kernel, which a
// launch uses whenever one of those fields or velocity distortion is requested. Per return point it
// also writes the beam's shared fields
// (reference optixPrograms.cu:288-326): ray index, azimuth and elevation of the sensor-frame pose,
// ring id and time stamps (the ray's time offset under velocity distortion, else 0).
template<bool SHADING>
__device__ __forceinline__ void writeReturns(const TraceParams& p, const SceneView& sc, const Mat34* samples, uint32_t beam,
                                             const Mat34& ray, const ReturnReducer& red)
{
	const TraceOutputs& out = p.out;
	const int32_t returnMode = p.returnMode;
	const int returnCount = p.returnCount;
	const Vec3 org = ray.rayOrigin();
	const Vec3 dn = normalized(ray.rayDir());
	float azimuth = 0.0f, elevation = 0.0f;
	if (out.azimuth || out.elevation) {
		const Mat34 local = mul(p.worldToSensor, ray);
		azimuth = rayAzimuth(local);
		elevation = rayElevation(local);
	}
	const uint16_t ring = (out.ringId && p.ringIds) ? (uint16_t) p.ringIds[beam % (uint32_t) p.nRingIds] : (uint16_t) 0;
	for (int r = 0; r < returnCount; ++r) {
		const size_t pi = (size_t) beam * returnCount + r;
		const uint32_t type = (((uint32_t) returnMode) >> (8 * r)) & 0xffu;
		if (out.rayIdx) {
			out.rayIdx[pi] = beam;
		}
		if (out.azimuth) out.azimuth[pi] = azimuth;
		if (out.elevation) out.elevation[pi] = elevation;
		if (out.ringId) out.ringId[pi] = ring;
		const bool stamped = p.distortion && p.timeOffsetsMs;
		if (out.timeStampF64) out.timeStampF64[pi] = stamped ? (double) fmul(p.timeOffsetsMs[beam], 1e-3f) : 0.0;
		if (out.timeStampU32) out.timeStampU32[pi] = stamped ? (uint32_t) fmul(p.timeOffsetsMs[beam], 1e6f) : 0u;
		if (!red.haveFirst) {
			const float nonHitDist = red.nonHitDist;
			Vec3 disp = dn * nonHitDist;
			disp.x = isnan(disp.x) ? 0.0f : disp.x;
			disp.y = isnan(disp.y) ? 0.0f : disp.y;
			disp.z = isnan(disp.z) ? 0.0f : disp.z;
			if (out.xyz) {
				const Vec3 q = org + disp;
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
			if (out.absVelocity) {
				out.absVelocity[3 * pi] = out.absVelocity[3 * pi + 1] = out.absVelocity[3 * pi + 2] = __int_as_float(0x7fc00000);
			}
			if (out.relVelocity) {
				out.relVelocity[3 * pi] = out.relVelocity[3 * pi + 1] = out.relVelocity[3 * pi + 2] = __int_as_float(0x7fc00000);
			}
			if (out.radialSpeed) out.radialSpeed[pi] = 0.0f;
			continue;
		}
		Selected sel;
		if (type == 4u) sel = red.first;
		else if (type == 3u) sel = red.second;
		else if (type == 2u) sel = red.last;
		else if (type == 1u) sel = red.strongest;
		else if (type == 5u) sel = red.secondStrongest;
		else continue;
		if (out.xyz) {
			const Vec3 q = org + dn * sel.dist;
			out.xyz[3 * pi] = q.x;
			out.xyz[3 * pi + 1] = q.y;
			out.xyz[3 * pi + 2] = q.z;
		}
		if (out.distance) out.distance[pi] = sel.dist;
		if (out.isHit) out.isHit[pi] = 1;
		const InstanceRec& hitInst = sc.instances[sel.inst & kInstMask];
		if (out.entityId) out.entityId[pi] = hitInst.entityId;
		if (out.returnType) out.returnType[pi] = (uint8_t) type;
		if (out.intensityF32) out.intensityF32[pi] = sel.intensity;
		if (out.intensityU8) out.intensityU8[pi] = sel.intensity < 255.0f ? (uint8_t) roundf(sel.intensity) : (uint8_t) 255;
		if (out.normal) {
			out.normal[3 * pi] = sel.nx;
			out.normal[3 * pi + 1] = sel.ny;
			out.normal[3 * pi + 2] = sel.nz;
		}
		if (out.incidentAngle) out.incidentAngle[pi] = acosf(sel.cosInc);
		if (out.laserRetro) out.laserRetro[pi] = hitInst.laserRetro;
		if (SHADING && (out.absVelocity || out.relVelocity || out.radialSpeed)) {
			const int sample = sel.inst >> kSampleShift;
			const Mat34 traced = distortRay(p, beam, ray);
			const Mat34 sr = sample == 0 ? traced : mul(traced, loadMat(samples + sample));
			Vec3 absV, relV;
			float radial;
			hitVelocities(p, hitInst, sr, sel.dist, sel.tri, absV, relV, radial);
			if (out.absVelocity) {
				out.absVelocity[3 * pi] = absV.x;
				out.absVelocity[3 * pi + 1] = absV.y;
				out.absVelocity[3 * pi + 2] = absV.z;
			}
			if (out.relVelocity) {
				out.relVelocity[3 * pi] = relV.x;
				out.relVelocity[3 * pi + 1] = relV.y;
				out.relVelocity[3 * pi + 2] = relV.z;
			}
			if (out.radialSpeed) out.radialSpeed[pi] = radial;
		}
	}
}

__device__ __forceinline__ float pick(int r, float a, float b) { return r == 0 ? a : b; }
__device__ __forceinline__ uint32_t pickU(int r, uint32_t a, uint32_t b) { return r == 0 ? a : b; }

// Lane-group packing: the S samples of a beam sit on G = min(S, 32) adjacent lanes (lane k of the
// group holds samples k and k + G in sv[0], sv[1]); every lane of the warp takes part in the
// shuffles, and the group's first lane (`leader`) feeds the samples in order to `red`.
template<int ROUNDS, bool SHADING>
__device__ __forceinline__ void reduceGroup(const SampleVal (&sv)[ROUNDS], int nSamples, int G, int groupLane0, bool leader,
                                            ReturnReducer& red)
{
	for (int s = 0; s < nSamples; ++s) {
		const int r = (ROUNDS == 1) ? 0 : s / G;
		const int src = groupLane0 + (s - r * G);
		const uint32_t hit = __shfl_sync(0xffffffffu, ROUNDS == 1 ? sv[0].hit : pickU(r, sv[0].hit, sv[ROUNDS - 1].hit), src);
		const float dist = __shfl_sync(0xffffffffu, ROUNDS == 1 ? sv[0].dist : pick(r, sv[0].dist, sv[ROUNDS - 1].dist), src);
		const int32_t ent = __shfl_sync(
		    0xffffffffu, ROUNDS == 1 ? sv[0].inst : (int32_t) pickU(r, (uint32_t) sv[0].inst, (uint32_t) sv[ROUNDS - 1].inst), src);
		Selected cur{dist, 0.0f, ent, 0.0f, 0.0f, 0.0f, 0.0f, -1};
		if (SHADING) {
			cur.intensity = __shfl_sync(0xffffffffu, ROUNDS == 1 ? sv[0].intensity : pick(r, sv[0].intensity, sv[ROUNDS - 1].intensity), src);
			cur.nx = __shfl_sync(0xffffffffu, ROUNDS == 1 ? sv[0].nx : pick(r, sv[0].nx, sv[ROUNDS - 1].nx), src);
			cur.ny = __shfl_sync(0xffffffffu, ROUNDS == 1 ? sv[0].ny : pick(r, sv[0].ny, sv[ROUNDS - 1].ny), src);
			cur.nz = __shfl_sync(0xffffffffu, ROUNDS == 1 ? sv[0].nz : pick(r, sv[0].nz, sv[ROUNDS - 1].nz), src);
			cur.cosInc = __shfl_sync(0xffffffffu, ROUNDS == 1 ? sv[0].cosInc : pick(r, sv[0].cosInc, sv[ROUNDS - 1].cosInc), src);
			cur.tri = __shfl_sync(0xffffffffu, ROUNDS == 1 ? sv[0].tri : (int32_t) pickU(r, (uint32_t) sv[0].tri, (uint32_t) sv[ROUNDS - 1].tri),
			                      src);
		}
		if (leader) {
			red.add(s, hit, cur);
		}
	}
}

} // namespace tracedev
} // namespace rgl
