// Closest-hit traversal of the two-level acceleration structure, written as host/device functions so
// the same code runs in the CUDA traversal kernel and in the CPU harness of the test-suite.
//
// Replaces OptiX's trace of reference src/gpu/optixPrograms.cu:222-228 (optixTrace with tmin = 0,
// tmax = maxRange, any-hit disabled, no face culling) and the closest-hit lookup of :96-118.
#pragma once

#include <cfloat>
#include "device_types.hpp"

namespace rgl {

struct HitRec
{
	float t;       // ray parameter (units of the unnormalised direction)
	int32_t inst;  // instance index, -1 when nothing was hit
	int32_t tri;   // index into the instance BLAS triangle records
	int32_t prim;  // the triangle's index in its mesh (breaks ties in t)
};

#if defined(__CUDA_ARCH__)
RGL_HD float ldgF(const float* p) { return __ldg(p); }
#else
RGL_HD float ldgF(const float* p) { return *p; }
#endif

RGL_HD float absf_(float x) { return x < 0.0f ? -x : x; }
RGL_HD float minf_(float a, float b) { return a < b ? a : b; }
RGL_HD float maxf_(float a, float b) { return a > b ? a : b; }
RGL_HD float comp(Vec3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

// Per-ray constants of the watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013), held as
// the rows of its shear: with the axes permuted so that kz is the direction's dominant one,
// (x, y, z) -> (x_kx - Sx z_kz, x_ky - Sy z_kz, Sz z_kz). Rows with one unit, one -S and one zero
// entry evaluate that map with FMAs and no per-triangle component selection.
struct Watertight
{
	Vec3 row0, row1, row2;
};

RGL_HD Watertight setupWatertight(Vec3 d)
{
	float ax = absf_(d.x), ay = absf_(d.y), az = absf_(d.z);
	int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
	int kx = kz == 2 ? 0 : kz + 1;
	int ky = kx == 2 ? 0 : kx + 1;
	float dz = comp(d, kz);
	if (dz < 0.0f) {
		int t = kx;
		kx = ky;
		ky = t;
	}
	// One reciprocal instead of three divisions (the traversal enters two to three instances per ray):
	// every vertex is still sheared by the same S for all triangles, which is what keeps the test
	// watertight.
	const float Sz = 1.0f / dz;
	const float Sx = fmul(comp(d, kx), Sz), Sy = fmul(comp(d, ky), Sz);
	auto unitAxis = [](int k, float v) { return Vec3{k == 0 ? v : 0.0f, k == 1 ? v : 0.0f, k == 2 ? v : 0.0f}; };
	Watertight w;
	w.row0 = unitAxis(kx, 1.0f) + unitAxis(kz, -Sx);
	w.row1 = unitAxis(ky, 1.0f) + unitAxis(kz, -Sy);
	w.row2 = unitAxis(kz, Sz);
	return w;
}

// One sheared coordinate: row . v with FMAs. The zero and unit entries contribute exact terms, so the
// result is x_k - S z_kz rounded at most twice, by the same steps for a vertex in every triangle.
RGL_HD float shear(Vec3 row, Vec3 v) { return fmaf(row.x, v.x, fmaf(row.y, v.y, row.z * v.z)); }

// The edge functions in double precision, for the rare case where one of them is exactly zero in
// float. Kept out of line on the device so the traversal loop's code stays small (measured: the
// traversal of the 1M-triangle scan 0.302 -> 0.296 ms).
#if defined(__CUDA_ARCH__)
#define RGL_COLD __device__ __noinline__
#else
#define RGL_COLD inline
#endif
RGL_COLD void edgesInDouble(float Ax, float Ay, float Bx, float By, float Cx, float Cy, float& U, float& V, float& W)
{
	double CxBy = (double) Cx * (double) By, CyBx = (double) Cy * (double) Bx;
	double AxCy = (double) Ax * (double) Cy, AyCx = (double) Ay * (double) Cx;
	double BxAy = (double) Bx * (double) Ay, ByAx = (double) By * (double) Ax;
	U = (float) (CxBy - CyBx);
	V = (float) (AxCy - AyCx);
	W = (float) (BxAy - ByAx);
}

// Watertight test of triangle (a, b, c) against a ray with origin o. On a hit with
// 0 < t <= tBest returns true and the new t. Each vertex is sheared by the same arithmetic in every
// triangle that holds it; edge functions are evaluated without FMA so a shared edge yields exactly
// opposite values in both triangles; exact zeros are re-evaluated in double.
RGL_HD bool intersectTriangle(Vec3 a, Vec3 b, Vec3 c, Vec3 o, const Watertight& w, float tBest, float& tOut)
{
	Vec3 A = a - o, B = b - o, C = c - o;
	float Ax = shear(w.row0, A), Ay = shear(w.row1, A);
	float Bx = shear(w.row0, B), By = shear(w.row1, B);
	float Cx = shear(w.row0, C), Cy = shear(w.row1, C);
	float U = fsub(fmul(Cx, By), fmul(Cy, Bx));
	float V = fsub(fmul(Ax, Cy), fmul(Ay, Cx));
	float W = fsub(fmul(Bx, Ay), fmul(By, Ax));
	if (U == 0.0f || V == 0.0f || W == 0.0f) {
		edgesInDouble(Ax, Ay, Bx, By, Cx, Cy, U, V, W);
	}
	if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) {
		return false;
	}
	float det = U + V + W;
	if (det == 0.0f) {
		return false;
	}
	float Az = shear(w.row2, A), Bz = shear(w.row2, B), Cz = shear(w.row2, C);
	float T = fadd(fadd(fmul(U, Az), fmul(V, Bz)), fmul(W, Cz));
	float t = T / det;
	if (!(t > 0.0f) || !(t <= tBest)) {
		return false;
	}
	tOut = t;
	return true;
}

RGL_HD float safeInv(float d)
{
	const float tiny = 1e-30f;
	if (absf_(d) < tiny) {
		d = d < 0.0f ? -tiny : tiny;
	}
	return 1.0f / d;
}

RGL_HD float exp2Byte(uint8_t e)
{
	// 2^(e - 127) as a float with exponent bits e; e in [1, 254].
	uint32_t bits = ((uint32_t) e) << 23;
	float f;
#if defined(__CUDA_ARCH__)
	f = __uint_as_float(bits);
#else
	__builtin_memcpy(&f, &bits, 4);
#endif
	return f;
}

RGL_HD int popc8(uint32_t x)
{
#if defined(__CUDA_ARCH__)
	return __popc(x);
#else
	return __builtin_popcount(x);
#endif
}

// ---------------------------------------------------------------- wide-node traversal
//
// One loop walks both levels: the TLAS and every BLAS are 8-wide nodes of the same format, so lanes
// of a warp at different levels execute the same node-visit code. Stack entries are two 32-bit words
// (after Ylitie et al., HPG 2017), told apart by the second word:
//   node group      (childBase, imask | remaining-hits << 8), remaining hits != 0, so >= 256;
//                   bit j of the hits selects slot j ^ octant of the frame the group was pushed in;
//   enter instance  (instance index, kEnterInstance): transform the ray into the instance's frame;
//   leave instance  (0, kLeaveInstance): back to the world frame.
// Entries pushed inside an instance sit above its leave entry, so each group is popped in the frame
// it was pushed in. `Stack` provides push(a, b), pop(a&, b&), size().

// Slab test of a dequantised child box. Per axis a plane distance is evaluated as
// fma(1 + q 2^-15, S, D -+ e) with S = 2^15 A, A = s * inv (one grid step in t, exact: s is a power of
// two), C = (p - o) * inv and D = C - S (see the node loop). Against the exact distance of the ray
// with direction 1/inv it errs by at most
//  * relative: inv, the FMA and the |t| share of the C terms, 6u|t| (u = 2^-24); entry and exit
//    together 12u, covered by entry <= exit * (1 + 2e-6) (34u);
//  * absolute: C rounds twice and D and D -+ e once each, 4u|C| + 2^-8 |A| with |C| <= |t| + 255 |A|,
//    i.e. (2^-8 + 1020u) |A| < 0.0041 |A| beyond the relative part; near planes are moved earlier and
//    far planes later by e = 0.01 |A| (kPlaneSlack).
// Child boxes are the builder's verified enclosures (bvh_core.hpp quantizeAxis), so no hit inside the
// exact child box is lost. Axis-parallel rays (inv = +-1e30 after safeInv) only yield +-huge plane
// distances on that axis: the slab there is all or nothing, as it must be.
constexpr float kSlabRelSlack = 1.000002f;
// Absolute slack of a plane distance: 0.01 grid steps, as a fraction of |S| = 2^15 |A|.
constexpr float kPlaneSlack = 0.01f / 32768.0f;

RGL_HD uint32_t lowestBit(uint32_t x)
{
#if defined(__CUDA_ARCH__)
	return (uint32_t) (__ffs((int) x) - 1);
#else
	return (uint32_t) __builtin_ctz(x);
#endif
}

RGL_HD float asFloat(uint32_t u)
{
#if defined(__CUDA_ARCH__)
	return __uint_as_float(u);
#else
	float f;
	__builtin_memcpy(&f, &u, 4);
	return f;
#endif
}

RGL_HD uint32_t asUint(float f)
{
#if defined(__CUDA_ARCH__)
	return __float_as_uint(f);
#else
	uint32_t u;
	__builtin_memcpy(&u, &f, 4);
	return u;
#endif
}

// Byte k of w placed in bits 8..15 of the mantissa of 1.0: the float 1 + q * 2^-15, exact for every
// byte q. One byte permute on the device.
RGL_HD float byteMantissa(uint32_t w, int k)
{
#if defined(__CUDA_ARCH__)
	return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | ((uint32_t) k << 4)));
#else
	return asFloat(0x3F800000u | (((w >> (8 * k)) & 0xffu) << 8));
#endif
}

// Bit j of each byte of x moves to bit j ^ oct (x holds two 8-bit child masks).
RGL_HD uint32_t octantPermute(uint32_t x, uint32_t oct)
{
	if (oct & 1u) {
		x = ((x & 0x5555u) << 1) | ((x >> 1) & 0x5555u);
	}
	if (oct & 2u) {
		x = ((x & 0x3333u) << 2) | ((x >> 2) & 0x3333u);
	}
	if (oct & 4u) {
		x = ((x & 0x0F0Fu) << 4) | ((x >> 4) & 0x0F0Fu);
	}
	return x;
}

// max(a, b, c, d) and min(a, b, c, d) of the slab test; three-input min/max on the device.
RGL_HD float max4(float a, float b, float c, float d)
{
#if defined(__CUDA_ARCH__)
	float m;
	asm("max.f32 %0, %1, %2, %3;" : "=f"(m) : "f"(a), "f"(b), "f"(c));
	return fmaxf(m, d);
#else
	return maxf_(maxf_(a, b), maxf_(c, d));
#endif
}
RGL_HD float min4(float a, float b, float c, float d)
{
#if defined(__CUDA_ARCH__)
	float m;
	asm("min.f32 %0, %1, %2, %3;" : "=f"(m) : "f"(a), "f"(b), "f"(c));
	return fminf(m, d);
#else
	return minf_(minf_(a, b), minf_(c, d));
#endif
}

constexpr uint32_t kLeaveInstance = 0u;
constexpr uint32_t kEnterInstance = 1u;

RGL_HD uint32_t highestBit(uint32_t x)
{
#if defined(__CUDA_ARCH__)
	return (uint32_t) (31 - __clz((int) x));
#else
	return (uint32_t) (31 - __builtin_clz(x));
#endif
}

// Closest-hit order: smaller t first; equal t goes to the smaller (instance, mesh triangle index) pair.
// The order depends neither on the traversal order nor on the order of the BLAS's triangle records
// (which a device build allocates with atomics), so every traversal that tests all triangles at the
// minimal t (every correct one does: their boxes are never culled) returns the same hit from every
// build of the same mesh.
RGL_HD bool closerHit(float t, int32_t inst, int32_t prim, const HitRec& best)
{
	if (t != best.t) {
		return t < best.t;
	}
	return (uint32_t) inst != (uint32_t) best.inst ? (uint32_t) inst < (uint32_t) best.inst : (uint32_t) prim < (uint32_t) best.prim;
}

// A ray in the frame being traversed: origin, direction, inverse direction and its octant.
struct FrameRay
{
	Vec3 o, d, inv;
	uint32_t oct;
};

RGL_HD FrameRay frameRay(Vec3 o, Vec3 d)
{
	FrameRay r;
	r.o = o;
	r.d = d;
	r.inv = {safeInv(d.x), safeInv(d.y), safeInv(d.z)};
	r.oct = (r.inv.x < 0.0f ? 1u : 0u) | (r.inv.y < 0.0f ? 2u : 0u) | (r.inv.z < 0.0f ? 4u : 0u);
	return r;
}

// Error-free transformations (Knuth's TwoSum, the FMA form of TwoProduct) and the compensated dot
// product built from them (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 2005, Dot2): the result is as accurate as if computed in twice the working precision.
RGL_HD void twoSum(float a, float b, float& s, float& e)
{
	s = fadd(a, b);
	const float bb = fsub(s, a);
	e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
}
RGL_HD void twoProd(float a, float b, float& p, float& e)
{
	p = fmul(a, b);
	e = fmaf(a, b, -p);
}
// a . (bh + bl), bl a small correction of bh.
RGL_HD float dotCompensated(Vec3 a, Vec3 bh, Vec3 bl)
{
	float p0, e0, p1, e1, p2, e2, s1, f1, s2, f2;
	twoProd(a.x, bh.x, p0, e0);
	twoProd(a.y, bh.y, p1, e1);
	twoProd(a.z, bh.z, p2, e2);
	twoSum(p0, p1, s1, f1);
	twoSum(s1, p2, s2, f2);
	const float err = fadd(fadd(fadd(e0, e1), fadd(e2, f1)), fadd(f2, fadd(fadd(fmul(a.x, bl.x), fmul(a.y, bl.y)), fmul(a.z, bl.z))));
	return fadd(s2, err);
}

// Ray parameter of the hit with triangle (a, b, c), normal n = (b - a) x (c - a), from its plane:
// t = n.(a - o) / n.d, with a - o exact (TwoSum) and both dot products compensated. The watertight
// test decides hit or miss exactly, but its t comes from barycentric weights of the sheared, projected
// triangle, whose relative error grows as 1 / sin(grazing angle): at 0.9 degrees over terrain 50 m
// away it reached 2.5e-5 of the distance. In the plane form a grazing angle only divides the normal's
// rounding, which is weighted by the hit's offset from the vertex (the triangle's size), not by the
// distance. Returns `t` when the plane form is undefined (ray in the plane).
RGL_HD float planeHitT(Vec3 a, Vec3 n, Vec3 o, Vec3 d, float t)
{
	Vec3 eh, el;
	twoSum(a.x, -o.x, eh.x, el.x);
	twoSum(a.y, -o.y, eh.y, el.y);
	twoSum(a.z, -o.z, eh.z, el.z);
	const float num = dotCompensated(n, eh, el);
	const float den = dotCompensated(n, d, v3(0.0f, 0.0f, 0.0f));
	const float tp = num / den;
	return (tp > 0.0f && tp < 3.0e38f) ? tp : t;
}

// m * v + translation with every product and sum error-free: hi + lo is m * v to about u^2 relative.
RGL_HD void compensatedPoint(const Mat34& m, Vec3 v, Vec3& hi, Vec3& lo)
{
	float r[3], q[3];
	for (int i = 0; i < 3; ++i) {
		float p0, e0, p1, e1, p2, e2, s1, f1, s2, f2, s3, f3;
		twoProd(m.m[i][0], v.x, p0, e0);
		twoProd(m.m[i][1], v.y, p1, e1);
		twoProd(m.m[i][2], v.z, p2, e2);
		twoSum(p0, p1, s1, f1);
		twoSum(s1, p2, s2, f2);
		twoSum(s2, m.m[i][3], s3, f3);
		r[i] = s3;
		q[i] = fadd(fadd(fadd(e0, e1), fadd(e2, f1)), fadd(f2, f3));
	}
	hi = v3(r[0], r[1], r[2]);
	lo = v3(q[0], q[1], q[2]);
}

// Sine of the angle between ray and triangle plane below which the closest hit's t is finished from
// the plane (refineClosest); at or above it the watertight t stands (its error, about 4e-7 / sine of
// the distance, stays below 4e-6), unless the hit is close on a transformed instance (below).
constexpr float kRefineSine = 0.1f;

// The closest hit's t finished from the hit triangle's plane when the ray grazes it. On an instance
// with the identity transform (a scene-sized mesh) the instance frame is the world frame and planeHitT
// is exact up to the rounding of the normal. A transformed instance rounds the ray into its frame by
// about u |o - instance origin|, and a grazing angle divides that offset along the ray (0.08 degrees:
// 4e-5 of the distance; a sensor inside a sphere 0.4 m from its wall at 1.2 degrees: 3e-5); there the
// plane is evaluated in the world frame: the vertex moved to the world by compensatedPoint, the normal
// by the transposed inverse, so the only remaining rounding is the normal's, weighted by the hit's
// offset from the vertex.
template<class NodeLoader>
RGL_HD HitRec refineClosest(const SceneView& sc, Vec3 oW, Vec3 dW, HitRec best, const NodeLoader& load)
{
	if (best.inst < 0) {
		return best;
	}
	const InstanceRec& ir = load.instance(sc.instances, best.inst);
	const bool identity = (ir.flags & kInstanceIdentity) != 0;
	const TriRecord tr = load.tri(ir.tris, best.tri);
	const Vec3 a = v3(tr.v0x, tr.v0y, tr.v0z);
	const Vec3 n = cross(v3(tr.v1x, tr.v1y, tr.v1z) - a, v3(tr.v2x, tr.v2y, tr.v2z) - a);
	const Vec3 d = identity ? dW : ir.worldToObject.vector(dW);
	const float nd = dot(n, d), nn = dot(n, n), dd = dot(d, d);
	const float s2 = fmul(nd, nd), q = fmul(nn, dd); // sin^2 = s2 / q
	const bool grazing = s2 < kRefineSine * kRefineSine * q;
	// On a transformed instance the ray's rounding into the instance frame, about u |o - instance
	// origin|, also weighs against a hit closer than half that offset (a sensor inside a large instance).
	const Vec3 off = oW - ir.objectToWorld.translation();
	const bool close = !identity && fmul(fmul(best.t, best.t), dot(dW, dW)) < 0.25f * dot(off, off);
	if (!grazing && !close) {
		return best;
	}
	if (identity) {
		best.t = planeHitT(a, n, oW, dW, best.t);
		return best;
	}
	Vec3 ah, al;
	compensatedPoint(ir.objectToWorld, a, ah, al);
	const Mat34& w = ir.worldToObject;
	const Vec3 nW = v3(fadd(fadd(fmul(w.m[0][0], n.x), fmul(w.m[1][0], n.y)), fmul(w.m[2][0], n.z)),
	                   fadd(fadd(fmul(w.m[0][1], n.x), fmul(w.m[1][1], n.y)), fmul(w.m[2][1], n.z)),
	                   fadd(fadd(fmul(w.m[0][2], n.x), fmul(w.m[1][2], n.y)), fmul(w.m[2][2], n.z)));
	Vec3 eh, el;
	twoSum(ah.x, -oW.x, eh.x, el.x);
	twoSum(ah.y, -oW.y, eh.y, el.y);
	twoSum(ah.z, -oW.z, eh.z, el.z);
	el = v3(fadd(el.x, al.x), fadd(el.y, al.y), fadd(el.z, al.z));
	const float num = dotCompensated(nW, eh, el);
	const float den = dotCompensated(nW, dW, v3(0.0f, 0.0f, 0.0f));
	const float tp = num / den;
	if (tp > 0.0f && tp < 3.0e38f) {
		best.t = tp;
	}
	return best;
}

// Closest hit over all instances for a world-space ray o + t d, t in (0, tmax].
template<class Stack, class NodeLoader>
RGL_HD HitRec traceClosest(const SceneView& sc, Vec3 oW, Vec3 dW, float tmax, Stack& st, const NodeLoader& load)
{
	HitRec best;
	best.t = tmax; // hits with t == tmax are accepted
	best.inst = -1;
	best.tri = -1;
	best.prim = -1;
	if (sc.nInstances <= 0) {
		return best;
	}
	const int base = st.size();
	FrameRay r = frameRay(oW, dW);
	Watertight wt = setupWatertight(dW); // valid inside an instance
	const WideNode* nodes = sc.tlas;
	const TriRecord* leaves = sc.tlasLeaves;
	int32_t inst = -1; // -1: the TLAS (world frame)
	uint32_t node = 0;
	for (;;) {
		uint4 w0, w1, w2, w3, w4;
		load.nodeWords(nodes, node, w0, w1, w2, w3, w4);
		const float sx = exp2Byte((uint8_t) (w0.w & 0xffu)), sy = exp2Byte((uint8_t) ((w0.w >> 8) & 0xffu)),
		            sz = exp2Byte((uint8_t) ((w0.w >> 16) & 0xffu));
		const uint32_t imask = w0.w >> 24;
		const uint32_t childBase = w1.x, triBase = w1.y;
		const float Ax = sx * r.inv.x, Ay = sy * r.inv.y, Az = sz * r.inv.z;
		const float Cx = (asFloat(w0.x) - r.o.x) * r.inv.x, Cy = (asFloat(w0.y) - r.o.y) * r.inv.y, Cz = (asFloat(w0.z) - r.o.z) * r.inv.z;
		// Plane distance q * A + C evaluated as fma(1 + q * 2^-15, 2^15 * A, C - 2^15 * A): 2^15 * A and
		// the product term are exact; the error bound and the slacks that cover it are derived above
		// kSlabRelSlack.
		const float Sx = 32768.0f * Ax, Sy = 32768.0f * Ay, Sz = 32768.0f * Az;
		const float Dx = Cx - Sx, Dy = Cy - Sy, Dz = Cz - Sz;
		// Near planes earlier, far planes later, by kPlaneSlack grid steps.
		const float ex = kPlaneSlack * absf_(Sx), ey = kPlaneSlack * absf_(Sy), ez = kPlaneSlack * absf_(Sz);
		const float Dnx = Dx - ex, Dny = Dy - ey, Dnz = Dz - ez, Dfx = Dx + ex, Dfy = Dy + ey, Dfz = Dz + ez;
		// near/far quantised planes per axis (packed bytes), swapped for negative directions
		const bool negx = (r.oct & 1u) != 0, negy = (r.oct & 2u) != 0, negz = (r.oct & 4u) != 0;
		const uint32_t nx0 = negx ? w3.z : w2.x, nx1 = negx ? w3.w : w2.y, fx0 = negx ? w2.x : w3.z, fx1 = negx ? w2.y : w3.w;
		const uint32_t ny0 = negy ? w4.x : w2.z, ny1 = negy ? w4.y : w2.w, fy0 = negy ? w2.z : w4.x, fy1 = negy ? w2.w : w4.y;
		const uint32_t nz0 = negz ? w4.z : w3.x, nz1 = negz ? w4.w : w3.y, fz0 = negz ? w3.x : w4.z, fz1 = negz ? w3.y : w4.w;
		uint32_t hitSlots = 0; // bit s: child slot s is hit
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
		for (int s = 0; s < kWideArity; ++s) {
			const int k = s & 3;
			const bool hiw = s >= 4;
			const float tnx = fmaf(byteMantissa(hiw ? nx1 : nx0, k), Sx, Dnx), tfx = fmaf(byteMantissa(hiw ? fx1 : fx0, k), Sx, Dfx);
			const float tny = fmaf(byteMantissa(hiw ? ny1 : ny0, k), Sy, Dny), tfy = fmaf(byteMantissa(hiw ? fy1 : fy0, k), Sy, Dfy);
			const float tnz = fmaf(byteMantissa(hiw ? nz1 : nz0, k), Sz, Dnz), tfz = fmaf(byteMantissa(hiw ? fz1 : fz0, k), Sz, Dfz);
			const float tEntry = max4(tnx, tny, tnz, 0.0f);
			const float tExit = min4(tfx, tfy, tfz, best.t);
			hitSlots |= (tEntry <= tExit * kSlabRelSlack) ? (1u << s) : 0u;
		}
		// Internal and leaf hits in traversal order j (slot = j ^ oct): one permutation for both.
		const uint32_t ordered = octantPermute((hitSlots & imask) | ((hitSlots & ~imask & 0xffu) << 8), r.oct);
		uint32_t internalHits = ordered & 0xffu, leafHits = ordered >> 8;
		const uint32_t metaLo = w1.z, metaHi = w1.w;
		if (inst < 0) {
			// TLAS leaves are instances (one per leaf child): queued, the nearest on top.
			while (leafHits) {
				const uint32_t j = highestBit(leafHits);
				leafHits &= ~(1u << j);
				const uint32_t s = j ^ r.oct;
				const uint32_t meta = ((s < 4 ? metaLo : metaHi) >> ((s & 3) * 8)) & 0xffu;
				st.push((uint32_t) load.leafPrim(leaves, (int) triBase + (int) (meta & 31u)), kEnterInstance);
			}
		} else {
			// BLAS leaves: their triangles now, in ray order.
			while (leafHits) {
				const uint32_t s = lowestBit(leafHits) ^ r.oct;
				leafHits &= leafHits - 1u;
				const uint32_t meta = ((s < 4 ? metaLo : metaHi) >> ((s & 3) * 8)) & 0xffu;
				const int first = (int) triBase + (int) (meta & 31u);
				const int cnt = (int) (meta >> 5);
				for (int k = 0; k < cnt; ++k) {
					TriRecord tr = load.tri(leaves, first + k);
					float t;
					if (intersectTriangle(v3(tr.v0x, tr.v0y, tr.v0z), v3(tr.v1x, tr.v1y, tr.v1z), v3(tr.v2x, tr.v2y, tr.v2z), r.o, wt,
					                      best.t, t) &&
					    closerHit(t, inst, tr.primId, best)) {
						best.t = t;
						best.inst = inst;
						best.tri = first + k;
						best.prim = tr.primId;
					}
				}
			}
		}
		uint32_t groupBase = childBase, groupMask = imask, hits = internalHits;
		bool enterRoot = false;
		while (hits == 0) {
			if (st.size() == base) {
				return refineClosest(sc, oW, dW, best, load);
			}
			uint32_t a, b;
			st.pop(a, b);
			if (b == kLeaveInstance) {
				r = frameRay(oW, dW);
				nodes = sc.tlas;
				leaves = sc.tlasLeaves;
				inst = -1;
			} else if (b == kEnterInstance) {
				const InstanceRec& ir = load.instance(sc.instances, (int32_t) a);
				st.push(0u, kLeaveInstance);
				const Vec3 od = ir.worldToObject.vector(dW);
				r = frameRay(worldToInstance(ir, oW), od);
				wt = setupWatertight(od);
				nodes = ir.nodes;
				leaves = ir.tris;
				inst = (int32_t) a;
				enterRoot = true;
				break;
			} else {
				groupBase = a;
				groupMask = b & 0xffu;
				hits = b >> 8;
			}
		}
		if (enterRoot) {
			node = 0;
			continue;
		}
		const uint32_t s = lowestBit(hits) ^ r.oct;
		hits &= hits - 1u;
		if (hits) {
			st.push(groupBase, groupMask | (hits << 8));
		}
		node = groupBase + (uint32_t) popc8(groupMask & ((1u << s) - 1u));
	}
}

} // namespace rgl
