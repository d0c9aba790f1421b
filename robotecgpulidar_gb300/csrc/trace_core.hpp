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

// Per-ray constants of the watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013).
struct Watertight
{
	int kx, ky, kz;
	float Sx, Sy, Sz;
};

RGL_HD Watertight setupWatertight(Vec3 d)
{
	Watertight w;
	float ax = absf_(d.x), ay = absf_(d.y), az = absf_(d.z);
	w.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
	w.kx = w.kz == 2 ? 0 : w.kz + 1;
	w.ky = w.kx == 2 ? 0 : w.kx + 1;
	float dz = comp(d, w.kz);
	if (dz < 0.0f) {
		int t = w.kx;
		w.kx = w.ky;
		w.ky = t;
	}
	w.Sx = comp(d, w.kx) / dz;
	w.Sy = comp(d, w.ky) / dz;
	w.Sz = 1.0f / dz;
	return w;
}

// Watertight test of triangle (a, b, c) against a ray with origin o. On a hit with
// 0 < t <= tBest returns true and the new t. Edge functions are evaluated without FMA so a shared edge
// yields exactly opposite values in both triangles; exact zeros are re-evaluated in double.
RGL_HD bool intersectTriangle(Vec3 a, Vec3 b, Vec3 c, Vec3 o, const Watertight& w, float tBest, float& tOut)
{
	Vec3 A = a - o, B = b - o, C = c - o;
	float Akz = comp(A, w.kz), Bkz = comp(B, w.kz), Ckz = comp(C, w.kz);
	float Ax = fsub(comp(A, w.kx), fmul(w.Sx, Akz));
	float Ay = fsub(comp(A, w.ky), fmul(w.Sy, Akz));
	float Bx = fsub(comp(B, w.kx), fmul(w.Sx, Bkz));
	float By = fsub(comp(B, w.ky), fmul(w.Sy, Bkz));
	float Cx = fsub(comp(C, w.kx), fmul(w.Sx, Ckz));
	float Cy = fsub(comp(C, w.ky), fmul(w.Sy, Ckz));
	float U = fsub(fmul(Cx, By), fmul(Cy, Bx));
	float V = fsub(fmul(Ax, Cy), fmul(Ay, Cx));
	float W = fsub(fmul(Bx, Ay), fmul(By, Ax));
	if (U == 0.0f || V == 0.0f || W == 0.0f) {
		double CxBy = (double) Cx * (double) By, CyBx = (double) Cy * (double) Bx;
		double AxCy = (double) Ax * (double) Cy, AyCx = (double) Ay * (double) Cx;
		double BxAy = (double) Bx * (double) Ay, ByAx = (double) By * (double) Ax;
		U = (float) (CxBy - CyBx);
		V = (float) (AxCy - AyCx);
		W = (float) (BxAy - ByAx);
	}
	if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) {
		return false;
	}
	float det = U + V + W;
	if (det == 0.0f) {
		return false;
	}
	float Az = w.Sz * Akz, Bz = w.Sz * Bkz, Cz = w.Sz * Ckz;
	float T = fadd(fadd(fmul(U, Az), fmul(V, Bz)), fmul(W, Cz));
	float t = T / det;
	if (!(t > 0.0f) || !(t <= tBest)) {
		return false;
	}
	tOut = t;
	return true;
}

struct BoxRay
{
	Vec3 o;
	Vec3 inv;
	bool negx, negy, negz;
};

RGL_HD float safeInv(float d)
{
	const float tiny = 1e-30f;
	if (absf_(d) < tiny) {
		d = d < 0.0f ? -tiny : tiny;
	}
	return 1.0f / d;
}

RGL_HD BoxRay makeBoxRay(Vec3 o, Vec3 d)
{
	BoxRay r;
	r.o = o;
	r.inv = {safeInv(d.x), safeInv(d.y), safeInv(d.z)};
	r.negx = r.inv.x < 0.0f;
	r.negy = r.inv.y < 0.0f;
	r.negz = r.inv.z < 0.0f;
	return r;
}

// Conservative slack on the exit distance of a slab test: covers the three roundings of
// (plane - o) * inv (Ize, "Robust BVH Ray Traversal", JCGT 2013).
constexpr float kSlabSlack = 1.0000004f;

// Slab test of a float box; returns entry distance or -1 when the box is missed within [0, tBest].
RGL_HD float slabEnter(const BoxRay& r, float lox, float loy, float loz, float hix, float hiy, float hiz, float tBest)
{
	float nx = r.negx ? hix : lox, fx = r.negx ? lox : hix;
	float ny = r.negy ? hiy : loy, fy = r.negy ? loy : hiy;
	float nz = r.negz ? hiz : loz, fz = r.negz ? loz : hiz;
	float t0 = maxf_(maxf_((nx - r.o.x) * r.inv.x, (ny - r.o.y) * r.inv.y), maxf_((nz - r.o.z) * r.inv.z, 0.0f));
	float t1 = minf_(minf_((fx - r.o.x) * r.inv.x, (fy - r.o.y) * r.inv.y), minf_((fz - r.o.z) * r.inv.z, tBest));
	return (t0 <= t1 * kSlabSlack) ? t0 : -1.0f;
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

// Dequantised box of child slot i of a wide node (same float expression the builder verified).
RGL_HD void childBox(const WideNode& n, int i, float& lox, float& loy, float& loz, float& hix, float& hiy, float& hiz)
{
	float sx = exp2Byte(n.ex), sy = exp2Byte(n.ey), sz = exp2Byte(n.ez);
	lox = fadd(n.px, (float) n.qlox[i] * sx);
	loy = fadd(n.py, (float) n.qloy[i] * sy);
	loz = fadd(n.pz, (float) n.qloz[i] * sz);
	hix = fadd(n.px, (float) n.qhix[i] * sx);
	hiy = fadd(n.py, (float) n.qhiy[i] * sy);
	hiz = fadd(n.pz, (float) n.qhiz[i] * sz);
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
// Stack entries are two 32-bit words. BLAS entries are node groups (after Ylitie et al., HPG 2017):
// (childBase, imask | remaining-hits << 8), where bit j of the hits selects slot j ^ octant. TLAS
// entries are (node or ~instance, entry distance bits). `Stack` provides push(a, b), pop(a&, b&),
// size().

// Slab test of a dequantised child box in the FMA form t = q * (s * inv) + (p - o) * inv. The computed
// t differs from the exact plane distance by at most 4u|t| + 3u * 255 * s * |inv| (u = 2^-24), plus
// the rounding of the folded offset described in traverseBlas. The builder widens every child box by
// one grid step s (bvh_core.hpp quantizeAxis), which moves each plane outward by s * |inv| in t and
// covers the absolute terms; entry <= exit * (1 + 5e-7) covers the relative ones.
// Axis-parallel rays (inv = +-1e30 after safeInv) stay exact: their slab only yields +-huge values.
constexpr float kSlabRelSlack = 1.0000005f;

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

template<class Stack, class NodeLoader>
RGL_HD void traverseBlas(const InstanceRec& inst, int32_t instIdx, Vec3 o, Vec3 d, Stack& st, HitRec& best,
                         const NodeLoader& load)
{
	const Watertight wt = setupWatertight(d);
	const Vec3 inv = {safeInv(d.x), safeInv(d.y), safeInv(d.z)};
	const bool negx = inv.x < 0.0f, negy = inv.y < 0.0f, negz = inv.z < 0.0f;
	const uint32_t oct = (negx ? 1u : 0u) | (negy ? 2u : 0u) | (negz ? 4u : 0u);
	const int base = st.size();
	uint32_t node = 0;
	for (;;) {
		uint4 w0, w1, w2, w3, w4;
		load.nodeWords(inst.nodes, node, w0, w1, w2, w3, w4);
		const float sx = exp2Byte((uint8_t) (w0.w & 0xffu)), sy = exp2Byte((uint8_t) ((w0.w >> 8) & 0xffu)),
		            sz = exp2Byte((uint8_t) ((w0.w >> 16) & 0xffu));
		const uint32_t imask = w0.w >> 24;
		const uint32_t childBase = w1.x, triBase = w1.y;
		const float Ax = sx * inv.x, Ay = sy * inv.y, Az = sz * inv.z;
		const float Cx = (asFloat(w0.x) - o.x) * inv.x, Cy = (asFloat(w0.y) - o.y) * inv.y, Cz = (asFloat(w0.z) - o.z) * inv.z;
		// Plane distance q * A + C evaluated as fma(1 + q * 2^-15, 2^15 * A, C - 2^15 * A): 2^15 * A is
		// exact and the product term is exact, so the only extra rounding is that of C - 2^15 * A,
		// at most u|C| + 2^-9 |A|. With |C| <= |t| + 255 |A|, the relative slack (5u of 8.4u used) and
		// the one-grid-step widening |A| (2^-9 + 1020u of 1 used) still cover every error.
		const float Sx = 32768.0f * Ax, Sy = 32768.0f * Ay, Sz = 32768.0f * Az;
		const float Dx = Cx - Sx, Dy = Cy - Sy, Dz = Cz - Sz;
		// near/far quantised planes per axis (packed bytes), swapped for negative directions
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
			const float tnx = fmaf(byteMantissa(hiw ? nx1 : nx0, k), Sx, Dx), tfx = fmaf(byteMantissa(hiw ? fx1 : fx0, k), Sx, Dx);
			const float tny = fmaf(byteMantissa(hiw ? ny1 : ny0, k), Sy, Dy), tfy = fmaf(byteMantissa(hiw ? fy1 : fy0, k), Sy, Dy);
			const float tnz = fmaf(byteMantissa(hiw ? nz1 : nz0, k), Sz, Dz), tfz = fmaf(byteMantissa(hiw ? fz1 : fz0, k), Sz, Dz);
			const float tEntry = max4(tnx, tny, tnz, 0.0f);
			const float tExit = min4(tfx, tfy, tfz, best.t);
			hitSlots |= (tEntry <= tExit * kSlabRelSlack) ? (1u << s) : 0u;
		}
		// Internal and leaf hits in traversal order j (slot = j ^ oct): one permutation for both.
		const uint32_t ordered = octantPermute((hitSlots & imask) | ((hitSlots & ~imask & 0xffu) << 8), oct);
		uint32_t internalHits = ordered & 0xffu, leafHits = ordered >> 8;
		// Triangles of hit leaf children, in ray order.
		const uint32_t metaLo = w1.z, metaHi = w1.w;
		while (leafHits) {
			const uint32_t s = lowestBit(leafHits) ^ oct;
			leafHits &= leafHits - 1u;
			const uint32_t meta = ((s < 4 ? metaLo : metaHi) >> ((s & 3) * 8)) & 0xffu;
			const int first = (int) triBase + (int) (meta & 31u);
			const int cnt = (int) (meta >> 5);
			for (int k = 0; k < cnt; ++k) {
				TriRecord tr = load.tri(inst.tris, first + k);
				float t;
				if (intersectTriangle(v3(tr.v0x, tr.v0y, tr.v0z), v3(tr.v1x, tr.v1y, tr.v1z), v3(tr.v2x, tr.v2y, tr.v2z), o, wt,
				                      best.t, t)) {
					best.t = t;
					best.inst = instIdx;
					best.tri = first + k;
				}
			}
		}
		uint32_t groupBase = childBase, groupMask = imask, hits = internalHits;
		if (hits == 0) {
			if (st.size() == base) {
				break;
			}
			uint32_t b;
			st.pop(groupBase, b);
			groupMask = b & 0xffu;
			hits = b >> 8;
		}
		const uint32_t s = lowestBit(hits) ^ oct;
		hits &= hits - 1u;
		if (hits) {
			st.push(groupBase, groupMask | (hits << 8));
		}
		node = groupBase + (uint32_t) popc8(groupMask & ((1u << s) - 1u));
	}
}

// Closest hit over all instances for a world-space ray o + t d, t in (0, tmax].
template<class Stack, class NodeLoader>
RGL_HD HitRec traceClosest(const SceneView& sc, Vec3 o, Vec3 d, float tmax, Stack& st, const NodeLoader& load)
{
	HitRec best;
	best.t = tmax; // hits with t == tmax are accepted
	best.inst = -1;
	best.tri = -1;
	if (sc.nInstances <= 0) {
		return best;
	}
	const BoxRay br = makeBoxRay(o, d);
	const int base = st.size();
	// TLAS entries: (value >= 0 internal node | value < 0 instance ~value, entry distance bits).
	st.push((uint32_t) (sc.nInstances == 1 ? ~0 : 0), 0u);
	while (st.size() > base) {
		uint32_t ev, tb;
		st.pop(ev, tb);
		const int32_t e = (int32_t) ev;
		if (asFloat(tb) > best.t) {
			continue;
		}
		if (e < 0) {
			const int32_t ii = ~e;
			const InstanceRec& inst = load.instance(sc.instances, ii);
			traverseBlas(inst, ii, inst.worldToObject.point(o), inst.worldToObject.vector(d), st, best, load);
			continue;
		}
		const BinNode bn = load.bin(sc.tlas, e);
		const int32_t ch[2] = {bn.left, bn.right};
		float te[2];
		for (int k = 0; k < 2; ++k) {
			const int32_t c = ch[k];
			float lx, ly, lz, hx, hy, hz;
			if (c >= 0) {
				const BinNode cn = load.bin(sc.tlas, c);
				lx = cn.lox;
				ly = cn.loy;
				lz = cn.loz;
				hx = cn.hix;
				hy = cn.hiy;
				hz = cn.hiz;
			} else {
				const InstanceRec& ci = load.instance(sc.instances, ~c);
				lx = ci.lox;
				ly = ci.loy;
				lz = ci.loz;
				hx = ci.hix;
				hy = ci.hiy;
				hz = ci.hiz;
			}
			te[k] = slabEnter(br, lx, ly, lz, hx, hy, hz, best.t);
		}
		const int farK = (te[0] >= 0.0f && te[1] >= 0.0f && te[1] < te[0]) ? 0 : 1;
		for (int q = 0; q < 2; ++q) {
			const int k = (q == 0) ? farK : 1 - farK;
			if (te[k] >= 0.0f) {
				st.push((uint32_t) ch[k], asUint(te[k]));
			}
		}
	}
	return best;
}

} // namespace rgl
