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

// Generic traversal stack interface: `Stack` provides push(idx, tnear), pop(idx&, tnear&), size(),
// and an `overflow` flag.
template<class Stack, class NodeLoader>
RGL_HD void traverseBlas(const InstanceRec& inst, int32_t instIdx, Vec3 o, Vec3 d, Stack& st, HitRec& best,
                         const NodeLoader& load)
{
	Watertight wt = setupWatertight(d);
	BoxRay br = makeBoxRay(o, d);
	int base = st.size();
	st.push(0, 0.0f);
	while (st.size() > base) {
		int32_t ni;
		float tn;
		st.pop(ni, tn);
		if (tn > best.t) {
			continue;
		}
		WideNode n = load.node(inst.nodes, ni);
		int32_t cidx[kWideArity];
		float ctn[kWideArity];
		int nc = 0;
		int internalRank = 0;
		for (int i = 0; i < kWideArity; ++i) {
			bool isInternal = (n.imask >> i) & 1u;
			uint8_t meta = n.meta[i];
			if (!isInternal && meta == 0) {
				continue;
			}
			float lx, ly, lz, hx, hy, hz;
			childBox(n, i, lx, ly, lz, hx, hy, hz);
			float te = slabEnter(br, lx, ly, lz, hx, hy, hz, best.t);
			if (isInternal) {
				int32_t child = (int32_t) n.childBase + internalRank;
				++internalRank;
				if (te >= 0.0f) {
					// insertion by ascending entry distance
					int k = nc++;
					while (k > 0 && ctn[k - 1] > te) {
						ctn[k] = ctn[k - 1];
						cidx[k] = cidx[k - 1];
						--k;
					}
					ctn[k] = te;
					cidx[k] = child;
				}
			} else if (te >= 0.0f) {
				int first = (int) n.triBase + (meta & 31);
				int cnt = meta >> 5;
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
		}
		for (int k = nc - 1; k >= 0; --k) {
			if (ctn[k] <= best.t) {
				st.push(cidx[k], ctn[k]);
			}
		}
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
	BoxRay br = makeBoxRay(o, d);
	int base = st.size();
	// TLAS entries: value >= 0 internal node, value < 0 instance ~value.
	st.push(sc.nInstances == 1 ? ~0 : 0, 0.0f);
	while (st.size() > base) {
		int32_t e;
		float tn;
		st.pop(e, tn);
		if (tn > best.t) {
			continue;
		}
		if (e < 0) {
			int32_t ii = ~e;
			const InstanceRec& inst = load.instance(sc.instances, ii);
			Vec3 oo = inst.worldToObject.point(o);
			Vec3 dd = inst.worldToObject.vector(d);
			traverseBlas(inst, ii, oo, dd, st, best, load);
			continue;
		}
		BinNode bn = load.bin(sc.tlas, e);
		int32_t ch[2] = {bn.left, bn.right};
		float te[2];
		for (int k = 0; k < 2; ++k) {
			int32_t c = ch[k];
			float lx, ly, lz, hx, hy, hz;
			if (c >= 0) {
				BinNode cn = load.bin(sc.tlas, c);
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
		// push far child first
		bool swap = te[1] >= 0.0f && te[0] >= 0.0f && te[1] < te[0];
		int firstK = swap ? 0 : 1;
		for (int q = 0; q < 2; ++q) {
			int k = (q == 0) ? firstK : 1 - firstK;
			if (te[k] >= 0.0f) {
				st.push(ch[k], te[k]);
			}
		}
	}
	return best;
}

} // namespace rgl
