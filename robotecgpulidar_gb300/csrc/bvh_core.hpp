// Per-item steps of the on-device BVH builder, as host/device functions (the CUDA kernels in bvh.cu
// are thin wrappers; the test-suite's CPU harness runs the same functions serially).
//
// Build = Morton codes (30 bit) -> radix sort -> LBVH (Karras, "Maximizing Parallelism in the
// Construction of BVHs, Octrees, and k-d Trees", HPG 2012) -> bottom-up bounds -> top-down collapse
// into 8-wide nodes (children chosen by repeatedly opening the child of largest surface area) with
// 8-bit child boxes rounded outward and verified in float.  It replaces OptiX's GAS/IAS builds at
// reference src/scene/GASBuilder.hpp:31-100 and src/scene/Scene.cpp:131-190.
#pragma once

#include <cfloat>
#include <cstdint>
#include "device_types.hpp"
#include "trace_core.hpp"

namespace rgl {

struct Box
{
	float lox, loy, loz, hix, hiy, hiz;
};

RGL_HD Box emptyBox() { return Box{FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX}; }
RGL_HD Box unite(const Box& a, const Box& b)
{
	return Box{a.lox < b.lox ? a.lox : b.lox, a.loy < b.loy ? a.loy : b.loy, a.loz < b.loz ? a.loz : b.loz,
	           a.hix > b.hix ? a.hix : b.hix, a.hiy > b.hiy ? a.hiy : b.hiy, a.hiz > b.hiz ? a.hiz : b.hiz};
}
// Half the surface area, evaluated in the same order without FMA contraction on host and device, so
// the device builders choose exactly what the host builder chooses.
RGL_HD float halfArea(const Box& b)
{
	const float dx = fsub(b.hix, b.lox), dy = fsub(b.hiy, b.loy), dz = fsub(b.hiz, b.loz);
	return fadd(fadd(fmul(dx, dy), fmul(dy, dz)), fmul(dz, dx));
}
RGL_HD Box binBox(const BinNode& n) { return Box{n.lox, n.loy, n.loz, n.hix, n.hiy, n.hiz}; }

RGL_HD uint32_t expandBits10(uint32_t v)
{
	v = (v * 0x00010001u) & 0xFF0000FFu;
	v = (v * 0x00000101u) & 0x0F00F00Fu;
	v = (v * 0x00000011u) & 0xC30C30C3u;
	v = (v * 0x00000005u) & 0x49249249u;
	return v;
}

// 30-bit Morton code of point c inside [lo, lo + 1/invExt].
RGL_HD uint32_t morton30(float cx, float cy, float cz, const Box& cb)
{
	float ex = cb.hix - cb.lox, ey = cb.hiy - cb.loy, ez = cb.hiz - cb.loz;
	float fx = ex > 0.0f ? (cx - cb.lox) / ex : 0.0f;
	float fy = ey > 0.0f ? (cy - cb.loy) / ey : 0.0f;
	float fz = ez > 0.0f ? (cz - cb.loz) / ez : 0.0f;
	auto q = [](float f) -> uint32_t {
		float s = f * 1024.0f;
		s = s < 0.0f ? 0.0f : (s > 1023.0f ? 1023.0f : s);
		return (uint32_t) s;
	};
	return (expandBits10(q(fx)) << 2) | (expandBits10(q(fy)) << 1) | expandBits10(q(fz));
}

RGL_HD int clz32(uint32_t x)
{
#if defined(__CUDA_ARCH__)
	return __clz((int) x);
#else
	return x == 0 ? 32 : __builtin_clz(x);
#endif
}

// Common-prefix length of sorted keys i and j, with the index as tie-break for equal keys.
RGL_HD int lbvhDelta(const uint32_t* codes, int n, int i, int j)
{
	if (j < 0 || j >= n) {
		return -1;
	}
	uint32_t a = codes[i], b = codes[j];
	if (a == b) {
		return 32 + clz32((uint32_t) i ^ (uint32_t) j);
	}
	return clz32(a ^ b);
}

// Internal node i of the LBVH over n >= 2 sorted keys. Children: >= 0 internal node, < 0 leaf ~k
// (k = sorted position). Also returns the covered sorted range [first, last].
RGL_HD void lbvhInternal(int i, const uint32_t* codes, int n, int32_t& left, int32_t& right, int32_t& first, int32_t& last)
{
	int d = (lbvhDelta(codes, n, i, i + 1) - lbvhDelta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
	int dmin = lbvhDelta(codes, n, i, i - d);
	int lmax = 2;
	while (lbvhDelta(codes, n, i, i + lmax * d) > dmin) {
		lmax *= 2;
	}
	int l = 0;
	for (int t = lmax / 2; t >= 1; t /= 2) {
		if (lbvhDelta(codes, n, i, i + (l + t) * d) > dmin) {
			l += t;
		}
	}
	int j = i + l * d;
	int dnode = lbvhDelta(codes, n, i, j);
	int s = 0;
	int div = 2;
	int t;
	do {
		t = (l + div - 1) / div;
		if (lbvhDelta(codes, n, i, i + (s + t) * d) > dnode) {
			s += t;
		}
		div *= 2;
	} while (t > 1);
	int gamma = i + s * d + (d < 0 ? -1 : 0);
	int lo = i < j ? i : j;
	int hi = i < j ? j : i;
	left = (lo == gamma) ? ~gamma : gamma;
	right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
	first = lo;
	last = hi;
}

// Quantisation grid of a wide node: origin p = lo - 2^(e-127) (rounded down to a float) and
// 2^(e-127) * kQuantSpan >= extent, so the node box spans grid steps 1 .. 253 at most. Child bounds
// are rounded outward to whole steps (quantizeAxis) and never widened further; the spare steps at
// both ends keep the outward-rounded bounds inside 0 .. 255 whatever the rounding of p.
constexpr double kQuantSpan = 252.0;

// Smallest power of two 2^(e-127) with kQuantSpan * 2^(e-127) >= ext, as the biased exponent byte e.
RGL_HD uint8_t quantExponent(float ext)
{
	double s = (double) ext / kQuantSpan;
	int e = 1; // 2^-126
	double p = 1.1754943508222875e-38;
	while (p < s && e < 254) {
		p *= 2.0;
		++e;
	}
	return (uint8_t) e;
}

RGL_HD void quantizeAxis(float p, float scale, float clo, float chi, uint8_t& qlo, uint8_t& qhi)
{
	double flo = ((double) clo - (double) p) / (double) scale;
	double fhi = ((double) chi - (double) p) / (double) scale;
	int lo = (int) flo; // flo >= 0
	if ((double) lo > flo) {
		--lo;
	}
	int hi = (int) fhi;
	if ((double) hi < fhi) {
		++hi;
	}
	lo = lo < 0 ? 0 : (lo > 255 ? 255 : lo);
	hi = hi < 0 ? 0 : (hi > 255 ? 255 : hi);
	// Verify the enclosure with the exact float sum p + q * scale.
	while (lo > 0 && fadd(p, (float) lo * scale) > clo) {
		--lo;
	}
	while (hi < 255 && fadd(p, (float) hi * scale) < chi) {
		++hi;
	}
	// No widening: the traversal moves every near plane earlier and every far plane later by a slack
	// that covers its plane-distance error (trace_core.hpp kPlaneSlack).
	qlo = (uint8_t) lo;
	qhi = (uint8_t) hi;
}

// Atomic counters used by the collapse step: device atomics on the GPU, plain adds on the host.
RGL_HD uint32_t atomicAddU32(uint32_t* p, uint32_t v)
{
#if defined(__CUDA_ARCH__)
	return atomicAdd(p, v);
#else
	uint32_t old = *p;
	*p = old + v;
	return old;
#endif
}

// Quantisation frame of a wide node over its box nb: per-axis exponents and an origin one grid step
// below the box (rounded down to a float), see kQuantSpan.
RGL_HD void setWideFrame(WideNode& w, const Box& nb)
{
	w.ex = quantExponent(nb.hix - nb.lox);
	w.ey = quantExponent(nb.hiy - nb.loy);
	w.ez = quantExponent(nb.hiz - nb.loz);
	auto originBelow = [](float lo, uint8_t e) {
		const double exact = (double) lo - (double) exp2Byte(e);
		float p = (float) exact;
		if ((double) p > exact) {
			p = nextafterf(p, -FLT_MAX);
		}
		return p;
	};
	w.px = originBelow(nb.lox, w.ex);
	w.py = originBelow(nb.loy, w.ey);
	w.pz = originBelow(nb.loz, w.ez);
}

// An empty child slot: a box that no ray enters.
RGL_HD void clearChild(WideNode& w, int k)
{
	w.qlox[k] = w.qloy[k] = w.qloz[k] = 255;
	w.qhix[k] = w.qhiy[k] = w.qhiz[k] = 0;
}

// Conservative 8-bit box of child slot k in the node's frame (rounded outward and verified, quantizeAxis).
RGL_HD void quantizeChild(WideNode& w, int k, const Box& b)
{
	const float sx = exp2Byte(w.ex), sy = exp2Byte(w.ey), sz = exp2Byte(w.ez);
	quantizeAxis(w.px, sx, b.lox, b.hix, w.qlox[k], w.qhix[k]);
	quantizeAxis(w.py, sy, b.loy, b.hiy, w.qloy[k], w.qhiy[k]);
	quantizeAxis(w.pz, sz, b.loz, b.hiz, w.qloz[k], w.qhiz[k]);
}

struct CollapseInputs
{
	const BinNode* bin;        // n-1 internal nodes with bounds (n >= 2)
	const int32_t* rangeFirst; // per internal node
	const int32_t* rangeLast;
	const int32_t* sortedIds;  // sorted position -> original triangle
	const float4* triLo;       // per original triangle
	const float4* triHi;
	const float* vertices;     // 3 floats per vertex; null: leaf records carry only primId (TLAS)
	const int32_t* indices;    // 3 ints per triangle
	int32_t leafMax;           // primitives per leaf child: kLeafMaxTris (BLAS) or 1 (TLAS)
};

struct CollapseOutputs
{
	WideNode* wide;
	TriRecord* tris;
	uint32_t* wideCounter;
	uint32_t* triCounter;
	int2* queueOut;
	uint32_t* queueOutCount;
	Box* wideBoxes; // optional: float box of every wide node (TLAS refit)
};

RGL_HD int binCount(const CollapseInputs& in, int32_t c) { return c < 0 ? 1 : (in.rangeLast[c] - in.rangeFirst[c] + 1); }

RGL_HD Box childBounds(const CollapseInputs& in, int32_t c)
{
	if (c >= 0) {
		return binBox(in.bin[c]);
	}
	int tid = in.sortedIds[~c];
	float4 lo = in.triLo[tid], hi = in.triHi[tid];
	return Box{lo.x, lo.y, lo.z, hi.x, hi.y, hi.z};
}

// Builds wide node `wideIdx` from the binary subtree rooted at `binRoot` (leaf ~k allowed).
RGL_HD void collapseItem(int32_t binRoot, uint32_t wideIdx, const CollapseInputs& in, const CollapseOutputs& out)
{
	int32_t ch[kWideArity];
	int n = 0;
	if (binRoot < 0) {
		ch[n++] = binRoot;
	} else {
		ch[n++] = in.bin[binRoot].left;
		ch[n++] = in.bin[binRoot].right;
	}
	while (n < kWideArity) {
		int bestK = -1;
		float bestA = -1.0f;
		for (int k = 0; k < n; ++k) {
			int32_t c = ch[k];
			if (c >= 0 && binCount(in, c) > in.leafMax) {
				float a = halfArea(binBox(in.bin[c]));
				if (a > bestA) {
					bestA = a;
					bestK = k;
				}
			}
		}
		if (bestK < 0) {
			break;
		}
		int32_t c = ch[bestK];
		ch[bestK] = in.bin[c].left;
		ch[n++] = in.bin[c].right;
	}

	Box cb0[kWideArity];
	Box nb = emptyBox();
	uint32_t nInternal = 0, nLeafTris = 0;
	for (int k = 0; k < n; ++k) {
		cb0[k] = childBounds(in, ch[k]);
		nb = unite(nb, cb0[k]);
		int cnt = binCount(in, ch[k]);
		if (ch[k] >= 0 && cnt > in.leafMax) {
			++nInternal;
		} else {
			nLeafTris += (uint32_t) cnt;
		}
	}
	// Slot assignment by octant: a child whose centre lies on the +x/+y/+z side of the node centre
	// prefers slot bit 0/1/2 set, so a ray visiting slots in order j ^ (ray direction sign bits)
	// meets children roughly front to back (the ordering idea of Ylitie et al., HPG 2017). Larger
	// children choose first; a taken slot falls back to the free slot nearest in Hamming distance.
	int32_t slotChild[kWideArity];
	for (int s = 0; s < kWideArity; ++s) {
		slotChild[s] = -1;
	}
	{
		float ncx = 0.5f * (nb.lox + nb.hix), ncy = 0.5f * (nb.loy + nb.hiy), ncz = 0.5f * (nb.loz + nb.hiz);
		bool placed[kWideArity] = {false, false, false, false, false, false, false, false};
		for (int round = 0; round < n; ++round) {
			int pick = -1;
			float pickArea = -1.0f;
			for (int k = 0; k < n; ++k) {
				float a = halfArea(cb0[k]);
				if (!placed[k] && a > pickArea) {
					pickArea = a;
					pick = k;
				}
			}
			const Box& b = cb0[pick];
			int oct = ((0.5f * (b.lox + b.hix) >= ncx) ? 1 : 0) | ((0.5f * (b.loy + b.hiy) >= ncy) ? 2 : 0) |
			          ((0.5f * (b.loz + b.hiz) >= ncz) ? 4 : 0);
			int best = -1, bestD = 99;
			for (int s = 0; s < kWideArity; ++s) {
				if (slotChild[s] < 0) {
					int dd = popc8((uint32_t) (s ^ oct));
					if (dd < bestD) {
						bestD = dd;
						best = s;
					}
				}
			}
			slotChild[best] = pick;
			placed[pick] = true;
		}
	}
	int32_t chs[kWideArity];
	Box cb[kWideArity];
	for (int s = 0; s < kWideArity; ++s) {
		chs[s] = slotChild[s] >= 0 ? ch[slotChild[s]] : 0;
		cb[s] = slotChild[s] >= 0 ? cb0[slotChild[s]] : emptyBox();
	}
	uint32_t childBase = nInternal ? atomicAddU32(out.wideCounter, nInternal) : 0;
	uint32_t triBase = nLeafTris ? atomicAddU32(out.triCounter, nLeafTris) : 0;
	uint32_t qBase = nInternal ? atomicAddU32(out.queueOutCount, nInternal) : 0;

	WideNode w;
	setWideFrame(w, nb);
	w.imask = 0;
	w.childBase = childBase;
	w.triBase = triBase;
	for (int k = 0; k < kWideArity; ++k) {
		w.meta[k] = 0;
		clearChild(w, k);
	}
	uint32_t rank = 0, triOff = 0;
	for (int k = 0; k < kWideArity; ++k) {
		if (slotChild[k] < 0) {
			continue;
		}
		quantizeChild(w, k, cb[k]);
		int32_t c = chs[k];
		int cnt = binCount(in, c);
		if (c >= 0 && cnt > in.leafMax) {
			w.imask |= (uint8_t) (1u << k);
			out.queueOut[qBase + rank] = make_int2(c, (int) (childBase + rank));
			++rank;
		} else {
			int firstPos = c < 0 ? ~c : in.rangeFirst[c];
			w.meta[k] = (uint8_t) ((cnt << 5) | (int) triOff);
			for (int m = 0; m < cnt; ++m) {
				int tid = in.sortedIds[firstPos + m];
				if (in.vertices == nullptr) { // TLAS leaf: the instance index only
					TriRecord tr{};
					tr.primId = tid;
					out.tris[triBase + triOff + m] = tr;
					continue;
				}
				const int32_t* ix = in.indices + 3 * (size_t) tid;
				const float* a = in.vertices + 3 * (size_t) ix[0];
				const float* b = in.vertices + 3 * (size_t) ix[1];
				const float* cc = in.vertices + 3 * (size_t) ix[2];
				TriRecord tr;
				tr.v0x = a[0];
				tr.v0y = a[1];
				tr.v0z = a[2];
				tr.primId = tid;
				tr.v1x = b[0];
				tr.v1y = b[1];
				tr.v1z = b[2];
				tr.pad1 = 0;
				tr.v2x = cc[0];
				tr.v2y = cc[1];
				tr.v2z = cc[2];
				tr.pad2 = 0;
				out.tris[triBase + triOff + m] = tr;
			}
			triOff += (uint32_t) cnt;
		}
	}
	out.wide[wideIdx] = w;
	if (out.wideBoxes) {
		out.wideBoxes[wideIdx] = nb;
	}
}

} // namespace rgl
