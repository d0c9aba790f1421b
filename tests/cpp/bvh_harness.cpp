// CPU harness of the test-suite: runs the library's BVH build steps (bvh_core.hpp) and closest-hit
// traversal (trace_core.hpp) serially on the host, so their logic can be checked against the oracle
// without a GPU. The CUDA kernels wrap exactly these functions.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "bvh_core.hpp"
#include "sah_build.hpp"
#include "trace_core.hpp"
#include "wave_split.hpp"

using namespace rgl;

namespace {

struct Blas
{
	std::vector<WideNode> wide;
	std::vector<TriRecord> tris;
	Box bounds;
};

void buildLbvh(const std::vector<uint32_t>& codes, std::vector<BinNode>& bin, std::vector<int32_t>& rf, std::vector<int32_t>& rl,
               std::vector<int32_t>& parentInt, std::vector<int32_t>& parentLeaf)
{
	int n = (int) codes.size();
	bin.assign(std::max(0, n - 1), BinNode{});
	rf.assign(std::max(0, n - 1), 0);
	rl.assign(std::max(0, n - 1), 0);
	parentInt.assign(std::max(0, n - 1), -1);
	parentLeaf.assign(n, -1);
	for (int i = 0; i < n - 1; ++i) {
		int32_t l, r, f, la;
		lbvhInternal(i, codes.data(), n, l, r, f, la);
		bin[i].left = l;
		bin[i].right = r;
		rf[i] = f;
		rl[i] = la;
		if (l >= 0)
			parentInt[l] = i;
		else
			parentLeaf[~l] = i;
		if (r >= 0)
			parentInt[r] = i;
		else
			parentLeaf[~r] = i;
	}
}

void bottomUp(std::vector<BinNode>& bin, const std::vector<int32_t>& parentInt, const std::vector<int32_t>& parentLeaf,
              const std::vector<Box>& leafBox)
{
	int n = (int) leafBox.size();
	std::vector<int> visits(bin.size(), 0);
	for (int k = 0; k < n; ++k) {
		int node = parentLeaf[k];
		while (node >= 0) {
			if (visits[node]++ == 0)
				break;
			Box a = bin[node].left >= 0 ? binBox(bin[bin[node].left]) : leafBox[~bin[node].left];
			Box b = bin[node].right >= 0 ? binBox(bin[bin[node].right]) : leafBox[~bin[node].right];
			Box u = unite(a, b);
			bin[node].lox = u.lox;
			bin[node].loy = u.loy;
			bin[node].loz = u.loz;
			bin[node].hix = u.hix;
			bin[node].hiy = u.hiy;
			bin[node].hiz = u.hiz;
			node = parentInt[node];
		}
	}
}

// Wide BVH over primitive boxes lo/hi, as the device builder makes it (bvh.cu buildWide): leaf records
// are triangles (v/idx given) or primitive indices (v null, the TLAS).
Blas buildWideHost(std::vector<float4> lo, std::vector<float4> hi, const float* v, const int32_t* idx, int leafMax)
{
	const int nt = (int) lo.size();
	Box cb = emptyBox();
	std::vector<float> cx(nt), cy(nt), cz(nt);
	for (int t = 0; t < nt; ++t) {
		cx[t] = 0.5f * (lo[t].x + hi[t].x);
		cy[t] = 0.5f * (lo[t].y + hi[t].y);
		cz[t] = 0.5f * (lo[t].z + hi[t].z);
		cb = unite(cb, Box{cx[t], cy[t], cz[t], cx[t], cy[t], cz[t]});
	}
	std::vector<uint32_t> code(nt);
	std::vector<int32_t> ids(nt);
	for (int t = 0; t < nt; ++t) {
		code[t] = morton30(cx[t], cy[t], cz[t], cb);
		ids[t] = t;
	}
	std::stable_sort(ids.begin(), ids.end(), [&](int a, int b) { return code[a] < code[b]; });
	std::vector<uint32_t> sortedCode(nt);
	for (int k = 0; k < nt; ++k)
		sortedCode[k] = code[ids[k]];
	std::vector<BinNode> bin;
	std::vector<int32_t> rf, rl, pi, pl;
	buildLbvh(sortedCode, bin, rf, rl, pi, pl);
	std::vector<Box> leafBox(nt);
	for (int k = 0; k < nt; ++k) {
		int t = ids[k];
		leafBox[k] = Box{lo[t].x, lo[t].y, lo[t].z, hi[t].x, hi[t].y, hi[t].z};
	}
	bottomUp(bin, pi, pl, leafBox);

	Blas out;
	out.wide.resize(std::max(1, nt));
	out.tris.resize(nt);
	uint32_t wideCounter = 1, triCounter = 0;
	std::vector<int2> qa(std::max(1, nt)), qb(std::max(1, nt));
	uint32_t qaCount = 1, qbCount = 0;
	qa[0] = make_int2(nt == 1 ? ~0 : 0, 0);
	CollapseInputs in{bin.data(), rf.data(), rl.data(), ids.data(), lo.data(), hi.data(), v, idx, leafMax};
	while (qaCount > 0) {
		qbCount = 0;
		CollapseOutputs o{out.wide.data(), out.tris.data(), &wideCounter, &triCounter, qb.data(), &qbCount, nullptr};
		for (uint32_t i = 0; i < qaCount; ++i)
			collapseItem(qa[i].x, (uint32_t) qa[i].y, in, o);
		std::swap(qa, qb);
		qaCount = qbCount;
	}
	out.wide.resize(wideCounter);
	out.bounds = nt == 1 ? leafBox[0] : binBox(bin[0]);
	return out;
}

// Wide TLAS from a host SAH topology (sah_build.hpp), collapsed like the device build.
Blas buildTlasSah(const std::vector<float4>& lo, const std::vector<float4>& hi)
{
	const int n = (int) lo.size();
	std::vector<Box> boxes(n);
	for (int i = 0; i < n; ++i) {
		boxes[i] = Box{lo[i].x, lo[i].y, lo[i].z, hi[i].x, hi[i].y, hi[i].z};
	}
	SahTree t = buildSahTree(boxes);
	Blas out;
	out.wide.resize(std::max(1, n));
	out.tris.resize(n);
	uint32_t wideCounter = 1, triCounter = 0;
	std::vector<int2> qa(std::max(1, n)), qb(std::max(1, n));
	uint32_t qaCount = 1, qbCount = 0;
	qa[0] = make_int2(n == 1 ? ~0 : 0, 0);
	CollapseInputs in{t.bin.data(), t.rangeFirst.data(), t.rangeLast.data(), t.sortedIds.data(), lo.data(), hi.data(), nullptr, nullptr, 1};
	while (qaCount > 0) {
		qbCount = 0;
		CollapseOutputs o{out.wide.data(), out.tris.data(), &wideCounter, &triCounter, qb.data(), &qbCount, nullptr};
		for (uint32_t i = 0; i < qaCount; ++i)
			collapseItem(qa[i].x, (uint32_t) qa[i].y, in, o);
		std::swap(qa, qb);
		qaCount = qbCount;
	}
	out.wide.resize(wideCounter);
	return out;
}

int gTlasSah = 1; // the product builds the TLAS topology by SAH (sah_build.hpp)

// Wide BLAS from the product's binned SAH topology (sah_build.hpp), collapsed like the product.
Blas buildBlasSah(const std::vector<float4>& lo, const std::vector<float4>& hi, const float* v, const int32_t* idx)
{
	const int n = (int) lo.size();
	std::vector<Box> boxes(n);
	for (int i = 0; i < n; ++i) {
		boxes[i] = Box{lo[i].x, lo[i].y, lo[i].z, hi[i].x, hi[i].y, hi[i].z};
	}
	SahTree t = buildBinnedSahTree(boxes);
	Blas out;
	out.wide.resize(std::max(1, n));
	out.tris.resize(n);
	uint32_t wideCounter = 1, triCounter = 0;
	std::vector<int2> qa(std::max(1, n)), qb(std::max(1, n));
	uint32_t qaCount = 1, qbCount = 0;
	qa[0] = make_int2(n == 1 ? ~0 : 0, 0);
	CollapseInputs in{t.bin.data(), t.rangeFirst.data(), t.rangeLast.data(), t.sortedIds.data(), lo.data(), hi.data(), v, idx, kLeafMaxTris};
	while (qaCount > 0) {
		qbCount = 0;
		CollapseOutputs o{out.wide.data(), out.tris.data(), &wideCounter, &triCounter, qb.data(), &qbCount, nullptr};
		for (uint32_t i = 0; i < qaCount; ++i)
			collapseItem(qa[i].x, (uint32_t) qa[i].y, in, o);
		std::swap(qa, qb);
		qaCount = qbCount;
	}
	out.wide.resize(wideCounter);
	out.bounds = n == 1 ? boxes[0] : binBox(t.bin[0]);
	return out;
}

int gBlasSah = 1; // the product builds mesh BLASes by binned SAH; 0: the device's Morton LBVH

Blas buildBlas(const float* v, int nv, const int32_t* idx, int nt)
{
	(void) nv;
	std::vector<float4> lo(nt), hi(nt);
	for (int t = 0; t < nt; ++t) {
		const float* a = v + 3 * idx[3 * t];
		const float* b = v + 3 * idx[3 * t + 1];
		const float* c = v + 3 * idx[3 * t + 2];
		lo[t] = make_float4(std::min({a[0], b[0], c[0]}), std::min({a[1], b[1], c[1]}), std::min({a[2], b[2], c[2]}), 0);
		hi[t] = make_float4(std::max({a[0], b[0], c[0]}), std::max({a[1], b[1], c[1]}), std::max({a[2], b[2], c[2]}), 0);
	}
	return gBlasSah ? buildBlasSah(lo, hi, v, idx) : buildWideHost(lo, hi, v, idx, kLeafMaxTris);
}

// Stack entries the device keeps on chip (shared memory); pushes and pops past them are counted.
int gStackOnChip = 24;
long gDeepPushes = 0, gDeepPops = 0;

struct HostStack
{
	uint32_t a[512], b[512];
	int sp = 0;
	int maxDepth = 0;
	bool overflow = false;
	void push(uint32_t x, uint32_t y)
	{
		if (sp >= 512) {
			overflow = true;
			return;
		}
		gDeepPushes += sp >= gStackOnChip ? 1 : 0;
		a[sp] = x;
		b[sp] = y;
		++sp;
		maxDepth = std::max(maxDepth, sp);
	}
	void pop(uint32_t& x, uint32_t& y)
	{
		--sp;
		gDeepPops += sp >= gStackOnChip ? 1 : 0;
		x = a[sp];
		y = b[sp];
	}
	int size() const { return sp; }
};

int gNodeVisits = 0;
int gRayTris = 0;                             // triangle tests of the current ray
std::vector<int> gVisitsPerRay, gTrisPerRay; // per ray of the last harness_cast (single-ray mode)
long gTriTests = 0, gBinLoads = 0, gInstLoads = 0, gTlasVisits = 0;
const WideNode* gTlasBase = nullptr;

struct HostLoader
{
	void nodeWords(const WideNode* base, uint32_t i, uint4& w0, uint4& w1, uint4& w2, uint4& w3, uint4& w4) const
	{
		++gNodeVisits;
		gTlasVisits += base == gTlasBase ? 1 : 0;
		const uint4* p = reinterpret_cast<const uint4*>(base + i);
		w0 = p[0];
		w1 = p[1];
		w2 = p[2];
		w3 = p[3];
		w4 = p[4];
	}
	TriRecord tri(const TriRecord* base, int32_t i) const
	{
		++gTriTests;
		++gRayTris;
		return base[i];
	}
	const InstanceRec& instance(const InstanceRec* base, int32_t i) const
	{
		++gInstLoads;
		return base[i];
	}
	int32_t leafPrim(const TriRecord* base, int32_t i) const
	{
		++gBinLoads;
		return base[i].primId;
	}
};

// ---------------------------------------------------------------- union traversal (test only)
//
// A second traversal order for the order-independence test: up to P rays sharing an origin walk the
// hierarchy together; every ray is tested against each visited node and a child is entered when any
// ray hits it, so the walk visits the union of the rays' nodes (in the first ray's octant order) and
// each ray tests at least the triangles its own traversal would. With closerHit() (trace_core.hpp)
// each ray's hit must then equal traceClosest's, bit for bit. Built only from the library's node
// decode, slab and triangle primitives.

// The set is held by one thread: nothing to share between lanes.
struct SoloGroup
{
	RGL_HD uint32_t unite(uint32_t v) const { return v; }
	RGL_HD uint32_t orderOctant(uint32_t oct) const { return oct; }
};

template<int P>
struct PacketFrame
{
	Vec3 o;
	Vec3 inv[P];
	uint32_t selOct; // octant of ray 0: near/far plane selection when the rays share it
	uint32_t ordOct; // child visiting order, common to the whole set
	bool mixed;      // the rays' octants differ: near and far planes are found per ray
};

// World directions and per-frame watertight constants of the set's rays are kept by `Scratch`
// (registers for one ray, shared memory or arrays for more), read once per frame change and once per
// triangle test. Scratch provides dir(r), setDir(r, v), wt(r) and setWt(r, w).
template<int P, class Scratch, class Group>
RGL_HD void setPacketFrame(PacketFrame<P>& f, Vec3 o, const Mat34* worldToObject, Scratch& sp, const Group& grp)
{
	f.o = o;
	uint32_t any = 0u, all = 7u;
	for (int r = 0; r < P; ++r) {
		const Vec3 d = worldToObject ? worldToObject->vector(sp.dir(r)) : sp.dir(r);
		f.inv[r] = {safeInv(d.x), safeInv(d.y), safeInv(d.z)};
		const uint32_t oc = (f.inv[r].x < 0.0f ? 1u : 0u) | (f.inv[r].y < 0.0f ? 2u : 0u) | (f.inv[r].z < 0.0f ? 4u : 0u);
		any |= oc;
		all &= oc;
		if (r == 0) {
			f.selOct = oc;
		}
		if (worldToObject) {
			sp.setWt(r, setupWatertight(d));
		}
	}
	f.mixed = any != all;
	f.ordOct = grp.orderOctant(f.selOct);
}

// Closest hits of the rays oW + t sp.dir(r), t in (0, tmax], r < n (n <= P; directions r >= n must be
// finite, e.g. copies of ray 0's, and get t = -1 with no hit). Every member of `grp` must make the
// call with the same oW, scene and stack depth.
template<int P, class Stack, class NodeLoader, class Scratch, class Group>
RGL_HD void traceClosestPacket(const SceneView& sc, Vec3 oW, int n, float tmax, Stack& st, const NodeLoader& load, Scratch& sp,
                               const Group& grp, HitRec (&best)[P])
{
	for (int r = 0; r < P; ++r) {
		best[r].t = r < n ? tmax : -1.0f; // an inactive ray culls every box and triangle
		best[r].inst = -1;
		best[r].tri = -1;
		best[r].prim = -1;
	}
	if (sc.nInstances <= 0) {
		return;
	}
	const int base = st.size();
	PacketFrame<P> f;
	setPacketFrame<P>(f, oW, nullptr, sp, grp);
	const WideNode* nodes = sc.tlas;
	const TriRecord* leaves = sc.tlasLeaves;
	int32_t inst = -1;
	uint32_t node = 0;
	for (;;) {
		uint4 w0, w1, w2, w3, w4;
		load.nodeWords(nodes, node, w0, w1, w2, w3, w4);
		const float sx = exp2Byte((uint8_t) (w0.w & 0xffu)), sy = exp2Byte((uint8_t) ((w0.w >> 8) & 0xffu)),
		            sz = exp2Byte((uint8_t) ((w0.w >> 16) & 0xffu));
		const uint32_t imask = w0.w >> 24;
		const uint32_t childBase = w1.x, triBase = w1.y;
		const float px = asFloat(w0.x) - f.o.x, py = asFloat(w0.y) - f.o.y, pz = asFloat(w0.z) - f.o.z;
		// Per ray the slab form of traceClosest: t = fma(1 + q 2^-15, 2^15 A, C - 2^15 A).
		float Sx[P], Sy[P], Sz[P], Dx[P], Dy[P], Dz[P];
		for (int r = 0; r < P; ++r) {
			Sx[r] = 32768.0f * (sx * f.inv[r].x);
			Sy[r] = 32768.0f * (sy * f.inv[r].y);
			Sz[r] = 32768.0f * (sz * f.inv[r].z);
			Dx[r] = px * f.inv[r].x - Sx[r];
			Dy[r] = py * f.inv[r].y - Sy[r];
			Dz[r] = pz * f.inv[r].z - Sz[r];
		}
		uint32_t hitSlots = 0;
		if (!f.mixed) {
			// One octant: near/far planes selected once for the packet.
			const bool negx = (f.selOct & 1u) != 0, negy = (f.selOct & 2u) != 0, negz = (f.selOct & 4u) != 0;
			const uint32_t nx0 = negx ? w3.z : w2.x, nx1 = negx ? w3.w : w2.y, fx0 = negx ? w2.x : w3.z, fx1 = negx ? w2.y : w3.w;
			const uint32_t ny0 = negy ? w4.x : w2.z, ny1 = negy ? w4.y : w2.w, fy0 = negy ? w2.z : w4.x, fy1 = negy ? w2.w : w4.y;
			const uint32_t nz0 = negz ? w4.z : w3.x, nz1 = negz ? w4.w : w3.y, fz0 = negz ? w3.x : w4.z, fz1 = negz ? w3.y : w4.w;
			for (int s = 0; s < kWideArity; ++s) {
				const int k = s & 3;
				const bool hiw = s >= 4;
				const float bnx = byteMantissa(hiw ? nx1 : nx0, k), bfx = byteMantissa(hiw ? fx1 : fx0, k);
				const float bny = byteMantissa(hiw ? ny1 : ny0, k), bfy = byteMantissa(hiw ? fy1 : fy0, k);
				const float bnz = byteMantissa(hiw ? nz1 : nz0, k), bfz = byteMantissa(hiw ? fz1 : fz0, k);
				uint32_t h = 0u; // no short circuit: every ray's test is straight-line code
				for (int r = 0; r < P; ++r) {
					// The traversal's plane slack: near planes earlier, far planes later.
					const float ex = kPlaneSlack * absf_(Sx[r]), ey = kPlaneSlack * absf_(Sy[r]), ez = kPlaneSlack * absf_(Sz[r]);
					const float tEntry = max4(fmaf(bnx, Sx[r], Dx[r] - ex), fmaf(bny, Sy[r], Dy[r] - ey), fmaf(bnz, Sz[r], Dz[r] - ez), 0.0f);
					const float tExit = min4(fmaf(bfx, Sx[r], Dx[r] + ex), fmaf(bfy, Sy[r], Dy[r] + ey), fmaf(bfz, Sz[r], Dz[r] + ez), best[r].t);
					h |= (tEntry <= tExit * kSlabRelSlack) ? 1u : 0u;
				}
				hitSlots |= h << s;
			}
		} else {
			// Mixed octants: both planes per axis, near = min, far = max, per ray.
			for (int s = 0; s < kWideArity; ++s) {
				const int k = s & 3;
				const bool hiw = s >= 4;
				const float lx = byteMantissa(hiw ? w2.y : w2.x, k), hx = byteMantissa(hiw ? w3.w : w3.z, k);
				const float ly = byteMantissa(hiw ? w2.w : w2.z, k), hy = byteMantissa(hiw ? w4.y : w4.x, k);
				const float lz = byteMantissa(hiw ? w3.y : w3.x, k), hz = byteMantissa(hiw ? w4.w : w4.z, k);
				uint32_t h = 0u;
				for (int r = 0; r < P; ++r) {
					const float ax = fmaf(lx, Sx[r], Dx[r]), bx = fmaf(hx, Sx[r], Dx[r]);
					const float ay = fmaf(ly, Sy[r], Dy[r]), by = fmaf(hy, Sy[r], Dy[r]);
					const float az = fmaf(lz, Sz[r], Dz[r]), bz = fmaf(hz, Sz[r], Dz[r]);
					const float ex = kPlaneSlack * absf_(Sx[r]), ey = kPlaneSlack * absf_(Sy[r]), ez = kPlaneSlack * absf_(Sz[r]);
					const float tEntry = max4(minf_(ax, bx) - ex, minf_(ay, by) - ey, minf_(az, bz) - ez, 0.0f);
					const float tExit = min4(maxf_(ax, bx) + ex, maxf_(ay, by) + ey, maxf_(az, bz) + ez, best[r].t);
					h |= (tEntry <= tExit * kSlabRelSlack) ? 1u : 0u;
				}
				hitSlots |= h << s;
			}
		}
		hitSlots = grp.unite(hitSlots);
		const uint32_t ordered = octantPermute((hitSlots & imask) | ((hitSlots & ~imask & 0xffu) << 8), f.ordOct);
		uint32_t internalHits = ordered & 0xffu, leafHits = ordered >> 8;
		const uint32_t metaLo = w1.z, metaHi = w1.w;
		if (inst < 0) {
			while (leafHits) {
				const uint32_t j = highestBit(leafHits);
				leafHits &= ~(1u << j);
				const uint32_t s = j ^ f.ordOct;
				const uint32_t meta = ((s < 4 ? metaLo : metaHi) >> ((s & 3) * 8)) & 0xffu;
				st.push((uint32_t) load.leafPrim(leaves, (int) triBase + (int) (meta & 31u)), kEnterInstance);
			}
		} else {
			while (leafHits) {
				const uint32_t s = lowestBit(leafHits) ^ f.ordOct;
				leafHits &= leafHits - 1u;
				const uint32_t meta = ((s < 4 ? metaLo : metaHi) >> ((s & 3) * 8)) & 0xffu;
				const int first = (int) triBase + (int) (meta & 31u);
				const int cnt = (int) (meta >> 5);
				for (int k = 0; k < cnt; ++k) {
					const TriRecord tr = load.tri(leaves, first + k);
					const Vec3 a = v3(tr.v0x, tr.v0y, tr.v0z), b = v3(tr.v1x, tr.v1y, tr.v1z), c = v3(tr.v2x, tr.v2y, tr.v2z);
					for (int r = 0; r < P; ++r) {
						float t;
						if (r < n && intersectTriangle(a, b, c, f.o, sp.wt(r), best[r].t, t) && closerHit(t, inst, tr.primId, best[r])) {
							best[r].t = t;
							best[r].inst = inst;
							best[r].tri = first + k;
							best[r].prim = tr.primId;
						}
					}
				}
			}
		}
		uint32_t groupBase = childBase, groupMask = imask, hits = internalHits;
		bool enterRoot = false;
		while (hits == 0) {
			if (st.size() == base) {
				return;
			}
			uint32_t a, b;
			st.pop(a, b);
			if (b == kLeaveInstance) {
				setPacketFrame<P>(f, oW, nullptr, sp, grp);
				nodes = sc.tlas;
				leaves = sc.tlasLeaves;
				inst = -1;
			} else if (b == kEnterInstance) {
				const InstanceRec& ir = load.instance(sc.instances, (int32_t) a);
				st.push(0u, kLeaveInstance);
				setPacketFrame<P>(f, worldToInstance(ir, oW), &ir.worldToObject, sp, grp);
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
		const uint32_t s = lowestBit(hits) ^ f.ordOct;
		hits &= hits - 1u;
		if (hits) {
			st.push(groupBase, groupMask | (hits << 8));
		}
		node = groupBase + (uint32_t) popc8(groupMask & ((1u << s) - 1u));
	}
}

template<int P>
struct HostPacketScratch
{
	Vec3 d[P];
	Watertight w[P];
	Vec3 dir(int r) const { return d[r]; }
	void setDir(int r, Vec3 v) { d[r] = v; }
	Watertight wt(int r) const { return w[r]; }
	void setWt(int r, const Watertight& x) { w[r] = x; }
};

// Casts groups of `group` consecutive rays (same origin) as packets; returns false on stack overflow.
template<int P>
bool castPackets(const SceneView& sv, int nRays, int group, const float* rays, HitRec* out)
{
	HostLoader ld;
	for (int g0 = 0; g0 < nRays; g0 += group) {
		const int n = std::min(group, nRays - g0);
		HostPacketScratch<P> sp;
		for (int r = 0; r < P; ++r) {
			const float* p = rays + 7 * (g0 + (r < n ? r : 0));
			sp.setDir(r, v3(p[3], p[4], p[5]));
		}
		const float* p0 = rays + 7 * g0;
		HostStack st;
		HitRec h[P];
		traceClosestPacket<P>(sv, v3(p0[0], p0[1], p0[2]), n, p0[6], st, ld, sp, SoloGroup{}, h);
		if (st.overflow) {
			return false;
		}
		for (int r = 0; r < n; ++r) {
			// the closest hit's distance from its plane, as the single-ray traversal finishes
			out[g0 + r] = refineClosest(sv, v3(p0[0], p0[1], p0[2]), sp.dir(r), h[r], ld);
		}
	}
	return true;
}

} // namespace

extern "C" {

// Largest number of wide-node visits of a single ray in the last harness_cast call.
int gMaxNodeVisits = 0;
long gTotalNodeVisits = 0;
int gMaxStackDepth = 0;
int harness_max_node_visits() { return gMaxNodeVisits; }
// 1: build the TLAS topology with the host SAH builder instead of the Morton-ordered LBVH.
void harness_set_tlas_sah(int on) { gTlasSah = on; }
// 1: build mesh BLASes with the binned SAH (as the product does); 0: with the Morton LBVH.
void harness_set_blas_sah(int on) { gBlasSah = on; }
// Deepest traversal stack of a single ray in the last harness_cast call.
int harness_max_stack_depth() { return gMaxStackDepth; }
long harness_total_node_visits() { return gTotalNodeVisits; }
// Stack entries held on chip (the rest would live in local memory on the device), and the pushes and
// pops of the last harness_cast call that went past them.
void harness_set_stack_on_chip(int entries) { gStackOnChip = entries; }
void harness_deep_stack_ops(long* out)
{
	out[0] = gDeepPushes;
	out[1] = gDeepPops;
}
// Totals of the last harness_cast call: triangle tests, TLAS leaf reads, instance entries, TLAS
// node visits.
void harness_work_counters(long* out)
{
	out[0] = gTriTests;
	out[1] = gBinLoads;
	out[2] = gInstLoads;
	out[3] = gTlasVisits;
}

// 0: every ray alone (traceClosest); g in 1..8: groups of g consecutive rays, which must share their
// origin and tmax, walk together (traceClosestPacket with the packet size the device uses for g).
int gPacketGroup = 0;
void harness_set_packet_group(int g) { gPacketGroup = g; }

// Builds BLASes for `nMeshes` meshes and a TLAS over `nInst` instances, then casts `nRays` world
// rays (origin, direction, tmax: 7 floats each). Outputs per ray: t, instance, original triangle id.
// Returns the number of wide nodes of mesh 0 (for diagnostics), or -1 on stack overflow.
int harness_cast(int nMeshes, const float* const* verts, const int* nVerts, const int32_t* const* idx, const int* nTris,
                 int nInst, const int* instMesh, const float* instTf, const int* instId, int nRays, const float* rays,
                 float* outT, int32_t* outInst, int32_t* outPrim)
{
	std::vector<Blas> blas;
	for (int m = 0; m < nMeshes; ++m)
		blas.push_back(buildBlas(verts[m], nVerts[m], idx[m], nTris[m]));
	std::vector<InstanceRec> inst(nInst);
	std::vector<Box> ib(nInst);
	Box cb = emptyBox();
	for (int i = 0; i < nInst; ++i) {
		Mat34 tf;
		std::memcpy(tf.m, instTf + 12 * i, 48);
		inst[i].objectToWorld = tf;
		inst[i].worldToObject = inverse(tf);
		inst[i].nodes = blas[instMesh[i]].wide.data();
		inst[i].tris = blas[instMesh[i]].tris.data();
		inst[i].entityId = instId[i];
		{
			const Mat34 id = Mat34::identity();
			inst[i].flags = std::memcmp(&tf, &id, sizeof(Mat34)) == 0 ? kInstanceIdentity : 0;
		}
		Box b = blas[instMesh[i]].bounds;
		Box w = emptyBox();
		for (int c = 0; c < 8; ++c) {
			Vec3 p = tf.point(v3((c & 1) ? b.hix : b.lox, (c & 2) ? b.hiy : b.loy, (c & 4) ? b.hiz : b.loz));
			w = unite(w, Box{p.x, p.y, p.z, p.x, p.y, p.z});
		}
		float pad = 4e-6f * (std::max({std::fabs(w.lox), std::fabs(w.hix), std::fabs(w.loy), std::fabs(w.hiy),
		                               std::fabs(w.loz), std::fabs(w.hiz)}) + 1.0f);
		w = Box{w.lox - pad, w.loy - pad, w.loz - pad, w.hix + pad, w.hiy + pad, w.hiz + pad};
		inst[i].lox = w.lox;
		inst[i].loy = w.loy;
		inst[i].loz = w.loz;
		inst[i].hix = w.hix;
		inst[i].hiy = w.hiy;
		inst[i].hiz = w.hiz;
		ib[i] = w;
		float c3[3] = {0.5f * (w.lox + w.hix), 0.5f * (w.loy + w.hiy), 0.5f * (w.loz + w.hiz)};
		cb = unite(cb, Box{c3[0], c3[1], c3[2], c3[0], c3[1], c3[2]});
	}
	std::vector<float4> ilo(nInst), ihi(nInst);
	for (int i = 0; i < nInst; ++i) {
		ilo[i] = make_float4(ib[i].lox, ib[i].loy, ib[i].loz, 0);
		ihi[i] = make_float4(ib[i].hix, ib[i].hiy, ib[i].hiz, 0);
	}
	(void) cb;
	Blas tlas = gTlasSah ? buildTlasSah(ilo, ihi) : buildWideHost(ilo, ihi, nullptr, nullptr, 1);
	SceneView sv{tlas.wide.data(), tlas.tris.data(), inst.data(), nInst, 0};
	gTlasBase = tlas.wide.data();
	HostLoader ld;
	bool overflow = false;
	gMaxNodeVisits = 0;
	gTotalNodeVisits = 0;
	gTriTests = gBinLoads = gInstLoads = gTlasVisits = 0;
	gMaxStackDepth = 0;
	gDeepPushes = gDeepPops = 0;
	gVisitsPerRay.assign(nRays, 0);
	gTrisPerRay.assign(nRays, 0);
	if (gPacketGroup > 0) {
		gNodeVisits = 0;
		std::vector<HitRec> hits(nRays);
		const bool ok = gPacketGroup <= 4 ? castPackets<4>(sv, nRays, gPacketGroup, rays, hits.data())
		                : gPacketGroup == 5 ? castPackets<5>(sv, nRays, gPacketGroup, rays, hits.data())
		                                    : castPackets<8>(sv, nRays, gPacketGroup, rays, hits.data());
		gTotalNodeVisits = gNodeVisits;
		for (int r = 0; r < nRays; ++r) {
			outT[r] = hits[r].t;
			outInst[r] = hits[r].inst;
			outPrim[r] = hits[r].inst >= 0 ? inst[hits[r].inst].tris[hits[r].tri].primId : -1;
		}
		return ok ? (nMeshes > 0 ? (int) blas[0].wide.size() : 0) : -1;
	}
	for (int r = 0; r < nRays; ++r) {
		const float* p = rays + 7 * r;
		HostStack st;
		gNodeVisits = 0;
		gRayTris = 0;
		HitRec h = traceClosest(sv, v3(p[0], p[1], p[2]), v3(p[3], p[4], p[5]), p[6], st, ld);
		overflow = overflow || st.overflow;
		gMaxStackDepth = std::max(gMaxStackDepth, st.maxDepth);
		gMaxNodeVisits = std::max(gMaxNodeVisits, gNodeVisits);
		gTotalNodeVisits += gNodeVisits;
		gVisitsPerRay[r] = gNodeVisits;
		gTrisPerRay[r] = gRayTris;
		outT[r] = h.t;
		outInst[r] = h.inst;
		outPrim[r] = h.inst >= 0 ? inst[h.inst].tris[h.tri].primId : -1;
	}
	if (overflow)
		return -1;
	return nMeshes > 0 ? (int) blas[0].wide.size() : 0;
}

// The wave cut of a batched frame (wave_split.hpp): first member of each wave, then n, into outFirst
// (room for n + 2 entries); returns the number of waves.
int harness_split_waves(const int64_t* rays, int n, int waves, int* outFirst)
{
	const std::vector<int> first = rgl::splitIntoWaves(std::vector<int64_t>(rays, rays + n), waves);
	std::copy(first.begin(), first.end(), outFirst);
	return (int) first.size() - 1;
}

// Node visits and triangle tests of each ray of the last harness_cast (single-ray mode).
void harness_ray_work(int* visits, int* tris, int n)
{
	for (int i = 0; i < n && i < (int) gVisitsPerRay.size(); ++i) {
		visits[i] = gVisitsPerRay[i];
		tris[i] = gTrisPerRay[i];
	}
}

} // extern "C"
