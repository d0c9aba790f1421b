// CPU harness of the test-suite: runs the library's BVH build steps (bvh_core.hpp) and closest-hit
// traversal (trace_core.hpp) serially on the host, so their logic can be checked against the oracle
// without a GPU. The CUDA kernels wrap exactly these functions.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "bvh_core.hpp"
#include "tlas_sah.hpp"
#include "trace_core.hpp"

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

// Wide TLAS from a host SAH topology (tlas_sah.hpp), collapsed like the device build.
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

int gTlasSah = 1; // the product builds the TLAS topology by SAH (tlas_sah.hpp)

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
	return buildWideHost(lo, hi, v, idx, kLeafMaxTris);
}

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
		a[sp] = x;
		b[sp] = y;
		++sp;
		maxDepth = std::max(maxDepth, sp);
	}
	void pop(uint32_t& x, uint32_t& y)
	{
		--sp;
		x = a[sp];
		y = b[sp];
	}
	int size() const { return sp; }
};

int gNodeVisits = 0;
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

} // namespace

extern "C" {

// Largest number of wide-node visits of a single ray in the last harness_cast call.
int gMaxNodeVisits = 0;
long gTotalNodeVisits = 0;
int gMaxStackDepth = 0;
int harness_max_node_visits() { return gMaxNodeVisits; }
// 1: build the TLAS topology with the host SAH builder instead of the Morton-ordered LBVH.
void harness_set_tlas_sah(int on) { gTlasSah = on; }
// Deepest traversal stack of a single ray in the last harness_cast call.
int harness_max_stack_depth() { return gMaxStackDepth; }
long harness_total_node_visits() { return gTotalNodeVisits; }
// Totals of the last harness_cast call: triangle tests, TLAS leaf reads, instance entries, TLAS
// node visits.
void harness_work_counters(long* out)
{
	out[0] = gTriTests;
	out[1] = gBinLoads;
	out[2] = gInstLoads;
	out[3] = gTlasVisits;
}

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
		Box b = blas[instMesh[i]].bounds;
		Box w = emptyBox();
		for (int c = 0; c < 8; ++c) {
			Vec3 p = tf.point(v3((c & 1) ? b.hix : b.lox, (c & 2) ? b.hiy : b.loy, (c & 4) ? b.hiz : b.loz));
			w = unite(w, Box{p.x, p.y, p.z, p.x, p.y, p.z});
		}
		float pad = 1e-6f * (std::max({std::fabs(w.lox), std::fabs(w.hix), std::fabs(w.loy), std::fabs(w.hiy),
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
	for (int r = 0; r < nRays; ++r) {
		const float* p = rays + 7 * r;
		HostStack st;
		gNodeVisits = 0;
		HitRec h = traceClosest(sv, v3(p[0], p[1], p[2]), v3(p[3], p[4], p[5]), p[6], st, ld);
		overflow = overflow || st.overflow;
		gMaxStackDepth = std::max(gMaxStackDepth, st.maxDepth);
		gMaxNodeVisits = std::max(gMaxNodeVisits, gNodeVisits);
		gTotalNodeVisits += gNodeVisits;
		outT[r] = h.t;
		outInst[r] = h.inst;
		outPrim[r] = h.inst >= 0 ? inst[h.inst].tris[h.tri].primId : -1;
	}
	if (overflow)
		return -1;
	return nMeshes > 0 ? (int) blas[0].wide.size() : 0;
}

} // extern "C"
