// CPU oracle for the RGL lidar ray-casting path — TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++ (FP64 where the reference leaves precision open, FP32 where the
// reference's semantics are defined by float arithmetic), what RobotecGPULidar computes on its ray
// casting path.  It is used by the test-suite, by __graft_entry__.smoke() and by bench.py's CPU
// baseline as the checker; the product library never links or calls it.
//
// Reference behaviour restated here (paths relative to the RobotecGPULidar tree):
//  * ray pose -> ray:        src/gpu/optixPrograms.cu:222-228 (origin = M*0, dir = M*z - origin, t in [0,maxRange])
//  * beam sub-ray pattern:   src/gpu/optixPrograms.cu:75-86,230-248, src/gpu/MultiReturn.hpp:19-21
//  * closest hit / min range src/gpu/optixPrograms.cu:96-136 (FP64 distance, near non-hit without continuation)
//  * miss:                   src/gpu/optixPrograms.cu:89-94 (far non-hit distance)
//  * intensity:              src/gpu/optixPrograms.cu:138-167 (default intensity * |cos incidence|)
//  * return selection:       src/gpu/nodeKernels.cu:334-422, saveReturnAsHit/NonHit :103-207
//  * return-mode encoding:   src/returnModeUtils.h:22-30
//  * ray transform:          src/gpu/nodeKernels.cu:45-49 (float), Mat3x4f operators src/math/Mat3x4f.hpp:253-267
//  * point transform:        src/gpu/nodeKernels.cu:51-56
//  * Gaussian noise algebra: src/gpu/gaussianNoiseKernels.cu:20-66; noise frames src/graph/NodesCore.hpp:123,280
//  * compaction:             src/gpu/nodeKernels.cu:58-68,424-436 (stable, keeps flag != 0)
//  * format:                 src/gpu/nodeKernels.cu:25-33, src/GPUFieldDescBuilder.hpp:57-69
//  * entity ids / instances: src/scene/Scene.cpp:143-153, src/scene/Entity.cpp:43-52
//
// The reference draws noise from cuRAND seeded by std::random_device (not reproducible).  The GB300
// build replaces it with Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11) keyed by (seed, point index, frame) and a Box-Muller transform; the oracle
// restates that specification so noise can be checked value by value.
//
// Triangle intersection uses the watertight algorithm of Woop, Benthin and Wald (JCGT 2013) in
// double precision over world-space triangles.  Every cast also reports an "ambiguous" flag: set
// when the FP64 answer is within 1e-6 (relative) of a decision boundary that FP32 cannot resolve —
// the hit lies near a triangle edge, a near-miss lies in front of the hit, two entities tie, the hit
// distance is at a range bound, or two sub-ray samples tie in the return selection.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- float ops in reference order
// Compiled with -ffp-contract=off: every float expression below rounds after each operation.

struct F3
{
	float x, y, z;
};
struct M34f
{
	float m[3][4];
};

M34f mulf(const M34f& a, const M34f& b)
{
	M34f r;
	for (int y = 0; y < 3; ++y) {
		for (int x = 0; x < 4; ++x) {
			float s = ((a.m[y][0] * b.m[0][x]) + (a.m[y][1] * b.m[1][x])) + (a.m[y][2] * b.m[2][x]);
			r.m[y][x] = (x == 3) ? s + a.m[y][3] : s;
		}
	}
	return r;
}

F3 pointf(const M34f& a, F3 p)
{
	return {((a.m[0][0] * p.x + a.m[0][1] * p.y) + a.m[0][2] * p.z) + a.m[0][3],
	        ((a.m[1][0] * p.x + a.m[1][1] * p.y) + a.m[1][2] * p.z) + a.m[1][3],
	        ((a.m[2][0] * p.x + a.m[2][1] * p.y) + a.m[2][2] * p.z) + a.m[2][3]};
}

F3 normalizedf(F3 v)
{
	float l = std::sqrt(((v.x * v.x) + (v.y * v.y)) + (v.z * v.z));
	return {v.x / l, v.y / l, v.z / l};
}

M34f loadM(const float* p)
{
	M34f r;
	std::memcpy(r.m, p, 48);
	return r;
}

// Sub-ray rotation Rx(v)*Ry(h); each entry is one rounded product of cosf/sinf values.
M34f sampleRotation(float h, float v)
{
	float ch = std::cos(h), sh = std::sin(h), cv = std::cos(v), sv = std::sin(v);
	M34f r = {{{ch, 0.0f, sh, 0.0f}, {sv * sh, cv, -(sv * ch), 0.0f}, {-(cv * sh), sv, cv * ch, 0.0f}}};
	return r;
}

// ---------------------------------------------------------------- double math

struct D3
{
	double x, y, z;
};
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double len(D3 a) { return std::sqrt(dot(a, a)); }
inline double comp(D3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

struct M34d
{
	double m[3][4];
};

M34d toD(const M34f& f)
{
	M34d r;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 4; ++j)
			r.m[i][j] = f.m[i][j];
	return r;
}

M34d mulD(const M34d& a, const M34d& b)
{
	M34d r;
	for (int y = 0; y < 3; ++y)
		for (int x = 0; x < 4; ++x) {
			double s = a.m[y][0] * b.m[0][x] + a.m[y][1] * b.m[1][x] + a.m[y][2] * b.m[2][x];
			r.m[y][x] = (x == 3) ? s + a.m[y][3] : s;
		}
	return r;
}

D3 pointD(const M34d& a, D3 p)
{
	return {a.m[0][0] * p.x + a.m[0][1] * p.y + a.m[0][2] * p.z + a.m[0][3],
	        a.m[1][0] * p.x + a.m[1][1] * p.y + a.m[1][2] * p.z + a.m[1][3],
	        a.m[2][0] * p.x + a.m[2][1] * p.y + a.m[2][2] * p.z + a.m[2][3]};
}

M34d inverseD(const M34d& a)
{
	const double(*m)[4] = a.m;
	double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
	double c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
	double c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
	double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
	M34d r{};
	if (det == 0.0) {
		return r;
	}
	double id = 1.0 / det;
	r.m[0][0] = c00 * id;
	r.m[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
	r.m[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
	r.m[1][0] = c01 * id;
	r.m[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
	r.m[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
	r.m[2][0] = c02 * id;
	r.m[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
	r.m[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
	for (int i = 0; i < 3; ++i)
		r.m[i][3] = -(r.m[i][0] * m[0][3] + r.m[i][1] * m[1][3] + r.m[i][2] * m[2][3]);
	return r;
}

M34d rotAxisD(int axis, double a)
{
	double c = std::cos(a), s = std::sin(a);
	M34d r = {{{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}}};
	if (axis == 1) {
		r.m[1][1] = c;
		r.m[1][2] = -s;
		r.m[2][1] = s;
		r.m[2][2] = c;
	} else if (axis == 2) {
		r.m[0][0] = c;
		r.m[0][2] = s;
		r.m[2][0] = -s;
		r.m[2][2] = c;
	} else {
		r.m[0][0] = c;
		r.m[0][1] = -s;
		r.m[1][0] = s;
		r.m[1][1] = c;
	}
	return r;
}

// ---------------------------------------------------------------- Philox4x32-10 (Salmon et al. SC'11)

void philox4x32_10(const uint32_t ctrIn[4], const uint32_t keyIn[2], uint32_t out[4])
{
	uint32_t c0 = ctrIn[0], c1 = ctrIn[1], c2 = ctrIn[2], c3 = ctrIn[3];
	uint32_t k0 = keyIn[0], k1 = keyIn[1];
	for (int r = 0; r < 10; ++r) {
		if (r > 0) {
			k0 += 0x9E3779B9u;
			k1 += 0xBB67AE85u;
		}
		uint64_t p0 = (uint64_t) 0xD2511F53u * c0;
		uint64_t p1 = (uint64_t) 0xCD9E8D57u * c2;
		uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
		uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
		c0 = hi1 ^ c1 ^ k0;
		c1 = lo1;
		c2 = hi0 ^ c3 ^ k1;
		c3 = lo0;
	}
	out[0] = c0;
	out[1] = c1;
	out[2] = c2;
	out[3] = c3;
}

// Standard normal for (seed, kind, index, frame): counter (index, frame lo, frame hi, kind),
// key (seed lo, seed hi); u1 = ((x0 >> 8) + 1) / 2^24 in (0,1], u2 = (x1 >> 8) / 2^24 in [0,1);
// n = sqrt(-2 ln u1) * cos(2 pi u2).
double normalSample(uint64_t seed, uint32_t kind, uint32_t index, uint64_t frame)
{
	uint32_t ctr[4] = {index, (uint32_t) frame, (uint32_t) (frame >> 32), kind};
	uint32_t key[2] = {(uint32_t) seed, (uint32_t) (seed >> 32)};
	uint32_t x[4];
	philox4x32_10(ctr, key, x);
	double u1 = ((double) (x[0] >> 8) + 1.0) * (1.0 / 16777216.0);
	double u2 = (double) (x[1] >> 8) * (1.0 / 16777216.0);
	return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
}

// ---------------------------------------------------------------- scene and FP64 BVH

struct Tri
{
	D3 v0, v1, v2;
	int entityId;
	int instance;
};

struct Node
{
	D3 lo, hi;
	int left = -1, right = -1; // internal: children; leaf: left = -1, [first, first+count)
	int first = 0, count = 0;
};

struct Scene
{
	std::vector<std::vector<float>> meshVerts; // xyz floats
	std::vector<std::vector<int>> meshIdx;     // 3 ints per triangle
	struct Inst
	{
		int mesh;
		M34f tf;
		int id;
	};
	std::vector<Inst> instances;
	std::vector<Tri> tris;
	std::vector<Node> nodes;
	double pad = 0.0; // conservative expansion of node boxes (so near misses are visited)
	double scale = 1.0;
};

void boundsOf(const Tri& t, D3& lo, D3& hi)
{
	lo = {std::min({t.v0.x, t.v1.x, t.v2.x}), std::min({t.v0.y, t.v1.y, t.v2.y}), std::min({t.v0.z, t.v1.z, t.v2.z})};
	hi = {std::max({t.v0.x, t.v1.x, t.v2.x}), std::max({t.v0.y, t.v1.y, t.v2.y}), std::max({t.v0.z, t.v1.z, t.v2.z})};
}

int buildRec(Scene& s, std::vector<int>& order, std::vector<D3>& cent, int first, int count, std::vector<Tri>& outTris)
{
	Node n;
	D3 lo{1e300, 1e300, 1e300}, hi{-1e300, -1e300, -1e300};
	for (int i = first; i < first + count; ++i) {
		D3 a, b;
		boundsOf(s.tris[order[i]], a, b);
		lo = {std::min(lo.x, a.x), std::min(lo.y, a.y), std::min(lo.z, a.z)};
		hi = {std::max(hi.x, b.x), std::max(hi.y, b.y), std::max(hi.z, b.z)};
	}
	n.lo = lo - D3{s.pad, s.pad, s.pad};
	n.hi = hi + D3{s.pad, s.pad, s.pad};
	int idx = (int) s.nodes.size();
	s.nodes.push_back(n);
	if (count <= 4) {
		s.nodes[idx].first = (int) outTris.size();
		s.nodes[idx].count = count;
		for (int i = first; i < first + count; ++i)
			outTris.push_back(s.tris[order[i]]);
		return idx;
	}
	D3 clo{1e300, 1e300, 1e300}, chi{-1e300, -1e300, -1e300};
	for (int i = first; i < first + count; ++i) {
		D3 c = cent[order[i]];
		clo = {std::min(clo.x, c.x), std::min(clo.y, c.y), std::min(clo.z, c.z)};
		chi = {std::max(chi.x, c.x), std::max(chi.y, c.y), std::max(chi.z, c.z)};
	}
	D3 ext = chi - clo;
	int axis = (ext.x >= ext.y && ext.x >= ext.z) ? 0 : (ext.y >= ext.z ? 1 : 2);
	int mid = first + count / 2;
	std::nth_element(order.begin() + first, order.begin() + mid, order.begin() + first + count,
	                 [&](int a, int b) { return comp(cent[a], axis) < comp(cent[b], axis); });
	int l = buildRec(s, order, cent, first, mid - first, outTris);
	int r = buildRec(s, order, cent, mid, first + count - mid, outTris);
	s.nodes[idx].left = l;
	s.nodes[idx].right = r;
	return idx;
}

void buildScene(Scene& s)
{
	s.tris.clear();
	s.nodes.clear();
	double maxc = 1.0;
	for (size_t ii = 0; ii < s.instances.size(); ++ii) {
		const auto& inst = s.instances[ii];
		M34d tf = toD(inst.tf);
		const auto& v = s.meshVerts[inst.mesh];
		const auto& ix = s.meshIdx[inst.mesh];
		for (size_t t = 0; t + 2 < ix.size(); t += 3) {
			D3 p[3];
			for (int k = 0; k < 3; ++k) {
				int vi = ix[t + k];
				p[k] = pointD(tf, D3{v[3 * vi], v[3 * vi + 1], v[3 * vi + 2]});
				maxc = std::max({maxc, std::fabs(p[k].x), std::fabs(p[k].y), std::fabs(p[k].z)});
			}
			s.tris.push_back(Tri{p[0], p[1], p[2], inst.id, (int) ii});
		}
	}
	s.scale = maxc;
	s.pad = 1e-5 * maxc;
	if (s.tris.empty()) {
		return;
	}
	std::vector<int> order(s.tris.size());
	std::vector<D3> cent(s.tris.size());
	for (size_t i = 0; i < s.tris.size(); ++i) {
		order[i] = (int) i;
		cent[i] = (s.tris[i].v0 + s.tris[i].v1 + s.tris[i].v2) * (1.0 / 3.0);
	}
	std::vector<Tri> sorted;
	sorted.reserve(s.tris.size());
	buildRec(s, order, cent, 0, (int) s.tris.size(), sorted);
	s.tris.swap(sorted);
}

struct Hit
{
	double t = std::numeric_limits<double>::infinity();
	int tri = -1;
	bool nearEdge = false;
	double nearMissT = std::numeric_limits<double>::infinity();
	int entity = -1;
	double secondT = std::numeric_limits<double>::infinity(); // closest hit of an entity other than `entity`
	double sinGraze = 1.0; // sine of the angle between the ray and the hit triangle's plane
};

inline bool slab(const Node& n, D3 o, D3 inv, double tmax)
{
	double t0 = 0.0, t1 = tmax;
	for (int a = 0; a < 3; ++a) {
		double oa = comp(o, a), ia = comp(inv, a);
		double ta = (comp(n.lo, a) - oa) * ia, tb = (comp(n.hi, a) - oa) * ia;
		if (std::isnan(ta) || std::isnan(tb)) {
			continue; // ray parallel and on the plane: no constraint
		}
		if (ta > tb)
			std::swap(ta, tb);
		t0 = std::max(t0, ta);
		t1 = std::min(t1, tb);
	}
	return t0 <= t1;
}

// Watertight ray/triangle test in double; returns barycentric "edge distances" for ambiguity checks.
void testTri(const Tri& tr, int triIdx, D3 o, D3 d, int kx, int ky, int kz, double Sx, double Sy, double Sz, double tmax,
             double eps, Hit& h)
{
	D3 A = tr.v0 - o, B = tr.v1 - o, C = tr.v2 - o;
	double Ax = comp(A, kx) - Sx * comp(A, kz), Ay = comp(A, ky) - Sy * comp(A, kz);
	double Bx = comp(B, kx) - Sx * comp(B, kz), By = comp(B, ky) - Sy * comp(B, kz);
	double Cx = comp(C, kx) - Sx * comp(C, kz), Cy = comp(C, ky) - Sy * comp(C, kz);
	double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
	double det = U + V + W;
	if (det == 0.0) {
		return;
	}
	double Az = Sz * comp(A, kz), Bz = Sz * comp(B, kz), Cz = Sz * comp(C, kz);
	double t = (U * Az + V * Bz + W * Cz) / det;
	// A hit at t == 0 (origin on the surface) is not reported (reference DistanceFieldTest.cpp:103-117
	// expects the far face of a cube whose near face contains the ray origin).
	if (!(t > 0.0) || t > tmax * (1.0 + 1e-6)) {
		return;
	}
	double b0 = U / det, b1 = V / det, b2 = W / det;
	// Distance of the hit point to each edge line = barycentric * corresponding triangle height.
	D3 e01 = tr.v1 - tr.v0, e12 = tr.v2 - tr.v1, e20 = tr.v0 - tr.v2;
	double area2 = len(cross(e01, tr.v2 - tr.v0));
	if (area2 == 0.0) {
		return;
	}
	double h0 = area2 / len(e12), h1 = area2 / len(e20), h2 = area2 / len(e01);
	double d0 = b0 * h0, d1 = b1 * h1, d2 = b2 * h2;
	double dmin = std::min({d0, d1, d2});
	double dlen = len(d);
	bool inside = (b0 >= 0 && b1 >= 0 && b2 >= 0);
	if (!inside) {
		if (dmin > -eps && t <= tmax * (1.0 + 1e-6)) {
			h.nearMissT = std::min(h.nearMissT, t);
		}
		return;
	}
	if (t > tmax) {
		// Beyond max range in FP64; if only barely, FP32 may accept it.
		h.nearMissT = std::min(h.nearMissT, t);
		return;
	}
	if (t < h.t) {
		// A new closest hit of another entity makes the previous closest (nearer than every other hit
		// seen) the closest hit of an entity other than the new one; within one entity it stays.
		if (h.tri >= 0 && h.entity != tr.entityId) {
			h.secondT = h.t;
		}
		h.t = t;
		h.tri = triIdx;
		h.entity = tr.entityId;
		h.nearEdge = dmin < eps;
		h.sinGraze = std::fabs(dot(cross(e01, tr.v2 - tr.v0), d)) / (area2 * dlen);
	} else if (tr.entityId != h.entity) {
		h.secondT = std::min(h.secondT, t);
	}
}

// Relative band within which two entities' surfaces are at the same depth for FP32: the watertight t
// errs by about 4e-7 / sin(grazing angle) of the distance, and distances carry the 1e-5 tolerance.
inline double depthBand(double sinGraze) { return std::max(1e-5, 4e-7 / std::max(sinGraze, 1e-6)); }

Hit castRay(const Scene& s, D3 o, D3 d, double tmax)
{
	Hit h;
	if (s.nodes.empty()) {
		return h;
	}
	int kz = (std::fabs(d.x) > std::fabs(d.y)) ? (std::fabs(d.x) > std::fabs(d.z) ? 0 : 2) : (std::fabs(d.y) > std::fabs(d.z) ? 1 : 2);
	int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
	if (comp(d, kz) < 0.0) {
		std::swap(kx, ky);
	}
	double dz = comp(d, kz);
	if (dz == 0.0) {
		return h; // zero direction
	}
	double Sx = comp(d, kx) / dz, Sy = comp(d, ky) / dz, Sz = 1.0 / dz;
	D3 inv{1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
	double eps = 1e-6 * std::max(s.scale, len(o) + tmax * len(d) * 0.0 + 1.0);
	int stack[256];
	int sp = 0;
	stack[sp++] = 0;
	while (sp > 0) {
		const Node& n = s.nodes[stack[--sp]];
		// hits of other entities within the depth band behind the closest one are still collected
		double tlim = std::min(tmax * (1.0 + 1e-6), h.t * (1.0 + depthBand(h.sinGraze)));
		if (!slab(n, o, inv, tlim)) {
			continue;
		}
		if (n.left < 0) {
			for (int i = n.first; i < n.first + n.count; ++i) {
				testTri(s.tris[i], i, o, d, kx, ky, kz, Sx, Sy, Sz, tmax, eps, h);
			}
		} else {
			stack[sp++] = n.left;
			stack[sp++] = n.right;
		}
	}
	return h;
}

// ---------------------------------------------------------------- return selection

// Relative distance tolerance of the GPU path against this oracle (the parity bound).
constexpr double kDistanceTolerance = 1e-5;

inline int returnCount(int32_t mode) { return (int) (((uint32_t) mode) >> 24); }
inline int returnType(int32_t mode, int r) { return (int) ((((uint32_t) mode) >> (8 * r)) & 0xffu); }

enum
{
	RT_UNKNOWN = 0,
	RT_STRONGEST = 1,
	RT_LAST = 2,
	RT_SECOND = 3,
	RT_FIRST = 4,
	RT_SECOND_STRONGEST = 5
};

struct Sample
{
	bool hit;
	float dist;
	float intensity;
	int entity;
	int tri;        // the hit triangle (scene triangle index), -1 for non-hits
	bool ambiguous;
	D3 normal;      // unit world normal of the hit triangle (edge v0v1 x edge v0v2)
	double cosInc;  // |normal . direction| with the sample's unnormalised direction
};

} // namespace

// ================================================================= C entry points (ctypes)

extern "C" {

void* orc_scene_create() { return new Scene(); }

void orc_scene_destroy(void* h) { delete static_cast<Scene*>(h); }

int orc_scene_add_mesh(void* h, const float* verts, int nv, const int* idx, int nt)
{
	auto* s = static_cast<Scene*>(h);
	s->meshVerts.emplace_back(verts, verts + 3 * (size_t) nv);
	s->meshIdx.emplace_back(idx, idx + 3 * (size_t) nt);
	return (int) s->meshVerts.size() - 1;
}

int orc_scene_add_instance(void* h, int mesh, const float* tf12, int entityId)
{
	auto* s = static_cast<Scene*>(h);
	s->instances.push_back({mesh, loadM(tf12), entityId});
	return (int) s->instances.size() - 1;
}

void orc_scene_set_instance(void* h, int inst, const float* tf12, int entityId)
{
	auto* s = static_cast<Scene*>(h);
	s->instances[inst].tf = loadM(tf12);
	s->instances[inst].id = entityId;
}

void orc_scene_build(void* h) { buildScene(*static_cast<Scene*>(h)); }

// Builds the sub-ray rotation table of a beam: entry 0 is the primary ray (identity), then
// layers x vertices entries in the reference's order (sample index 1 + layer*vertices + vertex).
int orc_beam_samples(float hDivergence, float vDivergence, int layers, int vertices, float* out12)
{
	M34f id = {{{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}}};
	std::memcpy(out12, id.m, 48);
	float hHalf = hDivergence / 2.0f, vHalf = vDivergence / 2.0f;
	if (!(hHalf > 0.0f && vHalf > 0.0f)) {
		return 1;
	}
	float step = 2.0f * static_cast<float>(M_PI) / (float) vertices;
	int n = 1;
	for (int l = 0; l < layers; ++l) {
		for (int k = 0; k < vertices; ++k) {
			float frac = 1.0f - (float) l / (float) layers;
			float hAngle = (hHalf * frac) * std::cos((float) k * step);
			float vAngle = (vHalf * frac) * std::sin((float) k * step);
			M34f r = sampleRotation(hAngle, vAngle);
			std::memcpy(out12 + 12 * n, r.m, 48);
			++n;
		}
	}
	return n;
}

// Full RaytraceNode semantics for `nRays` beams.
//   rays: nRays x 12 floats (ray poses before the transform), rayTf: 12 floats or NULL,
//   ranges: nRanges x 2 floats (nRanges == 1 or nRays; NULL -> {0, FLT_MAX}).
//   Outputs are sized returnCount * nRays; any output pointer may be NULL.
//   ambiguous: 1 byte per output point.
//   normal (3 floats per point) and incident angle (radians): reference optixPrograms.cu:138-150, the
//   world normal of the hit triangle and acos(|normal . ray direction|); NaN for non-hits
//   (nodeKernels.cu:196-201).
//   triTie: 1 byte per output point, 1 when two hit samples of the beam that hit different triangles
//   have distances within the unresolved band (twice the distance tolerance): the selected sample,
//   and with it the fields taken from its triangle (normal, incident angle, intensity), may then
//   differ from the FP32 path's although the distance and entity agree.
int orc_raytrace(void* h, const float* rays, int nRays, const float* rayTf, const float* ranges, int nRanges, int32_t returnMode,
                 float hDiv, float vDiv, int layers, int vertices, float nearDist, float farDist, float defaultIntensity,
                 int nThreads, float* outXyz, float* outDist, int32_t* outEntity, int32_t* outIsHit, uint8_t* outReturnType,
                 float* outIntensity, uint8_t* outAmbiguous, float* outNormal, float* outIncident, uint8_t* outTriTie)
{
	const Scene& s = *static_cast<Scene*>(h);
	const int R = returnCount(returnMode);
	std::vector<float> table(12 * (1 + (size_t) layers * vertices));
	int nSamples = orc_beam_samples(hDiv, vDiv, layers, vertices, table.data());
	M34f tf = rayTf ? loadM(rayTf) : M34f{{{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}}};
	std::atomic<int> next{0};
	const int chunk = 256;
	auto worker = [&]() {
		std::vector<Sample> smp(nSamples);
		for (;;) {
			int b0 = next.fetch_add(chunk);
			if (b0 >= nRays)
				break;
			for (int b = b0; b < std::min(nRays, b0 + chunk); ++b) {
				M34f ray = mulf(tf, loadM(rays + 12 * (size_t) b));
				float minR = 0.0f, maxR = std::numeric_limits<float>::max();
				if (ranges) {
					const float* rg = ranges + 2 * (nRanges == 1 ? 0 : b);
					minR = rg[0];
					maxR = rg[1];
				}
				F3 of = pointf(ray, F3{0, 0, 0});
				bool beamAmb = false;
				for (int si = 0; si < nSamples; ++si) {
					M34f sr = (si == 0) ? ray : mulf(ray, loadM(table.data() + 12 * si));
					F3 so = pointf(sr, F3{0, 0, 0});
					F3 sz = pointf(sr, F3{0, 0, 1});
					F3 sd = {sz.x - so.x, sz.y - so.y, sz.z - so.z};
					D3 o{so.x, so.y, so.z}, d{sd.x, sd.y, sd.z};
					Hit hit = castRay(s, o, d, (double) maxR);
					Sample& S = smp[si];
					S.ambiguous = false;
					S.tri = -1;
					if (hit.tri < 0) {
						S.hit = false;
						S.dist = farDist;
						S.intensity = 0.0f;
						S.entity = 0;
						if (hit.nearMissT < std::numeric_limits<double>::infinity())
							S.ambiguous = true;
						continue;
					}
					double dist = hit.t * len(d);
					const Tri& tr = s.tris[hit.tri];
					if (hit.nearEdge || hit.nearMissT <= hit.t * (1.0 + 1e-6)) {
						S.ambiguous = true;
					}
					// Decisions that compare a distance are ambiguous within what FP32 resolves: another
					// entity's surface at nearly the same depth (depthBand: FP32 picks the closer one by its
					// watertight t), and a hit at a range bound (the 1e-5 distance tolerance).
					if (hit.secondT <= hit.t * (1.0 + depthBand(hit.sinGraze))) {
						S.ambiguous = true;
					}
					if (std::fabs(hit.t - (double) maxR) <= kDistanceTolerance * (double) maxR ||
					    std::fabs(dist - (double) minR) <= kDistanceTolerance * std::max((double) minR, dist)) {
						S.ambiguous = true;
					}
					if (dist < (double) minR) {
						S.hit = false;
						S.dist = nearDist;
						S.intensity = 0.0f;
						S.entity = 0;
						continue;
					}
					S.hit = true;
					S.dist = (float) dist;
					S.entity = tr.entityId;
					S.tri = hit.tri;
					D3 n = cross(tr.v1 - tr.v0, tr.v2 - tr.v0);
					n = n * (1.0 / len(n));
					double cosI = std::fabs(dot(n, d));
					S.intensity = (float) ((double) defaultIntensity * cosI);
					S.normal = n;
					S.cosInc = cosI;
				}
				// Return selection, in sample order (reference nodeKernels.cu:334-399).
				int first = -1, second = -1, last = -1, strongest = -1, secondStrongest = -1;
				int i = 0;
				for (; i < nSamples; ++i) {
					if (smp[i].hit) {
						first = second = last = strongest = secondStrongest = i;
						break;
					}
				}
				for (int a = 0; a < nSamples; ++a) {
					beamAmb = beamAmb || smp[a].ambiguous;
				}
				bool triTie = false;
				if (first >= 0) {
					for (i = i + 1; i < nSamples; ++i) {
						if (!smp[i].hit)
							continue;
						float cd = smp[i].dist;
						if (cd < smp[first].dist) {
							second = first;
							first = i;
						} else if (smp[first].dist < cd && cd < smp[second].dist) {
							second = i;
						}
						if (cd > smp[last].dist) {
							last = i;
						}
						float ci = smp[i].intensity;
						if (ci > smp[strongest].intensity) {
							secondStrongest = strongest;
							strongest = i;
						} else if (smp[strongest].intensity > ci && ci > smp[secondStrongest].intensity) {
							secondStrongest = i;
						}
					}
					// Two hit samples whose float distances (or intensities) nearly tie make the selection
					// depend on rounding below FP32 resolution.
					for (int a = 0; a < nSamples && !beamAmb; ++a) {
						if (!smp[a].hit)
							continue;
						for (int c = a + 1; c < nSamples; ++c) {
							if (!smp[c].hit)
								continue;
							float da = smp[a].dist, dc = smp[c].dist;
							// Within twice the distance tolerance the order of two samples is not resolved.
							// It only changes the output's entity when they hit different entities; on one
							// entity a swap moves the point by less than the distance tolerance.
							if (std::fabs(da - dc) <= (float) (2.0 * kDistanceTolerance) * std::max(da, dc)) {
								if (smp[a].entity != smp[c].entity) {
									beamAmb = true;
									break;
								}
								triTie = triTie || smp[a].tri != smp[c].tri;
							}
						}
					}
				}
				F3 zf = pointf(ray, F3{0, 0, 1});
				F3 df = {zf.x - of.x, zf.y - of.y, zf.z - of.z};
				F3 nd = normalizedf(df);
				for (int r = 0; r < R; ++r) {
					size_t p = (size_t) b * R + r;
					int type = returnType(returnMode, r);
					if (outAmbiguous)
						outAmbiguous[p] = beamAmb ? 1 : 0;
					if (outTriTie)
						outTriTie[p] = triTie ? 1 : 0;
					if (first < 0) {
						float nh = smp[0].dist;
						F3 disp = {nd.x * nh, nd.y * nh, nd.z * nh};
						if (std::isnan(disp.x))
							disp.x = 0;
						if (std::isnan(disp.y))
							disp.y = 0;
						if (std::isnan(disp.z))
							disp.z = 0;
						if (outXyz) {
							outXyz[3 * p] = of.x + disp.x;
							outXyz[3 * p + 1] = of.y + disp.y;
							outXyz[3 * p + 2] = of.z + disp.z;
						}
						if (outDist)
							outDist[p] = nh;
						if (outEntity)
							outEntity[p] = 0;
						if (outIsHit)
							outIsHit[p] = 0;
						if (outReturnType)
							outReturnType[p] = (uint8_t) type;
						if (outIntensity)
							outIntensity[p] = 0.0f;
						if (outNormal)
							outNormal[3 * p] = outNormal[3 * p + 1] = outNormal[3 * p + 2] = std::numeric_limits<float>::quiet_NaN();
						if (outIncident)
							outIncident[p] = std::numeric_limits<float>::quiet_NaN();
						continue;
					}
					int sel = -1;
					if (type == RT_FIRST)
						sel = first;
					else if (type == RT_SECOND)
						sel = second;
					else if (type == RT_LAST)
						sel = last;
					else if (type == RT_STRONGEST)
						sel = strongest;
					else if (type == RT_SECOND_STRONGEST)
						sel = secondStrongest;
					if (sel < 0)
						continue;
					float dsel = smp[sel].dist;
					if (outXyz) {
						outXyz[3 * p] = of.x + nd.x * dsel;
						outXyz[3 * p + 1] = of.y + nd.y * dsel;
						outXyz[3 * p + 2] = of.z + nd.z * dsel;
					}
					if (outDist)
						outDist[p] = dsel;
					if (outEntity)
						outEntity[p] = smp[sel].entity;
					if (outIsHit)
						outIsHit[p] = 1;
					if (outReturnType)
						outReturnType[p] = (uint8_t) type;
					if (outIntensity)
						outIntensity[p] = smp[sel].intensity;
					if (outNormal) {
						outNormal[3 * p] = (float) smp[sel].normal.x;
						outNormal[3 * p + 1] = (float) smp[sel].normal.y;
						outNormal[3 * p + 2] = (float) smp[sel].normal.z;
					}
					if (outIncident)
						outIncident[p] = (float) std::acos(std::min(smp[sel].cosInc, 1.0));
				}
			}
		}
	};
	int nt = std::max(1, nThreads);
	std::vector<std::thread> th;
	for (int t = 0; t < nt; ++t)
		th.emplace_back(worker);
	for (auto& t : th)
		t.join();
	return nSamples;
}

// Ray poses after rgl_node_rays_transform: out = tf * ray (float, reference order).
void orc_transform_rays(const float* tf12, const float* rays, int n, float* out)
{
	M34f tf = loadM(tf12);
	for (int i = 0; i < n; ++i) {
		M34f r = mulf(tf, loadM(rays + 12 * (size_t) i));
		std::memcpy(out + 12 * (size_t) i, r.m, 48);
	}
}

// xyz <- tf * xyz (float, reference order).
void orc_transform_points(const float* tf12, const float* xyz, int n, float* out)
{
	M34f tf = loadM(tf12);
	for (int i = 0; i < n; ++i) {
		F3 p = pointf(tf, F3{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
		out[3 * i] = p.x;
		out[3 * i + 1] = p.y;
		out[3 * i + 2] = p.z;
	}
}

void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { philox4x32_10(ctr, key, out); }

void orc_normals(uint64_t seed, uint32_t kind, uint64_t frame, int n, double* out)
{
	for (int i = 0; i < n; ++i)
		out[i] = normalSample(seed, kind, (uint32_t) i, frame);
}

// Noise frame algebra in double. `lookAt` is the float frame L of the input point cloud
// (inverse of the cumulative ray transform, composed with inverse point transforms).
// kind 2: angular hitpoint; p' = L^-1 R(axis, mean + sd*n) L p; distance' = |R L p| when present.
void orc_noise_angular_hitpoint(const double* lookAt12, float mean, float stDev, int axis, uint64_t seed, uint64_t frame,
                                const float* xyz, int n, float* outXyz, float* outDist)
{
	M34d L;
	std::memcpy(L.m, lookAt12, 96);
	M34d Li = inverseD(L);
	for (int i = 0; i < n; ++i) {
		double e = (double) mean + normalSample(seed, 2, (uint32_t) i, frame) * (double) stDev;
		D3 q = pointD(rotAxisD(axis, e), pointD(L, D3{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}));
		if (outDist)
			outDist[i] = (float) len(q);
		D3 p = pointD(Li, q);
		outXyz[3 * i] = (float) p.x;
		outXyz[3 * i + 1] = (float) p.y;
		outXyz[3 * i + 2] = (float) p.z;
	}
}

// kind 3: distance; sigma = d*rise + base, e = mean + sigma*n, p' = L^-1 (Lp + Lp/|Lp| * e), d' = d + e.
void orc_noise_distance(const double* lookAt12, float mean, float stDevBase, float stDevRise, uint64_t seed, uint64_t frame,
                        const float* xyz, const float* dist, int n, float* outXyz, float* outDist)
{
	M34d L;
	std::memcpy(L.m, lookAt12, 96);
	M34d Li = inverseD(L);
	for (int i = 0; i < n; ++i) {
		double sigma = (double) dist[i] * (double) stDevRise + (double) stDevBase;
		double e = (double) mean + normalSample(seed, 3, (uint32_t) i, frame) * sigma;
		D3 pl = pointD(L, D3{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
		double l = len(pl);
		D3 p = pointD(Li, pl + pl * (e / l));
		outXyz[3 * i] = (float) p.x;
		outXyz[3 * i + 1] = (float) p.y;
		outXyz[3 * i + 2] = (float) p.z;
		outDist[i] = (float) ((double) dist[i] + e);
	}
}

// kind 1: angular ray; ray' = L^-1 R(axis, e) L ray with L = inverse of the cumulative ray transform.
void orc_noise_angular_ray(const double* lookAt12, float mean, float stDev, int axis, uint64_t seed, uint64_t frame,
                           const float* rays, int n, float* outRays)
{
	M34d L;
	std::memcpy(L.m, lookAt12, 96);
	M34d Li = inverseD(L);
	for (int i = 0; i < n; ++i) {
		double e = (double) mean + normalSample(seed, 1, (uint32_t) i, frame) * (double) stDev;
		M34f rf = loadM(rays + 12 * (size_t) i);
		M34d r = mulD(Li, mulD(rotAxisD(axis, e), mulD(L, toD(rf))));
		for (int a = 0; a < 3; ++a)
			for (int b = 0; b < 4; ++b)
				outRays[12 * (size_t) i + 4 * a + b] = (float) r.m[a][b];
	}
}

// Stable compaction: keeps element i when flags[i] != 0. Returns kept count.
int orc_compact(const int32_t* flags, int n, const uint8_t* src, int elemSize, uint8_t* dst)
{
	int w = 0;
	for (int i = 0; i < n; ++i) {
		if (flags[i] != 0) {
			std::memcpy(dst + (size_t) w * elemSize, src + (size_t) i * elemSize, elemSize);
			++w;
		}
	}
	return w;
}

// AoS packing: field k of point i goes to dst + i*pointSize + offset[k]; a NULL source is a padding
// field and its bytes are left untouched.
void orc_format(int n, int nFields, const uint8_t* const* src, const int* sizes, uint8_t* dst)
{
	int pointSize = 0;
	for (int k = 0; k < nFields; ++k)
		pointSize += sizes[k];
	for (int i = 0; i < n; ++i) {
		int off = 0;
		for (int k = 0; k < nFields; ++k) {
			if (src[k])
				std::memcpy(dst + (size_t) i * pointSize + off, src[k] + (size_t) i * sizes[k], sizes[k]);
			off += sizes[k];
		}
	}
}

} // extern "C"
