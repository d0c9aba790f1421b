// Host/device math shared by the C API layer and the CUDA kernels.
//
// Affine 3x4 matrices follow RGL's convention (reference src/math/Mat3x4f.hpp:25-267): row-major,
// column 3 is the translation, points are transformed as M * (x, y, z, 1).
//
// Ray construction and ray/point transforms are evaluated in float with an explicit operation order
// and no fused multiply-add, matching the expression order of the reference's Mat3x4f operators
// (Mat3x4f.hpp:253-267): ((m0*x + m1*y) + m2*z) + m3.  Doing so keeps the world-space rays built on
// the device bit-identical to the ones the host (and the CPU oracle) builds from the same inputs.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define RGL_HD __host__ __device__ __forceinline__
#else
#define RGL_HD inline
#endif

namespace rgl {

// Multiply/add without contraction into FMA, on host and device.
RGL_HD float fmul(float a, float b)
{
#if defined(__CUDA_ARCH__)
	return __fmul_rn(a, b);
#else
	volatile float r = a * b;
	return r;
#endif
}

RGL_HD float fadd(float a, float b)
{
#if defined(__CUDA_ARCH__)
	return __fadd_rn(a, b);
#else
	volatile float r = a + b;
	return r;
#endif
}

RGL_HD float fsub(float a, float b)
{
#if defined(__CUDA_ARCH__)
	return __fsub_rn(a, b);
#else
	volatile float r = a - b;
	return r;
#endif
}

struct Vec3
{
	float x, y, z;
};

RGL_HD Vec3 v3(float x, float y, float z) { return Vec3{x, y, z}; }
RGL_HD Vec3 operator+(Vec3 a, Vec3 b) { return {fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)}; }
RGL_HD Vec3 operator-(Vec3 a, Vec3 b) { return {fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)}; }
RGL_HD Vec3 operator*(Vec3 a, float s) { return {fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)}; }

// |v|^2 accumulated as ((0 + x*x) + y*y) + z*z without contraction (reference Vector.hpp:139-148).
RGL_HD float lengthSq(Vec3 v) { return fadd(fadd(fmul(v.x, v.x), fmul(v.y, v.y)), fmul(v.z, v.z)); }
RGL_HD float length(Vec3 v) { return sqrtf(lengthSq(v)); }
// v / |v| with correctly rounded division (reference Vector.hpp:152).
RGL_HD Vec3 normalized(Vec3 v)
{
	float l = length(v);
	return {v.x / l, v.y / l, v.z / l};
}
RGL_HD Vec3 cross(Vec3 a, Vec3 b)
{
	return {fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)), fsub(fmul(a.x, b.y), fmul(a.y, b.x))};
}
RGL_HD float dot(Vec3 a, Vec3 b) { return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z)); }

struct Mat34
{
	float m[3][4];

	static RGL_HD Mat34 identity() { return Mat34{{{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}}}; }
	static RGL_HD Mat34 zeros() { return Mat34{{{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}}}; }

	RGL_HD Vec3 translation() const { return {m[0][3], m[1][3], m[2][3]}; }

	// M * p for a point (translation applied).
	RGL_HD Vec3 point(Vec3 p) const
	{
		return {fadd(fadd(fadd(fmul(m[0][0], p.x), fmul(m[0][1], p.y)), fmul(m[0][2], p.z)), m[0][3]),
		        fadd(fadd(fadd(fmul(m[1][0], p.x), fmul(m[1][1], p.y)), fmul(m[1][2], p.z)), m[1][3]),
		        fadd(fadd(fadd(fmul(m[2][0], p.x), fmul(m[2][1], p.y)), fmul(m[2][2], p.z)), m[2][3])};
	}

	// Linear part only (directions).
	RGL_HD Vec3 vector(Vec3 v) const
	{
		return {fadd(fadd(fmul(m[0][0], v.x), fmul(m[0][1], v.y)), fmul(m[0][2], v.z)),
		        fadd(fadd(fmul(m[1][0], v.x), fmul(m[1][1], v.y)), fmul(m[1][2], v.z)),
		        fadd(fadd(fmul(m[2][0], v.x), fmul(m[2][1], v.y)), fmul(m[2][2], v.z))};
	}

	// Ray of this pose as RGL defines it (reference src/gpu/optixPrograms.cu:222-228):
	// origin = M*(0,0,0), direction = M*(0,0,1) - origin, left unnormalised.
	RGL_HD Vec3 rayOrigin() const { return point(v3(0.0f, 0.0f, 0.0f)); }
	RGL_HD Vec3 rayDir() const { return point(v3(0.0f, 0.0f, 1.0f)) - rayOrigin(); }
};

// lhs * rhs for affine matrices (reference Mat3x4f.hpp:253-260), same per-entry evaluation order.
RGL_HD Mat34 mul(const Mat34& a, const Mat34& b)
{
	Mat34 r;
	for (int y = 0; y < 3; ++y) {
		for (int x = 0; x < 4; ++x) {
			float s = fadd(fadd(fmul(a.m[y][0], b.m[0][x]), fmul(a.m[y][1], b.m[1][x])), fmul(a.m[y][2], b.m[2][x]));
			r.m[y][x] = (x == 3) ? fadd(s, a.m[y][3]) : s;
		}
	}
	return r;
}

// Inverse of an affine matrix: adjugate of the 3x3 block over its determinant, translation -R^-1 t.
// A singular matrix yields all zeros, as the reference does (Mat3x4f.hpp:186-191).
RGL_HD Mat34 inverse(const Mat34& a)
{
	const float(*m)[4] = a.m;
	float c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
	float c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
	float c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
	float det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
	if (det == 0.0f) {
		return Mat34::zeros();
	}
	float id = 1.0f / det;
	Mat34 r;
	r.m[0][0] = c00 * id;
	r.m[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
	r.m[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
	r.m[1][0] = c01 * id;
	r.m[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
	r.m[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
	r.m[2][0] = c02 * id;
	r.m[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
	r.m[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
	for (int i = 0; i < 3; ++i) {
		r.m[i][3] = -(r.m[i][0] * m[0][3] + r.m[i][1] * m[1][3] + r.m[i][2] * m[2][3]);
	}
	return r;
}

// Single-axis rotations; the entries equal the reference's Mat3x4f::rotationRad for a single
// non-zero angle (Mat3x4f.hpp:38-70): Rx = [1 0 0; 0 c -s; 0 s c], Ry = [c 0 s; 0 1 0; -s 0 c],
// Rz = [c -s 0; s c 0; 0 0 1].
RGL_HD Mat34 rotationAxis(int axis /*1=x,2=y,3=z*/, float c, float s)
{
	Mat34 r = Mat34::identity();
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

// Rotation of a beam sub-ray relative to its primary ray: Rx(vAngle) * Ry(hAngle)
// (reference src/gpu/optixPrograms.cu:230-248). Every entry of the product is a single rounded
// product, so writing it out directly gives the same floats as the reference's matrix product.
RGL_HD Mat34 beamSampleRotation(float hAngle, float vAngle)
{
	float ch = cosf(hAngle), sh = sinf(hAngle), cv = cosf(vAngle), sv = sinf(vAngle);
	Mat34 r;
	r.m[0][0] = ch;
	r.m[0][1] = 0.0f;
	r.m[0][2] = sh;
	r.m[0][3] = 0.0f;
	r.m[1][0] = fmul(sv, sh);
	r.m[1][1] = cv;
	r.m[1][2] = -fmul(sv, ch);
	r.m[1][3] = 0.0f;
	r.m[2][0] = -fmul(cv, sh);
	r.m[2][1] = sv;
	r.m[2][2] = fmul(cv, ch);
	r.m[2][3] = 0.0f;
	return r;
}

// Pose of a ray shifted by velocity distortion: translation t times the rotation Rz(z) Ry(y) Rx(x)
// given in degrees (reference Mat3x4f.hpp:38-97, TRS with unit scale; the entries of the rotation
// product are evaluated left to right as written there, so host and device agree bit for bit).
RGL_HD Mat34 translationRotationDeg(Vec3 t, Vec3 rDeg)
{
	const float toRad = 3.14159265358979323846f / 180.0f;
	const float x = fmul(rDeg.x, toRad), y = fmul(rDeg.y, toRad), z = fmul(rDeg.z, toRad);
	const float cr = cosf(x), sr = sinf(x), cp = cosf(y), sp = sinf(y), cy = cosf(z), sy = sinf(z);
	Mat34 m;
	m.m[0][0] = fmul(cp, cy);
	m.m[0][1] = fsub(fmul(fmul(sr, sp), cy), fmul(cr, sy));
	m.m[0][2] = fadd(fmul(sr, sy), fmul(fmul(cr, sp), cy));
	m.m[0][3] = t.x;
	m.m[1][0] = fmul(cp, sy);
	m.m[1][1] = fadd(fmul(cr, cy), fmul(fmul(sr, sp), sy));
	m.m[1][2] = fsub(fmul(fmul(cr, sp), sy), fmul(sr, cy));
	m.m[1][3] = t.y;
	m.m[2][0] = -sp;
	m.m[2][1] = fmul(sr, cp);
	m.m[2][2] = fmul(cr, cp);
	m.m[2][3] = t.z;
	return m;
}

} // namespace rgl
