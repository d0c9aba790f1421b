// Counter-based Philox4x32-10 generator (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11) and the standard normal used by the Gaussian noise nodes.
//
// The reference (src/gpu/helpersKernels.cu:22-27, src/gpu/gaussianNoiseKernels.cu:20-66) keeps a
// cuRAND state per point seeded from std::random_device, which makes runs irreproducible. Here each
// normal is a pure function of (seed, noise kind, point index, frame):
//   counter = (index, frame lo, frame hi, kind), key = (seed lo, seed hi)
//   u1 = ((x0 >> 8) + 1) / 2^24 in (0, 1],  u2 = (x1 >> 8) / 2^24 in [0, 1)
//   n  = sqrt(-2 ln u1) * cos(2 pi u2)                        (Box-Muller)
// Kinds: 1 angular ray noise, 2 angular hitpoint noise, 3 distance noise.
#pragma once

#include <cstdint>
#include "rgl_math.hpp"

namespace rgl {

RGL_HD void philoxRound(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3, uint32_t k0, uint32_t k1)
{
#if defined(__CUDA_ARCH__)
	uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
	uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
	uint64_t p0 = (uint64_t) 0xD2511F53u * c0, p1 = (uint64_t) 0xCD9E8D57u * c2;
	uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
	uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
#endif
	uint32_t n0 = hi1 ^ c1 ^ k0;
	uint32_t n2 = hi0 ^ c3 ^ k1;
	c0 = n0;
	c1 = lo1;
	c2 = n2;
	c3 = lo0;
}

RGL_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
	for (int r = 0; r < 10; ++r) {
		if (r > 0) {
			k0 += 0x9E3779B9u;
			k1 += 0xBB67AE85u;
		}
		philoxRound(c[0], c[1], c[2], c[3], k0, k1);
	}
}

RGL_HD float standardNormal(uint32_t seedLo, uint32_t seedHi, uint32_t kind, uint32_t index, uint32_t frameLo, uint32_t frameHi)
{
	uint32_t c[4] = {index, frameLo, frameHi, kind};
	philox4x32_10(c, seedLo, seedHi);
	float u1 = ((float) (c[0] >> 8) + 1.0f) * (1.0f / 16777216.0f);
	float u2 = (float) (c[1] >> 8) * (1.0f / 16777216.0f);
#if defined(__CUDA_ARCH__)
	return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
#else
	return (float) (std::sqrt(-2.0 * std::log((double) u1)) * std::cos(2.0 * 3.14159265358979323846 * (double) u2));
#endif
}

} // namespace rgl
