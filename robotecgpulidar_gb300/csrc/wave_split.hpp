// Cutting a batched frame's sensors into waves (batch.cpp), as a host-only function so the CPU test
// harness checks it too.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace rgl {

// Cuts n members with the given traced ray counts, in order, into min(W, n) (at least 1) contiguous
// waves of about equal rays: wave w ends at the first member whose running total reaches (w + 1) / W
// of all rays, or earlier when only one member is left for each later wave. No wave is empty.
// Returns the first member of each wave, then n.
inline std::vector<int> splitIntoWaves(const std::vector<int64_t>& rays, int W)
{
	const int n = (int) rays.size();
	int64_t total = 0;
	for (int64_t r : rays) {
		total += r;
	}
	W = std::max(1, std::min(W, n));
	std::vector<int> first(1, 0);
	int64_t acc = 0;
	for (int j = 0; j < n; ++j) {
		acc += rays[(size_t) j];
		const int w = (int) first.size() - 1;
		const int left = n - (j + 1);      // members after j
		const int wavesLeft = W - (w + 1); // waves after wave w
		if (w < W - 1 && left > 0 && left >= wavesLeft && (acc * W >= total * (w + 1) || left == wavesLeft)) {
			first.push_back(j + 1);
		}
	}
	first.push_back(n);
	return first;
}

} // namespace rgl
