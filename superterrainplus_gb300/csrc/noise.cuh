// Multi-biome fractal simplex heightfield: job descriptor and batched launch.
#pragma once

#include "internal.hpp"

namespace stpgb {

// One MapSize chunk: its histogram (offsets/bins) in, heights out.
struct NoiseJob {
	float* out;
	uint64_t pitch; // floats per output row
	const uint32_t* offsets;
	const stpgb_bin* bins;
	uint32_t W, H;
	float off_x, off_y;
};

// `block`: threads per block, 128, 256 or 512 (0 = 256)
int noise_launch(const NoiseJob* jobs, const NoiseJob& single, uint32_t njobs, uint64_t max_pixels,
	const stpgb_permutation& perm, const stpgb_biome_property* table, uint32_t biome_count, cudaStream_t stream,
	uint32_t block = 0u);

} // namespace stpgb
