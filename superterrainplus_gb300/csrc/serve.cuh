// Serving engine: job descriptors of its helper kernels.
#pragma once

#include "internal.hpp"

namespace stpgb {

// Voronoi biome tile of width x height at global pixel origin, row pitch = width.
struct VoronoiJob {
	uint16_t* out;
	int64_t origin_x, origin_y;
	uint32_t width, height;
	uint32_t cell;
};

// Nine S x S chunk heightfields (row-major chunk order) into a (3S)^2 map.
struct GatherJob {
	const float* chunk[9];
	float* merged;
	uint32_t S;
};

// Droplet starts uniform over the central chunk of a 3 x 3 neighbourhood.
struct StartsJob {
	float* out;
	uint64_t counter_base;
	uint32_t count;
	uint32_t S;
};

int voronoi_jobs_launch(const VoronoiJob* jobs, uint32_t njobs, uint32_t max_w, uint32_t max_h, uint64_t seed,
	uint32_t biomes, cudaStream_t s);
int gather_jobs_launch(const GatherJob* jobs, uint32_t njobs, uint32_t max_S, cudaStream_t s);
// the inverse of gather_jobs_launch: each merged map back into its nine chunks
int scatter_jobs_launch(const GatherJob* jobs, uint32_t njobs, uint32_t max_S, cudaStream_t s);
int starts_jobs_launch(const StartsJob* jobs, uint32_t njobs, uint32_t max_count, uint64_t seed, cudaStream_t s);

} // namespace stpgb
