// Droplet start positions (Philox4x32-10) and the seeded Voronoi biome map.
//
// Philox4x32-10 follows the published description (Salmon, Moraes, Dror,
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11): ten rounds of
// the 4x32 multiply-xor S-box with multipliers 0xD2511F53 / 0xCD9E8D57 and
// Weyl key increments 0x9E3779B9 / 0xBB67AE85.  Droplet i uses counter
// (i + base) and key = seed; its first two outputs become u in (0, 1] as
// ((x >> 8) + 1) * 2^-24 and are mapped to the central chunk exactly as
// SuperTerrain+/SuperTerrain+/Private/GPGPU/STPHeightfieldKernel.cu:93-104
// maps its two uniforms: pos = u * (MapSize - 1) + (NN / 2) * MapSize.
#include "internal.hpp"

namespace stpgb {

namespace {

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
	for (int round = 0; round < 10; round++) {
		const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
		const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
		const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
		c[0] = n0;
		c[1] = lo1;
		c[2] = n2;
		c[3] = lo0;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
}

__global__ void starts_kernel(float* __restrict__ xy, const uint32_t count, const uint64_t seed, const uint64_t base,
	const float base_x, const float base_y, const float range_x, const float range_y) {
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= count) {
		return;
	}
	const uint64_t ctr = base + i;
	uint32_t c[4] = { static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32), 0u, 0u };
	philox4x32_10(c, static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
	const float ux = static_cast<float>((c[0] >> 8) + 1u) * (1.0f / 16777216.0f);
	const float uy = static_cast<float>((c[1] >> 8) + 1u) * (1.0f / 16777216.0f);
	// separately rounded multiply then add, as the reference's
	// `initPos *= base; initPos += range;` (no fused multiply-add)
	const float x = __fadd_rn(__fmul_rn(ux, base_x), range_x);
	const float y = __fadd_rn(__fmul_rn(uy, base_y), range_y);
	reinterpret_cast<float2*>(xy)[i] = make_float2(x, y);
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
	z += 0x9E3779B97F4A7C15ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

__device__ __forceinline__ int64_t floordiv(const int64_t a, const int64_t b) {
	const int64_t q = a / b;
	return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

__global__ void voronoi_kernel(uint16_t* __restrict__ out, const uint32_t pitch, const uint32_t width,
	const uint32_t height, const int64_t ox, const int64_t oy, const uint32_t cell, const uint32_t biomes,
	const uint64_t seed) {
	const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= width || y >= height) {
		return;
	}
	const int64_t gx = ox + x, gy = oy + y;
	const int64_t cx = floordiv(gx, cell), cy = floordiv(gy, cell);
	int64_t best = INT64_MAX;
	uint64_t best_h = 0u;
	for (int dy = -1; dy <= 1; dy++) {
		for (int dx = -1; dx <= 1; dx++) {
			const int64_t nx = cx + dx, ny = cy + dy;
			const uint64_t h = splitmix64(seed ^ splitmix64(static_cast<uint64_t>(nx) * 0x9E3779B97F4A7C15ull
				^ static_cast<uint64_t>(ny) * 0xC2B2AE3D27D4EB4Full));
			const int64_t px = nx * cell + static_cast<int64_t>(h % cell), py = ny * cell + static_cast<int64_t>((h >> 32) % cell);
			const int64_t d = (px - gx) * (px - gx) + (py - gy) * (py - gy);
			if (d < best) {
				best = d;
				best_h = h;
			}
		}
	}
	out[static_cast<uint64_t>(y) * pitch + x] = static_cast<uint16_t>(splitmix64(best_h) % biomes);
}

} // namespace

int starts_launch(float* xy, uint32_t count, uint64_t seed, uint64_t base, uint32_t map_x, uint32_t map_y,
	uint32_t nn_x, uint32_t nn_y, cudaStream_t stream) {
	if (count == 0u) {
		return STPGB_OK;
	}
	starts_kernel<<<(count + 255u) / 256u, 256u, 0, stream>>>(xy, count, seed, base, static_cast<float>(map_x - 1u),
		static_cast<float>(map_y - 1u), static_cast<float>((nn_x / 2u) * map_x), static_cast<float>((nn_y / 2u) * map_y));
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int voronoi_launch(uint16_t* out, uint32_t pitch, uint32_t width, uint32_t height, int64_t ox, int64_t oy,
	uint32_t cell, uint32_t biomes, uint64_t seed, cudaStream_t stream) {
	if (width == 0u || height == 0u) {
		return STPGB_OK;
	}
	const dim3 block(32u, 8u), grid((width + 31u) / 32u, (height + 7u) / 8u);
	voronoi_kernel<<<grid, block, 0, stream>>>(out, pitch, width, height, ox, oy, cell, biomes, seed);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

} // namespace stpgb

using namespace stpgb;

extern "C" {

int stpgb_droplet_starts(float* starts_xy, uint32_t count, uint64_t seed, uint64_t counter_base,
	const stpgb_nn_info* nn, void* stream) {
	if ((count > 0u && !starts_xy) || !nn) {
		return inval("stpgb_droplet_starts: null pointer argument");
	}
	if (nn->MapSize[0] == 0u || nn->MapSize[1] == 0u) {
		return inval("stpgb_droplet_starts: empty map");
	}
	return starts_launch(starts_xy, count, seed, counter_base, nn->MapSize[0], nn->MapSize[1],
		nn->ChunkNearestNeighbour[0], nn->ChunkNearestNeighbour[1], as_stream(stream));
}

int stpgb_voronoi_biomemap(uint16_t* out, uint32_t pitch, uint32_t width, uint32_t height, int64_t origin_x,
	int64_t origin_y, uint32_t cell, uint32_t biome_count, uint64_t seed, void* stream) {
	if (!out || cell == 0u || biome_count == 0u || pitch < width) {
		return inval("stpgb_voronoi_biomemap: invalid argument");
	}
	return voronoi_launch(out, pitch, width, height, origin_x, origin_y, cell, biome_count, seed, as_stream(stream));
}

} // extern "C"
