// Multi-biome fractal simplex heightfield on sm_103a.
//
// Per pixel (x, y) of a chunk:  h = sum_bins Weight * (fractal(x, y) * Variation + Depth)
// (SuperDemo+/Script/STPMultiHeightGenerator.cu:35-72), with the 2D simplex
// noise and its fractal sum of SuperTerrain+/SuperAlgorithm+/Device/Private/
// STPSimplexNoise.cu:18-110.  The kernel is FP32-pipe bound.  Two exact
// rewrites take work out of the inner loop without changing a result:
//  * the reference hashes a corner as perm[a] % Gradient2DSize and then reads
//    the gradient; here a 512-entry table of the already-reduced gradient for
//    every perm slot lives in shared memory, so a corner costs one lookup;
//  * ((x - half) + offset) / Scale is the same for every octave (the
//    reference multiplies it by the octave frequency afterwards), so the IEEE
//    division is done once per bin instead of once per octave.
#include "noise.cuh"
#include "simplex.cuh"

namespace stpgb {

namespace {

constexpr uint32_t kNoiseBlock = 256u;

// one pixel per thread; the block size (128, 256 or 512) is the batch tuner's choice
template<uint32_t Block>
__global__ void __launch_bounds__(Block) multibiome_kernel(const NoiseJob* __restrict__ jobs,
	const NoiseJob single, const stpgb_permutation perm, const stpgb_biome_property* __restrict__ table,
	const uint32_t biome_count) {
	__shared__ uint8_t sperm[512];
	__shared__ float2 gtab[512];
	simplex::load_tables(perm, sperm, gtab);
	__syncthreads();

	const NoiseJob& J = jobs ? jobs[blockIdx.y] : single;
	const uint64_t npix = static_cast<uint64_t>(J.W) * J.H;
	const uint64_t idx = static_cast<uint64_t>(blockIdx.x) * Block + threadIdx.x;
	if (idx >= npix) {
		return;
	}
	const uint32_t x = static_cast<uint32_t>(idx % J.W), y = static_cast<uint32_t>(idx / J.W);
	// HalfDimension = vec2(MapSize) / 2 (SuperDemo+/World/Biomes/STPCommonCompiler.cpp:236)
	const float half_x = static_cast<float>(J.W) / 2.0f, half_y = static_cast<float>(J.H) / 2.0f;
	const float fx = (1.0f * x - half_x) + J.off_x, fy = (1.0f * y - half_y) + J.off_y;

	float height = 0.0f;
	const uint32_t b0 = J.offsets[idx], b1 = J.offsets[idx + 1u];
	for (uint32_t b = b0; b < b1; b++) {
		const uint2 raw = __ldg(reinterpret_cast<const uint2*>(J.bins) + b);
		const uint32_t id = raw.x & 0xFFFFu;
		const float weight = __uint_as_float(raw.y);
		if (id >= biome_count) {
			continue;
		}
		const stpgb_biome_property p = table[id];
		const float f = simplex::fractal(sperm, gtab, fx / p.Scale, fy / p.Scale, p.Octave, p.Persistence,
			p.Lacunarity);
		height += weight * (f * p.Variation + p.Depth);
	}
	J.out[static_cast<uint64_t>(y) * J.pitch + x] = height;
}

} // namespace

int noise_launch(const NoiseJob* jobs, const NoiseJob& single, uint32_t njobs, uint64_t max_pixels,
	const stpgb_permutation& perm, const stpgb_biome_property* table, uint32_t biome_count, cudaStream_t stream,
	const uint32_t block) {
	const uint32_t b = block == 0u ? kNoiseBlock : block;
	const dim3 grid(static_cast<uint32_t>((max_pixels + b - 1u) / b), njobs);
	switch (b) {
	case 128u:
		multibiome_kernel<128u><<<grid, 128u, 0, stream>>>(jobs, single, perm, table, biome_count);
		break;
	case 256u:
		multibiome_kernel<256u><<<grid, 256u, 0, stream>>>(jobs, single, perm, table, biome_count);
		break;
	case 512u:
		multibiome_kernel<512u><<<grid, 512u, 0, stream>>>(jobs, single, perm, table, biome_count);
		break;
	default:
		return inval("noise_launch: block size must be 128, 256 or 512");
	}
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

} // namespace stpgb

using namespace stpgb;

extern "C" int stpgb_multibiome_heightmap(float* heightmap, uint32_t pitch, const uint32_t* offsets,
	const stpgb_bin* bins, uint32_t map_x, uint32_t map_y, float offset_x, float offset_y,
	const stpgb_permutation* perm, const stpgb_biome_property* biome_table, uint32_t biome_count, void* stream) {
	if (!heightmap || !offsets || !perm || !perm->Permutation || !perm->Gradient2D || !biome_table) {
		return inval("stpgb_multibiome_heightmap: null pointer argument");
	}
	if (perm->Gradient2DSize == 0u) {
		return inval("stpgb_multibiome_heightmap: empty gradient table");
	}
	if (pitch < map_x) {
		return inval("stpgb_multibiome_heightmap: pitch below map width");
	}
	if (map_x == 0u || map_y == 0u) {
		return STPGB_OK;
	}
	NoiseJob job { heightmap, pitch, offsets, bins, map_x, map_y, offset_x, offset_y };
	return noise_launch(nullptr, job, 1u, static_cast<uint64_t>(map_x) * map_y, *perm, biome_table, biome_count,
		as_stream(stream));
}
