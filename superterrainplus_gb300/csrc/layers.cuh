// Biome layer chain on the GPU: shared description and launch entry points.
#pragma once

#include "internal.hpp"

namespace stpgb {

constexpr uint32_t kMaxLayers = STPGB_MAX_LAYERS;

// A validated linear chain with its per-layer seeds
// (STPLayer::seedLayer(global, salt)) computed on the host.
struct LayerChain {
	uint32_t count;
	uint16_t ocean, plains, forest, shallow[5];
	uint64_t voronoi_seed;
	uint32_t kind[kMaxLayers];
	uint32_t param[kMaxLayers];
	uint64_t seed[kMaxLayers];
};

// One biomemap rectangle: world pixels [x0, x0 + width) x [z0, z0 + height)
// into out[z * pitch + x], covered by `tiles` square tiles (tiles_x per row)
// of a grid whose first tile starts at (gx0, gz0) <= (x0, z0).
struct BiomemapJob {
	uint16_t* out;
	int32_t x0, z0;
	uint32_t pitch, width, height;
	int32_t gx0, gz0;
	uint32_t tiles_x, tiles;
};

int layer_chain_prepare(const stpgb_layer* chain, uint32_t count, uint64_t global_seed,
	const stpgb_layer_biomes* ids, LayerChain* out);

// Tile edge for a launch covering `pixels` output pixels in total.
uint32_t layer_tile_for(uint64_t pixels);

// The same, reduced until the chain's shared-memory plan fits.
uint32_t layer_tile(const LayerChain& chain, uint64_t pixels);

// The demo's 14-layer chain with the demo's biome IDs.
int layer_chain_demo(uint64_t global_seed, LayerChain* out);

// Fills the tiling fields of `job` for tile edge `tile`; EINVAL when the
// rectangle leaves the supported coordinate range.
int layer_job_tiling(BiomemapJob& job, uint32_t tile);

// One launch over njobs rectangles (grid.y = job); `jobs` is a device array,
// or null with njobs == 1 to pass `single` by value.
int layer_biomemap_launch(const LayerChain& chain, const BiomemapJob* jobs, const BiomemapJob& single,
	uint32_t njobs, uint32_t max_tiles, uint32_t tile, cudaStream_t stream);

} // namespace stpgb
