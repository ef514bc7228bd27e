// Plain per-chunk drop-in: the heightfield generator over host arrays,
// synchronous per call like the reference (SuperTerrain+/SuperTerrain+/
// Private/World/Chunk/STPHeightfieldGenerator.cpp:115-197), calling a
// diversity plugin for each chunk's heightmap (STPDiversityGenerator.hpp:
// 14-39), and the demo's multi-biome plugin as one such plugin
// (SuperDemo+/World/Biomes/STPBiomefieldGenerator.cpp:44-152).
//
// The reference merges the neighbour chunks into a pinned host buffer and
// then copies it to the device (STPNearestNeighbourTextureBuffer.cpp:18-113);
// here every chunk is copied straight into its place in the merged device
// buffer with one 2D copy, and back the same way.  The filter runs on the
// device, so its output never crosses the bus.  Concurrent callers each take
// a slot (stream + buffers) from a pool, as the reference takes a pooled
// stream per call (STPHeightfieldGenerator.cpp:152-156).
#include "internal.hpp"
#include "shf.cuh"

#include <algorithm>
#include <memory>
#include <mutex>
#include <vector>

namespace stpgb {

namespace {

template<typename T>
struct DevBuf {
	T* p = nullptr;
	size_t n = 0u;
	DevBuf() = default;
	DevBuf(const DevBuf&) = delete;
	DevBuf& operator=(const DevBuf&) = delete;
	~DevBuf() {
		if (p) {
			cudaFree(p);
		}
	}
	int alloc(size_t count) {
		if (count <= n && p) {
			return STPGB_OK;
		}
		if (p) {
			cudaFree(p);
			p = nullptr;
		}
		STPGB_CUDA_TRY(cudaMalloc(&p, std::max<size_t>(count, 1u) * sizeof(T)));
		n = count;
		return STPGB_OK;
	}
};

struct Slot {
	cudaStream_t stream = nullptr;
	// generate
	DevBuf<uint16_t> biome;
	DevBuf<float> height;
	// erode
	DevBuf<float> merged;
	DevBuf<uint16_t> fixed;
	DevBuf<float> starts;
	DevBuf<double> residual;
	DevBuf<uint32_t> status;
	~Slot() {
		if (stream) {
			cudaStreamDestroy(stream);
		}
	}
};

// Scratch of one call of the multi-biome plugin.
struct FieldScratch {
	DevBuf<unsigned char> ws;
	DevBuf<uint32_t> offsets;
	DevBuf<stpgb_bin> bins;
	DevBuf<uint32_t> status;
};

} // namespace


} // namespace stpgb

using namespace stpgb;

struct stpgb_biomefield {
	uint32_t radius = 0u;
	uint32_t biome_count = 0u;
	uint32_t max_items = 0u;
	DevBuf<uint8_t> perm;
	DevBuf<float> grad;
	stpgb_permutation permutation {};
	DevBuf<stpgb_biome_property> table;

	std::mutex mu;
	std::vector<std::unique_ptr<FieldScratch>> free_scratch;

	std::unique_ptr<FieldScratch> acquire() {
		std::lock_guard<std::mutex> lk(mu);
		if (free_scratch.empty()) {
			return std::make_unique<FieldScratch>();
		}
		auto s = std::move(free_scratch.back());
		free_scratch.pop_back();
		return s;
	}
	void release(std::unique_ptr<FieldScratch> s) {
		std::lock_guard<std::mutex> lk(mu);
		free_scratch.push_back(std::move(s));
	}
};

struct stpgb_generator {
	stpgb_chunk_setting chunk;
	stpgb_raindrop_setting rain;
	stpgb_nn_info div_nn {}, ero_nn {};
	int device = 0;
	stpgb_diversity_generator diversity {};
	// the demo plugin, when the generator was made with it
	std::unique_ptr<stpgb_biomefield> owned_plugin;
	DevBuf<int32_t> brush_index;
	DevBuf<float> brush_weight;
	uint32_t brush_size = 0u;
	uint64_t droplet_counter = 0u;

	std::mutex mu;
	std::vector<std::unique_ptr<Slot>> free_slots;

	int acquire(std::unique_ptr<Slot>& out) {
		{
			std::lock_guard<std::mutex> lk(mu);
			if (!free_slots.empty()) {
				out = std::move(free_slots.back());
				free_slots.pop_back();
				return STPGB_OK;
			}
		}
		out = std::make_unique<Slot>();
		STPGB_CUDA_TRY(cudaStreamCreateWithFlags(&out->stream, cudaStreamNonBlocking));
		return STPGB_OK;
	}
	void release(std::unique_ptr<Slot> s) {
		std::lock_guard<std::mutex> lk(mu);
		free_slots.push_back(std::move(s));
	}
	uint64_t take_droplets(uint32_t n) {
		std::lock_guard<std::mutex> lk(mu);
		const uint64_t base = droplet_counter;
		droplet_counter += n;
		return base;
	}
};

namespace {

stpgb_nn_info make_nn(const uint32_t map[2], const uint32_t nn[2]) {
	stpgb_nn_info i;
	i.MapSize[0] = map[0];
	i.MapSize[1] = map[1];
	i.ChunkNearestNeighbour[0] = nn[0];
	i.ChunkNearestNeighbour[1] = nn[1];
	i.TotalMapSize[0] = map[0] * nn[0];
	i.TotalMapSize[1] = map[1] * nn[1];
	return i;
}

// Copies chunk arrays (host) into / out of the merged device buffer
// (STPNearestNeighbourTextureBuffer.cpp:94-111, chunk i at local
// coordinate (i % nx, i / nx), STPChunk.cpp:71-73).
template<typename T>
int merge(T* merged, const T* const* chunks, const stpgb_nn_info& nn, cudaStream_t s) {
	const uint32_t nx = nn.ChunkNearestNeighbour[0], count = nx * nn.ChunkNearestNeighbour[1];
	const size_t row = static_cast<size_t>(nn.MapSize[0]) * sizeof(T), total_row = row * nx;
	for (uint32_t i = 0u; i < count; i++) {
		if (!chunks[i]) {
			return inval("neighbour chunk pointer is null");
		}
		const size_t ox = static_cast<size_t>(i % nx) * nn.MapSize[0], oy = static_cast<size_t>(i / nx) * nn.MapSize[1];
		T* const dst = merged + oy * nn.TotalMapSize[0] + ox;
		STPGB_CUDA_TRY(cudaMemcpy2DAsync(dst, total_row, chunks[i], row, row, nn.MapSize[1], cudaMemcpyHostToDevice, s));
	}
	return STPGB_OK;
}

template<typename T>
int unmerge(T* const* chunks, const T* merged, const stpgb_nn_info& nn, cudaStream_t s) {
	const uint32_t nx = nn.ChunkNearestNeighbour[0], count = nx * nn.ChunkNearestNeighbour[1];
	const size_t row = static_cast<size_t>(nn.MapSize[0]) * sizeof(T), total_row = row * nx;
	for (uint32_t i = 0u; i < count; i++) {
		if (!chunks[i]) {
			return inval("neighbour chunk pointer is null");
		}
		const size_t ox = static_cast<size_t>(i % nx) * nn.MapSize[0], oy = static_cast<size_t>(i / nx) * nn.MapSize[1];
		const T* const src = merged + oy * nn.TotalMapSize[0] + ox;
		STPGB_CUDA_TRY(cudaMemcpy2DAsync(chunks[i], row, src, total_row, row, nn.MapSize[1], cudaMemcpyDeviceToHost, s));
	}
	return STPGB_OK;
}

bool odd_positive(const uint32_t v[2]) {
	return v[0] > 0u && v[1] > 0u && (v[0] & 1u) && (v[1] & 1u);
}

int erode_common(stpgb_generator* g, float* const* heightfield, uint16_t* const* fixed, const float* starts_host,
	uint32_t count, double* residual_out) {
	if (!g || !heightfield || !fixed) {
		return inval("stpgb_generator_erode: null argument");
	}
	std::unique_ptr<Slot> slot;
	STPGB_TRY(g->acquire(slot));
	const cudaStream_t s = slot->stream;
	const stpgb_nn_info& nn = g->ero_nn;
	const size_t npix = static_cast<size_t>(nn.TotalMapSize[0]) * nn.TotalMapSize[1];
	int rc = STPGB_OK;
	auto body = [&]() -> int {
		STPGB_TRY(slot->merged.alloc(npix));
		STPGB_TRY(slot->fixed.alloc(npix));
		STPGB_TRY(slot->starts.alloc(2u * static_cast<size_t>(count)));
		STPGB_TRY(slot->residual.alloc(1u));
		STPGB_TRY(slot->status.alloc(1u));
		STPGB_TRY(merge<float>(slot->merged.p, heightfield, nn, s));
		if (starts_host) {
			STPGB_CUDA_TRY(cudaMemcpyAsync(slot->starts.p, starts_host, 2u * sizeof(float) * count,
				cudaMemcpyHostToDevice, s));
		} else {
			const uint64_t base = g->take_droplets(count);
			STPGB_TRY(stpgb_droplet_starts(slot->starts.p, count, g->rain.Seed, base, &nn, s));
		}
		STPGB_CUDA_TRY(cudaMemsetAsync(slot->residual.p, 0, sizeof(double), s));
		STPGB_CUDA_TRY(cudaMemsetAsync(slot->status.p, 0, sizeof(uint32_t), s));
		STPGB_TRY(stpgb_hydraulic_erosion(slot->merged.p, &nn, &g->rain, slot->starts.p, count, g->brush_index.p,
			g->brush_weight.p, g->brush_size, slot->residual.p, slot->status.p, s));
		STPGB_TRY(stpgb_format_heightmap(slot->merged.p, slot->fixed.p, nn.TotalMapSize[0], nn.TotalMapSize[1], s));
		STPGB_TRY(unmerge<float>(heightfield, slot->merged.p, nn, s));
		STPGB_TRY(unmerge<uint16_t>(fixed, slot->fixed.p, nn, s));
		double res = 0.0;
		STPGB_CUDA_TRY(cudaMemcpyAsync(&res, slot->residual.p, sizeof(double), cudaMemcpyDeviceToHost, s));
		STPGB_TRY(stpgb_status_check(slot->status.p, s));
		if (residual_out) {
			*residual_out = res;
		}
		return STPGB_OK;
	};
	rc = body();
	if (rc != STPGB_OK) {
		cudaStreamSynchronize(s);
	}
	g->release(std::move(slot));
	return rc;
}

} // namespace

extern "C" {

int stpgb_biomefield_create(const stpgb_simplex_setting* simplex, const stpgb_biome_property* biome_table,
	uint32_t biome_count, uint32_t interpolation_radius, stpgb_biomefield** out) {
	if (!simplex || !biome_table || !out || biome_count == 0u) {
		return inval("stpgb_biomefield_create: null argument or empty biome table");
	}
	STPGB_TRY(stpgb_simplex_setting_validate(simplex));
	auto f = std::make_unique<stpgb_biomefield>();
	f->radius = interpolation_radius;
	f->biome_count = biome_count;
	f->max_items = std::min<uint32_t>(biome_count, kShfMaxItems);
	// permutation (STPCommonCompiler.cpp:72 -> STPPermutationGenerator::generate)
	std::vector<uint8_t> perm(512);
	std::vector<float> grad(2u * simplex->Distribution);
	STPGB_TRY(stpgb_permutation_generate(simplex, perm.data(), grad.data(), static_cast<uint32_t>(grad.size())));
	STPGB_TRY(f->perm.alloc(512));
	STPGB_TRY(f->grad.alloc(grad.size()));
	STPGB_CUDA_TRY(cudaMemcpy(f->perm.p, perm.data(), 512, cudaMemcpyHostToDevice));
	STPGB_CUDA_TRY(cudaMemcpy(f->grad.p, grad.data(), grad.size() * sizeof(float), cudaMemcpyHostToDevice));
	f->permutation = stpgb_permutation { f->perm.p, f->grad.p, simplex->Distribution };
	STPGB_TRY(f->table.alloc(biome_count));
	STPGB_CUDA_TRY(cudaMemcpy(f->table.p, biome_table, biome_count * sizeof(stpgb_biome_property), cudaMemcpyHostToDevice));
	*out = f.release();
	return STPGB_OK;
}

int stpgb_biomefield_destroy(stpgb_biomefield* plugin) {
	delete plugin;
	return STPGB_OK;
}

// STPBiomefieldGenerator::operator() (STPBiomefieldGenerator.cpp:79-152): the
// filter of the biome neighbourhood, then the multi-biome heightmap kernel;
// the filter's output stays on the device.  The call waits for its own work
// (the filter's status is read back), so its scratch is free on return.
int stpgb_biomefield_generate(void* plugin, const stpgb_diversity_call* call) {
	auto* const f = static_cast<stpgb_biomefield*>(plugin);
	if (!f || !call || !call->heightmap || !call->biomemap) {
		return inval("stpgb_biomefield_generate: null argument");
	}
	const stpgb_nn_info& nn = call->biomemap_nn;
	const uint32_t W = nn.MapSize[0], H = nn.MapSize[1];
	if (call->heightmap_nn.MapSize[0] != W || call->heightmap_nn.MapSize[1] != H) {
		return inval("stpgb_biomefield_generate: heightmap and biome map chunk sizes differ");
	}
	const size_t npix = static_cast<size_t>(W) * H;
	const cudaStream_t s = as_stream(call->stream);
	std::unique_ptr<FieldScratch> sc = f->acquire();
	auto body = [&]() -> int {
		size_t ws = 0u;
		STPGB_TRY(stpgb_shf_workspace_size(&nn, f->radius, f->max_items, &ws));
		const uint64_t cap = npix * shf_kcap_h(f->radius, f->max_items);
		STPGB_TRY(sc->ws.alloc(ws));
		STPGB_TRY(sc->offsets.alloc(npix + 1u));
		STPGB_TRY(sc->bins.alloc(cap));
		STPGB_TRY(sc->status.alloc(1u));
		STPGB_TRY(stpgb_shf_filter(call->biomemap, &nn, f->radius, f->max_items, sc->ws.p, ws, sc->offsets.p,
			sc->bins.p, cap, sc->status.p, s));
		STPGB_TRY(stpgb_multibiome_heightmap(call->heightmap, W, sc->offsets.p, sc->bins.p, W, H, call->offset_x,
			call->offset_y, &f->permutation, f->table.p, f->biome_count, s));
		STPGB_TRY(stpgb_status_check(sc->status.p, s));
		return STPGB_OK;
	};
	const int rc = body();
	if (rc != STPGB_OK) {
		cudaStreamSynchronize(s);
	}
	f->release(std::move(sc));
	return rc;
}

int stpgb_generator_create_setup(const stpgb_generator_setup* setup, stpgb_generator** out) {
	if (!setup || !setup->ChunkSetting || !setup->RainDropSetting || !setup->DiversityGenerator
		|| !setup->DiversityGenerator->generate || !out) {
		return inval("stpgb_generator_create_setup: null argument or diversity generator without a function");
	}
	const stpgb_chunk_setting* const chunk = setup->ChunkSetting;
	const stpgb_raindrop_setting* const raindrop = setup->RainDropSetting;
	// STPChunkSetting::validate (SuperTerrain+/SuperTerrain+/Private/STPEnvironment.cpp:17-41), heightfield part
	if (chunk->MapSize[0] == 0u || chunk->MapSize[1] == 0u || !odd_positive(chunk->DiversityNearestNeighbour)
		|| !odd_positive(chunk->ErosionNearestNeighbour)) {
		return inval("STPChunkSetting: MapSize must be positive and neighbour counts positive and odd");
	}
	STPGB_TRY(stpgb_raindrop_setting_validate(raindrop));
	auto g = std::make_unique<stpgb_generator>();
	g->chunk = *chunk;
	g->rain = *raindrop;
	g->diversity = *setup->DiversityGenerator;
	g->div_nn = make_nn(chunk->MapSize, chunk->DiversityNearestNeighbour);
	g->ero_nn = make_nn(chunk->MapSize, chunk->ErosionNearestNeighbour);
	STPGB_CUDA_TRY(cudaGetDevice(&g->device));

	// erosion brush over the merged erosion map (STPHeightfieldGenerator.cpp:130-131)
	uint32_t bs = 0u;
	stpgb_erosion_brush_generate(g->ero_nn.TotalMapSize[0], raindrop->ErosionBrushRadius, nullptr, nullptr, 0u, &bs);
	std::vector<int32_t> bi(bs);
	std::vector<float> bw(bs);
	STPGB_TRY(stpgb_erosion_brush_generate(g->ero_nn.TotalMapSize[0], raindrop->ErosionBrushRadius, bi.data(),
		bw.data(), bs, &bs));
	STPGB_TRY(g->brush_index.alloc(bs));
	STPGB_TRY(g->brush_weight.alloc(bs));
	STPGB_CUDA_TRY(cudaMemcpy(g->brush_index.p, bi.data(), bs * sizeof(int32_t), cudaMemcpyHostToDevice));
	STPGB_CUDA_TRY(cudaMemcpy(g->brush_weight.p, bw.data(), bs * sizeof(float), cudaMemcpyHostToDevice));
	g->brush_size = bs;
	*out = g.release();
	return STPGB_OK;
}

int stpgb_generator_create(const stpgb_chunk_setting* chunk, const stpgb_raindrop_setting* raindrop,
	const stpgb_simplex_setting* simplex, const stpgb_biome_property* biome_table, uint32_t biome_count,
	uint32_t interpolation_radius, stpgb_generator** out) {
	if (!chunk || !raindrop || !simplex || !biome_table || !out || biome_count == 0u) {
		return inval("stpgb_generator_create: null argument or empty biome table");
	}
	// the filter's own checks of the radius against the diversity neighbourhood, at creation
	const stpgb_nn_info div = make_nn(chunk->MapSize, chunk->DiversityNearestNeighbour);
	if (chunk->MapSize[0] == 0u || chunk->MapSize[1] == 0u || !odd_positive(chunk->DiversityNearestNeighbour)
		|| !odd_positive(chunk->ErosionNearestNeighbour)) {
		return inval("STPChunkSetting: MapSize must be positive and neighbour counts positive and odd");
	}
	STPGB_TRY(stpgb_raindrop_setting_validate(raindrop));
	size_t ws = 0u;
	STPGB_TRY(stpgb_shf_workspace_size(&div, interpolation_radius, std::min<uint32_t>(biome_count, kShfMaxItems), &ws));
	stpgb_biomefield* plugin = nullptr;
	STPGB_TRY(stpgb_biomefield_create(simplex, biome_table, biome_count, interpolation_radius, &plugin));
	std::unique_ptr<stpgb_biomefield> owned(plugin);
	const stpgb_diversity_generator dg { stpgb_biomefield_generate, plugin };
	const stpgb_generator_setup setup { chunk, raindrop, &dg };
	stpgb_generator* g = nullptr;
	STPGB_TRY(stpgb_generator_create_setup(&setup, &g));
	g->owned_plugin = std::move(owned);
	*out = g;
	return STPGB_OK;
}

int stpgb_generator_destroy(stpgb_generator* gen) {
	delete gen;
	return STPGB_OK;
}

int stpgb_generator_generate(stpgb_generator* g, float* heightfield, const uint16_t* const* biomemap, float offset_x,
	float offset_y) {
	if (!g || !heightfield || !biomemap) {
		return inval("stpgb_generator_generate: null argument");
	}
	std::unique_ptr<Slot> slot;
	STPGB_TRY(g->acquire(slot));
	const cudaStream_t s = slot->stream;
	const stpgb_nn_info& nn = g->div_nn;
	const uint32_t W = nn.MapSize[0], H = nn.MapSize[1];
	const size_t npix = static_cast<size_t>(W) * H;
	auto body = [&]() -> int {
		STPGB_TRY(slot->biome.alloc(static_cast<size_t>(nn.TotalMapSize[0]) * nn.TotalMapSize[1]));
		STPGB_TRY(slot->height.alloc(npix));
		STPGB_TRY(merge<uint16_t>(slot->biome.p, biomemap, nn, s));
		stpgb_diversity_call call {};
		call.heightmap = slot->height.p;
		call.biomemap = slot->biome.p;
		call.biomemap_chunks_host = biomemap;
		const uint32_t one[2] = { 1u, 1u };
		call.heightmap_nn = make_nn(nn.MapSize, one);
		call.biomemap_nn = nn;
		call.offset_x = offset_x;
		call.offset_y = offset_y;
		call.stream = s;
		const int prc = g->diversity.generate(g->diversity.user, &call);
		if (prc != STPGB_OK) {
			if (prc < STPGB_OK || prc > STPGB_ECAPACITY) {
				return inval("diversity generator failed with code " + std::to_string(prc));
			}
			return prc;
		}
		STPGB_CUDA_TRY(cudaMemcpyAsync(heightfield, slot->height.p, npix * sizeof(float), cudaMemcpyDeviceToHost, s));
		STPGB_CUDA_TRY(cudaStreamSynchronize(s));
		return STPGB_OK;
	};
	const int rc = body();
	if (rc != STPGB_OK) {
		cudaStreamSynchronize(s);
	}
	g->release(std::move(slot));
	return rc;
}

int stpgb_generator_erode(stpgb_generator* gen, float* const* heightfield, uint16_t* const* heightfield_fixed) {
	if (!gen) {
		return inval("stpgb_generator_erode: null generator");
	}
	return erode_common(gen, heightfield, heightfield_fixed, nullptr, gen->rain.RainDropCount, nullptr);
}

int stpgb_generator_erode_starts(stpgb_generator* gen, float* const* heightfield, uint16_t* const* heightfield_fixed,
	const float* starts_xy, uint32_t count, double* residual_sediment) {
	if (!starts_xy && count > 0u) {
		return inval("stpgb_generator_erode_starts: null start array");
	}
	return erode_common(gen, heightfield, heightfield_fixed, starts_xy, count, residual_sediment);
}

} // extern "C"
