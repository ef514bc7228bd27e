/*
 * stpgb.h — C ABI of the GB300-native SuperTerrain+ heightfield pipeline.
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (STPGB_OK on success) and, on failure, leaves a message readable through
 * stpgb_last_error() on the calling thread.  Device pointers are CUDA device
 * addresses on the current device; `stream` is a cudaStream_t passed as a
 * void* so that this header needs no CUDA include.  Nothing here is globally
 * synchronous unless it says so: kernels are enqueued on `stream`.
 *
 * Status codes map onto the reference's exception types:
 *   STPGB_EINVAL   -> STPException::STPNumericDomainError / STPInvalidEnvironment
 *   STPGB_ECUDA    -> STPException::STPCUDAError
 *   STPGB_ETIMEOUT -> (new) a device loop hit its iteration cap
 *   STPGB_ENOMEM   -> allocation failure or an HBM budget refusal
 *   STPGB_ECAPACITY-> a caller-sized output or workspace was too small
 */
#ifndef STPGB_H_
#define STPGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define STPGB_API __attribute__((visibility("default")))
#else
#define STPGB_API
#endif

enum {
	STPGB_OK = 0,
	STPGB_EINVAL = 1,
	STPGB_ECUDA = 2,
	STPGB_ETIMEOUT = 3,
	STPGB_ENOMEM = 4,
	STPGB_ECAPACITY = 5
};

/* ---------------------------------------------------------------- types -- */

/* STPSingleHistogram::STPBin — SuperTerrain+/SuperAlgorithm+/Host/Public/
 * SuperAlgorithm+Host/STPSingleHistogram.hpp:23-33,35.  8 bytes: Item at 0,
 * two padding bytes, Weight at 4. */
typedef struct stpgb_bin {
	uint16_t Item;
	float Weight;
} stpgb_bin;

/* STPNearestNeighbourInformation —
 * SuperTerrain+/SuperTerrain+/Public/SuperTerrain+/World/Chunk/
 * STPNearestNeighbourInformation.hpp:13-25. */
typedef struct stpgb_nn_info {
	uint32_t MapSize[2];
	uint32_t ChunkNearestNeighbour[2];
	uint32_t TotalMapSize[2];
} stpgb_nn_info;

/* STPEnvironment::STPSimplexNoiseSetting —
 * SuperTerrain+/SuperAlgorithm+/Host/Public/SuperAlgorithm+Host/
 * STPSimplexNoiseSetting.h:13-27. */
typedef struct stpgb_simplex_setting {
	uint64_t Seed;
	uint32_t Distribution;
	double Offset;
} stpgb_simplex_setting;

/* STPEnvironment::STPRainDropSetting — SuperTerrain+/SuperTerrain+/Public/
 * SuperTerrain+/Environment/STPRainDropSetting.h:15-53 (same field order). */
typedef struct stpgb_raindrop_setting {
	uint64_t Seed;
	uint32_t RainDropCount;
	float Inertia;
	float SedimentCapacityFactor;
	float minSedimentCapacity;
	float initWaterVolume;
	float minWaterVolume;
	float Friction;
	float initSpeed;
	float ErodeSpeed;
	float DepositSpeed;
	float EvaporateSpeed;
	float Gravity;
	uint32_t ErosionBrushRadius;
} stpgb_raindrop_setting;

/* STPDemo::STPBiomeProperty — SuperDemo+/World/Biomes/STPBiomeProperty.hpp:10-27. */
typedef struct stpgb_biome_property {
	float Scale;
	uint32_t Octave;
	float Persistence;
	float Lacunarity;
	float Depth;
	float Variation;
} stpgb_biome_property;

/* STPAlgorithm::STPPermutation — .../SuperAlgorithm+Host/STPPermutation.hpp:9-22.
 * Both pointers are device addresses. */
typedef struct stpgb_permutation {
	const uint8_t* Permutation;
	const float* Gradient2D;
	uint32_t Gradient2DSize;
} stpgb_permutation;

/* Settings of one heightfield generator: the subset of STPChunkSetting
 * (SuperTerrain+/SuperTerrain+/Public/SuperTerrain+/Environment/
 * STPChunkSetting.h:15-45) the heightfield path reads. */
typedef struct stpgb_chunk_setting {
	uint32_t MapSize[2];
	uint32_t DiversityNearestNeighbour[2];
	uint32_t ErosionNearestNeighbour[2];
} stpgb_chunk_setting;

/* ------------------------------------------------------------- errors --- */

/* Message of the last failure on this thread ("" if none). */
STPGB_API const char* stpgb_last_error(void);
/* Library version string. */
STPGB_API const char* stpgb_version(void);

/* No counterpart in the reference: a copy of `bytes` between any two host or
 * device buffers, ordered on `stream` (cudaMemcpyAsync, the direction taken
 * from the addresses); with `wait` nonzero the call returns after the copy.
 * For callers that do not include the CUDA headers, such as the C++ façade's
 * texture buffers staged in host memory. */
STPGB_API int stpgb_copy(void* dst, const void* src, size_t bytes, void* stream, int wait);

/* --------------------------------------------------- host-side tables --- */

/* Validation of STPSimplexNoiseSetting
 * (SuperTerrain+/SuperAlgorithm+/Host/Private/STPAlgorithmEnvironment.cpp:13-17). */
STPGB_API int stpgb_simplex_setting_validate(const stpgb_simplex_setting* setting);

/* Validation of STPRainDropSetting
 * (SuperTerrain+/SuperTerrain+/Private/STPEnvironment.cpp:48-66). */
STPGB_API int stpgb_raindrop_setting_validate(const stpgb_raindrop_setting* setting);

/* Replaces STPPermutationGenerator::generate
 * (SuperTerrain+/SuperAlgorithm+/Host/Private/STPPermutationGenerator.cpp:40-94),
 * host half: writes the 512-byte permutation and 2*Distribution gradient
 * floats to host memory.  `grad_capacity` is the number of floats `grad`
 * holds (>= 2*Distribution).  The gradient loop of the reference runs one
 * extra time for some Distribution values and writes past its table; here the
 * extra entry is dropped. */
STPGB_API int stpgb_permutation_generate(const stpgb_simplex_setting* setting,
	uint8_t* perm512, float* grad, uint32_t grad_capacity);

/* Replaces generateErosionBrush
 * (SuperTerrain+/SuperTerrain+/Private/World/Chunk/STPHeightfieldGenerator.cpp:44-99),
 * host half: `index` / `weight` receive up to `capacity` entries, `*size` the
 * brush size.  Returns STPGB_ECAPACITY (and the needed size) if too small. */
STPGB_API int stpgb_erosion_brush_generate(uint32_t dimension_x, uint32_t radius,
	int32_t* index, float* weight, uint32_t capacity, uint32_t* size);

/* minWaterVolume that makes the droplet loop of
 * SuperTerrain+/SuperTerrain+/Private/GPGPU/STPRainDrop.cu:74 run exactly
 * `lifetime` steps (unless the droplet leaves the map first). */
STPGB_API float stpgb_lifetime_min_water_volume(float init_water_volume,
	float evaporate_speed, uint32_t lifetime);

/* ------------------------------------------------- chunk coordinates ---- */

/* The static coordinate functions of STPChunk
 * (SuperTerrain+/SuperTerrain+/Public/SuperTerrain+/World/Chunk/STPChunk.h:110-157,
 * SuperTerrain+/SuperTerrain+/Private/World/Chunk/STPChunk.cpp:63-108).  A
 * chunk coordinate is in world units (a multiple of the chunk size); vectors
 * are two-element arrays (x, then y / z).  Where the reference has undefined
 * behaviour (a zero size or range, an int32 overflow, a non-finite
 * position) these return STPGB_EINVAL. */

/* STPChunk::calcWorldChunkCoordinate (STPChunk.cpp:63-69): the coordinate of
 * the chunk holding world point (x, z), chunks scaled by `scale`. */
STPGB_API int stpgb_chunk_world_coordinate(double point_x, double point_z,
	const uint32_t* chunk_size, const double* scale, int32_t* out);
/* STPChunk::calcLocalChunkCoordinate (STPChunk.cpp:71-73): chunk index of a
 * row-major region -> (index % range.x, index / range.x). */
STPGB_API int stpgb_chunk_local_coordinate(uint32_t chunk_id, const uint32_t* chunk_range,
	uint32_t* out);
/* STPChunk::calcLocalChunkOrigin (STPChunk.cpp:75-79): the top-left chunk of
 * a neighbourhood of `neighbour_size` chunks around `centre`. */
STPGB_API int stpgb_chunk_local_origin(const int32_t* centre, const uint32_t* chunk_size,
	const uint32_t* neighbour_size, int32_t* out);
/* STPChunk::calcChunkMapOffset (STPChunk.cpp:81-85): the map offset a chunk's
 * maps are generated at, (coord / chunk_size) * map_size + map_offset in
 * double (a rounded product, then a rounded sum). */
STPGB_API int stpgb_chunk_map_offset(const int32_t* chunk_coord, const uint32_t* chunk_size,
	const uint32_t* map_size, const double* map_offset, double* out);
/* STPChunk::offsetChunk (STPChunk.cpp:87-89): coord + chunk_size * offset. */
STPGB_API int stpgb_chunk_offset(const int32_t* chunk_coord, const uint32_t* chunk_size,
	const int32_t* offset, int32_t* out);
/* STPChunk::calcChunkNeighbourOffset (STPChunk.cpp:91-108): the offset of
 * every chunk of a `region_size` neighbourhood from its centre chunk, in
 * chunk-index order, as `*count` (x, y) pairs in `offsets_xy` (STPGB_ECAPACITY
 * with the needed count when `capacity` pairs are too few). */
STPGB_API int stpgb_chunk_neighbour_offset(const uint32_t* chunk_size, const uint32_t* region_size,
	int32_t* offsets_xy, uint32_t capacity, uint32_t* count);

/* Host memory mode of STPNearestNeighbourTextureBuffer::STPMergedBuffer
 * (SuperTerrain+/SuperTerrain+/Private/World/Chunk/STPNearestNeighbourTextureBuffer.cpp:18-113):
 * pack the ChunkNearestNeighbour.x * .y host chunk maps (MapSize pixels of
 * `element_size` bytes each, row-major, chunk index order) into one merged
 * TotalMapSize map, chunk i at local chunk coordinate (i % nx, i / nx), and
 * unpack it back.  The device path merges on the GPU inside the generator,
 * the batch and the server. */
STPGB_API int stpgb_nn_merge_host(const void* const* chunks, uint32_t element_size, const stpgb_nn_info* nn,
	void* merged);
STPGB_API int stpgb_nn_unmerge_host(const void* merged, uint32_t element_size, const stpgb_nn_info* nn,
	void* const* chunks);

/* ----------------------------------------------- single histogram filter -- */

/* Workspace bytes stpgb_shf_filter needs for a chunk of `nn`, `radius`, and
 * at most `max_items` distinct sample values in any filter window
 * (0 = the library maximum, 256). */
STPGB_API int stpgb_shf_workspace_size(const stpgb_nn_info* nn, uint32_t radius,
	uint32_t max_items, size_t* bytes);

/* Replaces STPSingleHistogramFilter::operator()
 * (SuperTerrain+/SuperAlgorithm+/Host/Private/STPSingleHistogramFilter.cpp:870-902),
 * on the GPU.  Input: `samplemap` (device, TotalMapSize row-major uint16).
 * Output (device): `offsets` (MapSize.x*MapSize.y+1 uint32, the reference's
 * HistogramStartOffset) and `bins` (capacity `bins_capacity`), bit-identical to
 * the reference including bin order.  Radius must be positive, even and no
 * larger than the central chunk's start coordinate (reference :874-880).
 * A too-small `bins_capacity` or a window with more than `max_items` distinct
 * values is reported by stpgb_shf_check on `status` (device uint32, may be
 * NULL; it is cleared by this call).  Asynchronous on `stream`. */
STPGB_API int stpgb_shf_filter(const uint16_t* samplemap, const stpgb_nn_info* nn,
	uint32_t radius, uint32_t max_items, void* workspace, size_t workspace_bytes,
	uint32_t* offsets, stpgb_bin* bins, uint64_t bins_capacity, uint32_t* status,
	void* stream);

/* No counterpart in the reference.  stpgb_shf_filter for callers that may not
 * allocate device memory (a frame loop where cudaFree would stall on the whole
 * device, an engine whose own allocator owns every byte of its budget): the
 * filter's scratch comes from a fixed 16 MiB array inside the library, held
 * by every GPU that loads it until the process exits, instead of a caller
 * workspace.  Inputs and outputs are the caller's, as in stpgb_shf_filter.
 * Returns STPGB_ECAPACITY if stpgb_shf_workspace_size exceeds 16 MiB.  The
 * first call on a device looks up the array's address; make it before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller.  Allocates nothing. */
STPGB_API int stpgb_shf_filter_noalloc(const uint16_t* samplemap, const stpgb_nn_info* nn,
	uint32_t radius, uint32_t max_items, uint32_t* offsets, stpgb_bin* bins,
	uint64_t bins_capacity, uint32_t* status, void* stream);

/* Synchronous convenience: runs the filter into library-owned device memory
 * and copies offsets (W*H+1) and bins to HOST memory.  `*nbins` receives the
 * bin count; if `bins_capacity` is too small nothing is copied to `bins`
 * and STPGB_ECAPACITY is returned with `*nbins` set.  Input is HOST memory. */
STPGB_API int stpgb_shf_filter_host(const uint16_t* samplemap_host, const stpgb_nn_info* nn,
	uint32_t radius, uint32_t* offsets_host, stpgb_bin* bins_host, uint64_t bins_capacity,
	uint64_t* nbins);

/* No counterpart in the reference.  The path the last stpgb_shf_filter call
 * with this workspace (and the same nn, radius, max_items) took for its chunk:
 * `*path` = 0 when the general sequential slides filtered it; 1 or 2 when the
 * chunk's read region ((H+2r) x (W+2r) samples) held at most 8 distinct
 * values and the few-values kernels did: 1 their packed sequential slides
 * (launches of many chunks), 2 their row bands (launches of few).  All give
 * the same output.  Synchronises `stream`. */
STPGB_API int stpgb_shf_filter_path(const stpgb_nn_info* nn, uint32_t radius, uint32_t max_items,
	const void* workspace, uint32_t* path, void* stream);

/* No counterpart in the reference.  Process-wide choice of the filter's path
 * for every later launch (tuning and diagnostics): 0 = by chunk and launch
 * size (the default), 1 = few-values packed slides, 2 = few-values row
 * bands (chunks of more than 4096 - 2r columns still take the general
 * slides), 3 = the general slides for every chunk.  STPGB_EINVAL above 3. */
STPGB_API int stpgb_shf_set_path(uint32_t path);

/* Reads and decodes a device status word written by the kernels
 * (synchronises `stream`).  Returns STPGB_OK, STPGB_ECAPACITY or STPGB_ETIMEOUT. */
STPGB_API int stpgb_status_check(const uint32_t* status, void* stream);

/* ------------------------------------------------ multi-biome heightfield -- */

/* Replaces generateMultiBiomeHeightmap + sampleSimplexNoise
 * (SuperDemo+/Script/STPMultiHeightGenerator.cu:35-72) and
 * STPSimplexNoise::simplex2D / simplex2DFractal
 * (SuperTerrain+/SuperAlgorithm+/Device/Private/STPSimplexNoise.cu:18-110).
 * For every pixel (x,y) of a MapSize chunk:
 *   h = sum over its bins of Weight * (fractal_biome(x,y) * Variation + Depth)
 * `heightmap` is written with row pitch `pitch` floats (>= MapSize.x).
 * `perm` holds device pointers; `biome_table` is a device array of
 * `biome_count` entries indexed by bin Item. */
STPGB_API int stpgb_multibiome_heightmap(float* heightmap, uint32_t pitch,
	const uint32_t* offsets, const stpgb_bin* bins, uint32_t map_x, uint32_t map_y,
	float offset_x, float offset_y, const stpgb_permutation* perm,
	const stpgb_biome_property* biome_table, uint32_t biome_count, void* stream);

/* ------------------------------------------------------------- erosion --- */

/* Replaces the droplet-start draw of hydraulicErosionKERNEL
 * (SuperTerrain+/SuperTerrain+/Private/GPGPU/STPHeightfieldKernel.cu:93-104):
 * `count` (x,y) float pairs uniform in the central chunk, from a
 * Philox4x32-10 stream (Salmon et al., SC'11) keyed by `seed`, counter =
 * droplet index + `counter_base`. Device output. */
STPGB_API int stpgb_droplet_starts(float* starts_xy, uint32_t count, uint64_t seed,
	uint64_t counter_base, const stpgb_nn_info* nn, void* stream);

/* Replaces STPHeightfieldKernel::hydraulicErosion
 * (SuperTerrain+/SuperTerrain+/Private/GPGPU/STPHeightfieldKernel.cu:37-49,80-108)
 * and STPRainDrop (SuperTerrain+/SuperTerrain+/Private/GPGPU/STPRainDrop.cu:18-165):
 * free-slip particle erosion of the merged map `heightmap` (device,
 * TotalMapSize row-major float) by `count` droplets starting at `starts_xy`
 * (device).  `setting` is host memory.  `brush_index` / `brush_weight` are
 * device arrays of `brush_size` entries.  `residual_sediment` (device double,
 * may be NULL) accumulates the sediment that left with dying droplets, so
 * that sum(h_before) - sum(h_after) == *residual_sediment up to rounding.
 * `status` (device uint32, may be NULL) reports a droplet that hit the step
 * cap.  A brush point removes min(max(cell, 0), w) where the reference
 * removes min(cell, w) (STPRainDrop.cu:149): the same on every non-negative
 * cell, which is every cell of a map that starts non-negative unless racing
 * droplets take one below zero; there the reference's form gives the
 * negative height back once per racing reader, which grows without bound in
 * dense channels.  Asynchronous on `stream`. */
STPGB_API int stpgb_hydraulic_erosion(float* heightmap, const stpgb_nn_info* nn,
	const stpgb_raindrop_setting* setting, const float* starts_xy, uint32_t count,
	const int32_t* brush_index, const float* brush_weight, uint32_t brush_size,
	double* residual_sediment, uint32_t* status, void* stream);

/* stpgb_hydraulic_erosion with an explicit number of lanes carrying one
 * droplet (1, 2, 4, 8, 16 or 32; 0 = the default, see stpgb_erosion_choice),
 * droplets per lane group (1, or 2 / 4 with 4, 8 or 16 lanes, or 2 with 2 or
 * 4 brush-row lanes: the group advances its droplets together so their
 * memory round trips overlap) and flags.  Point by point, each lane erodes its
 * share of the brush in the reference's order (STPRainDrop.cu:146-157): read
 * a cell, subtract min(cell, w), next point; one lane per droplet is the
 * reference kernel itself.  With 2 or 4 lanes and 1 or 2 droplets per group,
 * on a 16-byte aligned map whose width is a multiple of four, a lane takes
 * whole brush rows (runs of consecutive cells) and updates them in aligned
 * 16-byte blocks instead: one vector read, then one vector reduction
 * subtracting min(cell, w) from the row's cells (-0.0 elsewhere); a droplet's
 * cells are distinct, so per droplet this is the same read-then-subtract,
 * with a quarter of the memory operations.  From brush radius 4, and with two
 * lanes, a block is instead updated by one returning vector atomic that
 * subtracts the amounts and yields the cells' values at that moment, and a
 * lane gives back what a cell lacked: the reference's c - min(c, w) on the
 * exact current value.  Where few droplets are in flight per pixel (at most
 * 3/4), a lane reads up to three blocks of a run per round trip.  The default
 * runs brush rows with two lanes per droplet (row blocks need at least four
 * points or blocks per lane; with fewer a step's reads happen nearly together
 * and densely packed droplets can run the map away), and, where few droplets
 * are in flight per pixel, the warp-cooperative row kernel: one droplet per
 * lane, the brush runs of a warp's eroding droplets shared out over all 32
 * lanes, each run's blocks taken by returning atomics (lanes_per_droplet = 1
 * without STPGB_EROSION_POINTWISE selects it explicitly).
 * STPGB_EROSION_POINTWISE keeps the point-by-point kernels.
 * STPGB_EROSION_EXACT_CLAMP erodes each point by compare-and-swap instead, so
 * racing droplets never remove more than a cell holds (closer to the serial
 * algorithm, slower).  No counterpart in the reference. */
enum { STPGB_EROSION_EXACT_CLAMP = 1, STPGB_EROSION_POINTWISE = 2 };

/* The kernel variant the default (lanes_per_droplet = 0) of
 * stpgb_hydraulic_erosion_ex takes for a brush of `brush_radius` and
 * `droplets` over `area` pixels (the chunk the starts cover).  Racing
 * droplets packed densely enough dig channels without bound, and the faster
 * a droplet's brush update completes, the lower that density: up to 3
 * droplets per pixel and 1.5 in flight at once brush rows are taken (the
 * warp-cooperative kernel up to 0.2 in flight, reported as 1 lane with
 * rows; else lanes keeping four 16-byte blocks each; point by point for
 * brushes too small for that), beyond it one lane per droplet (the reference
 * kernel).  No counterpart in the reference. */
STPGB_API int stpgb_erosion_choice(uint32_t brush_radius, uint32_t droplets, uint32_t area,
	uint32_t* lanes_per_droplet, uint32_t* vector_rows);
STPGB_API int stpgb_hydraulic_erosion_ex(float* heightmap, const stpgb_nn_info* nn,
	const stpgb_raindrop_setting* setting, const float* starts_xy, uint32_t count,
	const int32_t* brush_index, const float* brush_weight, uint32_t brush_size,
	double* residual_sediment, uint32_t* status, uint32_t lanes_per_droplet,
	uint32_t droplets_per_group, uint32_t flags, void* stream);

/* Replaces STPHeightfieldKernel::formatHeightmap
 * (SuperTerrain+/SuperTerrain+/Private/GPGPU/STPHeightfieldKernel.cu:51-57,112-122):
 * out[i] = uint16(rint(saturate(in[i]) * 65535)). Device buffers. */
STPGB_API int stpgb_format_heightmap(const float* in, uint16_t* out, uint32_t map_x,
	uint32_t map_y, void* stream);

/* ---------------------------------------------------- synthetic inputs --- */

/* Seeded Voronoi biome map over global pixel coordinates: nearest jittered
 * site of a `cell`-pixel grid, biome = hash(site) % biome_count.  Writes a
 * width x height uint16 tile whose top-left pixel is (origin_x, origin_y),
 * row pitch `pitch` elements.  Device output. Integer-only, so the CPU and
 * GPU agree bit for bit. */
STPGB_API int stpgb_voronoi_biomemap(uint16_t* out, uint32_t pitch, uint32_t width,
	uint32_t height, int64_t origin_x, int64_t origin_y, uint32_t cell,
	uint32_t biome_count, uint64_t seed, void* stream);

/* ------------------------------------------------ biome layer chain ----- */

/* Layer kinds of a biome layer chain, the demo layers of SuperTerrain+
 * (SuperDemo+/World/Layers/):
 *   CONTINENT  STPContinentLayer.h   first ancestor: Plains 1 in 10, else Ocean
 *   SCALE      STPScaleLayer.h       x2 zoom; Param STPGB_SCALE_NORMAL / _FUZZY
 *   LAND       STPLandLayer.h        diagonal-neighbour (STPXCrossLayer) land growth
 *   ISLAND     STPIslandLayer.h      4-neighbour (STPCrossLayer) islands in open ocean
 *   VORONOI    STPVoronoiLayer.h     x4 jittered-cell zoom, 2-D (Param 0) */
enum {
	STPGB_LAYER_CONTINENT = 1,
	STPGB_LAYER_SCALE = 2,
	STPGB_LAYER_LAND = 3,
	STPGB_LAYER_ISLAND = 4,
	STPGB_LAYER_VORONOI = 5
};
enum { STPGB_SCALE_NORMAL = 0, STPGB_SCALE_FUZZY = 1 };
enum { STPGB_MAX_LAYERS = 32 };

/* One layer: its kind, kind parameter and salt (the STPLayer constructor's
 * `salt`, SuperTerrain+/Public/SuperTerrain+/World/Diversity/STPLayer.h). */
typedef struct stpgb_layer {
	uint32_t Kind;
	uint32_t Param;
	uint64_t Salt;
} stpgb_layer;

/* Biome IDs the demo layers emit and test (STPBiomeRegistry: Ocean, Plains,
 * Forest, and the five shallow oceans of STPBiomeRegistry::isShallowOcean:
 * Ocean, FrozenOcean, WarmOcean, LukewarmOcean, ColdOcean). */
typedef struct stpgb_layer_biomes {
	uint16_t Ocean, Plains, Forest;
	uint16_t ShallowOcean[5];
} stpgb_layer_biomes;

/* The demo's production line (SuperDemo+/World/Layers/STPAllLayers.cpp:59-105,
 * the STPLayerChainBuilder pipeline), first ancestor first: 14 layers. */
STPGB_API int stpgb_layer_chain_demo(stpgb_layer* chain, uint32_t capacity, uint32_t* count);

/* The demo's biome IDs as its parameter loader sets them from Biome.ini
 * (ocean 0, plains 1, forest 3; registry biomes it does not load keep 0). */
STPGB_API void stpgb_layer_biomes_demo(stpgb_layer_biomes* ids);

/* Biomemap of a linear layer chain (chain[0] = first ancestor, chain[count-1]
 * = the layer sampled), the GPU replacement of
 * STPBiomeFactory::operator()(STPSample_t* biomemap, glm::ivec2 offset)
 * (SuperTerrain+/Private/World/Diversity/STPBiomeFactory.cpp:24-41):
 * biomemap[z * pitch + x] = sample(x + offset_x, 0, z + offset_z) for
 * x < width, z < height.  Device output, asynchronous on `stream`; bit-exact
 * with the reference's layers.  Voronoi layers use seed std::hash(global_seed),
 * the identity of libstdc++.  |offset| + size must stay below 2^30. */
STPGB_API int stpgb_layer_biomemap(const stpgb_layer* chain, uint32_t count, uint64_t global_seed,
	const stpgb_layer_biomes* ids, uint16_t* biomemap, uint32_t pitch, uint32_t width, uint32_t height,
	int32_t offset_x, int32_t offset_z, void* stream);

/* Same with a host output array of width x height (synchronous): the drop-in
 * for a host STPBiomeFactory caller. */
STPGB_API int stpgb_layer_biomemap_host(const stpgb_layer* chain, uint32_t count, uint64_t global_seed,
	const stpgb_layer_biomes* ids, uint16_t* biomemap, uint32_t width, uint32_t height, int32_t offset_x,
	int32_t offset_z);

/* ------------------------------------------------------------ splatmap --- */

/* Splat rules (SuperTerrain+/Public/SuperTerrain+/World/Diversity/Texture/
 * STPTextureInformation.hpp:27-106).  Rules are added per biome sample as
 * the reference's STPTextureSplatBuilder adds them
 * (SuperTerrain+/Private/World/Diversity/STPTextureDatabase.cpp:305-350):
 * an altitude rule makes RegionIndex active up to UpperBound; a gradient rule
 * makes it active for minGradient <= slope <= maxGradient and LowerBound <=
 * altitude <= UpperBound.  RegionIndex is the index the renderer's texture
 * region registry uses (the reference converts texture IDs to it). */
typedef struct stpgb_altitude_rule {
	uint16_t Sample;
	float UpperBound;
	uint32_t RegionIndex;
} stpgb_altitude_rule;

typedef struct stpgb_gradient_rule {
	uint16_t Sample;
	float minGradient, maxGradient, LowerBound, UpperBound;
	uint32_t RegionIndex;
} stpgb_gradient_rule;

/* The demo's rules (SuperDemo+/Script/STPBiomeSplatRule.tdl), regions
 * numbered in the script's texture order: redrock 0, grass 1, mossrock 2,
 * sand 3, soil 4, darkrock 5. */
STPGB_API int stpgb_splat_rules_demo(stpgb_altitude_rule* altitude, uint32_t altitude_capacity,
	uint32_t* altitude_count, stpgb_gradient_rule* gradient, uint32_t gradient_capacity,
	uint32_t* gradient_count);

/* STPSplatGeneratorInformation::STPLocalChunkInformation
 * (STPTextureInformation.hpp:114-135): which chunk of the rendering buffer
 * to splat, and its chunk map offset (the noise offset). */
typedef struct stpgb_splat_chunk {
	uint32_t LocalChunkCoordinateX, LocalChunkCoordinateY;
	float ChunkMapOffsetX, ChunkMapOffsetY;
} stpgb_splat_chunk;

typedef struct stpgb_splat_generator stpgb_splat_generator;

/* The splatmap generator (SuperDemo+/World/Biomes/STPSplatmapGenerator.cpp
 * with SuperDemo+/Script/STPSplatmapGenerator.cu and the rule database of
 * STPTextureFactory, SuperTerrain+/Private/World/Diversity/
 * STPTextureFactory.cpp:138-200): rules in host memory (sorted here as the
 * texture database sorts them: altitude rules by sample then upper bound,
 * gradient rules by sample in the order added), the simplex setting of the
 * world (permutation table) and the chunk MapSize. */
STPGB_API int stpgb_splat_generator_create(const stpgb_altitude_rule* altitude, uint32_t altitude_count,
	const stpgb_gradient_rule* gradient, uint32_t gradient_count, const stpgb_simplex_setting* simplex,
	uint32_t map_x, uint32_t map_y, stpgb_splat_generator** out);
STPGB_API int stpgb_splat_generator_destroy(stpgb_splat_generator* generator);

/* Replaces STPTextureFactory::operator() / generateTextureSplatmap
 * (STPTextureFactory.cpp:211-232, STPSplatmapGenerator.cu).  The rendering
 * buffer is width x height pixels of device memory: `biomemap` (uint16, rows
 * `biome_pitch` elements apart) and `heightmap` (uint16 fixed-point heights,
 * as formatHeightmap writes them, rows `height_pitch` elements apart);
 * `splatmap` (uint8 region per pixel, 255 = no region) rows `splat_pitch`
 * bytes apart.  Each of the `count` chunks
 * (host array) covers MapSize pixels at LocalChunkCoordinate * MapSize.  The
 * heightmap is read through a texture with the reference's sampler (linear
 * filter, normalised float, clamp, unnormalised coordinates), the biomemap
 * through a point-filtered one, so both buffers must start on a 512-byte
 * boundary with a row pitch that is a multiple of 32 bytes.  `slope` and
 * `altitude` (device float, may be NULL, rows `splat_pitch` elements apart)
 * receive the slope factor and the noisy altitude the rules are tested with.
 * Asynchronous on `stream`. */
STPGB_API int stpgb_splatmap(stpgb_splat_generator* generator, const uint16_t* biomemap,
	uint32_t biome_pitch, const uint16_t* heightmap, uint32_t height_pitch, uint8_t* splatmap,
	uint32_t splat_pitch, uint32_t width, uint32_t height, const stpgb_splat_chunk* chunks, uint32_t count,
	float* slope, float* altitude, void* stream);

/* ------------------------------------- plain per-chunk drop-in generator -- */

typedef struct stpgb_generator stpgb_generator;

/* One call of a multi-biome heightmap plugin: the arguments of
 * STPDiversityGenerator::operator()
 * (SuperTerrain+/SuperTerrain+/Public/SuperTerrain+/World/Chunk/
 * STPDiversityGenerator.hpp:14-39), whose texture buffers
 * (STPNearestNeighbourTextureBuffer.h) become plain buffers: the chunk's
 * heightmap to write and the merged biome neighbourhood to read, both already
 * on the device, with the caller's host chunk arrays beside them for plugins
 * that work on the host.  All work goes on `stream`. */
typedef struct stpgb_diversity_call {
	float* heightmap;                             /* device, MapSize floats, row-major: the chunk to write */
	const uint16_t* biomemap;                     /* device, the merged DiversityNearestNeighbour region */
	const uint16_t* const* biomemap_chunks_host;  /* the caller's host chunks, chunk i at (i % nx, i / nx) */
	stpgb_nn_info heightmap_nn;                   /* MapSize, a 1x1 neighbourhood */
	stpgb_nn_info biomemap_nn;                    /* MapSize, DiversityNearestNeighbour */
	float offset_x, offset_y;                     /* the chunk's map offset in world coordinates */
	void* stream;                                 /* cudaStream_t */
} stpgb_diversity_call;

/* The plugin's operator(): enqueues the heightmap's generation on
 * call->stream and returns STPGB_OK, or an STPGB_* error code, which the
 * generator returns to its caller.  Called from the thread that called
 * stpgb_generator_generate; concurrent generate calls call it concurrently. */
typedef int (*stpgb_diversity_fn)(void* user, const stpgb_diversity_call* call);

/* STPDiversityGenerator as a C object: the function and its state. */
typedef struct stpgb_diversity_generator {
	stpgb_diversity_fn generate;
	void* user;
} stpgb_diversity_generator;

/* STPHeightfieldGenerator::STPGeneratorSetup
 * (SuperTerrain+/SuperTerrain+/Public/SuperTerrain+/World/Chunk/STPHeightfieldGenerator.h:35-45). */
typedef struct stpgb_generator_setup {
	const stpgb_chunk_setting* ChunkSetting;
	const stpgb_raindrop_setting* RainDropSetting;
	const stpgb_diversity_generator* DiversityGenerator; /* not owned; must outlive the generator */
} stpgb_generator_setup;

/* Replaces STPHeightfieldGenerator::STPHeightfieldGenerator(const STPGeneratorSetup&)
 * (STPHeightfieldGenerator.h:121, STPHeightfieldGenerator.cpp:115-150): validates the
 * settings and builds the erosion brush on the device; generate() calls the
 * setup's diversity plugin for the heightmap. */
STPGB_API int stpgb_generator_create_setup(const stpgb_generator_setup* setup, stpgb_generator** out);

/* The demo's multi-biome diversity plugin, STPBiomefieldGenerator
 * (SuperDemo+/World/Biomes/STPBiomefieldGenerator.cpp:44-152): single
 * histogram filter of the biome neighbourhood, then the multi-biome fractal
 * simplex heightmap, both on the device.  stpgb_biomefield_generate is an
 * stpgb_diversity_fn whose user pointer is the plugin object; it is
 * thread-safe (each call takes its own scratch). */
typedef struct stpgb_biomefield stpgb_biomefield;
STPGB_API int stpgb_biomefield_create(const stpgb_simplex_setting* simplex, const stpgb_biome_property* biome_table,
	uint32_t biome_count, uint32_t interpolation_radius, stpgb_biomefield** out);
STPGB_API int stpgb_biomefield_destroy(stpgb_biomefield* plugin);
STPGB_API int stpgb_biomefield_generate(void* plugin, const stpgb_diversity_call* call);

/* Replaces STPHeightfieldGenerator::STPHeightfieldGenerator
 * (SuperTerrain+/SuperTerrain+/Private/World/Chunk/STPHeightfieldGenerator.cpp:115-150)
 * together with the demo diversity plugin STPBiomefieldGenerator
 * (SuperDemo+/World/Biomes/STPBiomefieldGenerator.cpp:44-65): validates the
 * settings, builds the erosion brush and permutation on the device.  The same
 * as stpgb_generator_create_setup with an stpgb_biomefield plugin that the
 * generator owns. */
STPGB_API int stpgb_generator_create(const stpgb_chunk_setting* chunk,
	const stpgb_raindrop_setting* raindrop, const stpgb_simplex_setting* simplex,
	const stpgb_biome_property* biome_table, uint32_t biome_count,
	uint32_t interpolation_radius, stpgb_generator** out);
STPGB_API int stpgb_generator_destroy(stpgb_generator* gen);

/* Replaces STPHeightfieldGenerator::generate (…/STPHeightfieldGenerator.cpp:158-169):
 * HOST arrays; `biomemap` holds DiversityNearestNeighbour.x*y chunk pointers
 * (MapSize uint16 each, row-major chunk order); `heightfield` receives the
 * MapSize float chunk.  Synchronous, like the reference. */
STPGB_API int stpgb_generator_generate(stpgb_generator* gen, float* heightfield,
	const uint16_t* const* biomemap, float offset_x, float offset_y);

/* Replaces STPHeightfieldGenerator::erode (…/STPHeightfieldGenerator.cpp:171-197):
 * HOST arrays, ErosionNearestNeighbour.x*y chunk pointers each.  Droplet
 * starts come from stpgb_droplet_starts keyed by the raindrop Seed, with the
 * counter advanced by RainDropCount on every call.  Synchronous. */
STPGB_API int stpgb_generator_erode(stpgb_generator* gen, float* const* heightfield,
	uint16_t* const* heightfield_fixed);

/* erode() with explicit HOST droplet starts (`count` xy pairs in merged-map
 * coordinates); `residual_sediment` (host, may be NULL) receives the mass
 * that left with dying droplets. */
STPGB_API int stpgb_generator_erode_starts(stpgb_generator* gen, float* const* heightfield,
	uint16_t* const* heightfield_fixed, const float* starts_xy, uint32_t count,
	double* residual_sediment);

/* -------------------------------------------------- roofline kernels -- */

/* No counterpart in the reference: the measurement kernels behind the
 * roofline denominators of the kernels that HBM copy bandwidth does not
 * bound.  Each launch is `blocks` blocks of 256 threads, asynchronous on
 * `stream`; time it with events on that stream.
 *   RED_F32     every thread adds 1.0f with a scalar red.global to `iters`
 *               pseudo-random floats of `buffer` (`elements` floats, a power
 *               of two): 4 bytes per operation;
 *   RED_V4_F32  the same with 16-byte vector reductions (red.global.add.v4.f32)
 *               to aligned groups of four floats: 16 bytes per operation;
 *   LOAD_V4_F32 `iters` pseudo-random 16-byte loads per thread, kept in L2
 *               (ld.global.cg); `sink` is one float that is never written for a
 *               map of zeros;
 *   CHASE       one thread follows the uint32 table `buffer` of `elements`
 *               entries from entry 0 for `iters` dependent loads and writes the
 *               elapsed clock64 ticks to sink[0] (uint64, then the last index);
 *   FMA_F32     eight independent chains of `iters` fused multiply-adds per
 *               thread (16 flop per thread and iteration); `buffer` is one
 *               float, never written;
 *   ATOM_V4_F32 RED_V4_F32 with returning atomics (atom.global.add.v4.f32, the
 *               erosion brush's operation), each result used before the
 *               thread's next atomic; `sink` as for LOAD_V4_F32. */
enum {
	STPGB_ROOFLINE_RED_F32 = 0,
	STPGB_ROOFLINE_RED_V4_F32 = 1,
	STPGB_ROOFLINE_LOAD_V4_F32 = 2,
	STPGB_ROOFLINE_CHASE = 3,
	STPGB_ROOFLINE_FMA_F32 = 4,
	STPGB_ROOFLINE_ATOM_V4_F32 = 5
};
STPGB_API int stpgb_roofline_launch(uint32_t kind, void* buffer, uint64_t elements, uint32_t blocks,
	uint32_t iters, void* sink, void* stream);

/* ------------------------------------------------------ batched pipeline -- */

/* No counterpart in the reference, which generates one chunk per call: many
 * eroded-chunk requests, each a 3x3 free-slip neighbourhood of MapSize^2
 * chunks around world chunk (ChunkX, ChunkY), filtered, generated and eroded
 * together by one fixed sequence of batched launches (every launch covers
 * every chunk of every request), optionally captured in a CUDA graph. */
typedef struct stpgb_batch stpgb_batch;

typedef struct stpgb_batch_request {
	uint32_t MapSize;             /* chunk side, a positive multiple of 8 */
	int32_t ChunkX, ChunkY;       /* world chunk coordinate of the centre chunk */
	uint32_t InterpolationRadius; /* filter radius (even, <= MapSize) */
	uint32_t DropletCount;
	uint32_t BrushRadius;
	uint32_t Lifetime;            /* droplet steps; 0 keeps the base minWaterVolume */
} stpgb_batch_request;

enum {
	STPGB_BATCH_GRAPH = 1,   /* capture the launch sequence into a CUDA graph */
	STPGB_BATCH_AUTOTUNE = 2 /* at the first stpgb_batch_run, time the erosion variants on the batch's inputs
	                          * (uploaded or synthesized by then) and keep the fastest per group */
};

/* Lays out and allocates every buffer of the batch on the current device in
 * one allocation (STPGB_ENOMEM if it exceeds `hbm_budget` bytes; 0 = no
 * budget), builds the job tables and, with STPGB_BATCH_GRAPH, captures the
 * launch sequence into a CUDA graph.  `base` supplies the droplet settings
 * a request does not override; `biome_table` is indexed by biome ID. */
STPGB_API int stpgb_batch_create(const stpgb_batch_request* requests, uint32_t count,
	const stpgb_raindrop_setting* base, const stpgb_simplex_setting* simplex,
	const stpgb_biome_property* biome_table, uint32_t biome_count, uint64_t hbm_budget,
	uint32_t flags, stpgb_batch** out);
STPGB_API int stpgb_batch_destroy(stpgb_batch* batch);
STPGB_API uint64_t stpgb_batch_device_bytes(const stpgb_batch* batch);

/* Device buffers of one request: the 5x5-chunk biome region (uint16,
 * (5*MapSize)^2 row-major, the diversity neighbourhoods of all nine chunks),
 * the merged 3x3 float heightmap and its uint16 format ((3*MapSize)^2), and
 * the droplet start array (2*DropletCount floats).  Any may be NULL. */
STPGB_API int stpgb_batch_buffers(stpgb_batch* batch, uint32_t request, uint16_t** biome_region,
	float** heightmap, uint16_t** heightmap_fixed, float** starts_xy);

/* Fills every request's biome region with the seeded Voronoi map (global
 * coordinates, so neighbouring requests agree) and its starts with the
 * Philox stream of the base Seed. Asynchronous. */
STPGB_API int stpgb_batch_synthesize_inputs(stpgb_batch* batch, uint32_t voronoi_cell, uint64_t seed,
	void* stream);

/* Replaces every request's biome region with the demo's biome layer chain
 * (stpgb_layer_chain_demo, demo IDs, `seed`), as the reference's world
 * pipeline generates biomemaps; call after stpgb_batch_synthesize_inputs
 * (which also makes the starts).  The biome table must cover IDs 0, 1, 3. */
STPGB_API int stpgb_batch_synthesize_layer_biomes(stpgb_batch* batch, uint64_t seed, void* stream);

/* Runs the whole batch (graph launch when captured). Asynchronous. */
STPGB_API int stpgb_batch_run(stpgb_batch* batch, void* stream);

/* Runs the same work as the plain per-chunk call sequence (one chunk's
 * filter + noise per call, one erosion per request, a stream synchronise
 * after every call).  Synchronous; the baseline the batched path is
 * compared with. */
STPGB_API int stpgb_batch_run_plain(stpgb_batch* batch, void* stream);

/* HOST <-> device copies of the inputs and results, enqueued on `stream`. */
STPGB_API int stpgb_batch_upload(stpgb_batch* batch, const uint16_t* const* biome_regions,
	const float* const* starts_xy, void* stream);
STPGB_API int stpgb_batch_download(stpgb_batch* batch, float* const* heightmaps,
	uint16_t* const* heightmaps_fixed, double* residual_sediment, void* stream);

/* Device -> HOST copies of the current inputs (biome regions, starts). */
STPGB_API int stpgb_batch_download_inputs(stpgb_batch* batch, uint16_t* const* biome_regions,
	float* const* starts_xy, void* stream);

/* Synchronises `stream` and decodes the batch's device status word. */
STPGB_API int stpgb_batch_status(stpgb_batch* batch, void* stream);

/* One stage of the batch on its own (0 filter, 1 noise, 2 erosion,
 * 3 format), for per-kernel timing. Asynchronous. */
STPGB_API int stpgb_batch_run_stage(stpgb_batch* batch, uint32_t stage, void* stream);

/* Runs the autotuner now, on the batch's current inputs (synchronous), and
 * re-captures the graph of a batch created with STPGB_BATCH_GRAPH. */
STPGB_API int stpgb_batch_tune(stpgb_batch* batch);

/* A batch erodes its requests in up to four variant groups (requests that may
 * take the warp-cooperative kernel, other row requests, radius-2 brushes,
 * requests too densely packed for more than one lane per droplet), each tuned
 * on its own.  Reports the group with the most droplets: its erosion lanes per
 * droplet, droplets per lane group and brush update (1 = brush rows in 16-byte
 * blocks, 0 = point by point; 1 lane with rows = the warp-cooperative kernel)
 * in use, and the autotuner's erosion time in ms per candidate: 36 floats,
 * index 18*rows + 3*log2(lanes) + {0, 1, 2} for 1, 2, 4 droplets per group
 * (0 = not tried).  Any output pointer may be NULL. */
STPGB_API int stpgb_batch_tuning(const stpgb_batch* batch, uint32_t* lanes_per_droplet,
	uint32_t* droplets_per_group, uint32_t* vector_rows, float* erosion_ms);

/* The autotuner's choices for the other stages: the filter's segment count
 * (0 = chosen from the launch size) with its time in ms for the candidates
 * 0, 1, 2, 4, 8, 16 (6 floats), and the noise kernel's block size with its
 * time for 128, 256, 512 threads (3 floats); 0 ms = not tried; and, where the
 * dominant erosion group runs the warp-cooperative kernel, the number of jobs
 * whose blocks it interleaves (else 0).  Any output pointer may be NULL. */
STPGB_API int stpgb_batch_tuning_stages(const stpgb_batch* batch, uint32_t* shf_segments, float* shf_ms,
	uint32_t* noise_block, float* noise_ms, uint32_t* coop_interleave);

/* No counterpart in the reference.  The filter path the autotuner chose for
 * the batch (`*path`: 0 by launch size, 1 few-values packed slides, 2 few-values
 * row bands, 3 general slides; see stpgb_shf_set_path) and the filter stage's
 * time with each (`path_ms`, 4 floats; zeros before tuning). */
STPGB_API int stpgb_batch_tuning_filter_path(const stpgb_batch* batch, uint32_t* path, float* path_ms);

/* No counterpart in the reference.  The kernels one stpgb_batch_run launches:
 * the kernel nodes of the batch's CUDA graph (the filter's nine launches,
 * noise, one erosion launch per variant group, format). */
STPGB_API int stpgb_batch_kernels_per_run(const stpgb_batch* batch, uint32_t* kernels);

/* Realised droplet steps and brush-erosion steps summed over the runs since
 * the last reset (synchronises the device). */
STPGB_API int stpgb_batch_counters(stpgb_batch* batch, uint64_t* realised_steps, uint64_t* erode_steps,
	int reset);

/* ---------------------------------------------------------- serving ---- */

/* No counterpart in the reference (its world pipeline, SuperTerrain+/
 * SuperTerrain+/Private/World/STPWorldPipeline.cpp:411-662, runs one
 * synchronous generate/erode call per chunk from a host thread pool).  A
 * continuous-batching server: requests are admitted against a fixed HBM
 * budget, batched with whatever else is admitted while earlier batches run
 * on other streams, and served from resident generated chunks shared by
 * overlapping neighbourhoods.  Each request erodes a private copy of its
 * 3x3 neighbourhood, so its result does not depend on the other requests. */
typedef struct stpgb_server stpgb_server;

typedef struct stpgb_server_config {
	uint64_t HbmBudget;    /* device bytes of the pool (results, resident chunks, scratch) */
	uint32_t MaxInFlight;  /* requests admitted and not yet complete */
	uint32_t MaxBatch;     /* requests per launch sequence */
	uint32_t Streams;      /* launch sequences in flight at once */
	uint32_t VoronoiCell;  /* synthetic biome-map cell, in pixels of a 512 chunk (scaled with the side) */
	uint64_t BiomeSeed;
	/* STPGB_BIOMES_VORONOI: the synthetic Voronoi map above; STPGB_BIOMES_LAYER_CHAIN:
	 * the demo's biome layer chain (stpgb_layer_chain_demo, seed BiomeSeed, the
	 * demo's IDs 0 / 1 / 3, which the biome table must cover), as the
	 * reference's world pipeline generates biomemaps */
	uint32_t BiomeSource;
	/* STPGB_EROSION_PRIVATE: each request erodes a private copy of its
	 * neighbourhood (results independent of the request mix).
	 * STPGB_EROSION_IN_PLACE: the reference's world-pipeline semantics
	 * (SuperTerrain+/SuperTerrain+/Private/World/STPWorldPipeline.cpp:
	 * 339-403,485-541,640-662): a request erodes the resident chunks of its
	 * neighbourhood in place, so a chunk carries its neighbours' erosion;
	 * a centre chunk is eroded once (later requests for it return the
	 * current state); the requests of one launch sequence are ordered by the
	 * reference's priority schedule (overlapping neighbourhoods in
	 * successive priority levels, smallest first, non-overlapping ones
	 * together) and sequences touching the same chunks run one after the
	 * other.  Evicting a chunk discards the erosion it carried. */
	uint32_t ErosionMode;
} stpgb_server_config;
enum { STPGB_BIOMES_VORONOI = 0, STPGB_BIOMES_LAYER_CHAIN = 1 };
enum { STPGB_EROSION_PRIVATE = 0, STPGB_EROSION_IN_PLACE = 1 };

typedef struct stpgb_serve_request {
	int32_t ChunkX, ChunkY;       /* centre chunk of the 3x3 neighbourhood */
	uint32_t MapSize;             /* chunk side (level of detail), a multiple of 8 */
	uint32_t InterpolationRadius; /* filter radius, even, <= MapSize */
	float DropletsPerPixel;       /* droplets = round(DropletsPerPixel * MapSize^2) */
	uint32_t BrushRadius;
	uint32_t Lifetime;            /* droplet steps; 0 keeps the base minWaterVolume */
	uint64_t UserTag;
} stpgb_serve_request;

typedef struct stpgb_serve_result {
	uint64_t Ticket, UserTag;
	int Status;
	uint32_t MapSize;
	double LatencyMs;              /* submission -> result complete on the device */
	const float* Heightmap;        /* device, eroded (3*MapSize)^2 neighbourhood */
	const uint16_t* HeightmapFixed; /* device, its uint16 format */
	double ResidualSediment;
	/* STPGB_EROSION_IN_PLACE: the request's place in the server's erosion
	 * order (1, 2, ...; requests of one priority level take consecutive
	 * places and erode together), or 0 if its centre chunk had been eroded
	 * already and it returned the current state; 0 in the private mode. */
	uint64_t ErosionOrder;
} stpgb_serve_result;

typedef struct stpgb_server_stats {
	uint64_t Submitted, Admitted, Completed, Launches, ChunksGenerated, ChunksEvicted;
	uint64_t PoolBytesUsed, ResidentChunks;
} stpgb_server_stats;

/* Allocates the pool (STPGB_ENOMEM if the budget cannot be had) and starts
 * the scheduler thread on the current device. */
STPGB_API int stpgb_server_create(const stpgb_server_config* config, const stpgb_raindrop_setting* base,
	const stpgb_simplex_setting* simplex, const stpgb_biome_property* biome_table, uint32_t biome_count,
	stpgb_server** out);
STPGB_API int stpgb_server_destroy(stpgb_server* server);
/* Thread-safe, non-blocking.  STPGB_ENOMEM if one request alone exceeds the budget. */
STPGB_API int stpgb_server_submit(stpgb_server* server, const stpgb_serve_request* request, uint64_t* ticket);
/* Several requests that enter the queue together, in order, as the chunks of
 * one STPWorldPipeline::requestChunk call do (STPWorldPipeline.cpp:640-662):
 * the scheduler sees all of them at once.  `tickets` (may be NULL) receives
 * `count` tickets.  Checks every request first and queues none if one fails. */
STPGB_API int stpgb_server_submit_batch(stpgb_server* server, const stpgb_serve_request* requests, uint32_t count,
	uint64_t* tickets);
/* Up to `capacity` completed results; waits up to `wait_ms` (-1 = until one completes). */
STPGB_API int stpgb_server_poll(stpgb_server* server, stpgb_serve_result* results, uint32_t capacity,
	uint32_t* count, int wait_ms);
/* Copies a completed, not yet released result to HOST memory ((3*MapSize)^2
 * floats and uint16; either may be NULL).  Synchronous. */
STPGB_API int stpgb_server_download(stpgb_server* server, uint64_t ticket, float* heightmap,
	uint16_t* heightmap_fixed);
/* Returns a completed result's device memory to the pool. */
STPGB_API int stpgb_server_release(stpgb_server* server, uint64_t ticket);
STPGB_API int stpgb_server_stats_get(stpgb_server* server, stpgb_server_stats* stats);
/* Submits `requests[i]` at `arrival_s[i]` seconds after the call (ascending),
 * releases every result as it completes, writes each request's latency and
 * the wall time until the last completed.  Synchronous. */
STPGB_API int stpgb_server_replay(stpgb_server* server, const stpgb_serve_request* requests,
	const double* arrival_s, uint32_t count, double* latency_ms, double* wall_s);

#ifdef __cplusplus
}
#endif

#endif /* STPGB_H_ */
