// C entry points over the reference's own device code compiled as host C++
// (SuperAlgorithm+/Device/Private/STPSimplexNoise.cu,
// SuperTerrain+/Private/GPGPU/STPRainDrop.cu and the demo's generator script
// SuperDemo+/Script/STPMultiHeightGenerator.cu), used only to pin the oracle
// restatement.  Kernels run as host loops, one block of one thread at a time,
// in block order; droplets run one after another in start order.
#include <SuperAlgorithm+Device/STPSimplexNoise.cuh>
#include <SuperAlgorithm+Host/STPSingleHistogram.hpp>
#include <SuperTerrain+/GPGPU/STPRainDrop.cuh>
#include <STPBiomeProperty>

#include <cstdint>
#include <cstring>

uint3 threadIdx = { 0u, 0u, 0u }, blockIdx = { 0u, 0u, 0u };
dim3 blockDim, gridDim;

using namespace SuperTerrainPlus;
using namespace SuperTerrainPlus::STPAlgorithm;

namespace SuperTerrainPlus {
// the droplet's dynamic shared memory (`extern __shared__ unsigned char ErosionBrush[]`,
// STPRainDrop.cu:57): brush indices then weights
alignas(16) unsigned char ErosionBrush[8192u * (sizeof(int) + sizeof(float))];
}

// the generator script's constant memory (STPCommonGenerator.cu, STPMultiHeightGenerator.cu:14)
namespace STPCommonGenerator {
extern uint2 Dimension[1];
extern float2 HalfDimension[1];
extern uint2 RenderedDimension[1];
extern STPPermutation Permutation[1];
}
extern STPDemo::STPBiomeProperty BiomeTable[2];
void generateMultiBiomeHeightmap(STPHeightFloat_t*, const STPSingleHistogram, const float2);

namespace {

STPPermutation permutation_of(const uint8_t* perm, const float* grad, const uint32_t grad_size) {
	STPPermutation p;
	p.Permutation = const_cast<unsigned char*>(perm);
	p.Gradient2D = const_cast<float*>(grad);
	p.Gradient2DSize = grad_size;
	return p;
}

} // namespace

extern "C" {

// the fields of STPRainDropSetting (STPRainDropSetting.h), in its order
typedef struct ref_raindrop {
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
} ref_raindrop;

float ref_simplex2d(const uint8_t* perm, const float* grad, uint32_t grad_size, float x, float y) {
	return STPSimplexNoise::simplex2D(permutation_of(perm, grad, grad_size), x, y);
}

float ref_fractal(const uint8_t* perm, const float* grad, uint32_t grad_size, float x, float y, float pers,
	float lacu, uint32_t oct, float scale, float off_x, float off_y, float half_x, float half_y) {
	STPSimplexNoise::STPFractalSimplexInformation desc = { };
	desc.Persistence = pers;
	desc.Lacunarity = lacu;
	desc.Octave = oct;
	desc.Scale = scale;
	desc.Offset = make_float2(off_x, off_y);
	desc.HalfDimension = make_float2(half_x, half_y);
	return STPSimplexNoise::simplex2DFractal(permutation_of(perm, grad, grad_size), x, y, desc);
}

// generateMultiBiomeHeightmap over a map_x * map_y chunk whose histogram uses biome IDs 0 and 1
// (the script's biome table holds two biomes); `table` holds the two STPBiomeProperty records.
// Returns 1 when a bin names another biome.
int ref_multibiome(float* out, const uint32_t* offsets, const void* bins, const void* table, const uint8_t* perm,
	const float* grad, uint32_t grad_size, uint32_t map_x, uint32_t map_y, float off_x, float off_y) {
	const STPSingleHistogram::STPBin* const bin = static_cast<const STPSingleHistogram::STPBin*>(bins);
	for (uint64_t b = 0u; b < offsets[static_cast<uint64_t>(map_x) * map_y]; b++) {
		if (bin[b].Item > 1u) {
			return 1;
		}
	}
	std::memcpy(BiomeTable, table, sizeof(BiomeTable));
	STPCommonGenerator::Dimension[0] = make_uint2(map_x, map_y);
	// STPCommonCompiler.cpp:235: Dimension / 2.0f
	STPCommonGenerator::HalfDimension[0] = make_float2(static_cast<float>(map_x) / 2.0f, static_cast<float>(map_y) / 2.0f);
	STPCommonGenerator::RenderedDimension[0] = make_uint2(map_x, map_y);
	STPCommonGenerator::Permutation[0] = permutation_of(perm, grad, grad_size);
	STPSingleHistogram histogram;
	histogram.Bin = bin;
	histogram.HistogramStartOffset = offsets;
	blockDim = dim3 { };
	gridDim = dim3 { map_x, map_y, 1u };
	threadIdx = uint3 { 0u, 0u, 0u };
	for (uint32_t y = 0u; y < map_y; y++) {
		for (uint32_t x = 0u; x < map_x; x++) {
			blockIdx = uint3 { x, y, 0u };
			generateMultiBiomeHeightmap(out, histogram, make_float2(off_x, off_y));
		}
	}
	return 0;
}

// STPRainDrop(start, initWaterVolume, initSpeed, (dim_x, dim_y)) then operator() for each start
// in order on the float map.  Returns 1 for a brush larger than the shared-memory stand-in.
int ref_erode(float* map, uint32_t dim_x, uint32_t dim_y, const ref_raindrop* s, const float* starts, uint32_t count,
	const int32_t* brush_index, const float* brush_weight, uint32_t brush_size) {
	if (static_cast<uint64_t>(brush_size) * (sizeof(int) + sizeof(float)) > sizeof(ErosionBrush)) {
		return 1;
	}
	STPEnvironment::STPRainDropSetting setting;
	setting.Seed = s->Seed;
	setting.RainDropCount = s->RainDropCount;
	setting.Inertia = s->Inertia;
	setting.SedimentCapacityFactor = s->SedimentCapacityFactor;
	setting.minSedimentCapacity = s->minSedimentCapacity;
	setting.initWaterVolume = s->initWaterVolume;
	setting.minWaterVolume = s->minWaterVolume;
	setting.Friction = s->Friction;
	setting.initSpeed = s->initSpeed;
	setting.ErodeSpeed = s->ErodeSpeed;
	setting.DepositSpeed = s->DepositSpeed;
	setting.EvaporateSpeed = s->EvaporateSpeed;
	setting.Gravity = s->Gravity;
	setting.ErosionBrushRadius = s->ErosionBrushRadius;
	STPErosionBrush brush;
	brush.Index = brush_index;
	brush.Weight = brush_weight;
	brush.BrushSize = brush_size;
	blockDim = dim3 { };
	threadIdx = uint3 { 0u, 0u, 0u };
	for (uint32_t d = 0u; d < count; d++) {
		blockIdx = uint3 { d, 0u, 0u };
		STPRainDrop droplet(glm::vec2(starts[2u * d], starts[2u * d + 1u]), setting.initWaterVolume, setting.initSpeed,
			glm::uvec2(dim_x, dim_y));
		droplet(map, setting, brush);
	}
	return 0;
}

} // extern "C"
