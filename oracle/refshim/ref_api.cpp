// C entry points over the reference's own compiled host classes
// (STPSingleHistogramFilter, STPPermutationGenerator, STPLayer and the demo's
// biome layer chain), used only to pin the oracle restatement and to produce
// golden fixtures.
#include <SuperAlgorithm+Host/STPSingleHistogramFilter.h>
#include <SuperAlgorithm+Host/STPPermutationGenerator.h>
#include <SuperTerrain+/Exception/STPNumericDomainError.h>
#include <SuperTerrain+/Exception/STPInvalidEnvironment.h>
#include <SuperTerrain+/World/Diversity/STPLayer.h>
#include <World/Layers/STPAllLayers.h>
#include <World/Biomes/STPBiomeRegistry.h>

#include <cstdint>
#include <cstring>
#include <memory>

using namespace SuperTerrainPlus;
using namespace SuperTerrainPlus::STPAlgorithm;

extern "C" {

typedef struct ref_bin {
	uint16_t Item;
	float Weight;
} ref_bin;

// parallel != 0 selects STPFilterBuffer::STPExecutionType::Parallel.
// Returns 0 ok, 1 STPNumericDomainError, 5 capacity too small, 9 other.
int ref_shf(const uint16_t* samplemap, uint32_t map_x, uint32_t map_y, uint32_t nn_x, uint32_t nn_y,
	uint32_t radius, int parallel, uint32_t* offsets, ref_bin* bins, uint64_t capacity, uint64_t* nbins) {
	try {
		static STPSingleHistogramFilter filter;
		STPSingleHistogramFilter::STPFilterBuffer buffer(parallel
			? STPSingleHistogramFilter::STPFilterBuffer::STPExecutionType::Parallel
			: STPSingleHistogramFilter::STPFilterBuffer::STPExecutionType::Serial);
		STPNearestNeighbourInformation info;
		info.MapSize = glm::uvec2(map_x, map_y);
		info.ChunkNearestNeighbour = glm::uvec2(nn_x, nn_y);
		info.TotalMapSize = info.MapSize * info.ChunkNearestNeighbour;
		const STPSingleHistogram h = filter(samplemap, info, buffer, radius);
		const auto [bin_count, offset_count] = buffer.size();
		*nbins = bin_count;
		std::memcpy(offsets, h.HistogramStartOffset, sizeof(uint32_t) * offset_count);
		if (bin_count > capacity) {
			return 5;
		}
		for (size_t i = 0; i < bin_count; i++) {
			bins[i].Item = h.Bin[i].Item;
			bins[i].Weight = h.Bin[i].Weight;
		}
		return 0;
	} catch (const STPException::STPNumericDomainError&) {
		return 1;
	} catch (...) {
		return 9;
	}
}

// Returns 0 ok, 1 STPInvalidEnvironment, 9 other. grad receives 2*distribution floats.
int ref_permutation(uint64_t seed, uint32_t distribution, double offset, uint8_t* perm, float* grad) {
	try {
		STPEnvironment::STPSimplexNoiseSetting setting;
		setting.Seed = seed;
		setting.Distribution = distribution;
		setting.Offset = offset;
		const auto table = STPPermutationGenerator::generate(setting);
		std::memcpy(perm, table.Permutation.Permutation, 512);
		std::memcpy(grad, table.Permutation.Gradient2D, sizeof(float) * 2u * distribution);
		return 0;
	} catch (const STPException::STPInvalidEnvironment&) {
		return 1;
	} catch (...) {
		return 9;
	}
}

// The demo's biome layer chain (STPDemo::STPLayerChainBuilder, a
// STPBiomeFactory) run through STPBiomeFactory::operator()(biomemap, offset).
// Biome IDs are set the way the demo's parameter loader sets them
// (SuperDemo+/Helpers/STPTerrainParaLoader.cpp:272-294); biomes it never
// loads keep ID 0.  Returns 0 ok, 9 error.
int ref_layer_biomemap(uint64_t seed, uint16_t ocean, uint16_t plains, uint16_t desert, uint16_t forest,
	uint32_t width, uint32_t height, int32_t offset_x, int32_t offset_z, uint16_t* out) {
	try {
		namespace BR = STPDemo::STPBiomeRegistry;
		BR::Ocean.ID = ocean;
		BR::Plains.ID = plains;
		BR::Desert.ID = desert;
		BR::Forest.ID = forest;
		STPDemo::STPLayerChainBuilder builder(glm::uvec2(width, height), seed);
		builder(out, glm::ivec2(offset_x, offset_z));
		return 0;
	} catch (...) {
		return 9;
	}
}

// One STPLayer::mixSeed step and STPLayer::seedLayer, exposed through a
// probe layer, for the local-RNG unit tests.
namespace {
class ProbeLayer : public STPDiversity::STPLayer {
	STPSample_t sample(int, int, int) override {
		return 0u;
	}

public:
	ProbeLayer(uint64_t global, uint64_t salt) : STPLayer(0u, global, salt) {}
	static uint64_t mix(uint64_t s, int64_t fac) {
		return STPLayer::mixSeed(s, fac);
	}
	uint64_t local(int x, int z) const {
		return this->seedLocal(x, z);
	}
};
}

uint64_t ref_mix_seed(uint64_t s, int64_t fac) {
	return ProbeLayer::mix(s, fac);
}

uint64_t ref_layer_seed(uint64_t global, uint64_t salt) {
	return ProbeLayer(global, salt).LayerSeed;
}

uint64_t ref_local_seed(uint64_t global, uint64_t salt, int32_t x, int32_t z) {
	return ProbeLayer(global, salt).local(x, z);
}

}
