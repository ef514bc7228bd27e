// C entry points over the reference's own compiled host classes
// (STPSingleHistogramFilter, STPPermutationGenerator), used only to pin the
// oracle restatement and to produce golden fixtures.
#include <SuperAlgorithm+Host/STPSingleHistogramFilter.h>
#include <SuperAlgorithm+Host/STPPermutationGenerator.h>
#include <SuperTerrain+/Exception/STPNumericDomainError.h>
#include <SuperTerrain+/Exception/STPInvalidEnvironment.h>

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

}
