// The reference's own erosion kernel (hydraulicErosionKERNEL,
// SuperTerrain+/Private/GPGPU/STPHeightfieldKernel.cu:80-108: the droplet's
// spawn in the central chunk, then STPRainDrop), whose text oracle/build_ref.sh
// extracts into the build folder as erosion_kernel.inc, run as a host loop
// over the droplets in index order (test infrastructure only).  The curand
// Philox state is replaced by a stand-in that hands out the caller's two
// uniforms in (0, 1] per droplet.
#include <SuperTerrain+/Utility/STPDeviceLaunchSetup.cuh>
#include <SuperTerrain+/World/Chunk/STPNearestNeighbourInformation.hpp>
#include <SuperTerrain+/GPGPU/STPRainDrop.cuh>

#include <cstdint>
#include <vector>

namespace SuperTerrainPlus::STPHeightfieldKernel {
struct STPRainDropGenerator {
	float Uniform[2];
	unsigned int Next;
};
}

static float curand_uniform(SuperTerrainPlus::STPHeightfieldKernel::STPRainDropGenerator* const state) {
	return state->Uniform[state->Next++ & 1u];
}

using namespace SuperTerrainPlus;
using glm::uvec2;
using glm::vec2;

#include "erosion_kernel.inc"

extern "C" {

// one launch of count droplets on the merged map of `nn` (map and neighbourhood sizes); `uniforms`
// holds the two draws of each droplet; the setting in the layout of STPRainDropSetting
int ref_erosion_kernel(float* map, const uint32_t* map_size, const uint32_t* nn, const void* setting,
	const float* uniforms, uint32_t count, const int32_t* brush_index, const float* brush_weight,
	uint32_t brush_size) {
	STPEnvironment::STPRainDropSetting s = *static_cast<const STPEnvironment::STPRainDropSetting*>(setting);
	s.RainDropCount = count;
	STPNearestNeighbourInformation info;
	info.MapSize = uvec2(map_size[0], map_size[1]);
	info.ChunkNearestNeighbour = uvec2(nn[0], nn[1]);
	info.TotalMapSize = info.MapSize * info.ChunkNearestNeighbour;
	STPErosionBrush brush;
	brush.Index = brush_index;
	brush.Weight = brush_weight;
	brush.BrushSize = brush_size;
	std::vector<STPHeightfieldKernel::STPRainDropGenerator> rng(count);
	for (uint32_t i = 0u; i < count; i++) {
		rng[i] = STPHeightfieldKernel::STPRainDropGenerator { { uniforms[2u * i], uniforms[2u * i + 1u] }, 0u };
	}
	blockDim = dim3 { };
	gridDim = dim3 { count, 1u, 1u };
	threadIdx = uint3 { 0u, 0u, 0u };
	for (uint32_t i = 0u; i < count; i++) {
		blockIdx = uint3 { i, 0u, 0u };
		hydraulicErosionKERNEL(map, &s, rng.data(), info, brush);
	}
	return 0;
}

} // extern "C"
