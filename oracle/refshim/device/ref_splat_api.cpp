// C entry point over the demo's splatmap script
// (SuperDemo+/Script/STPSplatmapGenerator.cu) and the reference's rule lookups
// (SuperAlgorithm+/Device/Private/STPTextureSplatRuleWrapper.cu), compiled as
// host C++ and run one pixel at a time (test infrastructure only).
//
// What is not the reference's own code: the texture fetches and rnormf.  The
// sampler follows STPWorldPipeline.cpp:682-696 (unnormalised coordinates,
// clamped addressing; the biomemap point-filtered and read as its element
// type, the heightmap linearly filtered and read as a normalised float).
// Linear filtering here is the texture unit's documented form: texels
// floor(u - 0.5) and the next one blended with weight frac(u - 0.5) held as
// a fixed-point fraction of 8 bits; the weighted sum of the uint16 texels is
// exact, rounded to the nearest integer (halves up) and divided by 65535.
#include <SuperAlgorithm+Device/STPSimplexNoise.cuh>
#include <SuperTerrain+/World/Diversity/Texture/STPTextureInformation.hpp>

#include <algorithm>
#include <cmath>
#include <cstdint>

using namespace SuperTerrainPlus;
using namespace SuperTerrainPlus::STPAlgorithm;
namespace STPTI = SuperTerrainPlus::STPDiversity::STPTextureInformation;

namespace STPCommonGenerator {
extern uint2 Dimension[1];
extern float2 HalfDimension[1];
extern uint2 RenderedDimension[1];
extern STPPermutation Permutation[1];
}
extern STPTI::STPSplatRuleDatabase SplatDatabase[1];
void generateTextureSplatmap(const cudaTextureObject_t, const cudaTextureObject_t, const cudaSurfaceObject_t,
	const STPTI::STPSplatGeneratorInformation);

namespace {

struct HostTexture {
	const uint16_t* data;
	uint32_t pitch, width, height;
};

struct HostSurface {
	uint8_t* data;
	uint32_t pitch, width, height;
	bool trapped;
};

int64_t texel(const HostTexture& t, int x, int y) {
	x = std::min(std::max(x, 0), static_cast<int>(t.width) - 1);
	y = std::min(std::max(y, 0), static_cast<int>(t.height) - 1);
	return t.data[static_cast<size_t>(y) * t.pitch + x];
}

} // namespace

// the heightmap: linear filter, normalised float
template<> float tex2D<float>(const cudaTextureObject_t obj, const float u, const float v) {
	const HostTexture& t = *reinterpret_cast<const HostTexture*>(obj);
	const float xb = u - 0.5f, yb = v - 0.5f;
	const float x0 = std::floor(xb), y0 = std::floor(yb);
	const int64_t a = std::lround((xb - x0) * 256.0f), b = std::lround((yb - y0) * 256.0f);
	const int i = static_cast<int>(x0), j = static_cast<int>(y0);
	const int64_t sum = (256 - a) * (256 - b) * texel(t, i, j) + a * (256 - b) * texel(t, i + 1, j)
		+ (256 - a) * b * texel(t, i, j + 1) + a * b * texel(t, i + 1, j + 1);
	return static_cast<float>((sum + 32768) >> 16) / 65535.0f;
}

// the biomemap: point filter, element type
template<> unsigned short tex2D<unsigned short>(const cudaTextureObject_t obj, const float u, const float v) {
	const HostTexture& t = *reinterpret_cast<const HostTexture*>(obj);
	return static_cast<unsigned short>(texel(t, static_cast<int>(std::floor(u)), static_cast<int>(std::floor(v))));
}

template<> void surf2Dwrite<unsigned char>(const unsigned char value, const cudaSurfaceObject_t obj, const int x_bytes,
	const int y, cudaSurfaceBoundaryMode) {
	HostSurface& s = *reinterpret_cast<HostSurface*>(obj);
	if (x_bytes < 0 || y < 0 || static_cast<uint32_t>(x_bytes) >= s.width || static_cast<uint32_t>(y) >= s.height) {
		s.trapped = true;  // a trap on the device
		return;
	}
	s.data[static_cast<size_t>(y) * s.pitch + x_bytes] = value;
}

float rnormf(const int n, const float* const a) {
	double sum = 0.0;
	for (int i = 0; i < n; i++) {
		sum += static_cast<double>(a[i]) * a[i];
	}
	return static_cast<float>(1.0 / std::sqrt(sum));
}

extern "C" {

// generateTextureSplatmap over `count` requested chunks (local chunk x, y, map offset x, y) of a
// width x height rendering buffer of map_x x map_y chunks; the rule tables in the layout of
// STPTextureInformation.hpp.  Returns 1 when a write left the surface (a trap on the device).
int ref_splatmap(const uint16_t* biomemap, const uint16_t* heightmap, uint32_t map_pitch, uint32_t width,
	uint32_t height, const void* chunks, uint32_t count, uint32_t map_x, uint32_t map_y, const uint16_t* dict,
	uint32_t dict_count, const void* reg, const void* alt, const void* gra, const uint8_t* perm, const float* grad,
	uint32_t grad_size, uint8_t* out, uint32_t out_pitch) {
	HostTexture biome { biomemap, map_pitch, width, height }, hm { heightmap, map_pitch, width, height };
	HostSurface surf { out, out_pitch, width, height, false };
	STPCommonGenerator::Dimension[0] = make_uint2(map_x, map_y);
	STPCommonGenerator::HalfDimension[0] = make_float2(static_cast<float>(map_x) / 2.0f, static_cast<float>(map_y) / 2.0f);
	STPCommonGenerator::RenderedDimension[0] = make_uint2(width, height);
	STPPermutation& p = STPCommonGenerator::Permutation[0];
	p.Permutation = const_cast<unsigned char*>(perm);
	p.Gradient2D = const_cast<float*>(grad);
	p.Gradient2DSize = grad_size;
	STPTI::STPSplatRuleDatabase& db = SplatDatabase[0];
	db.SplatRegistryDictionary = dict;
	db.DictionaryEntryCount = dict_count;
	db.SplatRegistry = static_cast<const STPTI::STPSplatRegistry*>(reg);
	db.AltitudeRegistry = static_cast<const STPTI::STPAltitudeNode*>(alt);
	db.GradientRegistry = static_cast<const STPTI::STPGradientNode*>(gra);
	STPTI::STPSplatGeneratorInformation info;
	info.RequestingLocalInfo = static_cast<const STPTI::STPSplatGeneratorInformation::STPLocalChunkInformation*>(chunks);
	info.LocalCount = count;
	blockDim = dim3 { };
	gridDim = dim3 { map_x, map_y, count };
	threadIdx = uint3 { 0u, 0u, 0u };
	for (uint32_t z = 0u; z < count; z++) {
		for (uint32_t y = 0u; y < map_y; y++) {
			for (uint32_t x = 0u; x < map_x; x++) {
				blockIdx = uint3 { x, y, z };
				generateTextureSplatmap(reinterpret_cast<cudaTextureObject_t>(&biome),
					reinterpret_cast<cudaTextureObject_t>(&hm), reinterpret_cast<cudaSurfaceObject_t>(&surf), info);
			}
		}
	}
	return surf.trapped ? 1 : 0;
}

} // extern "C"
