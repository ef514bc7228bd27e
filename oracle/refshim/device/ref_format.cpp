// The reference's own format kernel (formatHeightmapKERNEL,
// SuperTerrain+/Private/GPGPU/STPHeightfieldKernel.cu:110-121), whose text
// oracle/build_ref.sh extracts into the build folder as format_kernel.inc,
// run as a host loop over the pixels (test infrastructure only).
#include <SuperTerrain+/Utility/STPDeviceLaunchSetup.cuh>
#include <SuperTerrain+/World/STPWorldMapPixelFormat.hpp>
#include <glm/vec2.hpp>

#include <cstdint>

using namespace SuperTerrainPlus;
using glm::uvec2;

#include "format_kernel.inc"

extern "C" {

void ref_format(const float* in, uint16_t* out, uint32_t n) {
	blockDim = dim3 { };
	gridDim = dim3 { n, 1u, 1u };
	threadIdx = uint3 { 0u, 0u, 0u };
	for (uint32_t i = 0u; i < n; i++) {
		blockIdx = uint3 { i, 0u, 0u };
		formatHeightmapKERNEL(const_cast<float*>(in), out, uvec2(n, 1u));
	}
}

} // extern "C"
