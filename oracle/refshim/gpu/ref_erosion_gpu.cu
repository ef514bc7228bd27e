// The reference's own erosion kernel built for the GPU (test infrastructure
// only): hydraulicErosionKERNEL (SuperTerrain+/Private/GPGPU/
// STPHeightfieldKernel.cu:80-108, the droplet's spawn in the central chunk,
// then STPRainDrop) and STPRainDrop (STPRainDrop.cu, compiled unmodified in
// its own translation unit with relocatable device code, as the reference's
// build does), for sm_103a with -DNDEBUG so that the map is updated through
// float atomics as in the reference's release build.  oracle/build_ref.sh
// extracts the kernel's text into the build folder as erosion_kernel.inc.
//
// Droplets eat explicit starts: curand's Philox state is replaced by a
// stand-in that hands each droplet the caller's two uniforms in (0, 1], so
// the reference kernel and the library's kernels erode the same droplets.
// The run-to-run spread of this build (atomics from many droplets in flight
// land in a different order every run) is the erosion tolerance.
//
// Memory safety: the reference droplet is not NaN-safe.  Once a map runs
// away to infinity, a NaN position passes the border test (every comparison
// with NaN is false), converts to cell 0, and the brush's negative offsets
// wrap around in unsigned 32-bit arithmetic.  Every index the kernel forms is
// an unsigned int, so every address it can touch lies in map[0, 2^32).  The
// harness therefore runs the kernel on a copy of the map at the start of a
// 16 GiB arena (2^32 floats, allocated once per device and kept), so that no
// access can leave the allocation, and copies the result back.  The droplet
// loop ends on the water volume, which decays by (1 - EvaporateSpeed) per
// step whatever the map holds; the call refuses settings for which it would
// not (EvaporateSpeed outside (0, 1), minWaterVolume not above zero).
#include <SuperTerrain+/Utility/STPDeviceLaunchSetup.cuh>
#include <SuperTerrain+/World/Chunk/STPNearestNeighbourInformation.hpp>
#include <SuperTerrain+/GPGPU/STPRainDrop.cuh>

#include <cuda_runtime.h>

#include <cstdint>

namespace SuperTerrainPlus::STPHeightfieldKernel {
struct STPRainDropGenerator {
	float Uniform[2];
	unsigned int Next;
};
}

__device__ static float curand_uniform(SuperTerrainPlus::STPHeightfieldKernel::STPRainDropGenerator* const state) {
	return state->Uniform[state->Next++ & 1u];
}

using namespace SuperTerrainPlus;
using glm::uvec2;
using glm::vec2;

#include "erosion_kernel.inc"

__global__ static void fill_generators(STPHeightfieldKernel::STPRainDropGenerator* const rng,
	const float* const uniforms, const unsigned int count) {
	const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < count) {
		rng[i].Uniform[0] = uniforms[2u * i];
		rng[i].Uniform[1] = uniforms[2u * i + 1u];
		rng[i].Next = 0u;
	}
}

static constexpr size_t ArenaBytes = (size_t { 1 } << 32) * sizeof(float);
static constexpr int MaxDevices = 64;
static float* Arena[MaxDevices] = {};

extern "C" {

// One launch of `count` droplets on the device map `map` (merged neighbourhood of nn chunks of
// map_x x map_y), on `stream`.  `setting` is a host STPRainDropSetting; `uniforms` (device) holds
// each droplet's two draws; the brush arrays are device arrays of `brush_size` entries.  The block
// size is the occupancy-maximising one for the kernel and its dynamic shared memory, and the grid
// covers the droplets, as determineLaunchConfiguration<1u> resolves for a one-dimensional launch
// (STPHeightfieldKernel.cu:45-54).  Returns the CUDA error code of the call (0 on success); the
// call synchronises the stream.
int ref_gpu_erosion(float* const map, const uint32_t map_x, const uint32_t map_y, const uint32_t nn_x,
	const uint32_t nn_y, const void* const setting, const float* const uniforms, const uint32_t count,
	const int32_t* const brush_index, const float* const brush_weight, const uint32_t brush_size,
	void* const stream_handle) {
	const cudaStream_t stream = static_cast<cudaStream_t>(stream_handle);
	STPEnvironment::STPRainDropSetting s = *static_cast<const STPEnvironment::STPRainDropSetting*>(setting);
	s.RainDropCount = count;
	STPNearestNeighbourInformation info;
	info.MapSize = uvec2(map_x, map_y);
	info.ChunkNearestNeighbour = uvec2(nn_x, nn_y);
	info.TotalMapSize = info.MapSize * info.ChunkNearestNeighbour;
	STPErosionBrush brush;
	brush.Index = brush_index;
	brush.Weight = brush_weight;
	brush.BrushSize = brush_size;
	if (count == 0u) {
		return 0;
	}
	if (!(s.EvaporateSpeed > 0.0f && s.EvaporateSpeed < 1.0f && s.minWaterVolume > 0.0f)) {
		return static_cast<int>(cudaErrorInvalidValue);
	}
	const size_t map_bytes = sizeof(float) * map_x * nn_x * static_cast<size_t>(map_y) * nn_y;
	if (map_bytes == 0u || map_bytes > ArenaBytes) {
		return static_cast<int>(cudaErrorInvalidValue);
	}
	int device = 0;
	cudaError_t e = cudaGetDevice(&device);
	if (e != cudaSuccess || device >= MaxDevices) {
		return static_cast<int>(e != cudaSuccess ? e : cudaErrorInvalidDevice);
	}
	if (!Arena[device]) {
		e = cudaMalloc(&Arena[device], ArenaBytes);
		if (e != cudaSuccess) {
			Arena[device] = nullptr;
			return static_cast<int>(e);
		}
	}
	float* const arena = Arena[device];

	STPEnvironment::STPRainDropSetting* d_setting = nullptr;
	STPHeightfieldKernel::STPRainDropGenerator* d_rng = nullptr;
	e = cudaMalloc(&d_setting, sizeof(s));
	if (e == cudaSuccess) {
		e = cudaMemcpyAsync(arena, map, map_bytes, cudaMemcpyDeviceToDevice, stream);
	}
	if (e == cudaSuccess) {
		e = cudaMalloc(&d_rng, sizeof(STPHeightfieldKernel::STPRainDropGenerator) * count);
	}
	if (e == cudaSuccess) {
		e = cudaMemcpyAsync(d_setting, &s, sizeof(s), cudaMemcpyHostToDevice, stream);
	}
	if (e == cudaSuccess) {
		fill_generators<<<(count + 255u) / 256u, 256u, 0, stream>>>(d_rng, uniforms, count);
		e = cudaGetLastError();
	}
	const size_t smem = brush_size * (sizeof(int) + sizeof(float));
	int min_grid = 0, block = 0;
	if (e == cudaSuccess) {
		e = cudaOccupancyMaxPotentialBlockSize(&min_grid, &block, hydraulicErosionKERNEL, smem, 0);
	}
	if (e == cudaSuccess) {
		const unsigned int grid = (count + static_cast<unsigned int>(block) - 1u) / static_cast<unsigned int>(block);
		hydraulicErosionKERNEL<<<grid, block, smem, stream>>>(arena, d_setting, d_rng, info, brush);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) {
		e = cudaMemcpyAsync(map, arena, map_bytes, cudaMemcpyDeviceToDevice, stream);
	}
	const cudaError_t sync = cudaStreamSynchronize(stream);
	if (e == cudaSuccess) {
		e = sync;
	}
	cudaFree(d_rng);
	cudaFree(d_setting);
	return static_cast<int>(e);
}

// the block size the launch above takes for a brush of `brush_size` points (0 on error)
int ref_gpu_erosion_block_size(const uint32_t brush_size) {
	int min_grid = 0, block = 0;
	const size_t smem = brush_size * (sizeof(int) + sizeof(float));
	if (cudaOccupancyMaxPotentialBlockSize(&min_grid, &block, hydraulicErosionKERNEL, smem, 0) != cudaSuccess) {
		return 0;
	}
	return block;
}

} // extern "C"
