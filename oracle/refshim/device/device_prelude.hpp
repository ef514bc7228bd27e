// Host stand-ins for the CUDA C++ language extensions used by the reference's
// device sources (simplex noise, the droplet, the multi-biome generator
// script, the format kernel), so that those sources compile unchanged as
// plain host C++ for pinning the oracle.  Test infrastructure only: nothing
// here runs on a GPU.
//
// A kernel "launch" is a host loop that sets blockIdx before each call of the
// kernel body, with one thread per block; blocks run one after another, so an
// atomic add is a plain read-modify-write and a block barrier has nothing to
// wait for.
#pragma once
#include <math.h>
#include <cmath>
#include <new>
#include <utility>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __constant__
#define __shared__

struct uint1 { unsigned int x; };
struct uint2 { unsigned int x, y; };
struct uint3 { unsigned int x, y, z; };
struct float2 { float x, y; };
struct dim3 { unsigned int x = 1u, y = 1u, z = 1u; };

static inline uint1 make_uint1(unsigned int x) { return uint1 { x }; }
static inline uint2 make_uint2(unsigned int x, unsigned int y) { return uint2 { x, y }; }
static inline uint3 make_uint3(unsigned int x, unsigned int y, unsigned int z) { return uint3 { x, y, z }; }
static inline float2 make_float2(float x, float y) { return float2 { x, y }; }

// defined once by the harness (refshim/device/ref_device_api.cpp)
extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

static inline void __syncthreads() {}

static inline float atomicAdd(float* const address, const float value) {
	const float old = *address;
	*address = old + value;
	return old;
}

// the documented behaviour of __saturatef: clamp to [+0, 1], NaN gives +0
static inline float __saturatef(const float v) {
	return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f;
}

// Texture and surface objects of the splatmap script: handles to host
// descriptors that the harness (refshim/device/ref_splat_api.cpp) fills in;
// the fetches there restate the sampler the reference configures.
struct int2 { int x, y; };
typedef unsigned long long cudaTextureObject_t;
typedef unsigned long long cudaSurfaceObject_t;
enum cudaSurfaceBoundaryMode { cudaBoundaryModeZero = 0, cudaBoundaryModeClamp = 1, cudaBoundaryModeTrap = 2 };
template<class T> T tex2D(cudaTextureObject_t, float, float);
template<> float tex2D<float>(cudaTextureObject_t, float, float);
template<> unsigned short tex2D<unsigned short>(cudaTextureObject_t, float, float);
template<class T> void surf2Dwrite(T, cudaSurfaceObject_t, int, int, cudaSurfaceBoundaryMode);
template<> void surf2Dwrite<unsigned char>(unsigned char, cudaSurfaceObject_t, int, int, cudaSurfaceBoundaryMode);
// rnormf(n, a): 1 / sqrt(a[0]^2 + ... + a[n-1]^2), here the double-precision value rounded to float
float rnormf(int, const float*);
