// 2-D simplex noise and its fractal sum on sm_103a, shared by the
// multi-biome heightfield and the splatmap kernels
// (SuperTerrain+/SuperAlgorithm+/Device/Private/STPSimplexNoise.cu:5-110).
#pragma once

#include "internal.hpp"

namespace stpgb {
namespace simplex {

// STPSimplexNoise.cu:5-7
constexpr float kF2 = 0.3660254038f;
constexpr float kG2 = 0.2113248654f;
constexpr float kH2 = -1.0f + 2.0f * kG2;

// STPSimplexNoise.cu:14-16: not floorf (an exact negative integer maps one lower)
__device__ __forceinline__ int floori(const float x) {
	return x > 0.0f ? static_cast<int>(x) : static_cast<int>(x - 1.0f);
}

__device__ __forceinline__ float corner(const float dx, const float dy, const float2 g) {
	float w = 0.5f - dx * dx - dy * dy;
	if (w <= 0.0f) {
		return 0.0f;
	}
	w *= w;
	return w * w * (g.x * dx + g.y * dy);
}

// STPSimplexNoise.cu:18-82.  The skew and unskew (x + (x+y)*F2 and
// i - (i+j)*G2) are written with separately rounded operations: fused into
// one multiply-add they shift the cell origin by up to an ulp of the sample
// coordinate, which at world offsets of 10^4-10^5 pixels is a visible error.
__device__ __forceinline__ float simplex2d(const uint8_t* __restrict__ perm, const float2* __restrict__ gtab,
	const float x, const float y) {
	const float s = __fmul_rn(__fadd_rn(x, y), kF2);
	const int i = floori(__fadd_rn(x, s)), j = floori(__fadd_rn(y, s));
	const float t = __fmul_rn(static_cast<float>(i + j), kG2);
	const float dx0 = __fsub_rn(x, __fsub_rn(static_cast<float>(i), t));
	const float dy0 = __fsub_rn(y, __fsub_rn(static_cast<float>(j), t));
	const unsigned int i1 = (dx0 > dy0) ? 1u : 0u, j1 = 1u - i1;
	const float dx1 = dx0 - static_cast<float>(i1) + kG2, dy1 = dy0 - static_cast<float>(j1) + kG2;
	const float dx2 = dx0 + kH2, dy2 = dy0 + kH2;
	const unsigned int ii = static_cast<unsigned int>(i) & 255u, jj = static_cast<unsigned int>(j) & 255u;
	const float2 g0 = gtab[ii + perm[jj]];
	const float2 g1 = gtab[ii + i1 + perm[jj + j1]];
	const float2 g2 = gtab[ii + 1u + perm[jj + 1u]];
	return 70.0f * (corner(dx0, dy0, g0) + corner(dx1, dy1, g1) + corner(dx2, dy2, g2));
}

// Shared-memory tables of a block: the permutation and, for every
// permutation slot, its gradient (perm[k] % Gradient2DSize) already looked up.
__device__ __forceinline__ void load_tables(const stpgb_permutation& perm, uint8_t* sperm, float2* gtab) {
	for (uint32_t k = threadIdx.x; k < 512u; k += blockDim.x) {
		const uint32_t p = perm.Permutation[k];
		sperm[k] = static_cast<uint8_t>(p);
		const uint32_t g = p % perm.Gradient2DSize;
		gtab[k] = make_float2(perm.Gradient2D[2u * g], perm.Gradient2D[2u * g + 1u]);
	}
}

// STPSimplexNoise.cu:84-110 at sample (ux, uy) = ((x - half) + offset) / Scale:
// the saturated, normalised fractal sum in [0, 1].
__device__ __forceinline__ float fractal(const uint8_t* __restrict__ perm, const float2* __restrict__ gtab,
	const float ux, const float uy, const uint32_t octave, const float persistence, const float lacunarity) {
	float sum = 0.0f, amplitude = 1.0f, frequency = 1.0f, range = 0.0f;
	for (uint32_t o = 0u; o < octave; o++) {
		sum += simplex2d(perm, gtab, ux * frequency, uy * frequency) * amplitude;
		range += amplitude;
		amplitude *= persistence;
		frequency *= lacunarity;
	}
	return __saturatef((sum + range) / (2.0f * range));
}

} // namespace simplex
} // namespace stpgb
