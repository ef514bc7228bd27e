// Measurement kernels for the roofline denominators of the kernels that are
// not bound by HBM copy bandwidth: random float reductions into an
// L2-resident map (scalar and 16-byte vector, the operations of the erosion
// kernels' deposits and brush updates; 16-byte returning atomics, the
// brush's exact take), random 16-byte loads from it (their
// corner gathers), the latency of one dependent L2 load (the chain each
// droplet step waits on), and the FP32 fused multiply-add rate (the noise
// kernel's pipe).  No counterpart in the reference.  Plain kernels that touch
// only the buffers they are given; they change no clock or device setting.
#include "internal.hpp"

namespace stpgb {

namespace {

constexpr uint32_t kBlock = 256u;

// one step of a 32-bit linear congruential generator (Numerical Recipes'
// constants): two integer operations per address
__device__ __forceinline__ uint32_t lcg(const uint32_t h) {
	return h * 1664525u + 1013904223u;
}

__global__ void __launch_bounds__(kBlock) red_scalar_kernel(float* __restrict__ map, const uint32_t shift,
	const uint32_t iters) {
	uint32_t h = (blockIdx.x * kBlock + threadIdx.x) * 2654435761u;
	for (uint32_t i = 0u; i < iters; i++) {
		h = lcg(h);
		asm volatile("red.global.add.f32 [%0], %1;" ::"l"(map + (h >> shift)), "f"(1.0f) : "memory");
	}
}

__global__ void __launch_bounds__(kBlock) red_v4_kernel(float* __restrict__ map, const uint32_t shift,
	const uint32_t iters) {
	uint32_t h = (blockIdx.x * kBlock + threadIdx.x) * 2654435761u;
	for (uint32_t i = 0u; i < iters; i++) {
		h = lcg(h);
		float* const p = map + 4u * (h >> shift);
		asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(1.0f), "f"(1.0f), "f"(1.0f),
			"f"(1.0f) : "memory");
	}
}

__global__ void __launch_bounds__(kBlock) load_v4_kernel(const float4* __restrict__ map, const uint32_t shift,
	const uint32_t iters, float* __restrict__ sink) {
	uint32_t h = (blockIdx.x * kBlock + threadIdx.x) * 2654435761u;
	float acc = 0.0f;
	for (uint32_t i = 0u; i < iters; i++) {
		h = lcg(h);
		const float4 v = __ldcg(map + (h >> shift));
		acc += v.x + v.y + v.z + v.w;
	}
	if (acc == 12345.678f) {
		sink[0] = acc; // never taken for the zero map; keeps the loads
	}
}

// returning 16-byte atomics, each result summed before the next is issued
// (one in flight per thread, as a brush lane waits on its block's values)
__global__ void __launch_bounds__(kBlock) atom_v4_kernel(float* __restrict__ map, const uint32_t shift,
	const uint32_t iters, float* __restrict__ sink) {
	uint32_t h = (blockIdx.x * kBlock + threadIdx.x) * 2654435761u;
	float acc = 0.0f;
	for (uint32_t i = 0u; i < iters; i++) {
		h = lcg(h);
		float* const p = map + 4u * (h >> shift);
		float a, b, c, d;
		asm volatile("atom.global.add.v4.f32 {%0, %1, %2, %3}, [%4], {%5, %6, %7, %8};"
					 : "=f"(a), "=f"(b), "=f"(c), "=f"(d)
					 : "l"(p), "f"(1.0f), "f"(1.0f), "f"(1.0f), "f"(1.0f)
					 : "memory");
		acc += a + b + c + d;
	}
	if (acc == -12345.678f) {
		sink[0] = acc; // never taken: the map only grows from zero; keeps the results used
	}
}

// one thread follows `next` from 0 (an entry past the table restarts at 0);
// reports the clock64 ticks of all `steps` loads
__global__ void chase_kernel(const uint32_t* __restrict__ next, const uint32_t n, const uint32_t steps,
	uint64_t* __restrict__ out) {
	uint32_t j = 0u;
	const long long t0 = clock64();
	for (uint32_t i = 0u; i < steps; i++) {
		j = __ldcg(next + j);
		j = j < n ? j : 0u;
	}
	const long long t1 = clock64();
	out[0] = static_cast<uint64_t>(t1 - t0);
	out[1] = j;
}

// eight independent chains of fused multiply-adds per thread
__global__ void __launch_bounds__(kBlock) fma_kernel(float* __restrict__ out, const uint32_t iters, const float b,
	const float c) {
	float a[8];
#pragma unroll
	for (int k = 0; k < 8; k++) {
		a[k] = static_cast<float>(threadIdx.x + k);
	}
	for (uint32_t i = 0u; i < iters; i++) {
#pragma unroll
		for (int k = 0; k < 8; k++) {
			a[k] = __fmaf_rn(a[k], b, c);
		}
	}
	float s = 0.0f;
#pragma unroll
	for (int k = 0; k < 8; k++) {
		s += a[k];
	}
	if (s == 12345.678f) {
		out[0] = s;
	}
}

uint32_t log2_exact(const uint64_t v) {
	uint32_t l = 0u;
	while ((uint64_t { 1 } << l) < v) {
		l++;
	}
	return (uint64_t { 1 } << l) == v ? l : 0xFFFFFFFFu;
}

} // namespace

} // namespace stpgb

using namespace stpgb;

extern "C" int stpgb_roofline_launch(const uint32_t kind, void* buffer, const uint64_t elements, const uint32_t blocks,
	const uint32_t iters, void* sink, void* stream) {
	const cudaStream_t s = as_stream(stream);
	if (!buffer || blocks == 0u || iters == 0u) {
		return inval("stpgb_roofline_launch: null buffer or empty launch");
	}
	const uint32_t l = log2_exact(elements);
	switch (kind) {
	case STPGB_ROOFLINE_RED_F32:
		if (l == 0xFFFFFFFFu || l > 32u || l == 0u) {
			return inval("stpgb_roofline_launch: the map needs a power-of-two float count up to 2^32");
		}
		red_scalar_kernel<<<blocks, kBlock, 0, s>>>(static_cast<float*>(buffer), 32u - l, iters);
		break;
	case STPGB_ROOFLINE_RED_V4_F32:
	case STPGB_ROOFLINE_LOAD_V4_F32:
	case STPGB_ROOFLINE_ATOM_V4_F32:
		if (l == 0xFFFFFFFFu || l < 3u || l > 34u) {
			return inval("stpgb_roofline_launch: the map needs a power-of-two float count from 8 to 2^34");
		}
		if (kind == STPGB_ROOFLINE_RED_V4_F32) {
			red_v4_kernel<<<blocks, kBlock, 0, s>>>(static_cast<float*>(buffer), 32u - (l - 2u), iters);
		} else if (kind == STPGB_ROOFLINE_ATOM_V4_F32) {
			if (!sink) {
				return inval("stpgb_roofline_launch: the atomic kernel needs a sink");
			}
			atom_v4_kernel<<<blocks, kBlock, 0, s>>>(static_cast<float*>(buffer), 32u - (l - 2u), iters,
				static_cast<float*>(sink));
		} else {
			if (!sink) {
				return inval("stpgb_roofline_launch: the load kernel needs a sink");
			}
			load_v4_kernel<<<blocks, kBlock, 0, s>>>(static_cast<const float4*>(buffer), 32u - (l - 2u), iters,
				static_cast<float*>(sink));
		}
		break;
	case STPGB_ROOFLINE_CHASE:
		if (!sink || elements == 0u || elements > 0xFFFFFFFFull) {
			return inval("stpgb_roofline_launch: the chase needs a sink and at most 2^32 entries");
		}
		chase_kernel<<<1, 1, 0, s>>>(static_cast<const uint32_t*>(buffer), static_cast<uint32_t>(elements), iters,
			static_cast<uint64_t*>(sink));
		break;
	case STPGB_ROOFLINE_FMA_F32:
		fma_kernel<<<blocks, kBlock, 0, s>>>(static_cast<float*>(buffer), iters, 0.999f, 1e-3f);
		break;
	default:
		return inval("stpgb_roofline_launch: unknown kind");
	}
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}
