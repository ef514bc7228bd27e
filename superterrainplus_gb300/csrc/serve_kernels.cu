// Batched helper kernels of the serving engine: Voronoi biome regions,
// neighbourhood gathers (nine resident chunk heightfields into one merged
// free-slip map) and Philox droplet starts, each over a job array.
#include "serve.cuh"

namespace stpgb {

namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
	z += 0x9E3779B97F4A7C15ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

__device__ __forceinline__ int64_t floordiv(const int64_t a, const int64_t b) {
	const int64_t q = a / b;
	return (a % b != 0 && ((a < 0) != (b < 0))) ? q - 1 : q;
}

// the same map as stpgb_voronoi_biomemap (synth.cu), per job
__global__ void voronoi_jobs_kernel(const VoronoiJob* __restrict__ jobs, const uint64_t seed, const uint32_t biomes) {
	const VoronoiJob& J = jobs[blockIdx.z];
	const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
	if (x >= J.width || y >= J.height) {
		return;
	}
	const int64_t gx = J.origin_x + x, gy = J.origin_y + y, cell = J.cell;
	const int64_t cx = floordiv(gx, cell), cy = floordiv(gy, cell);
	int64_t best = INT64_MAX;
	uint64_t best_h = 0u;
	for (int dy = -1; dy <= 1; dy++) {
		for (int dx = -1; dx <= 1; dx++) {
			const int64_t nx = cx + dx, ny = cy + dy;
			const uint64_t h = splitmix64(seed ^ splitmix64(static_cast<uint64_t>(nx) * 0x9E3779B97F4A7C15ull
				^ static_cast<uint64_t>(ny) * 0xC2B2AE3D27D4EB4Full));
			const int64_t px = nx * cell + static_cast<int64_t>(h % static_cast<uint64_t>(cell)),
				py = ny * cell + static_cast<int64_t>((h >> 32) % static_cast<uint64_t>(cell));
			const int64_t d = (px - gx) * (px - gx) + (py - gy) * (py - gy);
			if (d < best) {
				best = d;
				best_h = h;
			}
		}
	}
	J.out[static_cast<uint64_t>(y) * J.width + x] = static_cast<uint16_t>(splitmix64(best_h) % biomes);
}

// nine S x S chunk heightfields -> one (3S)^2 merged map, four floats per thread
__global__ void gather_jobs_kernel(const GatherJob* __restrict__ jobs) {
	const GatherJob& J = jobs[blockIdx.y];
	const uint32_t S = J.S, W = 3u * S, quads = W / 4u;
	const uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
	if (t >= static_cast<uint64_t>(quads) * W) {
		return;
	}
	const uint32_t y = static_cast<uint32_t>(t / quads), x = static_cast<uint32_t>(t % quads) * 4u;
	const uint32_t c = (y / S) * 3u + x / S;
	const float4 v = __ldcs(reinterpret_cast<const float4*>(J.chunk[c] + static_cast<uint64_t>(y % S) * S + x % S));
	*reinterpret_cast<float4*>(J.merged + static_cast<uint64_t>(y) * W + x) = v;
}

// one (3S)^2 merged map -> its nine S x S chunk heightfields, the inverse of
// gather_jobs_kernel (the in-place mode's write-back of an eroded neighbourhood)
__global__ void scatter_jobs_kernel(const GatherJob* __restrict__ jobs) {
	const GatherJob& J = jobs[blockIdx.y];
	const uint32_t S = J.S, W = 3u * S, quads = W / 4u;
	const uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
	if (t >= static_cast<uint64_t>(quads) * W) {
		return;
	}
	const uint32_t y = static_cast<uint32_t>(t / quads), x = static_cast<uint32_t>(t % quads) * 4u;
	const uint32_t c = (y / S) * 3u + x / S;
	const float4 v = *reinterpret_cast<const float4*>(J.merged + static_cast<uint64_t>(y) * W + x);
	*reinterpret_cast<float4*>(const_cast<float*>(J.chunk[c]) + static_cast<uint64_t>(y % S) * S + x % S) = v;
}

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
	for (int round = 0; round < 10; round++) {
		const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
		const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
		const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
		c[0] = n0;
		c[1] = lo1;
		c[2] = n2;
		c[3] = lo0;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
}

// the same starts as stpgb_droplet_starts (synth.cu), per job, central chunk of a 3x3 neighbourhood
__global__ void starts_jobs_kernel(const StartsJob* __restrict__ jobs, const uint64_t seed) {
	const StartsJob& J = jobs[blockIdx.y];
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= J.count) {
		return;
	}
	const uint64_t ctr = J.counter_base + i;
	uint32_t c[4] = { static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32), 0u, 0u };
	philox4x32_10(c, static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
	const float ux = static_cast<float>((c[0] >> 8) + 1u) * (1.0f / 16777216.0f);
	const float uy = static_cast<float>((c[1] >> 8) + 1u) * (1.0f / 16777216.0f);
	const float base = static_cast<float>(J.S - 1u), range = static_cast<float>(J.S);
	reinterpret_cast<float2*>(J.out)[i] = make_float2(__fadd_rn(__fmul_rn(ux, base), range), __fadd_rn(__fmul_rn(uy, base), range));
}

} // namespace

int voronoi_jobs_launch(const VoronoiJob* jobs, uint32_t njobs, uint32_t max_w, uint32_t max_h, uint64_t seed,
	uint32_t biomes, cudaStream_t s) {
	if (njobs == 0u) {
		return STPGB_OK;
	}
	const dim3 block(32u, 8u), grid((max_w + 31u) / 32u, (max_h + 7u) / 8u, njobs);
	voronoi_jobs_kernel<<<grid, block, 0, s>>>(jobs, seed, biomes);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int gather_jobs_launch(const GatherJob* jobs, uint32_t njobs, uint32_t max_S, cudaStream_t s) {
	if (njobs == 0u) {
		return STPGB_OK;
	}
	const uint64_t threads = static_cast<uint64_t>(3u * max_S / 4u) * (3u * max_S);
	gather_jobs_kernel<<<dim3(static_cast<uint32_t>((threads + 255u) / 256u), njobs), 256u, 0, s>>>(jobs);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int scatter_jobs_launch(const GatherJob* jobs, uint32_t njobs, uint32_t max_S, cudaStream_t s) {
	if (njobs == 0u) {
		return STPGB_OK;
	}
	const uint64_t threads = static_cast<uint64_t>(3u * max_S / 4u) * (3u * max_S);
	scatter_jobs_kernel<<<dim3(static_cast<uint32_t>((threads + 255u) / 256u), njobs), 256u, 0, s>>>(jobs);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int starts_jobs_launch(const StartsJob* jobs, uint32_t njobs, uint32_t max_count, uint64_t seed, cudaStream_t s) {
	if (njobs == 0u || max_count == 0u) {
		return STPGB_OK;
	}
	starts_jobs_kernel<<<dim3((max_count + 255u) / 256u, njobs), 256u, 0, s>>>(jobs, seed);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

} // namespace stpgb
