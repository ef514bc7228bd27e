// Free-slip particle hydraulic erosion and height formatting on sm_103a.
//
// A group of 1-32 lanes per droplet, following STPRainDrop::operator()
// (SuperTerrain+/SuperTerrain+/Private/GPGPU/STPRainDrop.cu:53-165) step for
// step: bilinear height/gradient at the current cell (:23-51), inertia
// steering, unit move, death within BrushRadius of the merged-map border,
// deposit over the 4 corners of the OLD cell or erosion over the brush
// centred on the OLD cell, speed and volume update.  Like the reference the
// map is shared by all droplets and updated with float atomics (release
// build, :133-137,154); reads go through L2 (ld.global.cg) so a droplet sees
// the other droplets' completed updates.  Two additions:
//  * the sediment a droplet still carries when it dies (evaporated or left
//    the map) is summed into a double, which closes the mass balance
//    sum(h_before) - sum(h_after) = residual;
//  * the loop has a hard step cap (the reference loops while
//    Volume >= minWaterVolume); reaching it sets STATUS_TIMEOUT.
#include "erosion.cuh"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace stpgb {

namespace {

constexpr uint32_t kErodeBlock = 128u;

// Every brush update subtracts min(max(cell, 0), w) where the reference
// subtracts min(cell, w) (STPRainDrop.cu:149).  The two agree on every
// non-negative cell, and without concurrent droplets no cell goes negative:
// the maps start non-negative (normalised noise), deposits add, and an
// erosion removes at most what the cell holds.  Concurrent droplets that read
// the same cell before either update lands can take it below zero; the
// reference's min() then returns the negative height, so each droplet that
// read it adds its magnitude back, and with three or more such readers the
// magnitude grows with every such exchange: measured on 64^2 chunks of multi-biome
// terrain, 2.7 to 3 droplets per pixel with brush radius 3 drove heights to
// -10^5 and beyond in some runs.  With the clamp a negative cell is left to
// the deposits, and no feedback remains.

struct HG {
	float h, gx, gy;
};

// The four corner heights of a cell, identical in every lane of the group:
// the map changes under concurrent droplets, so the lanes must not read it
// separately.  With G >= 4 lane c of the group reads corner c, with G == 2
// each lane reads one row, and the values are broadcast over the group.
template<uint32_t G>
__device__ __forceinline__ float4 cell_corners(const float* __restrict__ base, const uint64_t pitch, const uint32_t g,
	const uint32_t gmask, const uint32_t glead) {
	if constexpr (G == 1u) {
		return make_float4(__ldcg(base), __ldcg(base + 1), __ldcg(base + pitch), __ldcg(base + pitch + 1));
	} else if constexpr (G == 2u) {
		const float* const row = base + (g ? pitch : 0u);
		const float a = __ldcg(row), b = __ldcg(row + 1);
		return make_float4(__shfl_sync(gmask, a, glead), __shfl_sync(gmask, b, glead), __shfl_sync(gmask, a, glead + 1),
			__shfl_sync(gmask, b, glead + 1));
	} else {
		const uint32_t c = g & 3u;
		const float v = __ldcg(base + ((c & 2u) ? pitch : 0u) + (c & 1u));
		return make_float4(__shfl_sync(gmask, v, glead), __shfl_sync(gmask, v, glead + 1),
			__shfl_sync(gmask, v, glead + 2), __shfl_sync(gmask, v, glead + 3));
	}
}

// STPRainDrop.cu:23-51
template<uint32_t G>
__device__ __forceinline__ HG height_gradient(const float* __restrict__ map, const uint64_t pitch, const float px,
	const float py, const uint32_t g, const uint32_t gmask, const uint32_t glead) {
	const uint32_t rx = static_cast<uint32_t>(px), ry = static_cast<uint32_t>(py);
	const float cx = px - static_cast<float>(rx), cy = py - static_cast<float>(ry);
	const float4 q = cell_corners<G>(map + static_cast<uint64_t>(ry) * pitch + rx, pitch, g, gmask, glead);
	const float h00 = q.x, h10 = q.y, h01 = q.z, h11 = q.w;
	HG r;
	r.h = h00 * (1.0f - cx) * (1.0f - cy) + h10 * cx * (1.0f - cy) + h01 * (1.0f - cx) * cy + h11 * cx * cy;
	// glm::mix(a, b, t) = a * (1 - t) + b * t
	r.gx = (h10 - h00) * (1.0f - cy) + (h11 - h01) * cy;
	r.gy = (h01 - h00) * (1.0f - cx) + (h11 - h10) * cx;
	return r;
}

// Brush points a lane has in flight at once (compare-and-swap mode), and
// the bound on failed swaps per batch before the plain subtraction.
constexpr uint32_t kBrushBatch = 8u;
constexpr uint32_t kCasRetries = 16u;

// G lanes (1, 2, 4, 8, 16 or 32) carry one droplet.  Every lane of a group
// holds the same droplet state and takes the same branches: the corner
// heights are read once and broadcast, so no lane sees a different racy
// value.  The brush points of an erosion step and the four deposit corners
// are split across the lanes, so one droplet's scattered updates leave the
// warp as a few coalesced requests instead of one request per point, and a
// step costs ceil(points / G) read-update round trips instead of one per
// point.  The eroded amounts are summed over the group with a butterfly,
// which gives every lane the same total.
template<uint32_t G, bool ExactClamp>
__global__ void __launch_bounds__(kErodeBlock) erosion_kernel(const ErosionJob* __restrict__ jobs,
	const ErosionJob single) {
	const ErosionJob& J = jobs ? jobs[blockIdx.y] : single;
	extern __shared__ unsigned char esm[];
	int32_t* const bidx = reinterpret_cast<int32_t*>(esm);
	float* const bw = reinterpret_cast<float*>(esm) + J.brush_size;
	for (uint32_t k = threadIdx.x; k < J.brush_size; k += kErodeBlock) {
		bidx[k] = J.brush_index[k];
		bw[k] = J.brush_weight[k];
	}
	__syncthreads();

	const RainParams& P = J.p;
	const uint32_t g = threadIdx.x % G;
	const uint32_t d = (blockIdx.x * kErodeBlock + threadIdx.x) / G;
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t gmask = G == 32u ? 0xFFFFFFFFu : (((1u << G) - 1u) << (lane & ~(G - 1u)));
	const uint32_t glead = lane & ~(G - 1u);
	double residual = 0.0;
	bool capped = false;
	uint32_t steps_done = 0u, erode_steps = 0u;
	if (d < J.count) {
		float* const map = J.map;
		const uint64_t pitch = J.pitch;
		const uint32_t bsize = J.brush_size;
		float px = J.starts[2u * d], py = J.starts[2u * d + 1u];
		float dirx = 0.0f, diry = 0.0f;
		float speed = P.initSpeed, vol = P.initWaterVolume, sed = 0.0f;
		const float lo = static_cast<float>(P.BrushRadius);
		const float hi_x = 1.0f * J.dim_x - P.BrushRadius, hi_y = 1.0f * J.dim_y - P.BrushRadius;
		uint32_t step = 0u;
		// A start whose 2x2 bilinear footprint is not inside the map (or is not
		// a number) dies before its first step, so no access leaves the map.
		if (!(px >= 0.0f && px < J.dim_x - 1.0f && py >= 0.0f && py < J.dim_y - 1.0f)) {
			vol = 0.0f;
		}
		while (vol >= P.minWaterVolume) {
			if (step++ >= P.MaxSteps) {
				capped = true;
				break;
			}
			const uint64_t mi = static_cast<uint64_t>(static_cast<uint32_t>(py)) * pitch + static_cast<uint32_t>(px);
			const float ox = px - static_cast<float>(static_cast<int>(px)), oy = py - static_cast<float>(static_cast<int>(py));
			const HG hg = height_gradient<G>(map, pitch, px, py, g, gmask, glead);
			dirx = (-hg.gx) * (1.0f - P.Inertia) + dirx * P.Inertia;
			diry = (-hg.gy) * (1.0f - P.Inertia) + diry * P.Inertia;
			const float len = sqrtf(dirx * dirx + diry * diry);
			if (len != 0.0f) {
				dirx /= len;
				diry /= len;
			}
			px += dirx;
			py += diry;
			// the reference's border test, written so that a NaN position also dies
			if ((dirx == 0.0f && diry == 0.0f) || !(px >= lo && px < hi_x && py >= lo && py < hi_y)) {
				vol = 0.0f;
				break; // the carried sediment leaves with the droplet
			}
			const float dh = height_gradient<G>(map, pitch, px, py, g, gmask, glead).h - hg.h;
			const float cap = fmaxf(-dh * speed * vol * P.SedimentCapacityFactor, P.minSedimentCapacity);
			if (sed > cap || dh > 0.0f) {
				const float dep = (dh > 0.0f) ? fminf(dh, sed) : (sed - cap) * P.DepositSpeed;
				sed -= dep;
				for (uint32_t c = g; c < 4u; c += G) {
					const float wx = (c & 1u) ? ox : 1.0f - ox, wy = (c & 2u) ? oy : 1.0f - oy;
					atomicAdd(map + mi + ((c & 2u) ? pitch : 0u) + (c & 1u), dep * wx * wy);
				}
			} else {
				erode_steps++;
				const float ero = fminf((cap - sed) * P.ErodeSpeed, -dh);
				float part = 0.0f;
				if constexpr (!ExactClamp) {
					// The reference's order (STPRainDrop.cu:146-157): read the
					// cell, subtract min(cell, w), then the next point; the next
					// read stays behind the previous atomic.  The amount is
					// clamped at 0, as noted at kErodeBlock.
#pragma unroll 1
					for (uint32_t p = g; p < bsize; p += G) {
						float* const cell = map + static_cast<int64_t>(mi) + bidx[p];
						const float we = ero * bw[p];
						const float cur = __ldcg(cell);
						const float ds = fminf(fmaxf(cur, 0.0f), we);
						atomicAdd(cell, -ds);
						part += ds;
						asm volatile("" ::: "memory");
					}
				} else {
					// The reference's min(cell, w) as one compare-and-swap per
					// point: read all of the lane's cells, then replace each
					// value v by v - clamp(v, 0, w) only if the cell still holds
					// v, retrying with the value found otherwise.  All of a
					// step's points are in flight at once, yet racing droplets
					// can never remove more than a cell holds -- reading every
					// cell first and subtracting later (or subtracting first and
					// giving back) lets densely packed droplets all remove the
					// same stale height, which drives the map unstable.  After
					// kCasRetries failed swaps the lane falls back to the
					// reference's unconditional subtraction of its last read.
					for (uint32_t base = g; base < bsize; base += G * kBrushBatch) {
						float cur[kBrushBatch], we[kBrushBatch];
						bool done[kBrushBatch];
#pragma unroll
						for (uint32_t k = 0u; k < kBrushBatch; k++) {
							const uint32_t p = base + k * G;
							done[k] = p >= bsize;
							if (!done[k]) {
								we[k] = ero * bw[p];
								cur[k] = __ldcg(map + static_cast<int64_t>(mi) + bidx[p]);
							}
						}
						for (uint32_t attempt = 0u; attempt < kCasRetries; attempt++) {
							bool pending = false;
#pragma unroll
							for (uint32_t k = 0u; k < kBrushBatch; k++) {
								if (!done[k]) {
									int* const cell = reinterpret_cast<int*>(map + static_cast<int64_t>(mi) + bidx[base + k * G]);
									const float ds = fminf(fmaxf(cur[k], 0.0f), we[k]);
									const int seen = atomicCAS(cell, __float_as_int(cur[k]), __float_as_int(cur[k] - ds));
									if (seen == __float_as_int(cur[k])) {
										part += ds;
										done[k] = true;
									} else {
										cur[k] = __int_as_float(seen);
										pending = true;
									}
								}
							}
							if (!pending) {
								break;
							}
						}
#pragma unroll
						for (uint32_t k = 0u; k < kBrushBatch; k++) {
							if (!done[k]) {
								const float ds = fminf(fmaxf(cur[k], 0.0f), we[k]);
								atomicAdd(map + static_cast<int64_t>(mi) + bidx[base + k * G], -ds);
								part += ds;
							}
						}
					}
				}
#pragma unroll
				for (uint32_t o = G / 2u; o > 0u; o >>= 1) {
					part += __shfl_xor_sync(gmask, part, o);
				}
				sed += part;
			}
			speed = sqrtf(fmaxf(0.0f, speed * speed + dh * P.Gravity));
			speed *= 1.0f - P.Friction;
			vol *= 1.0f - P.EvaporateSpeed;
			steps_done++;
			// the group leaves every step together (the deposit loop above runs
			// on some of its lanes only)
			__syncwarp(gmask);
		}
		residual = static_cast<double>(sed);
	}
	if (g != 0u) {
		// one lane per droplet reports
		residual = 0.0;
		steps_done = 0u;
		erode_steps = 0u;
		capped = false;
	}
	if (J.counters) {
		unsigned long long s = steps_done, e = erode_steps;
		for (int o = 16; o > 0; o >>= 1) {
			s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
			e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
		}
		if (lane == 0u) {
			atomicAdd(J.counters, s);
			atomicAdd(J.counters + 1, e);
		}
	}
	if (J.residual) {
		for (int o = 16; o > 0; o >>= 1) {
			residual += __shfl_xor_sync(0xFFFFFFFFu, residual, o);
		}
		if (lane == 0u && residual != 0.0) {
			atomicAdd(J.residual, residual);
		}
	}
	if (capped && J.status) {
		atomicOr(J.status, STATUS_TIMEOUT);
	}
}

// K droplets per group of G >= 4 lanes (reference order only).  The erosion
// kernel is bound by the latency of each lane's chain of brush reads; a
// droplet's chain cannot be shortened without changing how racing droplets
// see each other, so instead each group carries K independent droplets and
// advances them through every phase of a step together: the K corner reads,
// and the K reads of each brush position, are in flight at the same time.
// Each droplet still reads and updates its own brush points in order.
template<uint32_t G, uint32_t K>
// 8 resident blocks of 128 threads (64 registers) for two droplets per group:
// residency, not the few spilled registers, bounds this chain-latency kernel.
__global__ void __launch_bounds__(kErodeBlock, K == 2u ? 8 : 1) erosion_multi_kernel(const ErosionJob* __restrict__ jobs,
	const ErosionJob single) {
	static_assert(G >= 4u && K >= 2u, "one corner per lane needs four lanes");
	const ErosionJob& J = jobs ? jobs[blockIdx.y] : single;
	extern __shared__ unsigned char esm[];
	int32_t* const bidx = reinterpret_cast<int32_t*>(esm);
	float* const bw = reinterpret_cast<float*>(esm) + J.brush_size;
	for (uint32_t k = threadIdx.x; k < J.brush_size; k += kErodeBlock) {
		bidx[k] = J.brush_index[k];
		bw[k] = J.brush_weight[k];
	}
	__syncthreads();

	const RainParams& P = J.p;
	const uint32_t g = threadIdx.x % G;
	const uint32_t group = (blockIdx.x * kErodeBlock + threadIdx.x) / G;
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t gmask = G == 32u ? 0xFFFFFFFFu : (((1u << G) - 1u) << (lane & ~(G - 1u)));
	const uint32_t glead = lane & ~(G - 1u);
	const uint32_t corner = g & 3u;
	float* const map = J.map;
	const uint64_t pitch = J.pitch;
	const uint64_t corner_off = ((corner & 2u) ? pitch : 0u) + (corner & 1u);
	const uint32_t bsize = J.brush_size;
	const float lo = static_cast<float>(P.BrushRadius);
	const float hi_x = 1.0f * J.dim_x - P.BrushRadius, hi_y = 1.0f * J.dim_y - P.BrushRadius;

	float px[K], py[K], dirx[K], diry[K], speed[K], vol[K], sed[K];
	uint32_t step[K];
	bool alive[K];
	double residual = 0.0;
	bool capped = false;
	uint32_t steps_done = 0u, erode_steps = 0u;
#pragma unroll
	for (uint32_t k = 0u; k < K; k++) {
		const uint32_t d = group * K + k;
		alive[k] = d < J.count;
		px[k] = alive[k] ? J.starts[2u * d] : 0.0f;
		py[k] = alive[k] ? J.starts[2u * d + 1u] : 0.0f;
		// a start whose 2x2 bilinear footprint is not inside the map dies at once
		alive[k] = alive[k] && px[k] >= 0.0f && px[k] < J.dim_x - 1.0f && py[k] >= 0.0f && py[k] < J.dim_y - 1.0f;
		dirx[k] = diry[k] = 0.0f;
		speed[k] = P.initSpeed;
		vol[k] = P.initWaterVolume;
		sed[k] = 0.0f;
		step[k] = 0u;
	}
	auto bilinear = [](const float v, const uint32_t gm, const uint32_t gl, const float cx, const float cy) {
		const float h00 = __shfl_sync(gm, v, gl), h10 = __shfl_sync(gm, v, gl + 1), h01 = __shfl_sync(gm, v, gl + 2),
			h11 = __shfl_sync(gm, v, gl + 3);
		HG r;
		r.h = h00 * (1.0f - cx) * (1.0f - cy) + h10 * cx * (1.0f - cy) + h01 * (1.0f - cx) * cy + h11 * cx * cy;
		r.gx = (h10 - h00) * (1.0f - cy) + (h11 - h01) * cy;
		r.gy = (h01 - h00) * (1.0f - cx) + (h11 - h10) * cx;
		return r;
	};

	while (true) {
		bool any = false;
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (alive[k] && !(vol[k] >= P.minWaterVolume)) {
				alive[k] = false;
				residual += sed[k];
			} else if (alive[k] && step[k]++ >= P.MaxSteps) {
				alive[k] = false;
				capped = true;
				residual += sed[k];
			}
			any = any || alive[k];
		}
		if (!any) {
			break;
		}
		// phase 1: corners of the current cell of every droplet
		uint64_t mi[K];
		float ox[K], oy[K], v[K];
		HG hg[K];
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (alive[k]) {
				mi[k] = static_cast<uint64_t>(static_cast<uint32_t>(py[k])) * pitch + static_cast<uint32_t>(px[k]);
				ox[k] = px[k] - static_cast<float>(static_cast<int>(px[k]));
				oy[k] = py[k] - static_cast<float>(static_cast<int>(py[k]));
				v[k] = __ldcg(map + mi[k] + corner_off);
			}
		}
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (alive[k]) {
				hg[k] = bilinear(v[k], gmask, glead, ox[k], oy[k]);
				dirx[k] = (-hg[k].gx) * (1.0f - P.Inertia) + dirx[k] * P.Inertia;
				diry[k] = (-hg[k].gy) * (1.0f - P.Inertia) + diry[k] * P.Inertia;
				const float len = sqrtf(dirx[k] * dirx[k] + diry[k] * diry[k]);
				if (len != 0.0f) {
					dirx[k] /= len;
					diry[k] /= len;
				}
				px[k] += dirx[k];
				py[k] += diry[k];
				if ((dirx[k] == 0.0f && diry[k] == 0.0f)
					|| !(px[k] >= lo && px[k] < hi_x && py[k] >= lo && py[k] < hi_y)) {
					alive[k] = false; // the carried sediment leaves with the droplet
					residual += sed[k];
				}
			}
		}
		// phase 2: corners of the new cell, capacity, deposit or erode
		float v2[K];
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (alive[k]) {
				const uint64_t ni = static_cast<uint64_t>(static_cast<uint32_t>(py[k])) * pitch + static_cast<uint32_t>(px[k]);
				v2[k] = __ldcg(map + ni + corner_off);
			}
		}
		bool erode[K];
		float ero[K], dh[K];
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			erode[k] = false;
			if (alive[k]) {
				const float cx = px[k] - static_cast<float>(static_cast<uint32_t>(px[k]));
				const float cy = py[k] - static_cast<float>(static_cast<uint32_t>(py[k]));
				dh[k] = bilinear(v2[k], gmask, glead, cx, cy).h - hg[k].h;
				const float cap = fmaxf(-dh[k] * speed[k] * vol[k] * P.SedimentCapacityFactor, P.minSedimentCapacity);
				if (sed[k] > cap || dh[k] > 0.0f) {
					const float dep = (dh[k] > 0.0f) ? fminf(dh[k], sed[k]) : (sed[k] - cap) * P.DepositSpeed;
					sed[k] -= dep;
					if (g < 4u) {
						const float wx = (corner & 1u) ? ox[k] : 1.0f - ox[k], wy = (corner & 2u) ? oy[k] : 1.0f - oy[k];
						atomicAdd(map + mi[k] + corner_off, dep * wx * wy);
					}
				} else {
					erode[k] = true;
					erode_steps++;
					ero[k] = fminf((cap - sed[k]) * P.ErodeSpeed, -dh[k]);
				}
			}
		}
		// phase 3: the brush chains of the eroding droplets, interleaved.  Two
		// droplets of the group whose brushes overlap (droplets that flowed
		// into the same channel stay together) would read the same cells in
		// the same instruction and both remove the same stale height, step
		// after step; their chains then run one droplet after the other, so
		// the second reads the first one's updates.
		float part[K];
		bool serial = false;
		const int32_t reach = 2 * static_cast<int32_t>(P.BrushRadius) - 2;
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			part[k] = 0.0f;
#pragma unroll
			for (uint32_t q = k + 1u; q < K; q++) {
				if (erode[k] && erode[q]) {
					// 32-bit division (the launch checks that a map holds
					// fewer than 2^32 cells): a 64-bit division by a run-time
					// divisor runs on the narrow FP64 pipe
					const uint32_t a = static_cast<uint32_t>(mi[k]), b = static_cast<uint32_t>(mi[q]);
					const uint32_t p32 = static_cast<uint32_t>(pitch);
					const int32_t dx = static_cast<int32_t>(a % p32) - static_cast<int32_t>(b % p32);
					const int32_t dy = static_cast<int32_t>(a / p32) - static_cast<int32_t>(b / p32);
					serial = serial || (abs(dx) <= reach && abs(dy) <= reach);
				}
			}
		}
#pragma unroll 1
		for (uint32_t turn = 0u; turn < (serial ? K : 1u); turn++) {
#pragma unroll 1
			for (uint32_t p = g; p < bsize; p += G) {
				const int32_t off = bidx[p];
				const float wp = bw[p];
				float cur[K];
#pragma unroll
				for (uint32_t k = 0u; k < K; k++) {
					if (erode[k] && (!serial || k == turn)) {
						cur[k] = __ldcg(map + static_cast<int64_t>(mi[k]) + off);
					}
				}
#pragma unroll
				for (uint32_t k = 0u; k < K; k++) {
					if (erode[k] && (!serial || k == turn)) {
						const float we = ero[k] * wp;
						const float ds = fminf(fmaxf(cur[k], 0.0f), we);
						atomicAdd(map + static_cast<int64_t>(mi[k]) + off, -ds);
						part[k] += ds;
					}
				}
				asm volatile("" ::: "memory");
			}
		}
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (erode[k]) {
#pragma unroll
				for (uint32_t o = G / 2u; o > 0u; o >>= 1) {
					part[k] += __shfl_xor_sync(gmask, part[k], o);
				}
				sed[k] += part[k];
			}
			if (alive[k]) {
				speed[k] = sqrtf(fmaxf(0.0f, speed[k] * speed[k] + dh[k] * P.Gravity));
				speed[k] *= 1.0f - P.Friction;
				vol[k] *= 1.0f - P.EvaporateSpeed;
				steps_done++;
			}
		}
		__syncwarp(gmask);
	}
	if (g != 0u) {
		residual = 0.0;
		steps_done = 0u;
		erode_steps = 0u;
		capped = false;
	}
	if (J.counters) {
		unsigned long long s = steps_done, e = erode_steps;
		for (int o = 16; o > 0; o >>= 1) {
			s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
			e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
		}
		if (lane == 0u) {
			atomicAdd(J.counters, s);
			atomicAdd(J.counters + 1, e);
		}
	}
	if (J.residual) {
		for (int o = 16; o > 0; o >>= 1) {
			residual += __shfl_xor_sync(0xFFFFFFFFu, residual, o);
		}
		if (lane == 0u && residual != 0.0) {
			atomicAdd(J.residual, residual);
		}
	}
	if (capped && J.status) {
		atomicOr(J.status, STATUS_TIMEOUT);
	}
}

// Brush runs: maximal sequences of brush points whose cells are consecutive
// in memory (the rows of the reference's circular brush), found once per block.
struct BrushRun {
	int32_t first; // index of the run's first point
	int32_t len;
};

__device__ __forceinline__ float4 atom_add_v4(float4* addr, const float a, const float b, const float c,
	const float d) {
	float4 r;
	asm volatile("atom.global.add.v4.f32 {%0, %1, %2, %3}, [%4], {%5, %6, %7, %8};"
		: "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
		: "l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
		: "memory");
	return r;
}

__device__ __forceinline__ void red_add_v4(float4* addr, const float a, const float b, const float c, const float d) {
	asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
		: "memory");
}

// A deposit's two corners of one map row, c0[0] += d0 and c0[1] += d1: one
// 16-byte reduction when both lie in one aligned block (-0.0 to the block's
// other cells leaves them unchanged), else two scalar ones.  The L2 takes a
// reduction per request whatever its width, so this is 1.25 requests per row
// on average instead of 2.  Needs a map whose rows start 16-byte aligned.
__device__ __forceinline__ void deposit_row(float* const c0, const float d0, const float d1) {
	const uint32_t at = (static_cast<uint32_t>(reinterpret_cast<uintptr_t>(c0)) >> 2) & 3u;
	if (at != 3u) {
		float v[4] = { -0.0f, -0.0f, -0.0f, -0.0f };
#pragma unroll
		for (uint32_t k = 0u; k < 3u; k++) {
			if (k == at) {
				v[k] = d0;
				v[k + 1u] = d1;
			}
		}
		red_add_v4(reinterpret_cast<float4*>(c0 - at), v[0], v[1], v[2], v[3]);
	} else {
		atomicAdd(c0, d0);
		atomicAdd(c0 + 1, d1);
	}
}

// K droplets (1 or 2) per group of G lanes (2 or 4) as erosion_multi_kernel,
// with the erosion step done run by run in aligned 16-byte blocks: one
// vector read of four cells, then one vector reduction that subtracts
// min(cell, w) from the run's cells and adds -0.0 (which leaves any value,
// -0.0 included, unchanged) to the block's other cells.  A droplet's cells
// are distinct, so per droplet this is the reference's read-then-subtract
// for every point; a block costs one L2 read and one L2 reduction instead
// of one of each per point.  Needs a 16-byte aligned map whose pitch is a
// multiple of four floats, so that no block leaves its row.
// Residency bounds this chain-latency kernel more than the spilled registers
// do: 9 blocks of 128 threads (56 registers) with one droplet per group,
// 8 (64 registers) with two (measured: 10 blocks of 48 registers are 1 %
// slower with two blocks per round trip, 12 blocks of 40 registers slower
// still; 7 blocks of 72 registers and 6 of 80, without the spills, are as
// fast for two lanes and one droplet and 6-15 % slower for the others).
template<uint32_t G, uint32_t K>
__global__ void __launch_bounds__(kErodeBlock, K == 2u ? 8 : 9) erosion_rows_kernel(const ErosionJob* __restrict__ jobs,
	const ErosionJob single, const uint32_t resident, const bool wide, const bool atomic_brush) {
	static_assert((G == 2u || G == 4u) && (K == 1u || K == 2u), "2 or 4 lanes, 1 or 2 droplets");
	const ErosionJob& J = jobs ? jobs[blockIdx.y] : single;
	extern __shared__ unsigned char esm[];
	int32_t* const bidx = reinterpret_cast<int32_t*>(esm);
	float* const bw = reinterpret_cast<float*>(esm) + J.brush_size;
	BrushRun* const runs = reinterpret_cast<BrushRun*>(bw + J.brush_size);
	__shared__ uint32_t nruns;
	for (uint32_t k = threadIdx.x; k < J.brush_size; k += kErodeBlock) {
		bidx[k] = J.brush_index[k];
		bw[k] = J.brush_weight[k];
	}
	__syncthreads();
	if (threadIdx.x == 0u) {
		uint32_t n = 0u;
		for (uint32_t p = 0u; p < J.brush_size; p++) {
			if (p == 0u || bidx[p] != bidx[p - 1u] + 1) {
				runs[n].first = static_cast<int32_t>(p);
				runs[n].len = 0;
				n++;
			}
			runs[n - 1u].len++;
		}
		nruns = n;
	}
	__syncthreads();

	const RainParams& P = J.p;
	const uint32_t g = threadIdx.x % G;
	const uint32_t group = (blockIdx.x * kErodeBlock + threadIdx.x) / G;
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t gmask = G == 32u ? 0xFFFFFFFFu : (((1u << G) - 1u) << (lane & ~(G - 1u)));
	const uint32_t glead = lane & ~(G - 1u);
	float* const map = J.map;
	// cell offsets in 32 bits: a map holds fewer than 2^32 cells (checked at launch)
	const uint32_t pitch = static_cast<uint32_t>(J.pitch);
	// bilinear corners: with four lanes lane g reads corner g (x + (g & 1),
	// y + (g >> 1)); with two lanes lane g reads both corners of row y + g
	const uint32_t corner_off = G == 4u ? (((g & 2u) ? pitch : 0u) + (g & 1u)) : (g ? pitch : 0u);
	const uint32_t nrun = nruns;
	constexpr int32_t kTripMax = K == 1u ? 3 : 2;
	// blocks per round trip of this job: kTripMax where at most
	// kWideConcurrency droplets per pixel of its start area are in flight
	// (min(count, resident) droplets)
	const uint32_t trip = wide && J.start_area != 0u
			&& static_cast<double>(min(J.count, resident)) <= kWideConcurrency * J.start_area
		? static_cast<uint32_t>(kTripMax)
		: 1u;
	const float lo = static_cast<float>(P.BrushRadius);
	const float hi_x = 1.0f * J.dim_x - P.BrushRadius, hi_y = 1.0f * J.dim_y - P.BrushRadius;
	// cells whose brush (reach BrushRadius - 1) and deposit corners stay inside the map
	const uint32_t safe_lo = P.BrushRadius - 1u, safe_hx = J.dim_x - max(P.BrushRadius, 2u),
		safe_hy = J.dim_y - max(P.BrushRadius, 2u);

	float px[K], py[K], dirx[K], diry[K], speed[K], vol[K], sed[K];
	uint32_t step[K];
	bool alive[K];
	// sediment that left with this thread's (at most two) droplets; summed in
	// double per warp at the end (a double add per death would run on the
	// narrow FP64 pipe once per lane group)
	float residual = 0.0f;
	bool capped = false;
	uint32_t steps_done = 0u, erode_steps = 0u;
#pragma unroll
	for (uint32_t k = 0u; k < K; k++) {
		const uint32_t d = group * K + k;
		alive[k] = d < J.count;
		px[k] = alive[k] ? J.starts[2u * d] : 0.0f;
		py[k] = alive[k] ? J.starts[2u * d + 1u] : 0.0f;
		alive[k] = alive[k] && px[k] >= 0.0f && px[k] < J.dim_x - 1.0f && py[k] >= 0.0f && py[k] < J.dim_y - 1.0f;
		dirx[k] = diry[k] = 0.0f;
		speed[k] = P.initSpeed;
		vol[k] = P.initWaterVolume;
		sed[k] = 0.0f;
		step[k] = 0u;
	}
	auto corners = [&](const uint32_t cell) {
		const float* const c = map + cell + corner_off;
		return G == 4u ? make_float2(__ldcg(c), 0.0f) : make_float2(__ldcg(c), __ldcg(c + 1));
	};
	auto bilinear = [](const float2 v, const uint32_t gm, const uint32_t gl, const float cx, const float cy) {
		float h00, h10, h01, h11;
		if constexpr (G == 4u) {
			h00 = __shfl_sync(gm, v.x, gl);
			h10 = __shfl_sync(gm, v.x, gl + 1);
			h01 = __shfl_sync(gm, v.x, gl + 2);
			h11 = __shfl_sync(gm, v.x, gl + 3);
		} else {
			h00 = __shfl_sync(gm, v.x, gl);
			h10 = __shfl_sync(gm, v.y, gl);
			h01 = __shfl_sync(gm, v.x, gl + 1);
			h11 = __shfl_sync(gm, v.y, gl + 1);
		}
		HG r;
		r.h = h00 * (1.0f - cx) * (1.0f - cy) + h10 * cx * (1.0f - cy) + h01 * (1.0f - cx) * cy + h11 * cx * cy;
		r.gx = (h10 - h00) * (1.0f - cy) + (h11 - h01) * cy;
		r.gy = (h01 - h00) * (1.0f - cx) + (h11 - h10) * cx;
		return r;
	};

	while (true) {
		bool any = false;
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (alive[k] && !(vol[k] >= P.minWaterVolume)) {
				alive[k] = false;
				residual += sed[k];
			} else if (alive[k] && step[k]++ >= P.MaxSteps) {
				alive[k] = false;
				capped = true;
				residual += sed[k];
			}
			any = any || alive[k];
		}
		if (!any) {
			break;
		}
		// phase 1: corners of the current cell of every droplet
		uint32_t mi[K];
		float ox[K], oy[K];
		float2 v[K];
		bool safe[K];
		HG hg[K];
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (alive[k]) {
				const uint32_t cx = static_cast<uint32_t>(px[k]), cy = static_cast<uint32_t>(py[k]);
				safe[k] = cx >= safe_lo && cx <= safe_hx && cy >= safe_lo && cy <= safe_hy;
				mi[k] = cy * pitch + cx;
				ox[k] = px[k] - static_cast<float>(cx);
				oy[k] = py[k] - static_cast<float>(cy);
				v[k] = corners(mi[k]);
			}
		}
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (alive[k]) {
				hg[k] = bilinear(v[k], gmask, glead, ox[k], oy[k]);
				dirx[k] = (-hg[k].gx) * (1.0f - P.Inertia) + dirx[k] * P.Inertia;
				diry[k] = (-hg[k].gy) * (1.0f - P.Inertia) + diry[k] * P.Inertia;
				const float len = sqrtf(dirx[k] * dirx[k] + diry[k] * diry[k]);
				if (len != 0.0f) {
					dirx[k] /= len;
					diry[k] /= len;
				}
				px[k] += dirx[k];
				py[k] += diry[k];
				// the reference's border test (a NaN position also dies); a unit
				// move keeps the old cell's brush inside the map, `safe` also
				// covers a direction that rounded above unit length
				if ((dirx[k] == 0.0f && diry[k] == 0.0f)
					|| !(px[k] >= lo && px[k] < hi_x && py[k] >= lo && py[k] < hi_y) || !safe[k]) {
					alive[k] = false; // the carried sediment leaves with the droplet
					residual += sed[k];
				}
			}
		}
		// phase 2: corners of the new cell, capacity, deposit or erode
		float2 v2[K];
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (alive[k]) {
				const uint32_t ni = static_cast<uint32_t>(py[k]) * pitch + static_cast<uint32_t>(px[k]);
				v2[k] = corners(ni);
			}
		}
		bool erode[K];
		float ero[K], dh[K];
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			erode[k] = false;
			if (alive[k]) {
				const float cx = px[k] - static_cast<float>(static_cast<uint32_t>(px[k]));
				const float cy = py[k] - static_cast<float>(static_cast<uint32_t>(py[k]));
				dh[k] = bilinear(v2[k], gmask, glead, cx, cy).h - hg[k].h;
				const float cap = fmaxf(-dh[k] * speed[k] * vol[k] * P.SedimentCapacityFactor, P.minSedimentCapacity);
				if (sed[k] > cap || dh[k] > 0.0f) {
					const float dep = (dh[k] > 0.0f) ? fminf(dh[k], sed[k]) : (sed[k] - cap) * P.DepositSpeed;
					sed[k] -= dep;
					if constexpr (G == 4u) {
						const float wx = (g & 1u) ? ox[k] : 1.0f - ox[k], wy = (g & 2u) ? oy[k] : 1.0f - oy[k];
						atomicAdd(map + mi[k] + corner_off, dep * wx * wy);
					} else {
						const float wy = g ? oy[k] : 1.0f - oy[k];
						deposit_row(map + mi[k] + corner_off, dep * (1.0f - ox[k]) * wy, dep * ox[k] * wy);
					}
				} else {
					erode[k] = true;
					erode_steps++;
					ero[k] = fminf((cap - sed[k]) * P.ErodeSpeed, -dh[k]);
				}
			}
		}
		// phase 3: the brush runs of the eroding droplets, a run per lane; two
		// droplets whose brushes overlap run one after the other
		float part[K];
		bool serial = false;
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			part[k] = 0.0f;
		}
		if constexpr (K == 2u) {
			if (erode[0] && erode[1]) {
				const int32_t reach = 2 * static_cast<int32_t>(P.BrushRadius) - 2;
				const int32_t dx = static_cast<int32_t>(mi[0] % pitch) - static_cast<int32_t>(mi[1] % pitch);
				const int32_t dy = static_cast<int32_t>(mi[0] / pitch) - static_cast<int32_t>(mi[1] / pitch);
				serial = abs(dx) <= reach && abs(dy) <= reach;
			}
		}
#pragma unroll 1
		for (uint32_t turn = 0u; turn < (serial ? K : 1u); turn++) {
#pragma unroll 1
			for (uint32_t r = g; r < nrun; r += G) {
				const BrushRun R = runs[r];
				const int32_t off = bidx[R.first];
				float4* blk[K];
				int32_t lead[K], nb[K];
				int32_t nmax = 0;
#pragma unroll
				for (uint32_t k = 0u; k < K; k++) {
					nb[k] = 0;
					if (erode[k] && (!serial || k == turn)) {
						float* const first = map + (static_cast<int64_t>(mi[k]) + off);
						lead[k] = static_cast<int32_t>((reinterpret_cast<uintptr_t>(first) >> 2) & 3u);
						blk[k] = reinterpret_cast<float4*>(first - lead[k]);
						nb[k] = (lead[k] + R.len + 3) >> 2;
						nmax = max(nmax, nb[k]);
					}
				}
				// `trip` (1 to kTripMax) blocks per round trip: a run's blocks
				// are distinct cells, so reading the next ones before the first
				// one's update changes nothing for this droplet
#pragma unroll 1
				for (int32_t b0 = 0; b0 < nmax; b0 += static_cast<int32_t>(trip)) {
					float4 cur[K][kTripMax];
#pragma unroll
					for (uint32_t k = 0u; k < K; k++) {
#pragma unroll
						for (int32_t u = 0; u < kTripMax; u++) {
							const int32_t b = b0 + u;
							if (u < static_cast<int32_t>(trip) && b < nb[k]) {
								if (atomic_brush) {
									float d[4];
#pragma unroll
									for (int i = 0; i < 4; i++) {
										const int32_t j = 4 * b + i - lead[k];
										d[i] = (j >= 0 && j < R.len) ? -(ero[k] * bw[R.first + j]) : -0.0f;
									}
									cur[k][u] = atom_add_v4(blk[k] + b, d[0], d[1], d[2], d[3]);
								} else {
									cur[k][u] = __ldcg(blk[k] + b);
								}
							}
						}
					}
#pragma unroll
					for (uint32_t k = 0u; k < K; k++) {
#pragma unroll
						for (int32_t u = 0; u < kTripMax; u++) {
							const int32_t b = b0 + u;
							if (u < static_cast<int32_t>(trip) && b < nb[k]) {
								float c[4] = { cur[k][u].x, cur[k][u].y, cur[k][u].z, cur[k][u].w }, d[4];
								bool back = false;
#pragma unroll
								for (int i = 0; i < 4; i++) {
									const int32_t j = 4 * b + i - lead[k];
									d[i] = -0.0f;
									if (j >= 0 && j < R.len) {
										const float we = ero[k] * bw[R.first + j];
										const float ds = fminf(fmaxf(c[i], 0.0f), we);
										part[k] += ds;
										if (atomic_brush) {
											// w was taken; give back what the cell lacked
											if (ds < we) {
												d[i] = we - ds;
												back = true;
											}
										} else {
											d[i] = -ds;
										}
									}
								}
								if (!atomic_brush || back) {
									red_add_v4(blk[k] + b, d[0], d[1], d[2], d[3]);
								}
							}
						}
					}
				}
			}
		}
#pragma unroll
		for (uint32_t k = 0u; k < K; k++) {
			if (erode[k]) {
#pragma unroll
				for (uint32_t o = G / 2u; o > 0u; o >>= 1) {
					part[k] += __shfl_xor_sync(gmask, part[k], o);
				}
				sed[k] += part[k];
			}
			if (alive[k]) {
				speed[k] = sqrtf(fmaxf(0.0f, speed[k] * speed[k] + dh[k] * P.Gravity));
				speed[k] *= 1.0f - P.Friction;
				vol[k] *= 1.0f - P.EvaporateSpeed;
				steps_done++;
			}
		}
		__syncwarp(gmask);
	}
	if (g != 0u) {
		residual = 0.0f;
		steps_done = 0u;
		erode_steps = 0u;
		capped = false;
	}
	if (J.counters) {
		unsigned long long s = steps_done, e = erode_steps;
		for (int o = 16; o > 0; o >>= 1) {
			s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
			e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
		}
		if (lane == 0u) {
			atomicAdd(J.counters, s);
			atomicAdd(J.counters + 1, e);
		}
	}
	if (J.residual) {
		// the warp's 8 or 16 droplet residuals, gathered on lane 0 and summed in double
		double total = 0.0;
		for (uint32_t l = 0u; l < 32u; l += G) {
			const float r = __shfl_sync(0xFFFFFFFFu, residual, static_cast<int>(l));
			if (lane == 0u) {
				total += static_cast<double>(r);
			}
		}
		if (lane == 0u && total != 0.0) {
			atomicAdd(J.residual, total);
		}
	}
	if (capped && J.status) {
		atomicOr(J.status, STATUS_TIMEOUT);
	}
}

// One droplet per lane, the brush of every eroding droplet of a warp shared
// out over all 32 lanes.  Phases 1 and 2 (the corners of the current and of
// the new cell) are each lane's own four reads and twice as many droplets are
// in flight per SM as with two lanes per droplet.  In phase 3 the runs of the
// warp's eroding droplets form one task list -- (droplet, run) in the order
// of the droplets' lanes, then of the runs -- that the lanes take 32 at a
// time, so the lanes of depositing and finished droplets help and a step
// costs ceil(tasks / 32) round trips instead of one per run of a lane.  A
// run's 16-byte blocks are taken by returning vector atomics (the cells'
// values at that moment, w subtracted, the part of w a cell lacked given
// back): for the droplet this is c - min(max(c, 0), w) on the exact current
// value whichever lane takes the run and in whatever order.  Each run's
// eroded amount goes to a shared slot and the droplet's lane adds its runs up
// in run order, so the droplet's sediment does not depend on which lane took
// which run.  Every run of a droplet is in flight at once -- the brush update
// is more compressed in time than with two lanes per droplet -- so the
// default takes this kernel only where few droplets are in flight per pixel
// (erosion_variant_stable).  Needs what the row kernel needs: a 16-byte
// aligned map whose pitch is a multiple of four floats.
// The grid is one-dimensional, `blocks_per_job` blocks per job; with
// `interleave` > 1 the blocks of that many consecutive jobs alternate, so
// that several jobs share the droplets in flight and each keeps fewer of its
// own in flight per pixel (the blocks of a job still go out in order).
constexpr int32_t kCoopTrip = 3; // blocks of a run per round trip
// Blocks per SM the warp-cooperative kernel is compiled for: 8 (64 registers,
// no spill) ran the production batch's erosion in 59.95 ms, 7 (72) in 59.91,
// 6 (80) in 60.17, 9 (56, 32 bytes spilled) in 61.5, 10 and 12 slower still.
constexpr uint32_t kCoopBlocksPerSM = 8u;

__global__ void __launch_bounds__(kErodeBlock, kCoopBlocksPerSM) erosion_coop_kernel(const ErosionJob* __restrict__ jobs,
	const ErosionJob single, const uint32_t runcap, const uint32_t njobs, const uint32_t interleave,
	const uint32_t blocks_per_job) {
	constexpr uint32_t kWarps = kErodeBlock / 32u;
	uint32_t job = 0u, bx = blockIdx.x;
	if (jobs) {
		const uint32_t span = interleave * blocks_per_job;
		const uint32_t chunk = blockIdx.x / span, within = blockIdx.x - chunk * span;
		const uint32_t qn = min(interleave, njobs - chunk * interleave);
		job = chunk * interleave + within % qn;
		bx = within / qn;
	}
	const ErosionJob& J = jobs ? jobs[job] : single;
	extern __shared__ __align__(16) unsigned char esm[];
	int32_t* const bidx = reinterpret_cast<int32_t*>(esm);
	float* const bw = reinterpret_cast<float*>(esm) + J.brush_size;
	int2* const runs = reinterpret_cast<int2*>(esm + ((8u * J.brush_size + 7u) & ~7u)); // (first point, length)
	float* const parts = reinterpret_cast<float*>(runs + runcap);                         // [warp][32 * runcap]
	__shared__ uint32_t slot_cell[kWarps][32];
	__shared__ float slot_ero[kWarps][32];
	__shared__ uint32_t nruns;
	for (uint32_t k = threadIdx.x; k < J.brush_size; k += kErodeBlock) {
		bidx[k] = J.brush_index[k];
		bw[k] = J.brush_weight[k];
	}
	__syncthreads();
	if (threadIdx.x == 0u) {
		uint32_t n = 0u;
		for (uint32_t p = 0u; p < J.brush_size; p++) {
			if (p == 0u || bidx[p] != bidx[p - 1u] + 1) {
				if (n < runcap) {
					runs[n] = make_int2(static_cast<int32_t>(p), 0);
				}
				n++;
			}
			if (n <= runcap) {
				runs[n - 1u].y++;
			}
		}
		nruns = n;
	}
	__syncthreads();
	if (nruns > runcap) {
		// a brush of more runs than the shared slots were sized for (never one
		// made by stpgb_erosion_brush_generate): refused through the status word
		if (threadIdx.x == 0u && J.status) {
			atomicOr(J.status, STATUS_CAPACITY);
		}
		return;
	}

	const RainParams& P = J.p;
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	const uint32_t d = bx * kErodeBlock + threadIdx.x;
	const uint32_t nrun = nruns;
	float* const wparts = parts + static_cast<size_t>(warp) * 32u * runcap;
	float* const map = J.map;
	// cell offsets in 32 bits: a map holds fewer than 2^32 cells (checked at launch)
	const uint32_t pitch = static_cast<uint32_t>(J.pitch);
	const float lo = static_cast<float>(P.BrushRadius);
	const float hi_x = 1.0f * J.dim_x - P.BrushRadius, hi_y = 1.0f * J.dim_y - P.BrushRadius;
	// cells whose brush (reach BrushRadius - 1) and deposit corners stay inside the map
	const uint32_t safe_lo = P.BrushRadius - 1u, safe_hx = J.dim_x - max(P.BrushRadius, 2u),
		safe_hy = J.dim_y - max(P.BrushRadius, 2u);

	bool alive = d < J.count;
	float px = alive ? J.starts[2u * d] : 0.0f, py = alive ? J.starts[2u * d + 1u] : 0.0f;
	alive = alive && px >= 0.0f && px < J.dim_x - 1.0f && py >= 0.0f && py < J.dim_y - 1.0f;
	float dirx = 0.0f, diry = 0.0f, speed = P.initSpeed, vol = P.initWaterVolume, sed = 0.0f;
	uint32_t step = 0u;
	float residual = 0.0f;
	bool capped = false;
	uint32_t steps_done = 0u, erode_steps = 0u;
	auto corners = [&](const uint32_t cell) {
		const float* const c = map + cell;
		return make_float4(__ldcg(c), __ldcg(c + 1), __ldcg(c + pitch), __ldcg(c + pitch + 1));
	};

	while (true) {
		if (alive && !(vol >= P.minWaterVolume)) {
			alive = false;
			residual += sed;
		} else if (alive && step++ >= P.MaxSteps) {
			alive = false;
			capped = true;
			residual += sed;
		}
		// the lanes of finished droplets stay for the shared brush phase
		if (!__any_sync(0xFFFFFFFFu, alive)) {
			break;
		}
		bool erode = false;
		uint32_t mi = 0u;
		float ero = 0.0f, dh = 0.0f;
		if (alive) {
			// phase 1: corners of the current cell (STPRainDrop.cu:23-51)
			const uint32_t cx = static_cast<uint32_t>(px), cy = static_cast<uint32_t>(py);
			const bool safe = cx >= safe_lo && cx <= safe_hx && cy >= safe_lo && cy <= safe_hy;
			mi = cy * pitch + cx;
			const float ox = px - static_cast<float>(cx), oy = py - static_cast<float>(cy);
			const float4 q = corners(mi);
			HG hg;
			hg.h = q.x * (1.0f - ox) * (1.0f - oy) + q.y * ox * (1.0f - oy) + q.z * (1.0f - ox) * oy + q.w * ox * oy;
			hg.gx = (q.y - q.x) * (1.0f - oy) + (q.w - q.z) * oy;
			hg.gy = (q.z - q.x) * (1.0f - ox) + (q.w - q.y) * ox;
			dirx = (-hg.gx) * (1.0f - P.Inertia) + dirx * P.Inertia;
			diry = (-hg.gy) * (1.0f - P.Inertia) + diry * P.Inertia;
			const float len = sqrtf(dirx * dirx + diry * diry);
			if (len != 0.0f) {
				dirx /= len;
				diry /= len;
			}
			px += dirx;
			py += diry;
			// the reference's border test (a NaN position also dies); `safe`
			// also covers a direction that rounded above unit length
			if ((dirx == 0.0f && diry == 0.0f) || !(px >= lo && px < hi_x && py >= lo && py < hi_y) || !safe) {
				alive = false; // the carried sediment leaves with the droplet
				residual += sed;
			} else {
				// phase 2: corners of the new cell, capacity, deposit or erode
				const uint32_t nx = static_cast<uint32_t>(px), ny = static_cast<uint32_t>(py);
				const float4 q2 = corners(ny * pitch + nx);
				const float cx2 = px - static_cast<float>(nx), cy2 = py - static_cast<float>(ny);
				const float h2 = q2.x * (1.0f - cx2) * (1.0f - cy2) + q2.y * cx2 * (1.0f - cy2)
					+ q2.z * (1.0f - cx2) * cy2 + q2.w * cx2 * cy2;
				dh = h2 - hg.h;
				const float cap = fmaxf(-dh * speed * vol * P.SedimentCapacityFactor, P.minSedimentCapacity);
				if (sed > cap || dh > 0.0f) {
					const float dep = (dh > 0.0f) ? fminf(dh, sed) : (sed - cap) * P.DepositSpeed;
					sed -= dep;
#pragma unroll
					for (uint32_t row = 0u; row < 2u; row++) {
						const float wy = row ? oy : 1.0f - oy;
						deposit_row(map + mi + (row ? pitch : 0u), dep * (1.0f - ox) * wy, dep * ox * wy);
					}
				} else {
					erode = true;
					erode_steps++;
					ero = fminf((cap - sed) * P.ErodeSpeed, -dh);
				}
			}
		}
		// phase 3: the brush runs of the warp's eroding droplets over all lanes
		const uint32_t emask = __ballot_sync(0xFFFFFFFFu, erode);
		if (emask != 0u) {
			const uint32_t rank = __popc(emask & ((1u << lane) - 1u));
			if (erode) {
				slot_cell[warp][rank] = mi;
				slot_ero[warp][rank] = ero;
			}
			__syncwarp();
			const uint32_t ntask = static_cast<uint32_t>(__popc(emask)) * nrun;
#pragma unroll 1
			for (uint32_t t = lane; t < ntask; t += 32u) {
				const uint32_t di = t / nrun, r = t - di * nrun;
				const uint32_t cell = slot_cell[warp][di];
				const float e = slot_ero[warp][di];
				const int2 R = runs[r];
				float* const first = map + (static_cast<int64_t>(cell) + bidx[R.x]);
				const int32_t lead = static_cast<int32_t>((reinterpret_cast<uintptr_t>(first) >> 2) & 3u);
				float4* const blk = reinterpret_cast<float4*>(first - lead);
				const int32_t nb = (lead + R.y + 3) >> 2;
				float part = 0.0f;
#pragma unroll 1
				for (int32_t b0 = 0; b0 < nb; b0 += kCoopTrip) {
					float4 cur[kCoopTrip];
#pragma unroll
					for (int32_t u = 0; u < kCoopTrip; u++) {
						const int32_t b = b0 + u;
						if (b < nb) {
							float dd[4];
#pragma unroll
							for (int i = 0; i < 4; i++) {
								const int32_t j = 4 * b + i - lead;
								dd[i] = (j >= 0 && j < R.y) ? -(e * bw[R.x + j]) : -0.0f;
							}
							cur[u] = atom_add_v4(blk + b, dd[0], dd[1], dd[2], dd[3]);
						}
					}
#pragma unroll
					for (int32_t u = 0; u < kCoopTrip; u++) {
						const int32_t b = b0 + u;
						if (b < nb) {
							const float c[4] = { cur[u].x, cur[u].y, cur[u].z, cur[u].w };
							float dd[4];
							bool back = false;
#pragma unroll
							for (int i = 0; i < 4; i++) {
								const int32_t j = 4 * b + i - lead;
								dd[i] = -0.0f;
								if (j >= 0 && j < R.y) {
									const float we = e * bw[R.x + j];
									const float ds = fminf(fmaxf(c[i], 0.0f), we);
									part += ds;
									// w was taken; give back what the cell lacked
									if (ds < we) {
										dd[i] = we - ds;
										back = true;
									}
								}
							}
							if (back) {
								red_add_v4(blk + b, dd[0], dd[1], dd[2], dd[3]);
							}
						}
					}
				}
				wparts[t] = part;
			}
			__syncwarp();
			if (erode) {
				float sum = 0.0f;
				for (uint32_t r = 0u; r < nrun; r++) {
					sum += wparts[rank * nrun + r];
				}
				sed += sum;
			}
			__syncwarp();
		}
		if (alive) {
			speed = sqrtf(fmaxf(0.0f, speed * speed + dh * P.Gravity));
			speed *= 1.0f - P.Friction;
			vol *= 1.0f - P.EvaporateSpeed;
			steps_done++;
		}
	}
	if (J.counters) {
		unsigned long long s = steps_done, e = erode_steps;
		for (int o = 16; o > 0; o >>= 1) {
			s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
			e += __shfl_xor_sync(0xFFFFFFFFu, e, o);
		}
		if (lane == 0u) {
			atomicAdd(J.counters, s);
			atomicAdd(J.counters + 1, e);
		}
	}
	if (J.residual) {
		// the warp's 32 droplet residuals, gathered on lane 0 and summed in double
		double total = 0.0;
		for (uint32_t l = 0u; l < 32u; l++) {
			const float r = __shfl_sync(0xFFFFFFFFu, residual, static_cast<int>(l));
			if (lane == 0u) {
				total += static_cast<double>(r);
			}
		}
		if (lane == 0u && total != 0.0) {
			atomicAdd(J.residual, total);
		}
	}
	if (capped && J.status) {
		atomicOr(J.status, STATUS_TIMEOUT);
	}
}

// STPHeightfieldKernel.cu:112-122, eight pixels per thread where rows allow.
__device__ __forceinline__ uint32_t fmt1(const float h) {
	return static_cast<uint32_t>(rintf(__saturatef(h) * 65535.0f));
}

__device__ __forceinline__ void format_group(const float* __restrict__ in, const uint64_t in_pitch,
	uint16_t* __restrict__ out, const uint64_t out_pitch, const uint32_t W, const uint32_t H, const uint64_t t) {
	const uint32_t groups = (W + 7u) / 8u;
	if (t >= static_cast<uint64_t>(groups) * H) {
		return;
	}
	const uint32_t y = static_cast<uint32_t>(t / groups), x0 = static_cast<uint32_t>(t % groups) * 8u;
	const float* const src = in + y * in_pitch + x0;
	uint16_t* const dst = out + y * out_pitch + x0;
	const bool vec = x0 + 8u <= W && (reinterpret_cast<uintptr_t>(src) & 15u) == 0u
		&& (reinterpret_cast<uintptr_t>(dst) & 15u) == 0u;
	if (vec) {
		const float4 a = __ldcs(reinterpret_cast<const float4*>(src));
		const float4 b = __ldcs(reinterpret_cast<const float4*>(src) + 1);
		uint4 o;
		o.x = fmt1(a.x) | (fmt1(a.y) << 16);
		o.y = fmt1(a.z) | (fmt1(a.w) << 16);
		o.z = fmt1(b.x) | (fmt1(b.y) << 16);
		o.w = fmt1(b.z) | (fmt1(b.w) << 16);
		__stcs(reinterpret_cast<uint4*>(dst), o);
	} else {
		for (uint32_t x = x0; x < min(W, x0 + 8u); x++) {
			out[y * out_pitch + x] = static_cast<uint16_t>(fmt1(in[y * in_pitch + x]));
		}
	}
}

__global__ void format_kernel(const float* __restrict__ in, const uint64_t in_pitch, uint16_t* __restrict__ out,
	const uint64_t out_pitch, const uint32_t W, const uint32_t H) {
	format_group(in, in_pitch, out, out_pitch, W, H, static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x);
}

__global__ void format_batch_kernel(const FormatJob* __restrict__ jobs) {
	const FormatJob& J = jobs[blockIdx.y];
	format_group(J.in, J.in_pitch, J.out, J.out_pitch, J.W, J.H,
		static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x);
}

} // namespace

// Each lane of a group walks ceil(points / G) brush points one after another.
// Below four points per lane the reads of a step happen nearly together again,
// and on densely packed droplets (a 64^2 chunk with 9,000 droplets, brush 3)
// the map then runs away, as it does when all reads precede the updates; at
// four or more the grouped kernel stays within the one-lane kernel's
// run-to-run spread.  max_lanes() is the largest power of two that keeps four
// points per lane; the per-call entry point uses min(8, max_lanes()).
uint32_t max_lanes(uint32_t brush_size) {
	uint32_t g = 1u;
	while (g < 32u && 2u * g * 4u <= brush_size) {
		g *= 2u;
	}
	return g;
}

uint32_t default_lanes(uint32_t brush_size) {
	return std::min(8u, max_lanes(brush_size));
}

// The same rule for the brush-row update, in sequential 16-byte blocks per
// lane: the reference's circular brush of this radius has rows of
// 2 * floor(sqrt(r^2 - dy^2 - 1)) + 1 cells, a row of L cells spans
// ceil((lead + L) / 4) blocks for lead 0..3 (averaged), and 4 or 2 lanes are
// allowed while each keeps four blocks.  0 when even two lanes would not.
uint32_t rows_max_lanes(uint32_t radius) {
	const int64_t r = radius;
	double blocks = 0.0;
	for (int64_t dy = -(r - 1); dy <= r - 1; dy++) {
		int64_t half = 0;
		while ((half + 1) * (half + 1) + dy * dy < r * r) {
			half++;
		}
		const int64_t len = 2 * half + 1;
		for (int64_t lead = 0; lead < 4; lead++) {
			blocks += 0.25 * static_cast<double>((lead + len + 3) / 4);
		}
	}
	for (uint32_t g : { 4u, 2u }) {
		if (blocks >= 4.0 * g) {
			return g;
		}
	}
	return 0u;
}

// Stability envelope of the kernel variants against droplet density (droplets
// per pixel of the area the starts cover), measured on a 64^2 chunk of
// multi-biome terrain with brushes 3 and 4, ten runs each, the lowest height
// against the map's lowest start height: with the brush amount clamped at
// zero every row variant (one block per round trip) stays in range up to 3.5,
// and falls up to 0.1 below it at 7 (brush 3, four lanes); without the clamp
// brush 3 ran away to -10^5 at 2.7 to 3.  Four lanes point by point went out
// of range at 4.9 in some runs; one lane per droplet (the reference kernel)
// holds at 7.  Above kDenseRows, or kDenseInFlight droplets in flight per
// pixel, only the reference kernel is used.
bool erosion_variant_stable(const uint32_t lanes, const uint32_t droplets_per_group, const bool rows,
	const double density, const double in_flight) {
	(void)droplets_per_group;
	if (lanes == 1u && rows) {
		return density <= kDenseRows && in_flight <= kCoopInFlight;
	}
	return lanes == 1u || (density <= kDenseRows && in_flight <= kDenseInFlight);
}

double erosion_in_flight(const uint32_t count, const double area) {
	return area > 0.0 ? std::min<double>(count, erosion_resident_droplets(2u, 1u)) / area : 0.0;
}

uint32_t erosion_resident_droplets(const uint32_t lanes, const uint32_t dpg) {
	const uint32_t sms = current_sm_count();
	const uint32_t blocks = dpg == 2u ? 8u : 9u; // the row kernel's launch bounds
	return sms * blocks * kErodeBlock / std::max(lanes, 1u) * std::max(dpg, 1u);
}

uint32_t erosion_coop_interleave(const ErosionJob* jobs, const uint32_t njobs) {
	int dev = 0, l2 = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess
		|| l2 <= 0) {
		cudaGetLastError();
		l2 = 126 * 1024 * 1024;
	}
	// droplets the warp-cooperative kernel keeps resident (one per thread)
	const double resident = static_cast<double>(current_sm_count()) * kCoopBlocksPerSM * kErodeBlock;
	double worst = 0.0, map_bytes = 1.0;
	for (uint32_t j = 0u; j < njobs; j++) {
		const ErosionJob& J = jobs[j];
		if (J.start_area != 0u) {
			worst = std::max(worst, std::min<double>(J.count, resident) / J.start_area);
		}
		map_bytes = std::max(map_bytes, static_cast<double>(J.pitch) * J.dim_y * sizeof(float));
	}
	const double want = std::ceil(worst / kCoopInterleaveInFlight);
	const double fit = std::floor(0.5 * l2 / map_bytes);
	return static_cast<uint32_t>(std::max(1.0, std::min({ want, fit, static_cast<double>(njobs) })));
}

bool erosion_rows_wide(const uint32_t min_radius) {
	return min_radius >= kWideMinRadius;
}

bool erosion_rows_atomic(const uint32_t min_radius, const uint32_t lanes) {
	return min_radius >= kAtomicMinRadius || lanes == 2u;
}

ErosionChoice erosion_choice(const uint32_t radius, const uint32_t brush_size, const double density,
	const double in_flight, const bool rows_allowed) {
	if (!erosion_variant_stable(2u, 1u, true, density, in_flight)) {
		return ErosionChoice { 1u, 1u, false };
	}
	// brush rows where the brush allows them: the warp-cooperative kernel
	// where few droplets are in flight per pixel, else two lanes per droplet
	// (with the brush taken by returning atomics the fastest lane-group row
	// variant on the production chunk, 69 ms per 16 chunks against 76 ms with
	// four lanes, inside the one-thread kernel's band everywhere measured)
	if (rows_allowed && rows_max_lanes(radius) != 0u) {
		if (erosion_variant_stable(1u, 1u, true, density, in_flight) && in_flight <= kCoopDefaultInFlight) {
			return ErosionChoice { 1u, 1u, true };
		}
		return ErosionChoice { 2u, 1u, true };
	}
	return ErosionChoice { default_lanes(brush_size), 1u, false };
}

RainParams rain_params(const stpgb_raindrop_setting& s) {
	RainParams p;
	p.Inertia = s.Inertia;
	p.SedimentCapacityFactor = s.SedimentCapacityFactor;
	p.minSedimentCapacity = s.minSedimentCapacity;
	p.initWaterVolume = s.initWaterVolume;
	p.minWaterVolume = s.minWaterVolume;
	p.Friction = s.Friction;
	p.initSpeed = s.initSpeed;
	p.ErodeSpeed = s.ErodeSpeed;
	p.DepositSpeed = s.DepositSpeed;
	p.EvaporateSpeed = s.EvaporateSpeed;
	p.Gravity = s.Gravity;
	p.BrushRadius = s.ErosionBrushRadius;
	// The volume shrinks by (1 - EvaporateSpeed) per step: count the steps the
	// loop test allows, in float exactly as the kernel does, up to 1<<20.
	uint32_t steps = 0u;
	float v = s.initWaterVolume;
	const uint32_t limit = 1u << 20;
	while (v >= s.minWaterVolume && steps < limit) {
		v *= 1.0f - s.EvaporateSpeed;
		steps++;
	}
	p.MaxSteps = steps < limit ? steps + 1u : limit;
	return p;
}

int erosion_launch(const ErosionJob* jobs, const ErosionJob& single, uint32_t njobs, uint32_t max_count,
	uint32_t max_brush, cudaStream_t stream, uint32_t lanes_per_droplet, bool exact_clamp,
	uint32_t droplets_per_group, bool vector_rows, bool wide_trips, bool atomic_brush, uint32_t interleave) {
	if (max_count == 0u || njobs == 0u) {
		return STPGB_OK;
	}
	const size_t smem = static_cast<size_t>(max_brush) * (sizeof(int32_t) + sizeof(float));
	if (vector_rows && !exact_clamp && lanes_per_droplet == 1u && droplets_per_group == 1u) {
		// the warp-cooperative kernel: brush, runs and one eroded-amount slot per
		// (lane, run) of every warp; the reference's circular brush of radius r
		// has 2r - 1 runs, fewer than 2 * ceil(sqrt(size)) + 3
		uint32_t sq = 0u;
		while (sq * sq < max_brush) {
			sq++;
		}
		const uint32_t runcap = std::min(max_brush, 2u * sq + 3u);
		const size_t csmem = smem + static_cast<size_t>(runcap) * sizeof(int2)
			+ static_cast<size_t>(kErodeBlock) * runcap * sizeof(float);
		const uint64_t per_job = (static_cast<uint64_t>(max_count) + kErodeBlock - 1u) / kErodeBlock;
		if (per_job * njobs > 0x7FFFFFFFull) {
			return inval("erosion: too many droplets for one launch");
		}
		if (csmem > 48u * 1024u) {
			STPGB_CUDA_TRY(cudaFuncSetAttribute(erosion_coop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
				static_cast<int>(csmem)));
		}
		const uint32_t q = jobs ? std::max(1u, std::min(interleave, njobs)) : 1u;
		erosion_coop_kernel<<<static_cast<uint32_t>(per_job * njobs), kErodeBlock, csmem, stream>>>(jobs, single,
			runcap, njobs, q, static_cast<uint32_t>(per_job));
		STPGB_CUDA_TRY(cudaGetLastError());
		return STPGB_OK;
	}
	if (vector_rows && !exact_clamp && (droplets_per_group == 1u || droplets_per_group == 2u)
		&& (lanes_per_droplet == 2u || lanes_per_droplet == 4u)) {
		const size_t rsmem = smem + static_cast<size_t>(max_brush) * sizeof(BrushRun);
		const uint64_t groups = (static_cast<uint64_t>(max_count) + droplets_per_group - 1u) / droplets_per_group;
		const uint64_t rthreads = groups * lanes_per_droplet;
		if (rthreads > 0xFFFFFFFFull - kErodeBlock) {
			return inval("erosion: too many droplets for one launch");
		}
		const dim3 rgrid(static_cast<uint32_t>((rthreads + kErodeBlock - 1u) / kErodeBlock), njobs);
		auto go = [&](auto kernel) -> int {
			if (rsmem > 48u * 1024u) {
				STPGB_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
					static_cast<int>(rsmem)));
			}
			kernel<<<rgrid, kErodeBlock, rsmem, stream>>>(jobs, single,
				erosion_resident_droplets(lanes_per_droplet, droplets_per_group), wide_trips, atomic_brush);
			STPGB_CUDA_TRY(cudaGetLastError());
			return STPGB_OK;
		};
		switch (lanes_per_droplet * 8u + droplets_per_group) {
		case 2u * 8u + 1u:
			return go(erosion_rows_kernel<2u, 1u>);
		case 2u * 8u + 2u:
			return go(erosion_rows_kernel<2u, 2u>);
		case 4u * 8u + 1u:
			return go(erosion_rows_kernel<4u, 1u>);
		default:
			return go(erosion_rows_kernel<4u, 2u>);
		}
	}
	if (droplets_per_group > 1u) {
		if (exact_clamp || lanes_per_droplet < 4u || (droplets_per_group != 2u && droplets_per_group != 4u)) {
			return inval("erosion: 2 or 4 droplets per group need >= 4 lanes and the reference order");
		}
		const uint64_t groups = (static_cast<uint64_t>(max_count) + droplets_per_group - 1u) / droplets_per_group;
		const uint64_t mthreads = groups * lanes_per_droplet;
		if (mthreads > 0xFFFFFFFFull - kErodeBlock) {
			return inval("erosion: too many droplets for one launch");
		}
		const dim3 mgrid(static_cast<uint32_t>((mthreads + kErodeBlock - 1u) / kErodeBlock), njobs);
		auto go = [&](auto kernel) -> int {
			if (smem > 48u * 1024u) {
				STPGB_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
					static_cast<int>(smem)));
			}
			kernel<<<mgrid, kErodeBlock, smem, stream>>>(jobs, single);
			STPGB_CUDA_TRY(cudaGetLastError());
			return STPGB_OK;
		};
		const uint32_t key = lanes_per_droplet * 8u + droplets_per_group;
		switch (key) {
		case 4u * 8u + 2u:
			return go(erosion_multi_kernel<4u, 2u>);
		case 4u * 8u + 4u:
			return go(erosion_multi_kernel<4u, 4u>);
		case 8u * 8u + 2u:
			return go(erosion_multi_kernel<8u, 2u>);
		case 8u * 8u + 4u:
			return go(erosion_multi_kernel<8u, 4u>);
		case 16u * 8u + 2u:
			return go(erosion_multi_kernel<16u, 2u>);
		case 16u * 8u + 4u:
			return go(erosion_multi_kernel<16u, 4u>);
		default:
			return inval("erosion: droplets per group supported with 4, 8 or 16 lanes");
		}
	}
	const uint64_t threads = static_cast<uint64_t>(max_count) * lanes_per_droplet;
	if (threads > 0xFFFFFFFFull - kErodeBlock) {
		return inval("erosion: too many droplets for one launch");
	}
	const dim3 grid(static_cast<uint32_t>((threads + kErodeBlock - 1u) / kErodeBlock), njobs);
	auto go = [&](auto kernel) -> int {
		if (smem > 48u * 1024u) {
			STPGB_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
		}
		kernel<<<grid, kErodeBlock, smem, stream>>>(jobs, single);
		STPGB_CUDA_TRY(cudaGetLastError());
		return STPGB_OK;
	};
	auto pick = [&](auto ref_order) -> int {
		constexpr bool R = decltype(ref_order)::value;
		switch (lanes_per_droplet) {
		case 1u:
			return go(erosion_kernel<1u, R>);
		case 2u:
			return go(erosion_kernel<2u, R>);
		case 4u:
			return go(erosion_kernel<4u, R>);
		case 8u:
			return go(erosion_kernel<8u, R>);
		case 16u:
			return go(erosion_kernel<16u, R>);
		case 32u:
			return go(erosion_kernel<32u, R>);
		default:
			return inval("erosion: lanes per droplet must be 1, 2, 4, 8, 16 or 32");
		}
	};
	return exact_clamp ? pick(std::true_type {}) : pick(std::false_type {});
}

int format_launch(const float* in, uint64_t in_pitch, uint16_t* out, uint64_t out_pitch, uint32_t W, uint32_t H,
	cudaStream_t stream) {
	const uint64_t threads = static_cast<uint64_t>((W + 7u) / 8u) * H;
	if (threads == 0u) {
		return STPGB_OK;
	}
	format_kernel<<<static_cast<uint32_t>((threads + 255u) / 256u), 256u, 0, stream>>>(in, in_pitch, out, out_pitch, W, H);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int format_batch_launch(const FormatJob* jobs, uint32_t njobs, uint32_t max_W, uint32_t max_H, cudaStream_t stream) {
	const uint64_t threads = static_cast<uint64_t>((max_W + 7u) / 8u) * max_H;
	if (threads == 0u || njobs == 0u) {
		return STPGB_OK;
	}
	format_batch_kernel<<<dim3(static_cast<uint32_t>((threads + 255u) / 256u), njobs), 256u, 0, stream>>>(jobs);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

} // namespace stpgb

using namespace stpgb;

extern "C" {

int stpgb_hydraulic_erosion(float* heightmap, const stpgb_nn_info* nn, const stpgb_raindrop_setting* setting,
	const float* starts_xy, uint32_t count, const int32_t* brush_index, const float* brush_weight,
	uint32_t brush_size, double* residual_sediment, uint32_t* status, void* stream) {
	return stpgb_hydraulic_erosion_ex(heightmap, nn, setting, starts_xy, count, brush_index, brush_weight,
		brush_size, residual_sediment, status, 0u, 1u, 0u, stream);
}

int stpgb_hydraulic_erosion_ex(float* heightmap, const stpgb_nn_info* nn, const stpgb_raindrop_setting* setting,
	const float* starts_xy, uint32_t count, const int32_t* brush_index, const float* brush_weight,
	uint32_t brush_size, double* residual_sediment, uint32_t* status, uint32_t lanes_per_droplet,
	uint32_t droplets_per_group, uint32_t flags,
	void* stream) {
	STPGB_TRY(stpgb_raindrop_setting_validate(setting));
	if (!heightmap || !nn || (count > 0u && !starts_xy) || !brush_index || !brush_weight || brush_size == 0u) {
		return inval("stpgb_hydraulic_erosion: null pointer or empty brush");
	}
	const uint32_t dx = nn->TotalMapSize[0], dy = nn->TotalMapSize[1];
	if (dx <= 2u * setting->ErosionBrushRadius + 1u || dy <= 2u * setting->ErosionBrushRadius + 1u) {
		return inval("stpgb_hydraulic_erosion: map smaller than the erosion brush");
	}
	if (brush_size > 8192u) {
		return inval("stpgb_hydraulic_erosion: brush larger than 8192 points");
	}
	if (static_cast<uint64_t>(dx) * dy >= (uint64_t(1) << 32)) {
		return inval("stpgb_hydraulic_erosion: the map must hold fewer than 2^32 cells");
	}
	ErosionJob job;
	job.map = heightmap;
	job.dim_x = dx;
	job.dim_y = dy;
	job.pitch = dx;
	job.starts = starts_xy;
	job.count = count;
	job.brush_index = brush_index;
	job.brush_weight = brush_weight;
	job.brush_size = brush_size;
	job.p = rain_params(*setting);
	job.residual = residual_sediment;
	job.status = status;
	job.fixed = nullptr;
	job.counters = nullptr;
	job.start_area = nn->MapSize[0] * nn->MapSize[1];
	const bool exact = (flags & STPGB_EROSION_EXACT_CLAMP) != 0u;
	bool rows = !exact && (flags & STPGB_EROSION_POINTWISE) == 0u
		&& (reinterpret_cast<uintptr_t>(heightmap) & 15u) == 0u && (dx & 3u) == 0u;
	uint32_t lanes = lanes_per_droplet, dpg = droplets_per_group == 0u ? 1u : droplets_per_group;
	const double area = static_cast<double>(nn->MapSize[0]) * nn->MapSize[1];
	const double density = static_cast<double>(count) / area;
	if (lanes == 0u) {
		const ErosionChoice c = erosion_choice(setting->ErosionBrushRadius, brush_size, density,
			erosion_in_flight(count, area), rows);
		lanes = c.lanes;
		rows = c.rows;
	}
	return erosion_launch(nullptr, job, 1u, count, brush_size, as_stream(stream), lanes, exact, dpg, rows,
		erosion_rows_wide(setting->ErosionBrushRadius),
		erosion_rows_atomic(setting->ErosionBrushRadius, lanes));
}

int stpgb_erosion_choice(uint32_t brush_radius, uint32_t droplets, uint32_t area, uint32_t* lanes_per_droplet,
	uint32_t* vector_rows) {
	if (brush_radius == 0u || area == 0u || !lanes_per_droplet) {
		return inval("stpgb_erosion_choice: radius and area must be positive");
	}
	uint32_t bs = 0u;
	stpgb_erosion_brush_generate(4u * brush_radius + 4u, brush_radius, nullptr, nullptr, 0u, &bs);
	const ErosionChoice c = erosion_choice(brush_radius, bs, static_cast<double>(droplets) / area,
		erosion_in_flight(droplets, area), true);
	*lanes_per_droplet = c.lanes;
	if (vector_rows) {
		*vector_rows = c.rows ? 1u : 0u;
	}
	return STPGB_OK;
}

int stpgb_format_heightmap(const float* in, uint16_t* out, uint32_t map_x, uint32_t map_y, void* stream) {
	if (!in || !out) {
		return inval("stpgb_format_heightmap: null pointer argument");
	}
	return format_launch(in, map_x, out, map_x, map_x, map_y, as_stream(stream));
}

} // extern "C"
