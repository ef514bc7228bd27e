// Single histogram filter, few-values path, on sm_103a: the palette, the
// sequential-slide formulation for launches of many chunks, and the choice
// between it and the row-band formulation (shf_band.cu) for launches of few.
// Same output as the reference filter
// (SuperTerrain+/SuperAlgorithm+/Host/Private/STPSingleHistogramFilter.cpp),
// bin order included.
//
// In packed form (shf_fast.cuh) a slide step is a few SIMD operations: the
// vertical slide adds and removes one 4-bit index, the horizontal one adds and
// subtracts two columns' counts as eight 16-bit fields; an item that becomes
// present is appended (in the order of the column that brings it), one whose
// count drops to zero is erased, and both are rare on these maps.  The slides
// run as the reference runs them, one thread per column and per row, so the
// order is the reference's by construction.
//
//   shf_palette       block per (32-row tile of the read region, job):
//                     distinct values through a 65536-bit map in shared
//                     memory.
//   shf_route         thread per job: the path (few-values or general).
//   shf_vertical_fast thread per column: slides the column's vertical
//                     histogram down all rows and writes it to row-major
//                     planes in the job's vbuf.
//   shf_rows_fast     thread per row: the horizontal slide; COUNT writes the
//                     bins per row (before the row scan), WRITE the offsets
//                     and bins (after it).
#include "shf_fast.cuh"

#include <algorithm>

namespace stpgb {

using namespace shfx;

namespace {

constexpr uint32_t kPaletteBlock = 256u;
constexpr uint32_t kVertBlock = 64u;
constexpr uint32_t kRowBlock = 64u;
// rows of the vertical slide whose samples are loaded ahead of their use
constexpr uint32_t kVertAhead = 16u;
// local indices of a column's last kRing samples (>= 2r+2)
constexpr uint32_t kRing = 256u;
// Launches with fewer rows than this many per SM (rows of all chunks) take
// the row bands: one thread per row would leave the SMs nearly idle.
constexpr uint64_t kSlideRowsPerSM = 256u;

// ---------------------------------------------------------------- routing --

// Thread 0 per job: the union of its palette tiles decides its path -- the
// few-values path when it holds at most kShfFastItems values, no accumulator
// of the reference could overflow and the chunk is within the formulation's
// column bound, else the general slides.
__global__ void shf_route(const ShfJob* __restrict__ jobs, const ShfJob single, const uint32_t kcap_h,
	const uint32_t dense_max_cols, const uint32_t dense_form) {
	const ShfJob& J = pick(jobs, single);
	if (threadIdx.x != 0u) {
		return;
	}
	uint32_t vals[kShfFastItems];
	uint32_t n = 0u;
	const bool fits = palette_union(J, vals, n);
	const uint64_t side = 2ull * J.r + 1u;
	const uint64_t items = n;
	const bool radius_ok = J.r <= kFastMaxRadius;
	// the packed vertical histograms (12 bytes per column and row, or per band) fit in vbuf
	// (4 * kcap_v bytes per column and row)
	const bool dense = fits && radius_ok && J.W + 2u * J.r <= dense_max_cols
		&& min(items, side + 1u) <= J.kcap_v && min(items, (side + 1u) * side) <= kcap_h && J.kcap_v >= 3u;
	write_record(J, dense ? kShfModeFast : kShfModeSlide, dense ? n : 0u, vals, dense_form);
}

// ---------------------------------------------------------------- palette --

__global__ void __launch_bounds__(kPaletteBlock) shf_palette(const ShfJob* __restrict__ jobs, const ShfJob single) {
	const ShfJob& J = pick(jobs, single);
	const uint32_t NR = J.H + 2u * J.r, NC = J.W + 2u * J.r;
	const uint32_t r0 = blockIdx.x * kShfPaletteRows;
	if (r0 >= NR) {
		return;
	}
	const uint32_t r1 = min(NR, r0 + kShfPaletteRows);
	__shared__ uint32_t bits[2048];
	// distinct values found so far: every bit is counted once, by the thread whose atomicOr set it
	__shared__ uint32_t seen, fill;
	__shared__ uint32_t vals[kShfFastItems];
	for (uint32_t i = threadIdx.x; i < 2048u; i += kPaletteBlock) {
		bits[i] = 0u;
	}
	if (threadIdx.x == 0u) {
		seen = 0u;
		fill = 0u;
	}
	__syncthreads();
	const uint16_t* const base = read_region(J);
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t span = (NC + kPaletteBlock - 1u) / kPaletteBlock * kPaletteBlock;
	const volatile uint32_t& seen_now = seen;
	for (uint32_t row = r0; row < r1; row++) {
		// a tile past kShfFastItems values sends its job to the general slides: stop reading
		// (warp-uniform, so every lane of a warp leaves the match below together)
		if (__any_sync(0xFFFFFFFFu, seen_now > kShfFastItems)) {
			break;
		}
		const uint16_t* const src = base + static_cast<uint64_t>(row) * J.pitch;
		for (uint32_t c = threadIdx.x; c < span; c += kPaletteBlock) {
			const uint32_t v = c < NC ? static_cast<uint32_t>(__ldg(src + c)) : kNoValue;
			// one lane per distinct value of the warp sets its bit
			const uint32_t same = __match_any_sync(0xFFFFFFFFu, v);
			if (v != kNoValue && static_cast<uint32_t>(__ffs(same) - 1) == lane) {
				const uint32_t bit = 1u << (v & 31u);
				if (!(bits[v >> 5] & bit) && !(atomicOr(&bits[v >> 5], bit) & bit)) {
					atomicAdd(&seen, 1u);
				}
			}
		}
	}
	__syncthreads();
	const uint32_t n = seen;
	if (n <= kShfFastItems) {
		for (uint32_t i = threadIdx.x; i < 2048u; i += kPaletteBlock) {
			uint32_t w = bits[i];
			while (w) {
				const uint32_t b = static_cast<uint32_t>(__ffs(w) - 1);
				w &= w - 1u;
				vals[atomicAdd(&fill, 1u)] = i * 32u + b;
			}
		}
	}
	__syncthreads();
	if (threadIdx.x == 0u) {
		uint32_t* const slot = J.fast + kSlotWords * (1u + blockIdx.x);
		const bool fits = n <= kShfFastItems;
		slot[0] = fits ? n : kNoValue;
		for (uint32_t q = 0u; q < kShfFastItems / 2u; q++) {
			const uint32_t lo = fits && 2u * q < n ? vals[2u * q] : 0u;
			const uint32_t hi = fits && 2u * q + 1u < n ? vals[2u * q + 1u] : 0u;
			slot[2u + q] = lo | (hi << 16);
		}
	}
}

// --------------------------------------------------------------- vertical --

// Thread per column k of the read region: the vertical histogram of rows
// [y, y+2r] (relative to the region) for y = 0..H-1, slid as the reference
// slides it (:522-563), written for every row to two row-major planes in
// vbuf: counts [H][W+2r] (8 bytes) and orders [H][W+2r] (4-bit indices), so
// that a warp's stores are consecutive.  The local indices of a column's last
// kRing samples stay in shared memory, so only the entering sample is read
// from global memory, kVertAhead rows early.
__global__ void __launch_bounds__(kVertBlock) shf_vertical_fast(const ShfJob* __restrict__ jobs, const ShfJob single) {
	const ShfJob& J = pick(jobs, single);
	const ShfFastRecord* const rec = reinterpret_cast<const ShfFastRecord*>(J.fast);
	__shared__ uint8_t ring[kRing][kVertBlock];
	const uint32_t NC = J.W + 2u * J.r;
	const uint32_t k = blockIdx.x * kVertBlock + threadIdx.x;
	if (rec->mode != kShfModeFast || k >= NC) {
		return;
	}
	const Palette pal = record_palette(rec);
	const uint64_t pitch = J.pitch;
	const uint32_t H = J.H, r2 = 2u * J.r;
	const uint16_t* src = read_region(J) + k; // the next sample to load
	uint64_t* cv = reinterpret_cast<uint64_t*>(J.vbuf) + k;
	uint32_t* ov = reinterpret_cast<uint32_t*>(reinterpret_cast<uint64_t*>(J.vbuf) + static_cast<size_t>(NC) * H) + k;
	uint8_t* const mine = &ring[0][threadIdx.x];
	uint64_t cnt = 0ull;
	uint32_t order = 0u;
	for (uint32_t q = 0u; q <= r2; q++) {
		const uint32_t li = local_index(pal, __ldg(src));
		src += pitch;
		mine[(q & (kRing - 1u)) * kVertBlock] = static_cast<uint8_t>(li);
		hist_add(cnt, order, li);
	}
	cv[0] = cnt;
	ov[0] = order;
	// row y adds region row y+2r (prefetched) and removes row y-1 (from the ring)
	uint32_t pre[kVertAhead];
#pragma unroll
	for (uint32_t i = 0u; i < kVertAhead; i++) {
		pre[i] = 1u + i < H ? __ldg(src + i * pitch) : 0u;
	}
	src += kVertAhead * pitch;
	for (uint32_t y = 1u; y < H; y += kVertAhead) {
#pragma unroll
		for (uint32_t i = 0u; i < kVertAhead; i++) {
			const uint32_t yy = y + i;
			if (yy < H) {
				const uint32_t li = local_index(pal, pre[i]);
				if (yy + kVertAhead < H) {
					pre[i] = __ldg(src);
				}
				src += pitch;
				const uint32_t lo = mine[((yy - 1u) & (kRing - 1u)) * kVertBlock];
				mine[((yy + r2) & (kRing - 1u)) * kVertBlock] = static_cast<uint8_t>(li);
				if (li != lo) {
					hist_add(cnt, order, li);
					hist_sub(cnt, order, lo);
				}
				cv[static_cast<size_t>(yy) * NC] = cnt;
				ov[static_cast<size_t>(yy) * NC] = order;
			}
		}
	}
}

// ------------------------------------------------------------- horizontal --

// Thread per row y: the reference's horizontal slide (:608-679) over the
// packed vertical histograms of the row: counts as eight 16-bit fields, the
// accumulator's order as 4-bit indices.  A column's items enter in the order
// of its vertical histogram when they are absent, an item whose count drops to
// zero is erased; a step whose entering and leaving columns hold the same
// counts changes nothing.  The row's bins (item, weight) in order are kept in
// registers and rebuilt when the counts change.  COUNT: bins per row; WRITE:
// offsets and bins from the row's base, offsets four at a time and bins in
// pairs as 16-byte stores where the buffers are 16-byte aligned.
template<bool Write>
__global__ void __launch_bounds__(kRowBlock) shf_rows_fast(const ShfJob* __restrict__ jobs, const ShfJob single) {
	const ShfJob& J = pick(jobs, single);
	if (reinterpret_cast<const ShfFastRecord*>(J.fast)->mode != kShfModeFast) {
		return;
	}
	const uint32_t H = J.H, W = J.W, r2 = 2u * J.r, NC = W + r2;
	const uint32_t y = blockIdx.x * kRowBlock + threadIdx.x;
	if (y >= H) {
		return;
	}
	const ShfFastRecord* const rec = reinterpret_cast<const ShfFastRecord*>(J.fast);
	const uint64_t* const cv = reinterpret_cast<const uint64_t*>(J.vbuf) + static_cast<size_t>(y) * NC;
	const uint32_t* const ov = reinterpret_cast<const uint32_t*>(reinterpret_cast<const uint64_t*>(J.vbuf)
								   + static_cast<size_t>(NC) * H)
		+ static_cast<size_t>(y) * NC;
	uint4 hc = make_uint4(0u, 0u, 0u, 0u);
	uint32_t order = 0u, n = 0u;
	// absent items of column k (counts wa) enter in its vertical order
	auto insert = [&](const uint32_t k, const uint4 wa, uint32_t fresh) {
		uint32_t vo = __ldg(ov + k);
		for (uint32_t left = __popc(present_mask(wa)); left > 0u && fresh; left--, vo >>= 4) {
			const uint32_t j = vo & 15u;
			if ((fresh >> j) & 1u) {
				order |= j << (4u * n);
				n++;
				fresh &= ~(1u << j);
			}
		}
	};
	auto erase = [&](uint32_t gone) {
		while (gone) {
			const uint32_t j = static_cast<uint32_t>(__ffs(gone) - 1);
			gone &= gone - 1u;
			const uint32_t low = (1u << (4u * place_of(order, j))) - 1u;
			order = (order & low) | ((order >> 4) & ~low);
			n--;
		}
	};
	// one step: add column k's counts a, then remove counts b (b = 0 in the fill)
	auto step = [&](const uint32_t k, const uint64_t a, const uint64_t b) {
		const uint4 wa = widen(a), wb = widen(b);
		const uint4 za = zero4(hc);
		const uint4 h1 = add4(hc, wa);
		hc = sub4(h1, wb);
		const uint4 zw = zero4(wa), zb = zero4(wb), zh = zero4(hc);
		// fresh: zero before, brought by a; gone: brought by b (so present after the add), zero now
		const uint4 f = make_uint4(za.x & ~zw.x, za.y & ~zw.y, za.z & ~zw.z, za.w & ~zw.w);
		const uint4 g = make_uint4(zh.x & ~zb.x, zh.y & ~zb.y, zh.z & ~zb.z, zh.w & ~zb.w);
		if (f.x | f.y | f.z | f.w) {
			insert(k, wa, present_mask(f));
		}
		if (g.x | g.y | g.z | g.w) {
			erase(present_mask(g));
		}
	};
	for (uint32_t k = 0u; k <= r2; k++) {
		step(k, __ldg(cv + k), 0ull);
	}

	uint64_t o = 0u; // running bin index
	uint32_t* off_row = nullptr;
	uint2* bins = nullptr;
	bool off_vec = false, bin_vec = false;
	uint32_t q0 = 0u, q1 = 0u, q2 = 0u, q3 = 0u; // the last four offsets
	uint2 pend = make_uint2(0u, 0u);
	bool has_pend = false;
	uint4 items = make_uint4(0u, 0u, 0u, 0u); // the palette values as 16-bit fields
	float norm = 0.0f;
	uint2 e[kShfFastItems]; // the current bins in order
	// read once: the bins stores below could alias the job table as far as the compiler knows
	const uint64_t cap = J.bins_capacity;
	if constexpr (Write) {
		o = J.rows[y];
		off_row = J.offsets + static_cast<size_t>(y) * W;
		bins = reinterpret_cast<uint2*>(J.bins);
		off_vec = (reinterpret_cast<uintptr_t>(off_row) & 15u) == 0u;
		bin_vec = (reinterpret_cast<uintptr_t>(bins) & 15u) == 0u;
		const uint32_t* const iw = reinterpret_cast<const uint32_t*>(rec->item);
		items = make_uint4(iw[0], iw[1], iw[2], iw[3]);
		const uint32_t side = r2 + 1u;
		norm = __fdiv_rn(1.0f, static_cast<float>(side * side));
	}
	// the bins of the current state, n of them (most pixels hold one or two)
	auto rebuild = [&]() {
		if constexpr (Write) {
			uint32_t ord = order;
#pragma unroll
			for (uint32_t p = 0u; p < kShfFastItems; p++, ord >>= 4) {
				if (p >= n) {
					break;
				}
				const uint32_t j = ord & 15u;
				const float w = __fmul_rn(__uint2float_rn(field(hc, j)), norm);
				e[p] = make_uint2(field(items, j), __float_as_uint(w));
			}
		}
	};
	auto put_bin = [&](const uint2 b) {
		if (bin_vec && (o & 1u) && has_pend) {
			if (o < cap) {
				*reinterpret_cast<uint4*>(bins + o - 1u) = make_uint4(pend.x, pend.y, b.x, b.y);
			} else if (o - 1u < cap) {
				bins[o - 1u] = pend;
			}
			has_pend = false;
		} else if (bin_vec && !(o & 1u)) {
			pend = b;
			has_pend = true;
		} else if (o < cap) {
			bins[o] = b;
		}
		o++;
	};
	auto emit = [&](const uint32_t x) {
		if constexpr (Write) {
			const uint32_t v = static_cast<uint32_t>(o);
			if (off_vec) {
				q0 = q1;
				q1 = q2;
				q2 = q3;
				q3 = v;
				if ((x & 3u) == 3u) {
					*reinterpret_cast<uint4*>(off_row + x - 3u) = make_uint4(q0, q1, q2, q3);
				}
			} else {
				off_row[x] = v;
			}
#pragma unroll
			for (uint32_t p = 0u; p < kShfFastItems; p++) {
				if (p >= n) {
					break;
				}
				put_bin(e[p]);
			}
		} else {
			o += n;
		}
	};
	rebuild();
	emit(0u);
	// Step x adds column x+2r and removes column x-1.  Each row's counts are a
	// stream of its own (16 steps per 128-byte line); the line two ahead of
	// each stream is asked into L1 when a stream enters a line.
	const uint64_t* pa_src = cv + r2 + 1u;
	const uint64_t* pb_src = cv;
	for (uint32_t x = 1u; x < W; x++, pa_src++, pb_src++) {
		if (x + 32u < W) { // both prefetched addresses stay inside the row
			if ((reinterpret_cast<uintptr_t>(pa_src) & 127u) == 0u) {
				prefetch_l1(pa_src + 32);
			}
			if ((reinterpret_cast<uintptr_t>(pb_src) & 127u) == 0u) {
				prefetch_l1(pb_src + 32);
			}
		}
		const uint64_t a = __ldg(pa_src), b = __ldg(pb_src);
		if (a != b) {
			step(x + r2, a, b);
			rebuild();
		}
		emit(x);
	}
	if constexpr (Write) {
		// what is still held: offsets after the last full quad, and a bin without its pair
		if (off_vec) {
			const uint32_t rem = W & 3u;
			if (rem >= 3u) {
				off_row[W - 3u] = q1;
			}
			if (rem >= 2u) {
				off_row[W - 2u] = q2;
			}
			if (rem >= 1u) {
				off_row[W - 1u] = q3;
			}
		}
		if (has_pend && o - 1u < cap) {
			bins[o - 1u] = pend;
		}
	} else {
		J.rows[y] = static_cast<uint32_t>(min(o, static_cast<uint64_t>(0xFFFFFFFFu)));
	}
}

} // namespace

ShfFastPlan shf_fast_plan(const uint32_t njobs, const uint32_t max_W, const uint32_t max_H, const uint32_t max_r,
	const uint32_t path) {
	ShfFastPlan plan {};
	const uint32_t choice = path != 0u ? path : shf_path_override();
	plan.bands = choice == 2u
		|| (choice == 0u && static_cast<uint64_t>(njobs) * max_H < kSlideRowsPerSM * current_sm_count());
	plan.max_cols = choice == 3u ? 0u : plan.bands ? kShfBandMaxCols : 0xFFFFFFFFu;
	if (plan.bands) {
		plan.band = shf_band_config(njobs, max_W, max_H, max_r);
	}
	return plan;
}

int shf_fast_prepare(const ShfJob* jobs, const ShfJob& single, const uint32_t njobs, const uint32_t max_W,
	const uint32_t max_H, const uint32_t max_r, const uint32_t kcap_h, const ShfFastPlan& plan, cudaStream_t stream) {
	const uint32_t tiles = (max_H + 2u * max_r + kShfPaletteRows - 1u) / kShfPaletteRows;
	shf_palette<<<dim3(tiles, njobs), kPaletteBlock, 0, stream>>>(jobs, single);
	STPGB_CUDA_TRY(cudaGetLastError());
	shf_route<<<dim3(1u, njobs), 32u, 0, stream>>>(jobs, single, kcap_h, plan.max_cols,
		plan.bands ? kShfFormBands : kShfFormSlides);
	STPGB_CUDA_TRY(cudaGetLastError());
	if (plan.bands) {
		STPGB_TRY(shf_band_carry_launch(jobs, single, njobs, max_W, max_r, plan.band, stream));
	} else {
		const uint32_t ncols = max_W + 2u * max_r;
		shf_vertical_fast<<<dim3((ncols + kVertBlock - 1u) / kVertBlock, njobs), kVertBlock, 0, stream>>>(jobs,
			single);
		STPGB_CUDA_TRY(cudaGetLastError());
	}
	return STPGB_OK;
}

int shf_fast_pass(const ShfJob* jobs, const ShfJob& single, const uint32_t njobs, const uint32_t max_H,
	const ShfFastPlan& plan, const bool write, cudaStream_t stream) {
	if (plan.bands) {
		STPGB_TRY(shf_band_rows_launch(jobs, single, njobs, plan.band, write, stream));
	} else {
		const dim3 grid((max_H + kRowBlock - 1u) / kRowBlock, njobs);
		if (write) {
			shf_rows_fast<true><<<grid, kRowBlock, 0, stream>>>(jobs, single);
		} else {
			shf_rows_fast<false><<<grid, kRowBlock, 0, stream>>>(jobs, single);
		}
		STPGB_CUDA_TRY(cudaGetLastError());
	}
	return STPGB_OK;
}

} // namespace stpgb
