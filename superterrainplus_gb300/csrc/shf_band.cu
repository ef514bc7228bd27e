// Single histogram filter, few-values path, row-band formulation, on sm_103a:
// the one for launches of few chunks, where a thread per row or column would
// leave most of the GPU idle.  Same output as the reference filter
// (SuperTerrain+/SuperAlgorithm+/Host/Private/STPSingleHistogramFilter.cpp),
// bin order included.
//
// Horizontally the order follows from a rule that makes every pixel
// independent of the slide: when column k's vertical histogram is added, an
// item is inserted iff none of columns [max(0, k-2r-1), k-1] holds it (before
// the add, the window holds exactly those columns; the initial fill is the
// case k <= 2r).  An item present at pixel x was last inserted at the latest
// such column k0 <= x+2r, in the place it has in column k0's vertical
// histogram, and erasures keep the relative order of what remains, so the bins
// of pixel x are its present items sorted by (k0, place in column k0's
// histogram).  Windowed counts and "latest insertion column" are prefix scans
// over the columns of a row: one sum scan and one max scan of eight 16-bit
// fields per column, so a block computes a whole row at once.
//
//   shf_band_carry thread per column: slides the column's vertical histogram
//                  down all rows and keeps its state at the first row of
//                  every band.
//   shf_band_rows  block per (band of rows, job), thread per column(s): per
//                  row, the vertical step, the count scan, the insertion scan
//                  and the pixels' bins (COUNT: bins per row; WRITE: offsets
//                  and bins after the row scan).
#include "shf_fast.cuh"

#include <algorithm>

namespace stpgb {

using namespace shfx;

namespace {

constexpr uint32_t kCarryBlock = 64u;
constexpr uint32_t kFastMaxThreads = 1024u;
// rows of the carry's slide whose entering samples are loaded ahead of their
// use, and the ring of a column's last samples (>= 2r+2)
constexpr uint32_t kAhead = 16u;
constexpr uint32_t kRing = 256u;

// ------------------------------------------------------------------ carry --

// Thread per column k of the read region: the vertical histogram of rows
// [y, y+2r] (relative to the region) for y = 0..H-1, slid as the reference
// slides it (:522-563), stored at y = 0, band_rows, 2 band_rows, ...:
// counts [bands][W+2r] (8 bytes), then orders [bands][W+2r] (4-bit indices).
__global__ void __launch_bounds__(kCarryBlock) shf_band_carry(const ShfJob* __restrict__ jobs, const ShfJob single,
	const uint32_t band_rows) {
	const ShfJob& J = pick(jobs, single);
	const ShfFastRecord* const rec = reinterpret_cast<const ShfFastRecord*>(J.fast);
	const uint32_t NC = J.W + 2u * J.r;
	const uint32_t k = blockIdx.x * kCarryBlock + threadIdx.x;
	if (rec->mode != kShfModeFast || k >= NC) {
		return;
	}
	const Palette pal = record_palette(rec);
	const uint16_t* const col = read_region(J) + k;
	const uint64_t pitch = J.pitch;
	const uint32_t H = J.H, r2 = 2u * J.r;
	const uint32_t bands = (H + band_rows - 1u) / band_rows;
	uint64_t* const cvc = reinterpret_cast<uint64_t*>(J.vbuf);
	uint32_t* const cvo = reinterpret_cast<uint32_t*>(cvc + static_cast<size_t>(bands) * NC);
	auto at = [&](const uint32_t q) {
		return static_cast<uint32_t>(__ldg(col + static_cast<uint64_t>(q) * pitch));
	};
	// the local indices of the column's last kRing samples: the leaving sample
	// of a row is read from here, only the entering one from global memory,
	// kAhead rows early
	__shared__ uint8_t ring[kRing][kCarryBlock];
	uint8_t* const mine = &ring[0][threadIdx.x];
	uint64_t cnt = 0ull;
	uint32_t order = 0u;
	for (uint32_t q = 0u; q <= r2; q++) {
		const uint32_t li = local_index(pal, at(q));
		mine[(q & (kRing - 1u)) * kCarryBlock] = static_cast<uint8_t>(li);
		hist_add(cnt, order, li);
	}
	cvc[k] = cnt;
	cvo[k] = order;
	// row y adds region row y+2r and removes row y-1
	const uint16_t* src = col + static_cast<uint64_t>(r2 + 1u + kAhead) * pitch;
	uint32_t pre[kAhead];
#pragma unroll
	for (uint32_t i = 0u; i < kAhead; i++) {
		pre[i] = 1u + i < H ? at(r2 + 1u + i) : 0u;
	}
	uint32_t next_band = band_rows; // rows before the next band's first row
	size_t band_at = NC + k;
	for (uint32_t y = 1u; y < H; y += kAhead) {
#pragma unroll
		for (uint32_t i = 0u; i < kAhead; i++) {
			const uint32_t yy = y + i;
			if (yy < H) {
				const uint32_t li = local_index(pal, pre[i]);
				if (yy + kAhead < H) {
					pre[i] = __ldg(src);
				}
				src += pitch;
				const uint32_t lo = mine[((yy - 1u) & (kRing - 1u)) * kCarryBlock];
				mine[((yy + r2) & (kRing - 1u)) * kCarryBlock] = static_cast<uint8_t>(li);
				if (li != lo) {
					hist_add(cnt, order, li);
					hist_sub(cnt, order, lo);
				}
				if (--next_band == 0u) {
					cvc[band_at] = cnt;
					cvo[band_at] = order;
					band_at += NC;
					next_band = band_rows;
				}
			}
		}
	}
}

// ------------------------------------------------------------------- rows --

__device__ __forceinline__ uint4 max4(const uint4 a, const uint4 b) {
	return make_uint4(__vmaxu2(a.x, b.x), __vmaxu2(a.y, b.y), __vmaxu2(a.z, b.z), __vmaxu2(a.w, b.w));
}
__device__ __forceinline__ uint4 shfl_up4(const uint4 v, const uint32_t d) {
	return make_uint4(__shfl_up_sync(0xFFFFFFFFu, v.x, d), __shfl_up_sync(0xFFFFFFFFu, v.y, d),
		__shfl_up_sync(0xFFFFFFFFu, v.z, d), __shfl_up_sync(0xFFFFFFFFu, v.w, d));
}

struct AddOp {
	__device__ __forceinline__ uint4 operator()(const uint4 a, const uint4 b) const {
		return add4(a, b);
	}
};
struct MaxOp {
	__device__ __forceinline__ uint4 operator()(const uint4 a, const uint4 b) const {
		return max4(a, b);
	}
};

// Exclusive scan of one uint4 per thread over the block (identity 0), with
// `wt` (32 entries) for the warp totals; `total` gets the whole block's.
template<class Op>
__device__ __forceinline__ uint4 block_exscan(const uint4 v, uint4* const wt, uint4& total, const Op op) {
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
	uint4 inc = v;
#pragma unroll
	for (uint32_t d = 1u; d < 32u; d <<= 1) {
		const uint4 t = shfl_up4(inc, d);
		if (lane >= d) {
			inc = op(inc, t);
		}
	}
	uint4 ex = shfl_up4(inc, 1u);
	if (lane == 0u) {
		ex = zero;
	}
	if (lane == 31u) {
		wt[warp] = inc;
	}
	__syncthreads();
	if (warp == 0u) {
		uint4 s = lane < nw ? wt[lane] : zero;
#pragma unroll
		for (uint32_t d = 1u; d < 32u; d <<= 1) {
			const uint4 t = shfl_up4(s, d);
			if (lane >= d) {
				s = op(s, t);
			}
		}
		if (lane < nw) {
			wt[lane] = s;
		}
	}
	__syncthreads();
	total = wt[nw - 1u];
	return warp ? op(wt[warp - 1u], ex) : ex;
}

__device__ __forceinline__ uint32_t block_exscan_u32(const uint32_t v, uint32_t* const wt, uint32_t& total) {
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	uint32_t inc = v;
#pragma unroll
	for (uint32_t d = 1u; d < 32u; d <<= 1) {
		const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, d);
		if (lane >= d) {
			inc += t;
		}
	}
	if (lane == 31u) {
		wt[warp] = inc;
	}
	__syncthreads();
	if (warp == 0u) {
		uint32_t s = lane < nw ? wt[lane] : 0u;
#pragma unroll
		for (uint32_t d = 1u; d < 32u; d <<= 1) {
			const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, s, d);
			if (lane >= d) {
				s += t;
			}
		}
		if (lane < nw) {
			wt[lane] = s;
		}
	}
	__syncthreads();
	total = wt[nw - 1u];
	return (warp ? wt[warp - 1u] : 0u) + inc - v;
}

// Block (band of rows [b*band_rows, ...), job); thread t owns columns and
// pixels [t*cpt, t*cpt+cpt), cpt = ceil((W+2r) / threads) <= Cols.
// Shared memory: counts prefix P[W+2r+1], insertion scan M[W+2r] (uint4:
// eight 16-bit fields), three sets of 32 warp totals, orders[W+2r].
// Per row y: P[k] = counts of columns < k (the window of pixel x is
// P[x+2r+1] - P[x]); column k inserts item j iff it holds j and columns
// [max(0, k-2r-1), k-1] do not (P[k] - P[lo] == 0); M[k] = 1 + the latest
// such column <= k, per item.
template<bool Write, uint32_t Cols>
__global__ void __launch_bounds__(kFastMaxThreads) shf_band_rows(const ShfJob* __restrict__ jobs, const ShfJob single,
	const uint32_t band_rows, const uint32_t max_cols) {
	const ShfJob& J = pick(jobs, single);
	const ShfFastRecord* const rec = reinterpret_cast<const ShfFastRecord*>(J.fast);
	if (rec->mode != kShfModeFast) {
		return;
	}
	const uint32_t y0 = blockIdx.x * band_rows;
	if (y0 >= J.H) {
		return;
	}
	const uint32_t y1 = min(J.H, y0 + band_rows);
	const uint32_t W = J.W, r2 = 2u * J.r, NC = W + r2;
	const uint32_t cpt = (NC + blockDim.x - 1u) / blockDim.x;
	const uint32_t k0 = threadIdx.x * cpt;
	extern __shared__ uint4 fsm[];
	uint4* const P = fsm;
	uint4* const M = P + max_cols + 1u;
	uint4* const wt = M + max_cols;
	uint32_t* const ord = reinterpret_cast<uint32_t*>(wt + 96u);
	__shared__ uint32_t s_item[kShfFastItems];
	const uint32_t* const rw = reinterpret_cast<const uint32_t*>(rec->item);
	const uint32_t ncount = rec->count;
	auto half = [&](const uint32_t j) {
		return j < ncount ? ((rw[j / 2u] >> (16u * (j & 1u))) & 0xFFFFu) : 0xFFFFu;
	};
	const Palette pal = make_uint4(half(0) | (half(1) << 16), half(2) | (half(3) << 16), half(4) | (half(5) << 16),
		half(6) | (half(7) << 16));
	if (threadIdx.x < kShfFastItems) {
		s_item[threadIdx.x] = rec->item[threadIdx.x];
	}
	const uint32_t bands = (J.H + band_rows - 1u) / band_rows;
	const uint64_t* const cvc = reinterpret_cast<const uint64_t*>(J.vbuf);
	const uint32_t* const cvo = reinterpret_cast<const uint32_t*>(cvc + static_cast<size_t>(bands) * NC);
	const uint16_t* const base = read_region(J);
	const uint64_t pitch = J.pitch;
	uint64_t cnt[Cols];
	uint32_t order[Cols], na[Cols], nb[Cols];
	auto owned = [&](const uint32_t c) {
		return c < cpt && k0 + c < NC;
	};
#pragma unroll
	for (uint32_t c = 0u; c < Cols; c++) {
		if (owned(c)) {
			const size_t o = static_cast<size_t>(blockIdx.x) * NC + k0 + c;
			cnt[c] = cvc[o];
			order[c] = cvo[o];
		} else {
			cnt[c] = 0ull;
			order[c] = 0u;
		}
		na[c] = nb[c] = 0u;
	}
	// samples of row y: region row y+2r enters, row y-1 leaves
	auto load_row = [&](const uint32_t y) {
		if (y < y1) {
#pragma unroll
			for (uint32_t c = 0u; c < Cols; c++) {
				if (owned(c)) {
					na[c] = __ldg(base + static_cast<uint64_t>(y + r2) * pitch + k0 + c);
					nb[c] = __ldg(base + static_cast<uint64_t>(y - 1u) * pitch + k0 + c);
				}
			}
		}
	};
	load_row(y0 + 1u);
	const uint32_t side = r2 + 1u;
	const float norm = __fdiv_rn(1.0f, static_cast<float>(side * side));
	uint2* const bins = reinterpret_cast<uint2*>(J.bins);
	const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
	__syncthreads(); // s_item

	for (uint32_t y = y0; y < y1; y++) {
		if (y > y0) {
#pragma unroll
			for (uint32_t c = 0u; c < Cols; c++) {
				if (owned(c) && na[c] != nb[c]) {
					hist_add(cnt[c], order[c], local_index(pal, na[c]));
					hist_sub(cnt[c], order[c], local_index(pal, nb[c]));
				}
			}
			load_row(y + 1u);
		}
		// counts prefix
		uint4 run = zero;
#pragma unroll
		for (uint32_t c = 0u; c < Cols; c++) {
			if (owned(c)) {
				run = add4(run, widen(cnt[c]));
			}
		}
		uint4 tot;
		uint4 acc = block_exscan(run, wt, tot, AddOp {});
#pragma unroll
		for (uint32_t c = 0u; c < Cols; c++) {
			if (owned(c)) {
				P[k0 + c] = acc;
				ord[k0 + c] = order[c];
				acc = add4(acc, widen(cnt[c]));
			}
		}
		if (threadIdx.x == 0u) {
			P[NC] = tot;
		}
		__syncthreads();
		if constexpr (Write) {
			// insertion columns, as 1 + column per item, and their running maximum
			auto inserts = [&](const uint32_t c) {
				const uint32_t k = k0 + c;
				const uint4 win = sub4(P[k], P[k > r2 ? k - r2 - 1u : 0u]);
				const uint4 w = widen(cnt[c]);
				const uint32_t kk = (k + 1u) * 0x00010001u;
				return make_uint4(__vcmpeq2(win.x, 0u) & __vcmpne2(w.x, 0u) & kk,
					__vcmpeq2(win.y, 0u) & __vcmpne2(w.y, 0u) & kk, __vcmpeq2(win.z, 0u) & __vcmpne2(w.z, 0u) & kk,
					__vcmpeq2(win.w, 0u) & __vcmpne2(w.w, 0u) & kk);
			};
			uint4 mrun = zero;
#pragma unroll
			for (uint32_t c = 0u; c < Cols; c++) {
				if (owned(c)) {
					mrun = max4(mrun, inserts(c));
				}
			}
			uint4 mtot;
			uint4 macc = block_exscan(mrun, wt + 32u, mtot, MaxOp {});
#pragma unroll
			for (uint32_t c = 0u; c < Cols; c++) {
				if (owned(c)) {
					macc = max4(macc, inserts(c));
					M[k0 + c] = macc;
				}
			}
			__syncthreads();
		}
		// pixels x = k0 + c < W
		uint32_t mine = 0u;
#pragma unroll
		for (uint32_t c = 0u; c < Cols; c++) {
			const uint32_t x = k0 + c;
			if (c < cpt && x < W) {
				mine += __popc(present_mask(sub4(P[x + r2 + 1u], P[x])));
			}
		}
		uint32_t all;
		const uint32_t before = block_exscan_u32(mine, reinterpret_cast<uint32_t*>(wt + 64u), all);
		if constexpr (!Write) {
			if (threadIdx.x == 0u) {
				J.rows[y] = all;
			}
		} else {
			uint64_t o = static_cast<uint64_t>(J.rows[y]) + before;
			uint32_t* const off_row = J.offsets + static_cast<size_t>(y) * W;
			auto put = [&](const uint32_t j, const uint4 hc) {
				if (o < J.bins_capacity) {
					const float w = __fmul_rn(__uint2float_rn(field(hc, j)), norm);
					bins[o] = make_uint2(s_item[j], __float_as_uint(w));
				}
				o++;
			};
#pragma unroll
			for (uint32_t c = 0u; c < Cols; c++) {
				const uint32_t x = k0 + c;
				if (c < cpt && x < W) {
					const uint4 hc = sub4(P[x + r2 + 1u], P[x]);
					const uint32_t pm = present_mask(hc);
					off_row[x] = static_cast<uint32_t>(o);
					// a window always holds (2r+1)^2 samples, so pm != 0
					if (pm != 0u && (pm & (pm - 1u)) == 0u) {
						put(static_cast<uint32_t>(__ffs(pm) - 1), hc);
					} else if (pm != 0u) {
						// present items by (insertion column, place in its vertical histogram)
						const uint4 m = M[x + r2];
						uint32_t key[kShfFastItems];
#pragma unroll
						for (uint32_t j = 0u; j < kShfFastItems; j++) {
							key[j] = 0xFFFFFFFFu;
							if ((pm >> j) & 1u) {
								// every present item has an insertion column (the clamp only keeps a
								// broken invariant inside the tables)
								const uint32_t kc = min(field(m, j) - 1u, NC - 1u);
								key[j] = (kc << 3) | place_of(ord[kc], j);
							}
						}
						for (uint32_t left = __popc(pm); left > 0u; left--) {
							uint32_t best = 0u, bk = key[0];
#pragma unroll
							for (uint32_t j = 1u; j < kShfFastItems; j++) {
								if (key[j] < bk) {
									bk = key[j];
									best = j;
								}
							}
#pragma unroll
							for (uint32_t j = 0u; j < kShfFastItems; j++) {
								if (j == best) {
									key[j] = 0xFFFFFFFFu;
								}
							}
							put(best, hc);
						}
					}
				}
			}
		}
	}
}

template<bool Write>
int launch_rows(const ShfJob* jobs, const ShfJob& single, const uint32_t njobs, const ShfBandLaunch& cfg,
	cudaStream_t stream) {
	const dim3 grid(cfg.bands, njobs);
	switch (cfg.cols_per_thread) {
	case 1u:
		shf_band_rows<Write, 1u><<<grid, cfg.threads, cfg.smem, stream>>>(jobs, single, cfg.band_rows, cfg.max_cols);
		break;
	case 2u:
		shf_band_rows<Write, 2u><<<grid, cfg.threads, cfg.smem, stream>>>(jobs, single, cfg.band_rows, cfg.max_cols);
		break;
	default:
		shf_band_rows<Write, 4u><<<grid, cfg.threads, cfg.smem, stream>>>(jobs, single, cfg.band_rows, cfg.max_cols);
		break;
	}
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int band_set_smem_attributes() {
	const int bytes = 200 * 1024;
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_band_rows<false, 1u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_band_rows<false, 2u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_band_rows<false, 4u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_band_rows<true, 1u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_band_rows<true, 2u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_band_rows<true, 4u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	return STPGB_OK;
}

} // namespace

ShfBandLaunch shf_band_config(const uint32_t njobs, const uint32_t max_W, const uint32_t max_H, const uint32_t max_r) {
	ShfBandLaunch cfg {};
	const uint32_t ncols = std::min(max_W + 2u * max_r, kShfBandMaxCols);
	cfg.threads = ncols <= kFastMaxThreads ? (ncols + 31u) / 32u * 32u : kFastMaxThreads;
	const uint32_t need = (ncols + cfg.threads - 1u) / cfg.threads;
	cfg.cols_per_thread = need <= 1u ? 1u : need <= 2u ? 2u : 4u;
	// about three blocks per SM over the launch; bands of 4 to 64 rows
	const uint64_t want = (3ull * current_sm_count() + njobs - 1u) / std::max(njobs, 1u);
	const uint64_t rows = (static_cast<uint64_t>(max_H) + want - 1u) / std::max<uint64_t>(want, 1u);
	cfg.band_rows = static_cast<uint32_t>(std::min<uint64_t>(std::max<uint64_t>(rows, kShfBandMinRows), 64u));
	cfg.bands = (max_H + cfg.band_rows - 1u) / cfg.band_rows;
	cfg.max_cols = ncols;
	cfg.smem = (2u * static_cast<size_t>(ncols) + 1u + 96u) * sizeof(uint4) + static_cast<size_t>(ncols) * sizeof(uint32_t);
	return cfg;
}

int shf_band_carry_launch(const ShfJob* jobs, const ShfJob& single, const uint32_t njobs, const uint32_t max_W,
	const uint32_t max_r, const ShfBandLaunch& cfg, cudaStream_t stream) {
	const uint32_t ncols = max_W + 2u * max_r;
	shf_band_carry<<<dim3((ncols + kCarryBlock - 1u) / kCarryBlock, njobs), kCarryBlock, 0, stream>>>(jobs, single,
		cfg.band_rows);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int shf_band_rows_launch(const ShfJob* jobs, const ShfJob& single, const uint32_t njobs, const ShfBandLaunch& cfg,
	const bool write, cudaStream_t stream) {
	STPGB_TRY(once_per_device(SETUP_SHF_BAND_SMEM, band_set_smem_attributes));
	return write ? launch_rows<true>(jobs, single, njobs, cfg, stream) : launch_rows<false>(jobs, single, njobs, cfg, stream);
}

} // namespace stpgb
