// Single histogram filter, few-values path, on sm_103a.
//
// Same output as the reference filter
// (SuperTerrain+/SuperAlgorithm+/Host/Private/STPSingleHistogramFilter.cpp),
// bin order included, for chunks whose read region ((H+2r) x (W+2r)
// samples) holds at most kShfFastItems distinct values (biome maps: a
// Voronoi map of 8 biomes, the demo's layer chain).  Values are renamed to
// local indices 0..7 (their rank in the chunk's palette), which lets a
// histogram live in registers: eight byte counts in one 64-bit word and the
// accumulator's order as eight 4-bit indices in one 32-bit word.
//
// The order of a histogram is the reference accumulator's insertion order with
// erase-compaction (:400-450).  Vertically the slide is cheap in this form
// (one add and one remove of a 4-bit index per row and column) and is run as
// the reference runs it.  Horizontally the order follows from a rule that
// makes every pixel independent of the slide: when column k's vertical
// histogram is added, an item is inserted iff none of columns
// [max(0, k-2r-1), k-1] holds it (before the add, the window holds exactly
// those columns; the initial fill is the case k <= 2r).  An item present at
// pixel x was last inserted at the latest such column k0 <= x+2r, in the place
// it has in column k0's vertical histogram, and erasures keep the relative
// order of what remains, so the bins of pixel x are its present items sorted
// by (k0, place in column k0's histogram).  Windowed counts and "latest
// insertion column" are both prefix scans over the columns of a row: one sum
// scan and one max scan of eight 16-bit fields per column.
//
//   shf_palette   block per (32-row tile of the read region, job): distinct
//                 values through a 65536-bit map in shared memory.
//   shf_carry     thread per column: merges the palette tiles (every block
//                 does, block 0 records the job's path), then slides the
//                 column's vertical histogram down all rows and keeps its
//                 state at the first row of every band.
//   shf_fast_rows block per (band of rows, job), thread per column(s): per
//                 row, the vertical step, the count scan, the insertion scan
//                 and the pixels' bins (COUNT: bins per row; WRITE: offsets
//                 and bins after the row scan).
#include "shf.cuh"

#include <algorithm>

namespace stpgb {

namespace {

constexpr uint32_t kPaletteBlock = 256u;
constexpr uint32_t kCarryBlock = 64u;
constexpr uint32_t kFastMaxThreads = 1024u;
constexpr uint32_t kNoValue = 0xFFFFFFFFu;
// words per palette slot and per record: {count, 0, values as uint16 pairs x4, 0, 0}
constexpr uint32_t kSlotWords = 8u;
// the byte counts hold 2r+2 (add before remove), the 16-bit window sums (2r+1)^2
constexpr uint32_t kFastMaxRadius = 126u;

__device__ __forceinline__ const ShfJob& pick(const ShfJob* jobs, const ShfJob& single) {
	return jobs ? jobs[blockIdx.y] : single;
}

// first sample of the read region: row sy - r, column sx - r
__device__ __forceinline__ const uint16_t* read_region(const ShfJob& J) {
	return J.samplemap + static_cast<uint64_t>(J.sy - J.r) * J.pitch + (J.sx - J.r);
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
	__shared__ uint32_t total, fill;
	__shared__ uint32_t vals[kShfFastItems];
	for (uint32_t i = threadIdx.x; i < 2048u; i += kPaletteBlock) {
		bits[i] = 0u;
	}
	if (threadIdx.x == 0u) {
		total = 0u;
		fill = 0u;
	}
	__syncthreads();
	const uint16_t* const base = read_region(J);
	const uint32_t lane = threadIdx.x & 31u;
	const uint32_t span = (NC + kPaletteBlock - 1u) / kPaletteBlock * kPaletteBlock;
	for (uint32_t row = r0; row < r1; row++) {
		const uint16_t* const src = base + static_cast<uint64_t>(row) * J.pitch;
		for (uint32_t c = threadIdx.x; c < span; c += kPaletteBlock) {
			const uint32_t v = c < NC ? static_cast<uint32_t>(__ldg(src + c)) : kNoValue;
			// one lane per distinct value of the warp sets its bit
			const uint32_t same = __match_any_sync(0xFFFFFFFFu, v);
			if (v != kNoValue && static_cast<uint32_t>(__ffs(same) - 1) == lane) {
				const uint32_t bit = 1u << (v & 31u);
				if (!(bits[v >> 5] & bit)) {
					atomicOr(&bits[v >> 5], bit);
				}
			}
		}
	}
	__syncthreads();
	uint32_t mine = 0u;
	for (uint32_t i = threadIdx.x; i < 2048u; i += kPaletteBlock) {
		mine += __popc(bits[i]);
	}
	if (mine) {
		atomicAdd(&total, mine);
	}
	__syncthreads();
	const uint32_t n = total;
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

// ------------------------------------------------------ packed histograms --

// number of nonzero bytes (present items)
__device__ __forceinline__ uint32_t nonzero_bytes(const uint64_t v) {
	const uint64_t low7 = 0x7F7F7F7F7F7F7F7Full;
	return static_cast<uint32_t>(__popcll((((v & low7) + low7) | v) & 0x8080808080808080ull));
}

// place of item j in an order word (j is in its first nonzero_bytes nibbles):
// the lowest zero nibble of order ^ (j in every nibble)
__device__ __forceinline__ uint32_t place_of(const uint32_t order, const uint32_t j) {
	const uint32_t x = order ^ (j * 0x11111111u);
	const uint32_t z = (x - 0x11111111u) & ~x & 0x88888888u;
	return static_cast<uint32_t>(__ffs(z) - 1) >> 2;
}

// the reference accumulator's add of one sample of item a: appended when absent
__device__ __forceinline__ void hist_add(uint64_t& cnt, uint32_t& order, const uint32_t a) {
	const uint32_t sh = 8u * a;
	if (((cnt >> sh) & 0xFFull) == 0ull) {
		order |= a << (4u * nonzero_bytes(cnt));
	}
	cnt += 1ull << sh;
}

// its remove: an item whose count drops to zero is erased, later ones close up
__device__ __forceinline__ void hist_sub(uint64_t& cnt, uint32_t& order, const uint32_t b) {
	const uint32_t sh = 8u * b;
	cnt -= 1ull << sh;
	if (((cnt >> sh) & 0xFFull) == 0ull) {
		const uint32_t low = (1u << (4u * place_of(order, b))) - 1u;
		order = (order & low) | ((order >> 4) & ~low);
	}
}

// The palette as eight 16-bit fields (value j in word j/2, half j%2),
// ascending, 0xFFFF past the count.
using Palette = uint4;

__device__ __forceinline__ Palette make_palette(const uint32_t* const vals, const uint32_t n) {
	auto at = [&](const uint32_t j) {
		return j < n ? (vals[j] & 0xFFFFu) : 0xFFFFu;
	};
	return make_uint4(at(0) | (at(1) << 16), at(2) | (at(3) << 16), at(4) | (at(5) << 16), at(6) | (at(7) << 16));
}

// local index of a palette value: the number of palette values below it
// (a padding field, 0xFFFF, is never below a 16-bit value)
__device__ __forceinline__ uint32_t local_index(const Palette p, const uint32_t v) {
	const uint32_t vv = v * 0x00010001u;
	return (__popc(__vcmpgtu2(vv, p.x)) + __popc(__vcmpgtu2(vv, p.y)) + __popc(__vcmpgtu2(vv, p.z))
			   + __popc(__vcmpgtu2(vv, p.w)))
		>> 4;
}

// Union of a job's palette slots, ascending; kShfModeFast when it has at most
// kShfFastItems values and the job fits this path.
__device__ void merge_palette(const ShfJob& J, const uint32_t kcap_h, uint32_t& mode, uint32_t& count,
	uint32_t* const vals) {
	const uint32_t NR = J.H + 2u * J.r, NC = J.W + 2u * J.r;
	const uint32_t tiles = (NR + kShfPaletteRows - 1u) / kShfPaletteRows;
	uint32_t n = 0u;
	bool ok = NC <= kShfFastMaxCols && J.r <= kFastMaxRadius;
	for (uint32_t t = 0u; t < tiles && ok; t++) {
		const uint32_t* const slot = J.fast + kSlotWords * (1u + t);
		const uint32_t c = slot[0];
		if (c == kNoValue) {
			ok = false;
			break;
		}
		for (uint32_t i = 0u; i < c && ok; i++) {
			const uint32_t x = (slot[2u + i / 2u] >> (16u * (i & 1u))) & 0xFFFFu;
			uint32_t p = 0u;
			while (p < n && vals[p] < x) {
				p++;
			}
			if (p < n && vals[p] == x) {
				continue;
			}
			if (n == kShfFastItems) {
				ok = false;
				break;
			}
			for (uint32_t m = n; m > p; m--) {
				vals[m] = vals[m - 1u];
			}
			vals[p] = x;
			n++;
		}
	}
	// No accumulator of the slides could overflow (a vertical one holds at most
	// 2r+2 samples, a horizontal one (2r+2)(2r+1)), and the band states fit in
	// vbuf (bands * (W+2r) * 12 bytes against H * kcap_v * (W+2r) * 4).
	const uint64_t side = 2ull * J.r + 1u;
	const uint32_t max_bands = (J.H + kShfFastMinBandRows - 1u) / kShfFastMinBandRows;
	const uint64_t items = n;
	ok = ok && min(items, side + 1u) <= J.kcap_v && min(items, (side + 1u) * side) <= kcap_h
		&& 3ull * max_bands <= static_cast<uint64_t>(J.H) * J.kcap_v;
	for (uint32_t j = n; j < kShfFastItems; j++) {
		vals[j] = kNoValue;
	}
	mode = ok ? kShfModeFast : kShfModeSlide;
	count = n;
}

// ------------------------------------------------------------------ carry --

// Thread per column k of the read region: the vertical histogram of rows
// [y, y+2r] (relative to the region) for y = 0..H-1, slid as the reference
// slides it (:522-563), stored at y = 0, band_rows, 2 band_rows, ...:
// counts [bands][W+2r] (8 bytes), then orders [bands][W+2r] (4-bit indices).
__global__ void __launch_bounds__(kCarryBlock) shf_carry(const ShfJob* __restrict__ jobs, const ShfJob single,
	const uint32_t kcap_h, const uint32_t band_rows) {
	const ShfJob& J = pick(jobs, single);
	__shared__ uint32_t s_mode, s_count, s_val[kShfFastItems];
	if (threadIdx.x == 0u) {
		uint32_t vals[kShfFastItems];
		merge_palette(J, kcap_h, s_mode, s_count, vals);
		for (uint32_t j = 0u; j < kShfFastItems; j++) {
			s_val[j] = vals[j];
		}
		if (blockIdx.x == 0u) {
			ShfFastRecord* const rec = reinterpret_cast<ShfFastRecord*>(J.fast);
			rec->mode = s_mode;
			rec->count = s_count;
			rec->pad0 = 0u;
			rec->pad1 = 0u;
			for (uint32_t j = 0u; j < kShfFastItems; j++) {
				rec->item[j] = static_cast<uint16_t>(j < s_count ? vals[j] : 0u);
			}
		}
	}
	__syncthreads();
	const uint32_t NC = J.W + 2u * J.r;
	const uint32_t k = blockIdx.x * kCarryBlock + threadIdx.x;
	if (s_mode != kShfModeFast || k >= NC) {
		return;
	}
	const Palette pal = make_palette(s_val, s_count);
	const uint16_t* const col = read_region(J) + k;
	const uint64_t pitch = J.pitch;
	const uint32_t H = J.H, r2 = 2u * J.r;
	const uint32_t bands = (H + band_rows - 1u) / band_rows;
	uint64_t* const cvc = reinterpret_cast<uint64_t*>(J.vbuf);
	uint32_t* const cvo = reinterpret_cast<uint32_t*>(cvc + static_cast<size_t>(bands) * NC);
	auto at = [&](const uint32_t q) {
		return static_cast<uint32_t>(__ldg(col + static_cast<uint64_t>(q) * pitch));
	};
	uint64_t cnt = 0ull;
	uint32_t order = 0u;
	for (uint32_t q = 0u; q <= r2; q++) {
		hist_add(cnt, order, local_index(pal, at(q)));
	}
	cvc[k] = cnt;
	cvo[k] = order;
	// row y adds region row y+2r and removes row y-1; the samples of the next
	// four rows are loaded ahead (they do not depend on the histogram)
	constexpr uint32_t kAhead = 4u;
	uint32_t ra[kAhead], rb[kAhead];
#pragma unroll
	for (uint32_t i = 0u; i < kAhead; i++) {
		const uint32_t y = 1u + i;
		ra[i] = y < H ? at(y + r2) : 0u;
		rb[i] = y < H ? at(y - 1u) : 0u;
	}
	for (uint32_t y = 1u; y < H; y += kAhead) {
#pragma unroll
		for (uint32_t i = 0u; i < kAhead; i++) {
			const uint32_t yy = y + i;
			if (yy < H) {
				const uint32_t a = ra[i], b = rb[i];
				if (yy + kAhead < H) {
					ra[i] = at(yy + kAhead + r2);
					rb[i] = at(yy + kAhead - 1u);
				}
				if (a != b) {
					hist_add(cnt, order, local_index(pal, a));
					hist_sub(cnt, order, local_index(pal, b));
				}
				if (yy % band_rows == 0u) {
					const size_t o = static_cast<size_t>(yy / band_rows) * NC + k;
					cvc[o] = cnt;
					cvo[o] = order;
				}
			}
		}
	}
}

// ------------------------------------------------------------------- rows --

__device__ __forceinline__ uint4 add4(const uint4 a, const uint4 b) {
	return make_uint4(__vadd2(a.x, b.x), __vadd2(a.y, b.y), __vadd2(a.z, b.z), __vadd2(a.w, b.w));
}
__device__ __forceinline__ uint4 sub4(const uint4 a, const uint4 b) {
	return make_uint4(__vsub2(a.x, b.x), __vsub2(a.y, b.y), __vsub2(a.z, b.z), __vsub2(a.w, b.w));
}
__device__ __forceinline__ uint4 max4(const uint4 a, const uint4 b) {
	return make_uint4(__vmaxu2(a.x, b.x), __vmaxu2(a.y, b.y), __vmaxu2(a.z, b.z), __vmaxu2(a.w, b.w));
}
__device__ __forceinline__ uint4 shfl_up4(const uint4 v, const uint32_t d) {
	return make_uint4(__shfl_up_sync(0xFFFFFFFFu, v.x, d), __shfl_up_sync(0xFFFFFFFFu, v.y, d),
		__shfl_up_sync(0xFFFFFFFFu, v.z, d), __shfl_up_sync(0xFFFFFFFFu, v.w, d));
}

// eight byte counts -> eight 16-bit fields (item j in word j/2, half j%2)
__device__ __forceinline__ uint4 widen(const uint64_t c) {
	const uint32_t lo = static_cast<uint32_t>(c), hi = static_cast<uint32_t>(c >> 32);
	return make_uint4(__byte_perm(lo, 0u, 0x4140u), __byte_perm(lo, 0u, 0x4342u), __byte_perm(hi, 0u, 0x4140u),
		__byte_perm(hi, 0u, 0x4342u));
}

// bit j set where field j is nonzero
__device__ __forceinline__ uint32_t present_mask(const uint4 v) {
	const uint32_t a = __vcmpne2(v.x, 0u), b = __vcmpne2(v.y, 0u), c = __vcmpne2(v.z, 0u), d = __vcmpne2(v.w, 0u);
	return (a & 1u) | ((a >> 15) & 2u) | ((b & 1u) << 2) | ((b >> 13) & 8u) | ((c & 1u) << 4) | ((c >> 11) & 32u)
		| ((d & 1u) << 6) | ((d >> 9) & 128u);
}

__device__ __forceinline__ uint32_t field(const uint4 v, const uint32_t j) {
	const uint32_t w = (j & 4u) ? ((j & 2u) ? v.w : v.z) : ((j & 2u) ? v.y : v.x);
	return (w >> (16u * (j & 1u))) & 0xFFFFu;
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
__global__ void __launch_bounds__(kFastMaxThreads) shf_fast_rows(const ShfJob* __restrict__ jobs, const ShfJob single,
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
int launch_rows(const ShfJob* jobs, const ShfJob& single, const uint32_t njobs, const ShfFastLaunch& cfg,
	cudaStream_t stream) {
	const dim3 grid(cfg.bands, njobs);
	switch (cfg.cols_per_thread) {
	case 1u:
		shf_fast_rows<Write, 1u><<<grid, cfg.threads, cfg.smem, stream>>>(jobs, single, cfg.band_rows, cfg.max_cols);
		break;
	case 2u:
		shf_fast_rows<Write, 2u><<<grid, cfg.threads, cfg.smem, stream>>>(jobs, single, cfg.band_rows, cfg.max_cols);
		break;
	default:
		shf_fast_rows<Write, 4u><<<grid, cfg.threads, cfg.smem, stream>>>(jobs, single, cfg.band_rows, cfg.max_cols);
		break;
	}
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int fast_set_smem_attributes() {
	const int bytes = 200 * 1024;
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_fast_rows<false, 1u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_fast_rows<false, 2u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_fast_rows<false, 4u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_fast_rows<true, 1u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_fast_rows<true, 2u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_fast_rows<true, 4u>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
	return STPGB_OK;
}

} // namespace

ShfFastLaunch shf_fast_config(const uint32_t njobs, const uint32_t max_W, const uint32_t max_H, const uint32_t max_r) {
	ShfFastLaunch cfg {};
	const uint32_t ncols = std::min(max_W + 2u * max_r, kShfFastMaxCols);
	cfg.threads = ncols <= kFastMaxThreads ? (ncols + 31u) / 32u * 32u : kFastMaxThreads;
	const uint32_t need = (ncols + cfg.threads - 1u) / cfg.threads;
	cfg.cols_per_thread = need <= 1u ? 1u : need <= 2u ? 2u : 4u;
	// about three blocks per SM over the launch; bands of 4 to 64 rows
	const uint64_t want = (3ull * current_sm_count() + njobs - 1u) / std::max(njobs, 1u);
	const uint64_t rows = (static_cast<uint64_t>(max_H) + want - 1u) / std::max<uint64_t>(want, 1u);
	cfg.band_rows = static_cast<uint32_t>(std::min<uint64_t>(std::max<uint64_t>(rows, kShfFastMinBandRows), 64u));
	cfg.bands = (max_H + cfg.band_rows - 1u) / cfg.band_rows;
	cfg.max_cols = ncols;
	cfg.smem = (2u * static_cast<size_t>(ncols) + 1u + 96u) * sizeof(uint4) + static_cast<size_t>(ncols) * sizeof(uint32_t);
	return cfg;
}

int shf_fast_prepare(const ShfJob* jobs, const ShfJob& single, const uint32_t njobs, const uint32_t max_W,
	const uint32_t max_H, const uint32_t max_r, const uint32_t kcap_h, const ShfFastLaunch& cfg, cudaStream_t stream) {
	const uint32_t tiles = (max_H + 2u * max_r + kShfPaletteRows - 1u) / kShfPaletteRows;
	shf_palette<<<dim3(tiles, njobs), kPaletteBlock, 0, stream>>>(jobs, single);
	STPGB_CUDA_TRY(cudaGetLastError());
	const uint32_t ncols = max_W + 2u * max_r;
	shf_carry<<<dim3((ncols + kCarryBlock - 1u) / kCarryBlock, njobs), kCarryBlock, 0, stream>>>(jobs, single, kcap_h,
		cfg.band_rows);
	STPGB_CUDA_TRY(cudaGetLastError());
	return STPGB_OK;
}

int shf_fast_pass(const ShfJob* jobs, const ShfJob& single, const uint32_t njobs, const ShfFastLaunch& cfg,
	const bool write, cudaStream_t stream) {
	STPGB_TRY(once_per_device(SETUP_SHF_FAST_SMEM, fast_set_smem_attributes));
	return write ? launch_rows<true>(jobs, single, njobs, cfg, stream) : launch_rows<false>(jobs, single, njobs, cfg, stream);
}

} // namespace stpgb
