// Single histogram filter on sm_103a.
//
// Replaces the CPU filter of
// SuperTerrain+/SuperAlgorithm+/Host/Private/STPSingleHistogramFilter.cpp.
// The output must be bit-identical to the reference, including the order of
// the bins inside every histogram.  That order is the insertion order of the
// reference's accumulator (:400-450): a new item is appended, an item whose
// count drops to zero is erased and the rest close up.  It depends on the
// whole history of a sliding window, so each pass keeps the reference's
// sequential slide per column (vertical pass) and per row (horizontal pass),
// with the accumulator in shared memory.  When few chunks are filtered at
// once, a column / row is cut into segments that slide in parallel: each
// segment rebuilds its first accumulator from the window's counts and, for
// the order, the start of every present item's current run, found by one
// sweep back (an item's place is fixed by the step that last inserted it).
//
//   shf_vertical   thread per (column k in [0, W+2r), segment): window of
//                  rows [y-r, y+r] of column sx-r+k, slid down the segment's
//                  rows of the central chunk (reference :522-563).  Output:
//                  ordered (item, count) lists per (k, y) in the workspace.
//   shf_horizontal thread per (row y, segment): window of vertical histograms
//                  of columns [x, x+2r], slid across the segment's columns
//                  (reference :608-679).  COUNT mode sums the bins of the
//                  segment, WRITE mode writes offsets and normalised bins.
//   shf_rowscan    exclusive prefix over the (row, segment) totals -> bases.
//
// Every pixel's counts sum to (2r+1)^2, so the reference's normalisation
// factor 1.0f / float(sum) (:495-497) is the same for every pixel.
#include "shf.cuh"

#include <algorithm>
#include <atomic>

namespace stpgb {

namespace {

constexpr uint32_t kVBlock = 64u;
// steps of the vertical slide whose samples are loaded ahead of their use
constexpr uint32_t kVAhead = 8u;
constexpr uint32_t kHBlock = 32u;
// columns (rows) a segment's start sweep loads ahead of their use
constexpr uint32_t kSweepAhead = 8u;
constexpr uint32_t kScanBlock = 256u;
// consecutive (row, segment) counts a scan thread takes per pass
constexpr uint32_t kScanPer = 16u;
// threads per SM the segmented passes aim for
constexpr uint64_t kShfThreadsPerSM = 1024u;

size_t align256(size_t v) {
	return (v + 255u) & ~static_cast<size_t>(255u);
}

__device__ __forceinline__ const ShfJob& pick(const ShfJob* jobs, const ShfJob& single) {
	return jobs ? jobs[blockIdx.y] : single;
}

// Flag of an accumulator entry whose run start is known (segment start).
constexpr uint32_t kResolved = 0x80000000u;

// Thread (column k, segment s) of a job: rows [s*L, min(H, s*L+L)) of column
// sx - r + k.  Segment 0 starts as the reference does (fill rows -r..r);
// a later segment rebuilds the accumulator of its first row: the counts of
// the window, and the order the sequential slide would have produced.  An
// item's place is fixed by the step that last inserted it: it stays present
// while its occurrences in the column are at most 2r+1 rows apart (the
// window always holds one of them; add before remove keeps a 2r+1 gap
// joined), so the order of the present items is the order of the first
// occurrences of their current runs (an item present from step 0 starts its
// run at its first occurrence in rows -r..r, which orders the initial fill).
// One upward sweep from the window finds every run start.
__global__ void __launch_bounds__(kVBlock) shf_vertical(const ShfJob* __restrict__ jobs, const ShfJob single,
	const uint32_t kcap, const uint32_t segs, const uint32_t seg_len) {
	const ShfJob& J = pick(jobs, single);
	if (!shf_job_general(J)) {
		return; // filtered by the few-values path
	}
	const uint32_t ncols = J.W + 2u * J.r;
	const uint32_t t = blockIdx.x * kVBlock + threadIdx.x;
	const uint32_t k = t % ncols, s = t / ncols;
	const uint32_t y_a = s * seg_len;
	if (s >= segs || y_a >= J.H) {
		return;
	}
	const uint32_t y_b = min(J.H, y_a + seg_len);
	extern __shared__ uint32_t vsm[];
	uint32_t* const acc = vsm + threadIdx.x;              // entry j at acc[j * kVBlock]
	uint32_t* const key = vsm + kcap * kVBlock + threadIdx.x; // run start of entry j (segment start)
	uint32_t n = 0u;
	bool overflow = false;

	auto inc = [&](const uint32_t v) {
		for (uint32_t j = 0u; j < n; j++) {
			const uint32_t e = acc[j * kVBlock];
			if ((e >> 16) == v) {
				acc[j * kVBlock] = e + 1u;
				return;
			}
		}
		if (n < kcap) {
			acc[n * kVBlock] = (v << 16) | 1u;
			n++;
		} else {
			overflow = true;
		}
	};
	auto dec = [&](const uint32_t v) {
		for (uint32_t j = 0u; j < n; j++) {
			const uint32_t e = acc[j * kVBlock];
			if ((e >> 16) == v) {
				if ((e & 0xFFFFu) <= 1u) {
					for (uint32_t m = j; m + 1u < n; m++) {
						acc[m * kVBlock] = acc[(m + 1u) * kVBlock];
					}
					n--;
				} else {
					acc[j * kVBlock] = e - 1u;
				}
				return;
			}
		}
	};
	const uint16_t* const col = J.samplemap + (J.sx - J.r + k);
	const uint64_t pitch = J.pitch;
	// sample of window row q (relative to the chunk's first row, q >= -r)
	auto at = [&](const int q) {
		return static_cast<uint32_t>(__ldg(col + static_cast<uint64_t>(static_cast<int64_t>(J.sy) + q) * pitch));
	};
	// column-major output ([column][entry][row]): the horizontal pass's warps
	// (consecutive rows) read one line per entry plane and column
	uint16_t* const vn_col = J.vn + static_cast<size_t>(k) * J.H;
	uint32_t* const vb_col = J.vbuf + static_cast<size_t>(k) * kcap * J.H;
	auto write_row = [&](const uint32_t y, const uint32_t cnt, const uint32_t* const src, const uint32_t stride) {
		vn_col[y] = static_cast<uint16_t>(cnt);
		for (uint32_t j = 0u; j < cnt; j++) {
			vb_col[static_cast<size_t>(j) * J.H + y] = src[j * stride];
		}
	};
	// Writes go straight to the column-major buffers.  Staging rows in shared
	// memory to write whole sectors made this pass faster alone, but its
	// 18 KB per block of shared memory kept the pass's blocks off the SMs
	// that run another stream's erosion kernel, and batches that overlap on
	// two streams lost far more than the pass gained.
	auto emit = [&](const uint32_t y) {
		write_row(y, n, acc, kVBlock);
	};

	const int r = static_cast<int>(J.r);
	// The window of the segment's first row, rows [y_a - r, y_a + r], its
	// samples loaded kSweepAhead rows ahead (a ring of registers).
	auto for_window = [&](auto&& f) {
		const int q_a = static_cast<int>(y_a) - r, q_b = static_cast<int>(y_a) + r;
		uint32_t sv[kSweepAhead];
#pragma unroll
		for (uint32_t u = 0u; u < kSweepAhead; u++) {
			if (q_a + static_cast<int>(u) <= q_b) {
				sv[u] = at(q_a + static_cast<int>(u));
			}
		}
		for (int q0 = q_a; q0 <= q_b; q0 += static_cast<int>(kSweepAhead)) {
#pragma unroll
			for (uint32_t u = 0u; u < kSweepAhead; u++) {
				const int q = q0 + static_cast<int>(u);
				if (q <= q_b) {
					const uint32_t v = sv[u];
					if (q + static_cast<int>(kSweepAhead) <= q_b) {
						sv[u] = at(q + static_cast<int>(kSweepAhead));
					}
					f(q, v);
				}
			}
		}
	};
	if (y_a == 0u) {
		for_window([&](const int, const uint32_t v) { inc(v); });
	} else {
		// counts of the window, each item keyed by its topmost row in it (+r, >= 0)
		for_window([&](const int q, const uint32_t v) {
			const uint32_t before = n;
			inc(v);
			if (n > before) {
				key[(n - 1u) * kVBlock] = static_cast<uint32_t>(q + r);
			}
		});
		// upward sweep: extend each run while its occurrences stay within 2r+1
		// rows; the samples are loaded kSweepAhead rows ahead
		uint32_t open = n;
		uint32_t sv[kSweepAhead];
		const int q_top = static_cast<int>(y_a) - r - 1;
#pragma unroll
		for (uint32_t u = 0u; u < kSweepAhead; u++) {
			if (q_top - static_cast<int>(u) >= -r) {
				sv[u] = at(q_top - static_cast<int>(u));
			}
		}
		for (int q0 = q_top; q0 >= -r && open > 0u; q0 -= static_cast<int>(kSweepAhead)) {
#pragma unroll
			for (uint32_t u = 0u; u < kSweepAhead; u++) {
				const int q = q0 - static_cast<int>(u);
				if (q >= -r && open > 0u) {
					const uint32_t v = sv[u], qk = static_cast<uint32_t>(q + r);
					if (q - static_cast<int>(kSweepAhead) >= -r) {
						sv[u] = at(q - static_cast<int>(kSweepAhead));
					}
					for (uint32_t j = 0u; j < n; j++) {
						const uint32_t kj = key[j * kVBlock];
						if (kj & kResolved) {
							continue;
						}
						if (kj - qk >= 2u * J.r + 2u) {
							// 2r+1 rows without the item: an earlier occurrence starts another run
							key[j * kVBlock] = kj | kResolved;
							open--;
						} else if ((acc[j * kVBlock] >> 16) == v) {
							key[j * kVBlock] = qk;
						}
					}
				}
			}
		}
		// order by run start (insertion sort, entries are few)
		for (uint32_t j = 1u; j < n; j++) {
			const uint32_t e = acc[j * kVBlock], kj = key[j * kVBlock] & ~kResolved;
			uint32_t m = j;
			while (m > 0u && (key[(m - 1u) * kVBlock] & ~kResolved) > kj) {
				acc[m * kVBlock] = acc[(m - 1u) * kVBlock];
				key[m * kVBlock] = key[(m - 1u) * kVBlock];
				m--;
			}
			acc[m * kVBlock] = e;
			key[m * kVBlock] = kj;
		}
	}
	emit(y_a);
	// A step whose added and removed samples are equal leaves the accumulator
	// as it was (the item is present throughout, so nothing is inserted or
	// erased); the two samples of a step are loaded kVAhead steps ahead (a
	// ring of registers: the loads do not depend on the accumulator).
	uint32_t va[kVAhead], vr[kVAhead];
#pragma unroll
	for (uint32_t i = 0u; i < kVAhead; i++) {
		const uint32_t y = y_a + 1u + i;
		va[i] = y < y_b ? at(static_cast<int>(y) + r) : 0u;
		vr[i] = y < y_b ? at(static_cast<int>(y) - 1 - r) : 0u;
	}
	for (uint32_t y0 = y_a + 1u; y0 < y_b; y0 += kVAhead) {
#pragma unroll
		for (uint32_t i = 0u; i < kVAhead; i++) {
			const uint32_t y = y0 + i;
			if (y < y_b) {
				const uint32_t add = va[i], sub = vr[i];
				if (y + kVAhead < y_b) {
					va[i] = at(static_cast<int>(y + kVAhead) + r);
					vr[i] = at(static_cast<int>(y + kVAhead) - 1 - r);
				}
				if (add != sub) {
					inc(add);
					dec(sub);
				}
				emit(y);
			}
		}
	}
	if (overflow) {
		atomicOr(J.status, STATUS_CAPACITY);
	}
}

// Thread (row y, segment s): output columns [s*L, min(W, s*L+L)).  A later
// segment rebuilds its first accumulator as the vertical pass does, over
// columns of vertical histograms: an item stays present while the columns
// holding it are at most 2r+1 apart, and the items a step adds enter in the
// order of the added column's histogram, so the order is by (first column of
// the item's current run, its place in that column's histogram).
template<bool Write>
__global__ void __launch_bounds__(kHBlock) shf_horizontal(const ShfJob* __restrict__ jobs, const ShfJob single,
	const uint32_t kcap_v, const uint32_t kcap, const uint32_t segs, const uint32_t seg_len) {
	const ShfJob& J = pick(jobs, single);
	if (!shf_job_general(J)) {
		return;
	}
	const uint32_t t = blockIdx.x * kHBlock + threadIdx.x;
	const uint32_t y = t % J.H, s = t / J.H;
	const uint32_t x_a = s * seg_len;
	if (s >= segs) {
		return;
	}
	if (x_a >= J.W) {
		if constexpr (!Write) {
			J.rows[static_cast<size_t>(y) * segs + s] = 0u; // a segment past this job's width
		}
		return;
	}
	const uint32_t x_b = min(J.W, x_a + seg_len);
	extern __shared__ uint32_t hsm[];
	// staging words of the write pass after the accumulator (an even count, for 8-byte alignment)
	const uint32_t hstage = 2u * kcap * kHBlock + ((kcap * kHBlock + 3u) / 4u) * 2u;
	uint32_t* const cnt = hsm + threadIdx.x;                                               // [kcap][kHBlock]
	uint32_t* const key = hsm + kcap * kHBlock + threadIdx.x;                              // [kcap][kHBlock]
	uint16_t* const item = reinterpret_cast<uint16_t*>(hsm + 2u * kcap * kHBlock) + threadIdx.x; // [kcap][kHBlock]
	uint32_t n = 0u;
	bool overflow = false;

	auto inc = [&](const uint32_t v, const uint32_t c) {
		for (uint32_t j = 0u; j < n; j++) {
			if (item[j * kHBlock] == v) {
				cnt[j * kHBlock] += c;
				return;
			}
		}
		if (n < kcap) {
			item[n * kHBlock] = static_cast<uint16_t>(v);
			cnt[n * kHBlock] = c;
			n++;
		} else {
			overflow = true;
		}
	};
	auto dec = [&](const uint32_t v, const uint32_t c) {
		for (uint32_t j = 0u; j < n; j++) {
			if (item[j * kHBlock] == v) {
				if (cnt[j * kHBlock] <= c) {
					for (uint32_t m = j; m + 1u < n; m++) {
						item[m * kHBlock] = item[(m + 1u) * kHBlock];
						cnt[m * kHBlock] = cnt[(m + 1u) * kHBlock];
					}
					n--;
				} else {
					cnt[j * kHBlock] -= c;
				}
				return;
			}
		}
	};
	// the vertical histogram of column kc for this row: vn_at(kc) entries, entry j at ent(kc, j)
	const uint64_t H = J.H;
	const uint16_t* const vn = J.vn + y;
	const uint32_t* const vcol = J.vbuf + y;
	auto vn_at = [&](const uint32_t kc) {
		return min(static_cast<uint32_t>(vn[kc * H]), kcap_v); // the vertical pass never writes more
	};
	auto ent = [&](const uint32_t kc, const uint32_t j) {
		return vcol[(kc * static_cast<uint64_t>(kcap_v) + j) * H];
	};

	// A column's entry count and first two entries (ColData): entry slots past
	// the count hold stale data and are not used.
	struct ColData {
		uint32_t n, e0, e1;
	};
	const bool two = kcap_v >= 2u;
	auto fetch = [&](const uint32_t kc) {
		ColData c;
		c.n = vn_at(kc);
		c.e0 = ent(kc, 0u);
		c.e1 = two ? ent(kc, 1u) : 0u;
		return c;
	};

	const uint32_t side = 2u * J.r + 1u;
	// The window of the segment's first column, columns [x_a, x_a + 2r], with
	// each column's data loaded kSweepAhead columns ahead (a ring of registers);
	// f(kc, j, entry) for every entry in column then entry order.
	auto for_window = [&](auto&& f) {
		const uint32_t k_b = x_a + side;
		ColData sw[kSweepAhead];
#pragma unroll
		for (uint32_t u = 0u; u < kSweepAhead; u++) {
			if (x_a + u < k_b) {
				sw[u] = fetch(x_a + u);
			}
		}
		for (uint32_t k0 = x_a; k0 < k_b; k0 += kSweepAhead) {
#pragma unroll
			for (uint32_t u = 0u; u < kSweepAhead; u++) {
				const uint32_t kc = k0 + u;
				if (kc < k_b) {
					const ColData c = sw[u];
					if (kc + kSweepAhead < k_b) {
						sw[u] = fetch(kc + kSweepAhead);
					}
					for (uint32_t j = 0u; j < c.n; j++) {
						f(kc, j, j == 0u ? c.e0 : (j == 1u ? c.e1 : ent(kc, j)));
					}
				}
			}
		}
	};
	if (x_a == 0u) {
		for_window([&](const uint32_t, const uint32_t, const uint32_t e) { inc(e >> 16, e & 0xFFFFu); });
	} else {
		// counts of the window, each item keyed by (first column, place in its histogram)
		for_window([&](const uint32_t kc, const uint32_t j, const uint32_t e) {
			const uint32_t before = n;
			inc(e >> 16, e & 0xFFFFu);
			if (n > before) {
				key[(n - 1u) * kHBlock] = (kc << 12) | j;
			}
		});
		// leftward sweep: extend each run while its columns stay within 2r+1;
		// the columns' data is loaded kSweepAhead columns ahead (their loads do
		// not depend on the sweep), so the sweep is not a chain of round trips
		uint32_t open = n;
		ColData sw[kSweepAhead];
#pragma unroll
		for (uint32_t u = 0u; u < kSweepAhead; u++) {
			if (x_a >= 1u + u) {
				sw[u] = fetch(x_a - 1u - u);
			}
		}
		for (int kc0 = static_cast<int>(x_a) - 1; kc0 >= 0 && open > 0u; kc0 -= static_cast<int>(kSweepAhead)) {
#pragma unroll
			for (uint32_t u = 0u; u < kSweepAhead; u++) {
				const int kc = kc0 - static_cast<int>(u);
				if (kc >= 0 && open > 0u) {
					const ColData c = sw[u];
					if (kc >= static_cast<int>(kSweepAhead)) {
						sw[u] = fetch(static_cast<uint32_t>(kc) - kSweepAhead);
					}
					for (uint32_t i = 0u; i < n; i++) {
						const uint32_t ki = key[i * kHBlock];
						if (ki & kResolved) {
							continue;
						}
						if ((ki >> 12) - static_cast<uint32_t>(kc) >= 2u * J.r + 2u) {
							// 2r+1 columns without the item: an earlier one starts another run
							key[i * kHBlock] = ki | kResolved;
							open--;
							continue;
						}
						const uint32_t v = item[i * kHBlock];
						for (uint32_t j = 0u; j < c.n; j++) {
							const uint32_t e = j == 0u ? c.e0 : (j == 1u ? c.e1 : ent(static_cast<uint32_t>(kc), j));
							if ((e >> 16) == v) {
								key[i * kHBlock] = (static_cast<uint32_t>(kc) << 12) | j;
								break;
							}
						}
					}
				}
			}
		}
		for (uint32_t j = 1u; j < n; j++) {
			const uint16_t v = item[j * kHBlock];
			const uint32_t c = cnt[j * kHBlock], kj = key[j * kHBlock] & ~kResolved;
			uint32_t m = j;
			while (m > 0u && (key[(m - 1u) * kHBlock] & ~kResolved) > kj) {
				item[m * kHBlock] = item[(m - 1u) * kHBlock];
				cnt[m * kHBlock] = cnt[(m - 1u) * kHBlock];
				key[m * kHBlock] = key[(m - 1u) * kHBlock];
				m--;
			}
			item[m * kHBlock] = v;
			cnt[m * kHBlock] = c;
			key[m * kHBlock] = kj;
		}
	}

	const float norm = 1.0f / static_cast<float>(side * side);
	const size_t slot = static_cast<size_t>(y) * segs + s;
	uint64_t running = Write ? J.rows[slot] : 0u;
	uint32_t* const off_row = J.offsets + static_cast<size_t>(y) * J.W;
	uint2* const bins = reinterpret_cast<uint2*>(J.bins);
	// Write pass: a lane's bins and offsets are contiguous runs of the output;
	// four of each are staged and leave as 16-byte stores (two per 32-byte
	// sector of bins), after single stores up to the first aligned position.
	uint2* const bst = reinterpret_cast<uint2*>(hsm + hstage) + threadIdx.x; // [4][kHBlock]
	uint32_t* const ost = hsm + hstage + 8u * kHBlock + threadIdx.x;        // [4][kHBlock]
	const bool bvec = (reinterpret_cast<uintptr_t>(J.bins) % 16u) == 0u;
	const bool ovec = (reinterpret_cast<uintptr_t>(off_row) % 16u) == 0u;
	uint64_t bpos = running;
	uint32_t bpend = 0u, opend = 0u;
	auto bin_single = [&](const uint64_t o, const uint2 b) {
		if (o < J.bins_capacity) {
			bins[o] = b;
		}
	};
	auto put_bin = [&](const uint2 b) {
		if (bpend == 0u && ((bpos & 1u) || !bvec)) {
			bin_single(bpos++, b);
			return;
		}
		bst[bpend * kHBlock] = b;
		if (++bpend == 4u) {
			if (bpos + 4u <= J.bins_capacity) {
				uint4* const dst = reinterpret_cast<uint4*>(bins + bpos);
				const uint2 b0 = bst[0], b1 = bst[kHBlock], b2 = bst[2u * kHBlock], b3 = bst[3u * kHBlock];
				dst[0] = make_uint4(b0.x, b0.y, b1.x, b1.y);
				dst[1] = make_uint4(b2.x, b2.y, b3.x, b3.y);
			} else {
				for (uint32_t i = 0u; i < 4u; i++) {
					bin_single(bpos + i, bst[i * kHBlock]);
				}
			}
			bpos += 4u;
			bpend = 0u;
		}
	};
	auto put_off = [&](const uint32_t x, const uint32_t v) {
		if (opend == 0u && (!ovec || (x & 3u))) {
			off_row[x] = v;
			return;
		}
		ost[opend * kHBlock] = v;
		if (++opend == 4u) {
			*reinterpret_cast<uint4*>(off_row + x - 3u) = make_uint4(ost[0], ost[kHBlock], ost[2u * kHBlock],
				ost[3u * kHBlock]);
			opend = 0u;
		}
	};
	uint32_t last_x = x_a;
	auto emit = [&](const uint32_t x) {
		if constexpr (Write) {
			put_off(x, static_cast<uint32_t>(running));
			for (uint32_t j = 0u; j < n; j++) {
				const float w = __fmul_rn(__uint2float_rn(cnt[j * kHBlock]), norm);
				put_bin(make_uint2(item[j * kHBlock], __float_as_uint(w)));
			}
			last_x = x;
		}
		running += n;
	};
	auto drain = [&]() {
		if constexpr (Write) {
			for (uint32_t i = 0u; i < bpend; i++) {
				bin_single(bpos + i, bst[i * kHBlock]);
			}
			for (uint32_t i = 0u; i < opend; i++) {
				off_row[last_x + 1u - opend + i] = ost[i * kHBlock];
			}
		}
	};

	// The slide proper.  A step adds column x + 2r and removes column x - 1.
	// Their entry counts and first two entries do not depend on the
	// accumulator, so they are loaded kAhead steps early (a ring of register
	// slots) and the loads overlap the steps in between; entries past the
	// second (few columns hold more than two items) are loaded when applied.
	auto apply = [&](const uint32_t kc, const ColData& c, const bool add) {
		if (c.n > 0u) {
			add ? inc(c.e0 >> 16, c.e0 & 0xFFFFu) : dec(c.e0 >> 16, c.e0 & 0xFFFFu);
		}
		if (c.n > 1u) {
			add ? inc(c.e1 >> 16, c.e1 & 0xFFFFu) : dec(c.e1 >> 16, c.e1 & 0xFFFFu);
		}
		for (uint32_t j = 2u; j < c.n; j++) {
			const uint32_t e = ent(kc, j);
			add ? inc(e >> 16, e & 0xFFFFu) : dec(e >> 16, e & 0xFFFFu);
		}
	};
	const uint32_t r2 = 2u * J.r;
	ColData a0 {}, a1 {}, a2 {}, a3 {}, s0 {}, s1 {}, s2 {}, s3 {};
	auto prefetch = [&](const uint32_t xx, ColData& a, ColData& sb) {
		if (xx < x_b) {
			a = fetch(xx + r2);
			sb = fetch(xx - 1u);
		}
	};
	// a step whose added and removed columns hold the same histogram (at most
	// two entries, equal item and count in order) changes nothing: every item
	// of the removed column is present before the step and stays present
	auto step = [&](const uint32_t xx, ColData& a, ColData& sb) {
		if (xx < x_b) {
			const bool same = a.n == sb.n && a.n <= 2u && (a.n < 1u || a.e0 == sb.e0) && (a.n < 2u || a.e1 == sb.e1);
			if (!same) {
				apply(xx + r2, a, true);
				apply(xx - 1u, sb, false);
			}
			emit(xx);
			prefetch(xx + 4u, a, sb);
		}
	};
	emit(x_a);
	prefetch(x_a + 1u, a0, s0);
	prefetch(x_a + 2u, a1, s1);
	prefetch(x_a + 3u, a2, s2);
	prefetch(x_a + 4u, a3, s3);
	for (uint32_t x = x_a + 1u; x < x_b; x += 4u) {
		step(x, a0, s0);
		step(x + 1u, a1, s1);
		step(x + 2u, a2, s2);
		step(x + 3u, a3, s3);
	}
	drain();
	if constexpr (!Write) {
		J.rows[slot] = static_cast<uint32_t>(min(running, static_cast<uint64_t>(0xFFFFFFFFu)));
	}
	if (overflow) {
		atomicOr(J.status, STATUS_CAPACITY);
	}
}

// One block per job: rows[0..H*segs) (row-major over row, segment) ->
// exclusive prefix, rows[H*segs] = total; offsets[W*H] = total.  A job of
// the few-values path has one count per row (segs = 1).
__global__ void __launch_bounds__(kScanBlock) shf_rowscan(const ShfJob* __restrict__ jobs, const ShfJob single,
	const uint32_t segs_slide) {
	const ShfJob& J = pick(jobs, single);
	const uint32_t segs = shf_job_general(J) ? segs_slide : 1u;
	const uint32_t slots = J.H * segs;
	__shared__ uint64_t warp_sum[kScanBlock / 32u];
	__shared__ uint64_t carry_s;
	if (threadIdx.x == 0u) {
		carry_s = 0u;
	}
	__syncthreads();
	const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
	// kScanPer consecutive slots per thread and pass: the thread's own running sum, then one
	// block-wide scan of the threads' totals
	for (uint32_t base = 0u; base < slots; base += kScanBlock * kScanPer) {
		const uint32_t first = base + threadIdx.x * kScanPer;
		uint32_t v[kScanPer];
#pragma unroll
		for (uint32_t k = 0u; k < kScanPer; k++) {
			v[k] = first + k < slots ? J.rows[first + k] : 0u;
		}
		uint64_t mine = 0u;
#pragma unroll
		for (uint32_t k = 0u; k < kScanPer; k++) {
			mine += v[k];
		}
		uint64_t s = mine;
#pragma unroll
		for (uint32_t d = 1u; d < 32u; d <<= 1) {
			const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, s, d);
			if (lane >= d) {
				s += t;
			}
		}
		if (lane == 31u) {
			warp_sum[warp] = s;
		}
		__syncthreads();
		uint64_t wbase = 0u;
		for (uint32_t w = 0u; w < warp; w++) {
			wbase += warp_sum[w];
		}
		const uint64_t carry = carry_s;
		uint64_t excl = carry + wbase + s - mine;
#pragma unroll
		for (uint32_t k = 0u; k < kScanPer; k++) {
			if (first + k < slots) {
				J.rows[first + k] = static_cast<uint32_t>(min(excl, static_cast<uint64_t>(0xFFFFFFFFu)));
			}
			excl += v[k];
		}
		__syncthreads();
		if (threadIdx.x == kScanBlock - 1u) {
			carry_s = carry + wbase + s;
		}
		__syncthreads();
	}
	if (threadIdx.x == 0u) {
		const uint64_t total = carry_s;
		J.rows[slots] = static_cast<uint32_t>(min(total, static_cast<uint64_t>(0xFFFFFFFFu)));
		J.offsets[static_cast<size_t>(J.W) * J.H] = static_cast<uint32_t>(min(total, static_cast<uint64_t>(0xFFFFFFFFu)));
		if (total > J.bins_capacity || total > 0xFFFFFFFFull) {
			atomicOr(J.status, STATUS_CAPACITY);
		}
	}
}

// the passes' dynamic shared memory above the default 48 KB (a per-device attribute)
int shf_set_smem_attributes() {
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_vertical, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_horizontal<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
	STPGB_CUDA_TRY(cudaFuncSetAttribute(shf_horizontal<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
	return STPGB_OK;
}

} // namespace

// The reference adds the incoming row / column before it removes the
// outgoing one, so an accumulator briefly holds the window plus one row
// (vertical: 2r+2 samples) or one column (horizontal: (2r+2)(2r+1)).
uint32_t shf_kcap_v(uint32_t r, uint32_t max_items) {
	return std::min<uint32_t>(2u * r + 2u, max_items);
}

uint32_t shf_kcap_h(uint32_t r, uint32_t max_items) {
	const uint64_t side = 2ull * r + 1ull;
	return static_cast<uint32_t>(std::min<uint64_t>((side + 1u) * side, max_items));
}

namespace {
std::atomic<uint32_t> g_shf_path { 0u };
} // namespace

uint32_t shf_path_override() {
	return g_shf_path.load();
}

ShfLayout shf_layout(uint32_t W, uint32_t H, uint32_t r, uint32_t kcap_v) {
	const size_t ncols = static_cast<size_t>(W) + 2u * r;
	ShfLayout l;
	l.vbuf = 0u;
	l.vn = align256(static_cast<size_t>(H) * kcap_v * ncols * sizeof(uint32_t));
	l.rows = l.vn + align256(static_cast<size_t>(H) * ncols * sizeof(uint16_t));
	l.fast = l.rows + align256((static_cast<size_t>(H) * kShfMaxSegments + 1u) * sizeof(uint32_t));
	const size_t tiles = (static_cast<size_t>(H) + 2u * r + kShfPaletteRows - 1u) / kShfPaletteRows;
	l.total = l.fast + align256((1u + tiles) * sizeof(ShfFastRecord));
	return l;
}

void shf_bind_workspace(ShfJob& job, unsigned char* ws, const ShfLayout& l) {
	job.vbuf = reinterpret_cast<uint32_t*>(ws + l.vbuf);
	job.vn = reinterpret_cast<uint16_t*>(ws + l.vn);
	job.rows = reinterpret_cast<uint32_t*>(ws + l.rows);
	job.fast = reinterpret_cast<uint32_t*>(ws + l.fast);
}

int shf_launch(const ShfJob* jobs, const ShfJob& single, uint32_t njobs, uint32_t max_W, uint32_t max_H,
	uint32_t max_r, uint32_t kcap_v, uint32_t kcap_h, cudaStream_t stream, const uint32_t segments_wanted,
	const uint32_t path) {
	STPGB_TRY(once_per_device(SETUP_SHF_SMEM, shf_set_smem_attributes));
	const uint64_t target_threads = uint64_t { current_sm_count() } * kShfThreadsPerSM;
	// Segments per column / row: enough threads to fill the GPU when few
	// chunks are filtered at once, none while the launch already has a
	// quarter of that (a segment start sweeps back to the start of every run:
	// on the 16-request production batch, 2-3 segments made the filter 40 %
	// slower; on one chunk, 16 make it several times faster).
	const uint64_t ncols = static_cast<uint64_t>(max_W) + 2u * max_r;
	auto segments = [&](const uint64_t lanes, const uint32_t len) {
		if (segments_wanted != 0u) {
			return std::max(1u, std::min({ segments_wanted, kShfMaxSegments, std::max(len, 1u) }));
		}
		const uint64_t want = (target_threads + lanes * njobs - 1u) / (lanes * njobs);
		if (want < 4u) {
			return 1u;
		}
		return static_cast<uint32_t>(std::min<uint64_t>({ want, uint64_t(kShfMaxSegments), uint64_t(len) }));
	};
	const uint32_t segs_v = segments(ncols, max_H), segs_h = segments(max_H, max_W);
	const uint32_t len_v = (max_H + segs_v - 1u) / segs_v, len_h = (max_W + segs_h - 1u) / segs_h;
	const size_t vsmem = static_cast<size_t>(kcap_v) * kVBlock * 2u * sizeof(uint32_t);
	const size_t hsmem = (2u * static_cast<size_t>(kcap_h) * kHBlock + ((kcap_h * kHBlock + 3u) / 4u) * 2u
		+ 12u * kHBlock) * sizeof(uint32_t);
	const dim3 vgrid(static_cast<uint32_t>((ncols * segs_v + kVBlock - 1u) / kVBlock), njobs);
	const dim3 hgrid(static_cast<uint32_t>((static_cast<uint64_t>(max_H) * segs_h + kHBlock - 1u) / kHBlock), njobs);
	// Every job first takes the palette of its read region: at most
	// kShfFastItems values go the few-values path (shf_fast.cu), the others
	// the sequential slides; each kernel returns at once for jobs of the other.
	const ShfFastPlan fast = shf_fast_plan(njobs, max_W, max_H, max_r, path);
	STPGB_TRY(shf_fast_prepare(jobs, single, njobs, max_W, max_H, max_r, kcap_h, fast, stream));
	STPGB_TRY(shf_fast_pass(jobs, single, njobs, max_H, fast, false, stream));
	shf_vertical<<<vgrid, kVBlock, vsmem, stream>>>(jobs, single, kcap_v, segs_v, len_v);
	STPGB_CUDA_TRY(cudaGetLastError());
	shf_horizontal<false><<<hgrid, kHBlock, hsmem, stream>>>(jobs, single, kcap_v, kcap_h, segs_h, len_h);
	STPGB_CUDA_TRY(cudaGetLastError());
	shf_rowscan<<<dim3(1u, njobs), kScanBlock, 0, stream>>>(jobs, single, segs_h);
	STPGB_CUDA_TRY(cudaGetLastError());
	shf_horizontal<true><<<hgrid, kHBlock, hsmem, stream>>>(jobs, single, kcap_v, kcap_h, segs_h, len_h);
	STPGB_CUDA_TRY(cudaGetLastError());
	STPGB_TRY(shf_fast_pass(jobs, single, njobs, max_H, fast, true, stream));
	return STPGB_OK;
}

namespace {

int check_shf_args(const stpgb_nn_info* nn, uint32_t radius, uint32_t max_items, uint32_t& sx, uint32_t& sy) {
	if (!nn) {
		return inval("stpgb_shf: null neighbour information");
	}
	if (nn->MapSize[0] == 0u || nn->MapSize[1] == 0u || nn->ChunkNearestNeighbour[0] == 0u
		|| nn->ChunkNearestNeighbour[1] == 0u) {
		return inval("stpgb_shf: empty map or neighbourhood");
	}
	if (nn->TotalMapSize[0] != nn->MapSize[0] * nn->ChunkNearestNeighbour[0]
		|| nn->TotalMapSize[1] != nn->MapSize[1] * nn->ChunkNearestNeighbour[1]) {
		return inval("stpgb_shf: TotalMapSize must equal MapSize * ChunkNearestNeighbour");
	}
	// STPSingleHistogramFilter.cpp:874-880
	if (!(radius > 0u && (radius & 1u) == 0u)) {
		return inval("radius should be an positive even number");
	}
	sx = nn->MapSize[0] * (nn->ChunkNearestNeighbour[0] / 2u);
	sy = nn->MapSize[1] * (nn->ChunkNearestNeighbour[1] / 2u);
	if (radius > sx || radius > sy) {
		return inval("radius is too large and will overflow nearest neighbour boundary");
	}
	if (max_items > kShfMaxItems) {
		return inval("stpgb_shf: max_items above the library bound of 256");
	}
	return STPGB_OK;
}

} // namespace

} // namespace stpgb

using namespace stpgb;

extern "C" {

int stpgb_shf_workspace_size(const stpgb_nn_info* nn, uint32_t radius, uint32_t max_items, size_t* bytes) {
	uint32_t sx, sy;
	STPGB_TRY(check_shf_args(nn, radius, max_items, sx, sy));
	if (max_items == 0u) {
		max_items = kShfMaxItems;
	}
	*bytes = shf_layout(nn->MapSize[0], nn->MapSize[1], radius, shf_kcap_v(radius, max_items)).total;
	return STPGB_OK;
}

int stpgb_shf_filter(const uint16_t* samplemap, const stpgb_nn_info* nn, uint32_t radius, uint32_t max_items,
	void* workspace, size_t workspace_bytes, uint32_t* offsets, stpgb_bin* bins, uint64_t bins_capacity,
	uint32_t* status, void* stream) {
	uint32_t sx, sy;
	STPGB_TRY(check_shf_args(nn, radius, max_items, sx, sy));
	if (max_items == 0u) {
		max_items = kShfMaxItems;
	}
	if (!samplemap || !offsets || (!bins && bins_capacity > 0u) || !status) {
		return inval("stpgb_shf_filter: null pointer argument");
	}
	const uint32_t W = nn->MapSize[0], H = nn->MapSize[1];
	const uint32_t kv = shf_kcap_v(radius, max_items), kh = shf_kcap_h(radius, max_items);
	const ShfLayout l = shf_layout(W, H, radius, kv);
	if (!workspace || workspace_bytes < l.total) {
		set_error("stpgb_shf_filter: workspace smaller than stpgb_shf_workspace_size");
		return STPGB_ECAPACITY;
	}
	const cudaStream_t s = as_stream(stream);
	STPGB_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(uint32_t), s));
	unsigned char* ws = static_cast<unsigned char*>(workspace);
	ShfJob job;
	job.samplemap = samplemap;
	job.pitch = nn->TotalMapSize[0];
	job.W = W;
	job.H = H;
	job.sx = sx;
	job.sy = sy;
	job.r = radius;
	job.kcap_v = kv;
	shf_bind_workspace(job, ws, l);
	job.offsets = offsets;
	job.bins = bins;
	job.bins_capacity = bins_capacity;
	job.status = status;
	return shf_launch(nullptr, job, 1u, W, H, radius, kv, kh, s);
}

int stpgb_shf_filter_path(const stpgb_nn_info* nn, uint32_t radius, uint32_t max_items, const void* workspace,
	uint32_t* path, void* stream) {
	uint32_t sx, sy;
	STPGB_TRY(check_shf_args(nn, radius, max_items, sx, sy));
	if (!workspace || !path) {
		return inval("stpgb_shf_filter_path: null workspace or result");
	}
	if (max_items == 0u) {
		max_items = kShfMaxItems;
	}
	const ShfLayout l = shf_layout(nn->MapSize[0], nn->MapSize[1], radius, shf_kcap_v(radius, max_items));
	ShfFastRecord rec {};
	const cudaStream_t s = as_stream(stream);
	STPGB_CUDA_TRY(cudaMemcpyAsync(&rec, static_cast<const unsigned char*>(workspace) + l.fast, sizeof(rec),
		cudaMemcpyDeviceToHost, s));
	STPGB_CUDA_TRY(cudaStreamSynchronize(s));
	*path = rec.mode == kShfModeSlide ? 0u : rec.form;
	return STPGB_OK;
}

int stpgb_shf_set_path(uint32_t path) {
	if (path > 3u) {
		return inval("stpgb_shf_set_path: 0 (by size), 1 (packed slides), 2 (row bands) or 3 (general slides)");
	}
	g_shf_path.store(path);
	return STPGB_OK;
}

int stpgb_status_check(const uint32_t* status, void* stream) {
	uint32_t h = 0u;
	STPGB_CUDA_TRY(cudaMemcpyAsync(&h, status, sizeof(uint32_t), cudaMemcpyDeviceToHost, as_stream(stream)));
	STPGB_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
	if (h & STATUS_CAPACITY) {
		set_error("device status: an output capacity or the per-window item bound was exceeded");
		return STPGB_ECAPACITY;
	}
	if (h & STATUS_TIMEOUT) {
		set_error("device status: a droplet reached the step cap");
		return STPGB_ETIMEOUT;
	}
	return STPGB_OK;
}

int stpgb_shf_filter_host(const uint16_t* samplemap_host, const stpgb_nn_info* nn, uint32_t radius,
	uint32_t* offsets_host, stpgb_bin* bins_host, uint64_t bins_capacity, uint64_t* nbins) {
	uint32_t sx, sy;
	STPGB_TRY(check_shf_args(nn, radius, 0u, sx, sy));
	const uint32_t W = nn->MapSize[0], H = nn->MapSize[1];
	const size_t in_bytes = static_cast<size_t>(nn->TotalMapSize[0]) * nn->TotalMapSize[1] * sizeof(uint16_t);
	const size_t npix = static_cast<size_t>(W) * H;
	size_t ws_bytes = 0u;
	STPGB_TRY(stpgb_shf_workspace_size(nn, radius, 0u, &ws_bytes));
	// a window holds at most min((2r+1)^2, 256) distinct values
	const uint64_t cap = npix * shf_kcap_h(radius, kShfMaxItems);
	struct Scoped {
		void* p = nullptr;
		~Scoped() {
			if (p) {
				cudaFree(p);
			}
		}
	} d_in, d_ws, d_off, d_bins, d_status;
	STPGB_CUDA_TRY(cudaMalloc(&d_in.p, in_bytes));
	STPGB_CUDA_TRY(cudaMalloc(&d_ws.p, ws_bytes));
	STPGB_CUDA_TRY(cudaMalloc(&d_off.p, (npix + 1u) * sizeof(uint32_t)));
	STPGB_CUDA_TRY(cudaMalloc(&d_bins.p, std::max<uint64_t>(cap, 1u) * sizeof(stpgb_bin)));
	STPGB_CUDA_TRY(cudaMalloc(&d_status.p, sizeof(uint32_t)));
	cudaStream_t s = nullptr;
	STPGB_CUDA_TRY(cudaMemcpy(d_in.p, samplemap_host, in_bytes, cudaMemcpyHostToDevice));
	STPGB_TRY(stpgb_shf_filter(static_cast<uint16_t*>(d_in.p), nn, radius, 0u, d_ws.p, ws_bytes,
		static_cast<uint32_t*>(d_off.p), static_cast<stpgb_bin*>(d_bins.p), cap, static_cast<uint32_t*>(d_status.p), s));
	STPGB_TRY(stpgb_status_check(static_cast<uint32_t*>(d_status.p), s));
	STPGB_CUDA_TRY(cudaMemcpy(offsets_host, d_off.p, (npix + 1u) * sizeof(uint32_t), cudaMemcpyDeviceToHost));
	const uint64_t total = offsets_host[npix];
	*nbins = total;
	if (total > bins_capacity) {
		set_error("stpgb_shf_filter_host: bins capacity too small");
		return STPGB_ECAPACITY;
	}
	if (total > 0u) {
		STPGB_CUDA_TRY(cudaMemcpy(bins_host, d_bins.p, total * sizeof(stpgb_bin), cudaMemcpyDeviceToHost));
	}
	return STPGB_OK;
}

} // extern "C"
