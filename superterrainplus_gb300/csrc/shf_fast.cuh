// Single histogram filter, few-values path: device helpers shared by its two
// formulations (shf_fast.cu: sequential slides in packed form for launches of
// many chunks; shf_band.cu: row bands with prefix scans for launches of few).
//
// A chunk qualifies when its read region ((H+2r) x (W+2r) samples) holds at
// most kShfFastItems distinct values (biome maps: a Voronoi map of 8 biomes,
// the demo's layer chain).  Values are renamed to local indices 0..7 (their
// rank in the chunk's palette), so a histogram lives in registers: eight byte
// counts in one 64-bit word (or eight 16-bit fields in four words), and the
// reference accumulator's order (STPSingleHistogramFilter.cpp:400-450:
// insertion order with erase-compaction) as eight 4-bit indices in one
// 32-bit word.
#pragma once

#include "shf.cuh"

namespace stpgb {
namespace shfx {

constexpr uint32_t kNoValue = 0xFFFFFFFFu;
// words per palette slot and per record: {count, 0, values as uint16 pairs x4, 0, 0}
constexpr uint32_t kSlotWords = 8u;
// the byte counts hold 2r+2 (add before remove), the 16-bit fields
// (2r+1)(2r+2), a column's ring of local indices 2r+2
constexpr uint32_t kFastMaxRadius = 126u;

__device__ __forceinline__ const ShfJob& pick(const ShfJob* jobs, const ShfJob& single) {
	return jobs ? jobs[blockIdx.y] : single;
}

// first sample of the read region: row sy - r, column sx - r
__device__ __forceinline__ const uint16_t* read_region(const ShfJob& J) {
	return J.samplemap + static_cast<uint64_t>(J.sy - J.r) * J.pitch + (J.sx - J.r);
}

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

// local index of a palette value: the number of palette values below it
// (a padding field, 0xFFFF, is never below a 16-bit value)
__device__ __forceinline__ uint32_t local_index(const Palette p, const uint32_t v) {
	const uint32_t vv = v * 0x00010001u;
	return (__popc(__vcmpgtu2(vv, p.x)) + __popc(__vcmpgtu2(vv, p.y)) + __popc(__vcmpgtu2(vv, p.z))
			   + __popc(__vcmpgtu2(vv, p.w)))
		>> 4;
}

// Union of a job's palette slots, ascending, in vals[0..n) (kNoValue after);
// false when a tile or the union holds more than kShfFastItems values.
__device__ __forceinline__ bool palette_union(const ShfJob& J, uint32_t* const vals, uint32_t& n) {
	const uint32_t NR = J.H + 2u * J.r;
	const uint32_t tiles = (NR + kShfPaletteRows - 1u) / kShfPaletteRows;
	n = 0u;
	bool ok = true;
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
	for (uint32_t j = n; j < kShfFastItems; j++) {
		vals[j] = kNoValue;
	}
	return ok;
}

// The palette of a job routed to the dense path, from its record.
__device__ __forceinline__ Palette record_palette(const ShfFastRecord* const rec) {
	const uint32_t n = rec->count;
	const uint32_t* const rw = reinterpret_cast<const uint32_t*>(rec->item);
	auto half = [&](const uint32_t j) {
		return j < n ? ((rw[j / 2u] >> (16u * (j & 1u))) & 0xFFFFu) : 0xFFFFu;
	};
	return make_uint4(half(0) | (half(1) << 16), half(2) | (half(3) << 16), half(4) | (half(5) << 16),
		half(6) | (half(7) << 16));
}

// the job's path record (the routing kernel writes it)
__device__ __forceinline__ void write_record(const ShfJob& J, const uint32_t mode, const uint32_t count,
	const uint32_t* const vals, const uint32_t form) {
	ShfFastRecord* const rec = reinterpret_cast<ShfFastRecord*>(J.fast);
	rec->mode = mode;
	rec->count = count;
	rec->form = mode == kShfModeSlide ? 0u : form;
	rec->pad = 0u;
	for (uint32_t j = 0u; j < kShfFastItems; j++) {
		rec->item[j] = static_cast<uint16_t>(j < count ? vals[j] : 0u);
	}
}

// ----------------------------------------------------- eight 16-bit fields --

__device__ __forceinline__ uint4 add4(const uint4 a, const uint4 b) {
	return make_uint4(__vadd2(a.x, b.x), __vadd2(a.y, b.y), __vadd2(a.z, b.z), __vadd2(a.w, b.w));
}
__device__ __forceinline__ uint4 sub4(const uint4 a, const uint4 b) {
	return make_uint4(__vsub2(a.x, b.x), __vsub2(a.y, b.y), __vsub2(a.z, b.z), __vsub2(a.w, b.w));
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

// fields of a that are zero, as 0xFFFF halves
__device__ __forceinline__ uint4 zero4(const uint4 a) {
	return make_uint4(__vcmpeq2(a.x, 0u), __vcmpeq2(a.y, 0u), __vcmpeq2(a.z, 0u), __vcmpeq2(a.w, 0u));
}

// a hint to bring the line of p into L1 (callers keep p inside the buffer)
__device__ __forceinline__ void prefetch_l1(const void* p) {
	asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

} // namespace shfx
} // namespace stpgb
