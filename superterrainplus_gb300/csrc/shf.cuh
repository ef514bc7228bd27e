// Single histogram filter: job descriptor and batched launch entry shared by
// the per-chunk C ABI (shf.cu) and the batched pipeline.
#pragma once

#include "internal.hpp"

namespace stpgb {

// Library bound on the number of distinct sample values inside one filter
// window; it sizes the per-thread accumulators in shared memory.
constexpr uint32_t kShfMaxItems = 256u;

// Most segments a column (vertical pass) or row (horizontal pass) is cut
// into; the workspace holds one bin count per (row, segment).
constexpr uint32_t kShfMaxSegments = 16u;

// One filter invocation over one chunk.  `samplemap` points at the top-left
// pixel of the chunk's nearest-neighbour region (TotalMapSize), rows `pitch`
// elements apart; the central chunk starts at (sx, sy).
struct ShfJob {
	const uint16_t* samplemap;
	uint64_t pitch;
	uint32_t W, H, sx, sy, r;
	uint32_t kcap_v; // accumulator capacity of the vertical pass (<= 2r+1)
	// workspace
	uint32_t* vbuf;  // [W+2r][kcap_v][H] packed (item << 16 | count), column-major
	uint16_t* vn;    // [W+2r][H] entries per vertical histogram
	uint32_t* rows;  // [H*segments+1] bins per (row, segment), then exclusive prefix + total
	// output
	uint32_t* offsets;  // [W*H+1]
	stpgb_bin* bins;
	uint64_t bins_capacity;
	uint32_t* status;
};

struct ShfLayout {
	size_t vbuf, vn, rows, total;
};

// Workspace layout for one job (256-byte aligned sub-buffers).
ShfLayout shf_layout(uint32_t W, uint32_t H, uint32_t r, uint32_t kcap_v);
uint32_t shf_kcap_v(uint32_t r, uint32_t max_items);
uint32_t shf_kcap_h(uint32_t r, uint32_t max_items);

// Runs the whole filter for `njobs` jobs (device array `jobs`, or `single`
// when jobs == nullptr). max_W/max_H/max_r bound the grids.
// `segments`: columns and rows cut into this many segments (clamped to
// [1, kShfMaxSegments] and the slide length); 0 = chosen from the launch size.
int shf_launch(const ShfJob* jobs, const ShfJob& single, uint32_t njobs, uint32_t max_W, uint32_t max_H,
	uint32_t max_r, uint32_t kcap_v, uint32_t kcap_h, cudaStream_t stream, uint32_t segments = 0u);

} // namespace stpgb
