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
	uint32_t* fast;  // [8] path record (ShfFastRecord), then [palette tiles][8] palette slots
	// output
	uint32_t* offsets;  // [W*H+1]
	stpgb_bin* bins;
	uint64_t bins_capacity;
	uint32_t* status;
};

// The few-values path (shf_fast.cu, shf_band.cu) filters a chunk whose read
// region holds at most kShfFastItems distinct sample values; other chunks
// take the general slides.  Its packed vertical histograms (12 bytes per
// column and row, or per band) overlay `vbuf`, which that chunk does not
// otherwise use.
constexpr uint32_t kShfFastItems = 8u;
// A job's path: the general slides or the few-values path.
constexpr uint32_t kShfModeSlide = 0u, kShfModeFast = 1u;
// Rows of the read region per palette tile.
constexpr uint32_t kShfPaletteRows = 32u;
// The row-band formulation keeps a row's tables in shared memory: at most
// this many columns (W + 2r), bands of at least this many rows.
constexpr uint32_t kShfBandMaxCols = 4096u;
constexpr uint32_t kShfBandMinRows = 4u;

// Record of the path a job takes, written by the routing kernel: words
// {mode, distinct values, formulation (kShfForm*, 0 for the general slides),
// 0, then the values as 8 uint16, ascending}.
struct ShfFastRecord {
	uint32_t mode, count, form, pad;
	uint16_t item[kShfFastItems];
};
static_assert(sizeof(ShfFastRecord) == 32u, "record is 8 words");

// the general slides' kernels filter only the jobs routed to them
__device__ __forceinline__ bool shf_job_general(const ShfJob& J) {
	return reinterpret_cast<const volatile ShfFastRecord*>(J.fast)->mode == kShfModeSlide;
}

struct ShfLayout {
	size_t vbuf, vn, rows, fast, total;
};

// Workspace layout for one job (256-byte aligned sub-buffers).
ShfLayout shf_layout(uint32_t W, uint32_t H, uint32_t r, uint32_t kcap_v);
// Points the job's workspace fields at the sub-buffers of `ws` (laid out by shf_layout).
void shf_bind_workspace(ShfJob& job, unsigned char* ws, const ShfLayout& l);
uint32_t shf_kcap_v(uint32_t r, uint32_t max_items);
uint32_t shf_kcap_h(uint32_t r, uint32_t max_items);

// Runs the whole filter for `njobs` jobs (device array `jobs`, or `single`
// when jobs == nullptr). max_W/max_H/max_r bound the grids.
// `segments`: the general slides' columns and rows cut into this many
// segments (clamped to [1, kShfMaxSegments] and the slide length); 0 = chosen
// from the launch size.  `path`: 0 = the process-wide choice
// (stpgb_shf_set_path, by size by default), else that choice for this launch
// (1 packed slides, 2 row bands, 3 general slides).
int shf_launch(const ShfJob* jobs, const ShfJob& single, uint32_t njobs, uint32_t max_W, uint32_t max_H,
	uint32_t max_r, uint32_t kcap_v, uint32_t kcap_h, cudaStream_t stream, uint32_t segments = 0u,
	uint32_t path = 0u);

// The few-values path's launches around the general slides: palette and
// vertical histograms, then the bin count per row (before the row scan), and
// the write pass (after it).  Jobs that do not qualify return at once.  Two
// formulations: sequential slides in packed form (a thread per column, then
// per row) for launches of many chunks, row bands with prefix scans (a block
// per band of rows) for launches of few.
struct ShfBandLaunch {
	uint32_t band_rows, bands, threads, cols_per_thread, max_cols;
	size_t smem;
};
struct ShfFastPlan {
	bool bands;
	uint32_t max_cols; // widest chunk (W + 2r) the dense path takes; 0: none
	ShfBandLaunch band;
};
// stpgb_shf_set_path's choice (0 = by size)
uint32_t shf_path_override();
// the record's form: the few-values formulation that filtered the job
constexpr uint32_t kShfFormSlides = 1u, kShfFormBands = 2u;
ShfFastPlan shf_fast_plan(uint32_t njobs, uint32_t max_W, uint32_t max_H, uint32_t max_r, uint32_t path = 0u);
int shf_fast_prepare(const ShfJob* jobs, const ShfJob& single, uint32_t njobs, uint32_t max_W, uint32_t max_H,
	uint32_t max_r, uint32_t kcap_h, const ShfFastPlan& plan, cudaStream_t stream);
int shf_fast_pass(const ShfJob* jobs, const ShfJob& single, uint32_t njobs, uint32_t max_H, const ShfFastPlan& plan,
	bool write, cudaStream_t stream);
// the row-band formulation (shf_band.cu)
ShfBandLaunch shf_band_config(uint32_t njobs, uint32_t max_W, uint32_t max_H, uint32_t max_r);
int shf_band_carry_launch(const ShfJob* jobs, const ShfJob& single, uint32_t njobs, uint32_t max_W, uint32_t max_r,
	const ShfBandLaunch& cfg, cudaStream_t stream);
int shf_band_rows_launch(const ShfJob* jobs, const ShfJob& single, uint32_t njobs, const ShfBandLaunch& cfg,
	bool write, cudaStream_t stream);

} // namespace stpgb
