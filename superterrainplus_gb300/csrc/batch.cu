// Batched heightfield pipeline: many eroded-chunk requests (each a 3x3
// free-slip neighbourhood, chunks of uneven side, own filter radius, droplet
// count and brush) generated, filtered and eroded by one fixed sequence of
// batched kernel launches -- every launch covers every chunk of every
// request (grid.y = job; the erosion is one launch per variant group, side by
// side, and the warp-cooperative kernel interleaves the blocks of several
// jobs in a one-dimensional grid) -- captured once into a CUDA graph and
// replayed.
//
// Device layout per request (side S, all buffers resident, one allocation):
//   biome region   (5S)^2 uint16   the 3x3 diversity neighbourhoods of all
//                                   nine chunks overlap inside a 5x5 region
//   merged height  (3S)^2 float    noise writes each chunk straight into its
//                                   place, erosion runs on it in place
//   fixed height   (3S)^2 uint16   formatted output
//   per chunk      filter workspace, offsets (S^2+1), bins
//   starts, brush, residual sediment
// No merge/unmerge copies are needed: a chunk's filter input is a window of
// the biome region and its heightmap a window of the merged map.
#include "erosion.cuh"
#include "layers.cuh"
#include "noise.cuh"
#include "shf.cuh"

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

namespace stpgb {
int starts_launch(float* xy, uint32_t count, uint64_t seed, uint64_t base, uint32_t map_x, uint32_t map_y,
	uint32_t nn_x, uint32_t nn_y, cudaStream_t stream);
int voronoi_launch(uint16_t* out, uint32_t pitch, uint32_t width, uint32_t height, int64_t ox, int64_t oy,
	uint32_t cell, uint32_t biomes, uint64_t seed, cudaStream_t stream);
} // namespace stpgb

using namespace stpgb;

namespace {

// 512-byte sub-allocations: a fixed heightmap or a biome region can then be
// bound to a texture as it is (the texture base alignment of the GPU)
size_t al(size_t v) {
	return (v + 511u) & ~static_cast<size_t>(511u);
}

struct RequestLayout {
	size_t biome, height, fixed, starts, brush_idx, brush_w;
	size_t shf_ws[9], offsets[9], bins[9];
	uint64_t bins_cap;
	size_t end;
};

// Erosion variant groups: requests whose brush takes the row kernels
// (rows_max_lanes() >= 2) with few enough droplets in flight per pixel for the
// warp-cooperative kernel; the other requests that may take several lanes per
// droplet (erosion_variant_stable) with row blocks; those whose brush is too
// small for rows (radius 2); and requests too densely packed for anything but
// the one-lane reference kernel.  Each group has its own job
// array, kernel variant and autotuning, and the erosion stage launches the
// groups side by side.  One variant for the whole batch would hold every
// request to the most restricted one: a single radius-2 brush, or one small
// chunk with all of its droplets in flight, would put them all on the
// point-wise kernels.
struct ErosionGroup {
	std::vector<ErosionJob> h;
	ErosionJob* jobs = nullptr;    // device copy of h
	uint32_t max_count = 0u, max_brush = 0u;
	uint32_t lane_limit = 32u;     // max_lanes() of the smallest brush
	uint32_t rows_limit = 4u;      // rows_max_lanes() of the smallest brush
	uint32_t min_radius = 0xFFFFFFFFu;
	// largest droplet density (droplets per centre-chunk pixel); the
	// autotuner only tries the variants stable at this density
	double density = 0.0;
	double in_flight = 0.0; // largest droplets in flight per pixel
	uint64_t droplets = 0u;
	uint32_t lanes = 8u; // lanes per droplet
	uint32_t dpg = 1u;   // droplets per lane group
	bool rows = true;    // brush rows in 16-byte blocks
	// warp-cooperative kernel: jobs interleaved beyond erosion_coop_interleave's
	// rule (the autotuner's choice; more jobs keep fewer droplets of each in flight)
	uint32_t interleave_extra = 0u;
	// autotuner's erosion time per candidate, [rows 0, 1][lanes 1..32][droplets 1, 2, 4] (0 = not tried)
	float tune_ms[36] = {};

	void add(const ErosionJob& e, const uint32_t radius, const double d, const double f) {
		h.push_back(e);
		max_count = std::max(max_count, e.count);
		max_brush = std::max(max_brush, e.brush_size);
		lane_limit = std::min(lane_limit, max_lanes(e.brush_size));
		rows_limit = std::min(rows_limit, rows_max_lanes(radius));
		min_radius = std::min(min_radius, radius);
		density = std::max(density, d);
		in_flight = std::max(in_flight, f);
		droplets += e.count;
		// the default until the autotuner runs: brush rows (the warp-cooperative
		// kernel where it is stable, else two lanes per droplet), else several
		// lanes point by point, else the reference kernel
		const bool multi = erosion_variant_stable(2u, 1u, true, density, in_flight);
		rows = multi && rows_limit != 0u;
		lanes = rows ? (erosion_variant_stable(1u, 1u, true, density, in_flight) && in_flight <= kCoopDefaultInFlight
							   ? 1u
							   : 2u)
			: multi  ? std::min(8u, lane_limit)
					 : 1u;
		dpg = 1u;
	}

	int launch(cudaStream_t s) const {
		return erosion_launch(jobs, h[0], static_cast<uint32_t>(h.size()), max_count, max_brush, s, lanes, false, dpg,
			rows, erosion_rows_wide(min_radius), erosion_rows_atomic(min_radius, lanes),
			coop_interleave());
	}

	uint32_t coop_interleave() const {
		return erosion_coop_interleave(h.data(), static_cast<uint32_t>(h.size())) + interleave_extra;
	}
};

} // namespace

struct stpgb_batch {
	std::vector<stpgb_batch_request> req;
	stpgb_raindrop_setting base {};
	uint32_t biome_count = 0u, max_items = 0u;
	unsigned char* mem = nullptr;
	size_t bytes = 0u;
	std::vector<RequestLayout> layout;
	// device tables
	uint8_t* perm = nullptr;
	float* grad = nullptr;
	stpgb_permutation permutation {};
	stpgb_biome_property* table = nullptr;
	double* residual = nullptr;
	uint32_t* status = nullptr;
	unsigned long long* counters = nullptr; // realised droplet steps, brush-erosion steps
	// job arrays (device) and launch bounds
	ShfJob* shf_jobs = nullptr;
	NoiseJob* noise_jobs = nullptr;
	FormatJob* fmt_jobs = nullptr;
	std::vector<ShfJob> shf_h;
	std::vector<NoiseJob> noise_h;
	std::vector<ErosionJob> ero_h; // per request, request order (the plain sequence)
	std::vector<FormatJob> fmt_h;
	uint32_t max_S = 0u, max_r = 0u, kcap_v = 0u, kcap_h = 0u;
	// the filter's path (0 = by size, 1 few-values packed slides, 2 row bands,
	// 3 general slides), the general slides' segment count (0 = from the
	// launch size) and the noise kernel's block size, chosen by the autotuner;
	// its times per candidate
	static constexpr uint32_t kShfPathCands = 4u, kShfSegCands = 6u, kNoiseBlockCands = 3u;
	static constexpr uint32_t shf_seg_cands[kShfSegCands] = { 0u, 1u, 2u, 4u, 8u, 16u };
	static constexpr uint32_t noise_block_cands[kNoiseBlockCands] = { 128u, 256u, 512u };
	uint32_t shf_path = 0u, shf_segments = 0u, noise_block = 256u;
	float shf_path_ms[kShfPathCands] = {}, shf_tune_ms[kShfSegCands] = {}, noise_tune_ms[kNoiseBlockCands] = {};
	// erosion variant groups (brush rows in 16-byte blocks need aligned maps:
	// every merged map of a batch is 512-byte aligned with a pitch of
	// 3 * MapSize, a multiple of 24 floats); group_of[n] is request n's group
	static constexpr uint32_t kGroups = 4u;
	ErosionGroup grp[kGroups];
	uint32_t ngroups = 0u;
	std::vector<uint32_t> group_of;
	// launch streams of the groups after the first, and the events that fork
	// them from the batch's stream and join them back
	cudaStream_t aux[kGroups - 1u] = {};
	cudaEvent_t fork = nullptr, join[kGroups - 1u] = {};
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
	bool use_graph = false;
	// STPGB_BATCH_AUTOTUNE: the autotuner runs at the first stpgb_batch_run,
	// on the inputs the caller has uploaded or synthesized by then
	bool tune_pending = false;

	// (re)captures the launch sequence into a graph
	int capture() {
		if (exec) {
			cudaGraphExecDestroy(exec);
			exec = nullptr;
		}
		if (graph) {
			cudaGraphDestroy(graph);
			graph = nullptr;
		}
		cudaStream_t cs;
		STPGB_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
		STPGB_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
		const int rc = enqueue(cs);
		cudaGraph_t g = nullptr;
		const cudaError_t ce = cudaStreamEndCapture(cs, &g);
		cudaStreamDestroy(cs);
		if (rc != STPGB_OK) {
			if (g) {
				cudaGraphDestroy(g);
			}
			return rc;
		}
		STPGB_CUDA_TRY(ce);
		graph = g;
		STPGB_CUDA_TRY(cudaGraphInstantiate(&exec, g, 0));
		return STPGB_OK;
	}

	~stpgb_batch() {
		if (exec) {
			cudaGraphExecDestroy(exec);
		}
		if (graph) {
			cudaGraphDestroy(graph);
		}
		for (void* p : { static_cast<void*>(mem), static_cast<void*>(perm), static_cast<void*>(grad),
				 static_cast<void*>(table), static_cast<void*>(residual), static_cast<void*>(status),
				 static_cast<void*>(counters),
				 static_cast<void*>(shf_jobs), static_cast<void*>(noise_jobs), static_cast<void*>(grp[0].jobs),
				 static_cast<void*>(grp[1].jobs), static_cast<void*>(grp[2].jobs), static_cast<void*>(grp[3].jobs),
				 static_cast<void*>(fmt_jobs) }) {
			if (p) {
				cudaFree(p);
			}
		}
		if (fork) {
			cudaEventDestroy(fork);
		}
		for (uint32_t k = 0u; k + 1u < kGroups; k++) {
			if (join[k]) {
				cudaEventDestroy(join[k]);
			}
			if (aux[k]) {
				cudaStreamDestroy(aux[k]);
			}
		}
	}

	// the erosion stage: one launch per group, the later groups on their own
	// streams so that the groups run side by side
	int erode(cudaStream_t s) {
		if (ngroups == 1u) {
			return grp[0].launch(s);
		}
		STPGB_CUDA_TRY(cudaEventRecord(fork, s));
		for (uint32_t g = 1u; g < ngroups; g++) {
			STPGB_CUDA_TRY(cudaStreamWaitEvent(aux[g - 1u], fork, 0));
		}
		int rc = grp[0].launch(s);
		for (uint32_t g = 1u; g < ngroups; g++) {
			const int rg = grp[g].launch(aux[g - 1u]);
			rc = rc != STPGB_OK ? rc : rg;
			STPGB_CUDA_TRY(cudaEventRecord(join[g - 1u], aux[g - 1u]));
			STPGB_CUDA_TRY(cudaStreamWaitEvent(s, join[g - 1u], 0));
		}
		return rc;
	}

	// the group the tuning report describes: the one with the most droplets
	const ErosionGroup& dominant() const {
		uint32_t best = 0u;
		for (uint32_t g = 1u; g < ngroups; g++) {
			if (grp[g].droplets > grp[best].droplets) {
				best = g;
			}
		}
		return grp[best];
	}

	// the whole pipeline as a fixed launch sequence
	int enqueue(cudaStream_t s) {
		STPGB_CUDA_TRY(cudaMemsetAsync(residual, 0, sizeof(double) * req.size(), s));
		STPGB_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(uint32_t), s));
		for (uint32_t st = 0u; st < 4u; st++) {
			STPGB_TRY(stage(st, s));
		}
		return STPGB_OK;
	}

	// stage 0: filter, 1: noise, 2: erosion, 3: format
	int stage(uint32_t st, cudaStream_t s) {
		const uint32_t nchunks = static_cast<uint32_t>(shf_h.size());
		switch (st) {
		case 0u:
			return shf_launch(shf_jobs, shf_h[0], nchunks, max_S, max_S, max_r, kcap_v, kcap_h, s, shf_segments,
				shf_path);
		case 1u:
			return noise_launch(noise_jobs, noise_h[0], nchunks, static_cast<uint64_t>(max_S) * max_S, permutation,
				table, biome_count, s, noise_block);
		case 2u:
			return erode(s);
		case 3u:
			return format_batch_launch(fmt_jobs, static_cast<uint32_t>(req.size()), 3u * max_S, 3u * max_S, s);
		default:
			return inval("stpgb_batch_run_stage: stage must be 0..3");
		}
	}

	// Autotuner: the filter's segment count and the noise kernel's block size
	// (each candidate timed twice, the faster kept; every candidate gives the
	// same output), then each group's erosion launch with every candidate
	// variant (noise regenerates the heights before each trial, so every
	// trial erodes the same map), keeping the fastest per group.
	int autotune() {
		cudaStream_t s;
		STPGB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
		cudaEvent_t e0, e1;
		STPGB_CUDA_TRY(cudaEventCreate(&e0));
		STPGB_CUDA_TRY(cudaEventCreate(&e1));
		int rc = STPGB_OK;
		auto time_stage = [&](const uint32_t st, float& out) {
			for (int rep = 0; rep < 3 && rc == STPGB_OK; rep++) {
				cudaEventRecord(e0, s);
				rc = stage(st, s);
				cudaEventRecord(e1, s);
				if (cudaStreamSynchronize(s) != cudaSuccess) {
					rc = cuda_fail(cudaGetLastError(), "autotune");
				}
				float ms = 0.0f;
				cudaEventElapsedTime(&ms, e0, e1);
				if (rep > 0) { // the first run warms the caches and the code
					out = rep == 1 ? ms : std::min(out, ms);
				}
			}
		};
		float best_path = 0.0f;
		uint32_t pick_path = shf_path;
		for (uint32_t c = 0u; c < kShfPathCands && rc == STPGB_OK; c++) {
			shf_path = c;
			time_stage(0u, shf_path_ms[c]);
			if (rc == STPGB_OK && (best_path == 0.0f || shf_path_ms[c] < best_path)) {
				best_path = shf_path_ms[c];
				pick_path = shf_path;
			}
		}
		shf_path = pick_path;
		float best_shf = 0.0f;
		uint32_t pick_seg = shf_segments;
		for (uint32_t c = 0u; c < kShfSegCands && rc == STPGB_OK; c++) {
			shf_segments = shf_seg_cands[c];
			time_stage(0u, shf_tune_ms[c]);
			if (rc == STPGB_OK && (best_shf == 0.0f || shf_tune_ms[c] < best_shf)) {
				best_shf = shf_tune_ms[c];
				pick_seg = shf_segments;
			}
		}
		shf_segments = pick_seg;
		if (rc == STPGB_OK) {
			rc = stage(0u, s);
		}
		float best_noise = 0.0f;
		uint32_t pick_block = noise_block;
		for (uint32_t c = 0u; c < kNoiseBlockCands && rc == STPGB_OK; c++) {
			noise_block = noise_block_cands[c];
			time_stage(1u, noise_tune_ms[c]);
			if (rc == STPGB_OK && (best_noise == 0.0f || noise_tune_ms[c] < best_noise)) {
				best_noise = noise_tune_ms[c];
				pick_block = noise_block;
			}
		}
		noise_block = pick_block;
		const uint32_t cands[6] = { 1u, 2u, 4u, 8u, 16u, 32u };
		const uint32_t dcands[3] = { 1u, 2u, 4u };
		for (uint32_t gi = 0u; gi < ngroups && rc == STPGB_OK; gi++) {
			ErosionGroup& G = grp[gi];
			float best = 0.0f;
			uint32_t best_lanes = G.lanes, best_dpg = G.dpg, best_extra = 0u;
			G.interleave_extra = 0u;
			bool best_rows = G.rows;
			for (int c = 0; c < 36 && rc == STPGB_OK; c++) {
				const bool cr = c >= 18;
				const uint32_t cl = cands[(c % 18) / 3], cd = dcands[c % 3];
				// lane counts above the brush limit, and several droplets per group
				// below four lanes or above sixteen, are not candidates; brush rows
				// run with 2 or 4 lanes (up to rows_limit) and 1 or 2 droplets, or
				// warp-cooperatively (1 lane, 1 droplet) where the brush allows rows
				if (!cr && (cl > G.lane_limit || (cd > 1u && (cl < 4u || cl > 16u)))) {
					continue;
				}
				if (cr && !(G.rows_limit != 0u
							   && ((cl == 1u && cd == 1u) || (cl >= 2u && cl <= G.rows_limit && cd <= 2u)))) {
					continue;
				}
				if (!erosion_variant_stable(cl, cd, cr, G.density, G.in_flight)) {
					continue;
				}
				G.lanes = cl;
				G.dpg = cd;
				G.rows = cr;
				float t = 0.0f;
				for (int rep = 0; rep < 2 && rc == STPGB_OK; rep++) {
					rc = stage(1u, s);
					if (rc == STPGB_OK) {
						cudaEventRecord(e0, s);
						rc = G.launch(s);
						cudaEventRecord(e1, s);
					}
					if (cudaStreamSynchronize(s) != cudaSuccess) {
						rc = cuda_fail(cudaGetLastError(), "autotune");
					}
					float ms = 0.0f;
					cudaEventElapsedTime(&ms, e0, e1);
					t = rep == 0 ? ms : std::min(t, ms);
				}
				G.tune_ms[c] = t;
				if (rc == STPGB_OK && (best == 0.0f || t < best)) {
					best = t;
					best_lanes = cl;
					best_dpg = cd;
					best_rows = cr;
				}
			}
			G.lanes = best_lanes;
			G.dpg = best_dpg;
			G.rows = best_rows;
			// the warp-cooperative kernel over several jobs: also with 1, 2, 4, 8 and 12
			// more jobs interleaved than the rule gives, and with every job of the group
			// (a remainder group of a few jobs at the end of the launch runs dense and long)
			if (rc == STPGB_OK && G.rows && G.lanes == 1u && G.dpg == 1u) {
				const uint32_t base_q = G.coop_interleave();
				const uint32_t njob = static_cast<uint32_t>(G.h.size());
				uint32_t extras[6];
				uint32_t ne = 0u;
				for (const uint32_t e : { 1u, 2u, 4u, 8u, 12u }) {
					if (base_q + e <= njob) {
						extras[ne++] = e;
					}
				}
				if (njob > base_q && (ne == 0u || extras[ne - 1u] != njob - base_q)) {
					extras[ne++] = njob - base_q;
				}
				for (uint32_t xi = 0u; xi < ne && rc == STPGB_OK; xi++) {
					const uint32_t extra = extras[xi];
					G.interleave_extra = extra;
					float t = 0.0f;
					for (int rep = 0; rep < 2 && rc == STPGB_OK; rep++) {
						rc = stage(1u, s);
						if (rc == STPGB_OK) {
							cudaEventRecord(e0, s);
							rc = G.launch(s);
							cudaEventRecord(e1, s);
						}
						if (cudaStreamSynchronize(s) != cudaSuccess) {
							rc = cuda_fail(cudaGetLastError(), "autotune");
						}
						float ms = 0.0f;
						cudaEventElapsedTime(&ms, e0, e1);
						t = rep == 0 ? ms : std::min(t, ms);
					}
					if (rc == STPGB_OK && t < best) {
						best = t;
						best_extra = extra;
					}
				}
				G.interleave_extra = best_extra;
			}
		}
		cudaEventDestroy(e0);
		cudaEventDestroy(e1);
		cudaStreamDestroy(s);
		return rc;
	}

	// the same work as the per-chunk drop-in call sequence: one chunk's filter
	// + noise per call, then one erosion + format per request, the stream
	// synchronised after every call as the reference's generate()/erode() do
	int enqueue_plain(cudaStream_t s) {
		for (size_t n = 0; n < req.size(); n++) {
			for (uint32_t c = 0u; c < 9u; c++) {
				const ShfJob& j = shf_h[9u * n + c];
				STPGB_CUDA_TRY(cudaMemsetAsync(j.status, 0, sizeof(uint32_t), s));
				STPGB_TRY(shf_launch(nullptr, j, 1u, j.W, j.H, j.r, kcap_v, kcap_h, s));
				const NoiseJob& nj = noise_h[9u * n + c];
				STPGB_TRY(noise_launch(nullptr, nj, 1u, static_cast<uint64_t>(nj.W) * nj.H, permutation, table, biome_count, s));
				STPGB_CUDA_TRY(cudaStreamSynchronize(s));
			}
			const ErosionJob& e = ero_h[n];
			const ErosionGroup& G = grp[group_of[n]];
			STPGB_CUDA_TRY(cudaMemsetAsync(e.residual, 0, sizeof(double), s));
			STPGB_TRY(erosion_launch(nullptr, e, 1u, e.count, e.brush_size, s, G.lanes, false, G.dpg, G.rows,
				erosion_rows_wide(G.min_radius), erosion_rows_atomic(G.min_radius, G.lanes)));
			const FormatJob& f = fmt_h[n];
			STPGB_TRY(format_launch(f.in, f.in_pitch, f.out, f.out_pitch, f.W, f.H, s));
			STPGB_CUDA_TRY(cudaStreamSynchronize(s));
		}
		return STPGB_OK;
	}
};

namespace {

int check_request(const stpgb_batch_request& r) {
	if (r.MapSize == 0u || (r.MapSize & 7u) != 0u || r.MapSize > 16384u) {
		return inval("stpgb_batch: MapSize must be a positive multiple of 8, at most 16384");
	}
	if (r.InterpolationRadius == 0u || (r.InterpolationRadius & 1u) || r.InterpolationRadius > r.MapSize) {
		return inval("stpgb_batch: radius must be positive, even and at most MapSize");
	}
	if (r.BrushRadius == 0u || 2u * r.BrushRadius + 2u >= 3u * r.MapSize) {
		return inval("stpgb_batch: brush radius must be positive and fit the merged map");
	}
	return STPGB_OK;
}

template<typename T>
int upload(T*& dst, const std::vector<T>& src) {
	STPGB_CUDA_TRY(cudaMalloc(&dst, std::max<size_t>(src.size(), 1u) * sizeof(T)));
	STPGB_CUDA_TRY(cudaMemcpy(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
	return STPGB_OK;
}

} // namespace

extern "C" {

int stpgb_batch_create(const stpgb_batch_request* requests, uint32_t count, const stpgb_raindrop_setting* base,
	const stpgb_simplex_setting* simplex, const stpgb_biome_property* biome_table, uint32_t biome_count,
	uint64_t hbm_budget, uint32_t flags, stpgb_batch** out) {
	if (!requests || count == 0u || !base || !simplex || !biome_table || biome_count == 0u || !out) {
		return inval("stpgb_batch_create: null argument or empty batch");
	}
	STPGB_TRY(stpgb_simplex_setting_validate(simplex));
	STPGB_TRY(stpgb_raindrop_setting_validate(base));
	auto b = std::make_unique<stpgb_batch>();
	b->req.assign(requests, requests + count);
	b->base = *base;
	b->biome_count = biome_count;
	b->max_items = std::min<uint32_t>(biome_count, kShfMaxItems);
	for (const auto& r : b->req) {
		STPGB_TRY(check_request(r));
		b->max_S = std::max(b->max_S, r.MapSize);
		b->max_r = std::max(b->max_r, r.InterpolationRadius);
	}
	b->kcap_v = shf_kcap_v(b->max_r, b->max_items);
	b->kcap_h = shf_kcap_h(b->max_r, b->max_items);

	// layout
	size_t off = 0u;
	std::vector<std::vector<int32_t>> brush_i(count);
	std::vector<std::vector<float>> brush_w(count);
	for (uint32_t n = 0u; n < count; n++) {
		const auto& r = b->req[n];
		const size_t S = r.MapSize;
		RequestLayout L {};
		L.biome = off;
		off += al(25u * S * S * sizeof(uint16_t));
		L.height = off;
		off += al(9u * S * S * sizeof(float));
		L.fixed = off;
		off += al(9u * S * S * sizeof(uint16_t));
		L.starts = off;
		off += al(2u * static_cast<size_t>(r.DropletCount) * sizeof(float));
		uint32_t bs = 0u;
		stpgb_erosion_brush_generate(3u * r.MapSize, r.BrushRadius, nullptr, nullptr, 0u, &bs);
		brush_i[n].resize(bs);
		brush_w[n].resize(bs);
		STPGB_TRY(stpgb_erosion_brush_generate(3u * r.MapSize, r.BrushRadius, brush_i[n].data(), brush_w[n].data(), bs, &bs));
		L.brush_idx = off;
		off += al(bs * sizeof(int32_t));
		L.brush_w = off;
		off += al(bs * sizeof(float));
		const ShfLayout sl = shf_layout(r.MapSize, r.MapSize, r.InterpolationRadius, b->kcap_v);
		L.bins_cap = S * S * std::min<uint64_t>(shf_kcap_h(r.InterpolationRadius, b->max_items),
			(2ull * r.InterpolationRadius + 1u) * (2ull * r.InterpolationRadius + 1u));
		for (int c = 0; c < 9; c++) {
			L.shf_ws[c] = off;
			off += al(sl.total);
			L.offsets[c] = off;
			off += al((S * S + 1u) * sizeof(uint32_t));
			L.bins[c] = off;
			off += al(L.bins_cap * sizeof(stpgb_bin));
		}
		L.end = off;
		b->layout.push_back(L);
	}
	b->bytes = off;
	if (hbm_budget != 0u && off > hbm_budget) {
		set_error("stpgb_batch_create: the batch needs " + std::to_string(off) + " bytes, above the HBM budget");
		return STPGB_ENOMEM;
	}
	{
		const cudaError_t e = cudaMalloc(&b->mem, off);
		if (e != cudaSuccess) {
			cudaGetLastError();
			set_error("stpgb_batch_create: device allocation of " + std::to_string(off) + " bytes failed");
			return STPGB_ENOMEM;
		}
	}

	// tables
	std::vector<uint8_t> perm(512);
	std::vector<float> grad(2u * simplex->Distribution);
	STPGB_TRY(stpgb_permutation_generate(simplex, perm.data(), grad.data(), static_cast<uint32_t>(grad.size())));
	STPGB_TRY(upload(b->perm, perm));
	STPGB_TRY(upload(b->grad, grad));
	b->permutation = stpgb_permutation { b->perm, b->grad, simplex->Distribution };
	STPGB_TRY(upload(b->table, std::vector<stpgb_biome_property>(biome_table, biome_table + biome_count)));
	STPGB_CUDA_TRY(cudaMalloc(&b->residual, sizeof(double) * count));
	STPGB_CUDA_TRY(cudaMalloc(&b->status, sizeof(uint32_t)));
	STPGB_CUDA_TRY(cudaMalloc(&b->counters, 2u * sizeof(unsigned long long)));
	STPGB_CUDA_TRY(cudaMemset(b->counters, 0, 2u * sizeof(unsigned long long)));

	// jobs
	for (uint32_t n = 0u; n < count; n++) {
		const auto& r = b->req[n];
		const RequestLayout& L = b->layout[n];
		const uint32_t S = r.MapSize;
		unsigned char* const m = b->mem;
		STPGB_CUDA_TRY(cudaMemcpy(m + L.brush_idx, brush_i[n].data(), brush_i[n].size() * sizeof(int32_t), cudaMemcpyHostToDevice));
		STPGB_CUDA_TRY(cudaMemcpy(m + L.brush_w, brush_w[n].data(), brush_w[n].size() * sizeof(float), cudaMemcpyHostToDevice));
		uint16_t* const biome = reinterpret_cast<uint16_t*>(m + L.biome);
		float* const height = reinterpret_cast<float*>(m + L.height);
		for (uint32_t c = 0u; c < 9u; c++) {
			const uint32_t cx = c % 3u, cy = c / 3u;
			const ShfLayout sl = shf_layout(S, S, r.InterpolationRadius, b->kcap_v);
			ShfJob j {};
			j.samplemap = biome + static_cast<size_t>(cy) * S * (5u * S) + static_cast<size_t>(cx) * S;
			j.pitch = 5u * S;
			j.W = S;
			j.H = S;
			j.sx = S;
			j.sy = S;
			j.r = r.InterpolationRadius;
			j.kcap_v = b->kcap_v;
			shf_bind_workspace(j, m + L.shf_ws[c], sl);
			j.offsets = reinterpret_cast<uint32_t*>(m + L.offsets[c]);
			j.bins = reinterpret_cast<stpgb_bin*>(m + L.bins[c]);
			j.bins_capacity = L.bins_cap;
			j.status = b->status;
			b->shf_h.push_back(j);
			NoiseJob nj {};
			nj.out = height + static_cast<size_t>(cy) * S * (3u * S) + static_cast<size_t>(cx) * S;
			nj.pitch = 3u * S;
			nj.offsets = j.offsets;
			nj.bins = j.bins;
			nj.W = S;
			nj.H = S;
			// chunk map offset of neighbour (cx-1, cy-1) around the request's centre chunk
			// (STPChunk::calcChunkMapOffset: chunk unit * MapSize)
			nj.off_x = static_cast<float>((static_cast<int64_t>(r.ChunkX) + cx - 1) * S);
			nj.off_y = static_cast<float>((static_cast<int64_t>(r.ChunkY) + cy - 1) * S);
			b->noise_h.push_back(nj);
		}
		stpgb_raindrop_setting rs = b->base;
		rs.RainDropCount = r.DropletCount;
		rs.ErosionBrushRadius = r.BrushRadius;
		if (r.Lifetime != 0u) {
			rs.minWaterVolume = stpgb_lifetime_min_water_volume(rs.initWaterVolume, rs.EvaporateSpeed, r.Lifetime);
		}
		ErosionJob e {};
		e.map = height;
		e.dim_x = 3u * S;
		e.dim_y = 3u * S;
		e.pitch = 3u * S;
		e.starts = reinterpret_cast<float*>(m + L.starts);
		e.count = r.DropletCount;
		e.brush_index = reinterpret_cast<int32_t*>(m + L.brush_idx);
		e.brush_weight = reinterpret_cast<float*>(m + L.brush_w);
		e.brush_size = static_cast<uint32_t>(brush_i[n].size());
		e.p = rain_params(rs);
		e.residual = b->residual + n;
		e.status = b->status;
		e.counters = b->counters;
		e.start_area = S * S;
		e.fixed = reinterpret_cast<uint16_t*>(m + L.fixed);
		b->ero_h.push_back(e);
		b->fmt_h.push_back(FormatJob { height, 3ull * S, e.fixed, 3ull * S, 3u * S, 3u * S });
		const double area = static_cast<double>(S) * S;
		const double density = r.DropletCount / area, in_flight = erosion_in_flight(r.DropletCount, area);
		const uint32_t cls = !erosion_variant_stable(2u, 1u, true, density, in_flight) ? 3u
			: rows_max_lanes(r.BrushRadius) == 0u                                        ? 2u
			: erosion_variant_stable(1u, 1u, true, density, in_flight)                   ? 0u
																						  : 1u;
		b->group_of.push_back(cls);
		b->grp[cls].add(e, r.BrushRadius, density, in_flight);
	}
	{
		// the non-empty groups first, in their order
		uint32_t remap[stpgb_batch::kGroups] = {}, k = 0u;
		ErosionGroup packed[stpgb_batch::kGroups];
		for (uint32_t g = 0u; g < stpgb_batch::kGroups; g++) {
			if (!b->grp[g].h.empty()) {
				remap[g] = k;
				packed[k++] = std::move(b->grp[g]);
			}
		}
		for (uint32_t g = 0u; g < stpgb_batch::kGroups; g++) {
			b->grp[g] = std::move(packed[g]);
		}
		for (auto& g : b->group_of) {
			g = remap[g];
		}
		b->ngroups = k;
	}
	STPGB_TRY(upload(b->shf_jobs, b->shf_h));
	STPGB_TRY(upload(b->noise_jobs, b->noise_h));
	for (uint32_t g = 0u; g < b->ngroups; g++) {
		STPGB_TRY(upload(b->grp[g].jobs, b->grp[g].h));
	}
	STPGB_TRY(upload(b->fmt_jobs, b->fmt_h));
	if (b->ngroups > 1u) {
		STPGB_CUDA_TRY(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
		for (uint32_t g = 1u; g < b->ngroups; g++) {
			STPGB_CUDA_TRY(cudaStreamCreateWithFlags(&b->aux[g - 1u], cudaStreamNonBlocking));
			STPGB_CUDA_TRY(cudaEventCreateWithFlags(&b->join[g - 1u], cudaEventDisableTiming));
		}
	}

	b->tune_pending = (flags & STPGB_BATCH_AUTOTUNE) != 0u;
	b->use_graph = (flags & STPGB_BATCH_GRAPH) != 0u;
	if (b->use_graph) {
		STPGB_TRY(b->capture());
	}
	*out = b.release();
	return STPGB_OK;
}

int stpgb_batch_tune(stpgb_batch* b) {
	if (!b) {
		return inval("stpgb_batch_tune: null batch");
	}
	STPGB_CUDA_TRY(cudaDeviceSynchronize());
	b->tune_pending = false;
	STPGB_TRY(b->autotune());
	return b->use_graph ? b->capture() : STPGB_OK;
}

int stpgb_batch_destroy(stpgb_batch* b) {
	delete b;
	return STPGB_OK;
}

uint64_t stpgb_batch_device_bytes(const stpgb_batch* b) {
	return b ? b->bytes : 0u;
}

int stpgb_batch_buffers(stpgb_batch* b, uint32_t request, uint16_t** biome_region, float** heightmap,
	uint16_t** heightmap_fixed, float** starts_xy) {
	if (!b || request >= b->req.size()) {
		return inval("stpgb_batch_buffers: request out of range");
	}
	const RequestLayout& L = b->layout[request];
	if (biome_region) {
		*biome_region = reinterpret_cast<uint16_t*>(b->mem + L.biome);
	}
	if (heightmap) {
		*heightmap = reinterpret_cast<float*>(b->mem + L.height);
	}
	if (heightmap_fixed) {
		*heightmap_fixed = reinterpret_cast<uint16_t*>(b->mem + L.fixed);
	}
	if (starts_xy) {
		*starts_xy = reinterpret_cast<float*>(b->mem + L.starts);
	}
	return STPGB_OK;
}

int stpgb_batch_synthesize_inputs(stpgb_batch* b, uint32_t voronoi_cell, uint64_t seed, void* stream) {
	if (!b || voronoi_cell == 0u) {
		return inval("stpgb_batch_synthesize_inputs: invalid argument");
	}
	const cudaStream_t s = as_stream(stream);
	for (size_t n = 0; n < b->req.size(); n++) {
		const auto& r = b->req[n];
		const RequestLayout& L = b->layout[n];
		const uint32_t S = r.MapSize;
		STPGB_TRY(voronoi_launch(reinterpret_cast<uint16_t*>(b->mem + L.biome), 5u * S, 5u * S, 5u * S,
			(static_cast<int64_t>(r.ChunkX) - 2) * S, (static_cast<int64_t>(r.ChunkY) - 2) * S, voronoi_cell,
			b->biome_count, seed, s));
		// droplet counter space: the request's centre chunk coordinate keeps starts distinct per chunk
		const uint64_t base = (static_cast<uint64_t>(static_cast<uint32_t>(r.ChunkX)) << 40)
			^ (static_cast<uint64_t>(static_cast<uint32_t>(r.ChunkY)) << 20);
		STPGB_TRY(starts_launch(reinterpret_cast<float*>(b->mem + L.starts), r.DropletCount, b->base.Seed, base, S, S,
			3u, 3u, s));
	}
	return STPGB_OK;
}

int stpgb_batch_synthesize_layer_biomes(stpgb_batch* b, uint64_t seed, void* stream) {
	if (!b) {
		return inval("stpgb_batch_synthesize_layer_biomes: null batch");
	}
	LayerChain chain;
	STPGB_TRY(layer_chain_demo(seed, &chain));
	const cudaStream_t s = as_stream(stream);
	for (size_t n = 0; n < b->req.size(); n++) {
		const auto& r = b->req[n];
		const uint32_t S = r.MapSize;
		BiomemapJob job {};
		job.out = reinterpret_cast<uint16_t*>(b->mem + b->layout[n].biome);
		job.x0 = static_cast<int32_t>((static_cast<int64_t>(r.ChunkX) - 2) * S);
		job.z0 = static_cast<int32_t>((static_cast<int64_t>(r.ChunkY) - 2) * S);
		job.pitch = job.width = job.height = 5u * S;
		const uint32_t tile = layer_tile(chain, 25ull * S * S);
		STPGB_TRY(layer_job_tiling(job, tile));
		STPGB_TRY(layer_biomemap_launch(chain, nullptr, job, 1u, job.tiles, tile, s));
	}
	return STPGB_OK;
}

int stpgb_batch_run(stpgb_batch* b, void* stream) {
	if (!b) {
		return inval("stpgb_batch_run: null batch");
	}
	const cudaStream_t s = as_stream(stream);
	if (b->tune_pending) {
		// the caller's uploads on `s` complete before the tuner reads the inputs
		STPGB_CUDA_TRY(cudaStreamSynchronize(s));
		b->tune_pending = false;
		STPGB_TRY(b->autotune());
		if (b->use_graph) {
			STPGB_TRY(b->capture());
		}
	}
	if (b->exec) {
		STPGB_CUDA_TRY(cudaGraphLaunch(b->exec, s));
		return STPGB_OK;
	}
	return b->enqueue(s);
}

int stpgb_batch_run_plain(stpgb_batch* b, void* stream) {
	if (!b) {
		return inval("stpgb_batch_run_plain: null batch");
	}
	return b->enqueue_plain(as_stream(stream));
}

int stpgb_batch_upload(stpgb_batch* b, const uint16_t* const* biome_regions, const float* const* starts_xy,
	void* stream) {
	if (!b || !biome_regions) {
		return inval("stpgb_batch_upload: null argument");
	}
	const cudaStream_t s = as_stream(stream);
	for (size_t n = 0; n < b->req.size(); n++) {
		const size_t S = b->req[n].MapSize;
		STPGB_CUDA_TRY(cudaMemcpyAsync(b->mem + b->layout[n].biome, biome_regions[n], 25u * S * S * sizeof(uint16_t),
			cudaMemcpyHostToDevice, s));
		if (starts_xy && starts_xy[n]) {
			STPGB_CUDA_TRY(cudaMemcpyAsync(b->mem + b->layout[n].starts, starts_xy[n],
				2u * sizeof(float) * b->req[n].DropletCount, cudaMemcpyHostToDevice, s));
		}
	}
	return STPGB_OK;
}

int stpgb_batch_download(stpgb_batch* b, float* const* heightmaps, uint16_t* const* heightmaps_fixed,
	double* residual_sediment, void* stream) {
	if (!b) {
		return inval("stpgb_batch_download: null batch");
	}
	const cudaStream_t s = as_stream(stream);
	for (size_t n = 0; n < b->req.size(); n++) {
		const size_t S = b->req[n].MapSize;
		if (heightmaps && heightmaps[n]) {
			STPGB_CUDA_TRY(cudaMemcpyAsync(heightmaps[n], b->mem + b->layout[n].height, 9u * S * S * sizeof(float),
				cudaMemcpyDeviceToHost, s));
		}
		if (heightmaps_fixed && heightmaps_fixed[n]) {
			STPGB_CUDA_TRY(cudaMemcpyAsync(heightmaps_fixed[n], b->mem + b->layout[n].fixed,
				9u * S * S * sizeof(uint16_t), cudaMemcpyDeviceToHost, s));
		}
	}
	if (residual_sediment) {
		STPGB_CUDA_TRY(cudaMemcpyAsync(residual_sediment, b->residual, sizeof(double) * b->req.size(),
			cudaMemcpyDeviceToHost, s));
	}
	return STPGB_OK;
}

int stpgb_batch_tuning(const stpgb_batch* b, uint32_t* lanes_per_droplet, uint32_t* droplets_per_group,
	uint32_t* vector_rows, float* erosion_ms) {
	if (!b) {
		return inval("stpgb_batch_tuning: null batch");
	}
	const ErosionGroup& G = b->dominant();
	if (lanes_per_droplet) {
		*lanes_per_droplet = G.lanes;
	}
	if (droplets_per_group) {
		*droplets_per_group = G.dpg;
	}
	if (vector_rows) {
		*vector_rows = G.rows ? 1u : 0u;
	}
	if (erosion_ms) {
		for (int c = 0; c < 36; c++) {
			erosion_ms[c] = G.tune_ms[c];
		}
	}
	return STPGB_OK;
}

int stpgb_batch_tuning_stages(const stpgb_batch* b, uint32_t* shf_segments, float* shf_ms, uint32_t* noise_block,
	float* noise_ms, uint32_t* coop_interleave) {
	if (!b) {
		return inval("stpgb_batch_tuning_stages: null batch");
	}
	if (coop_interleave) {
		const ErosionGroup& G = b->dominant();
		*coop_interleave = G.rows && G.lanes == 1u && G.dpg == 1u ? G.coop_interleave() : 0u;
	}
	if (shf_segments) {
		*shf_segments = b->shf_segments;
	}
	if (noise_block) {
		*noise_block = b->noise_block;
	}
	for (uint32_t c = 0u; c < stpgb_batch::kShfSegCands && shf_ms; c++) {
		shf_ms[c] = b->shf_tune_ms[c];
	}
	for (uint32_t c = 0u; c < stpgb_batch::kNoiseBlockCands && noise_ms; c++) {
		noise_ms[c] = b->noise_tune_ms[c];
	}
	return STPGB_OK;
}

int stpgb_batch_kernels_per_run(const stpgb_batch* b, uint32_t* kernels) {
	if (!b || !kernels) {
		return inval("stpgb_batch_kernels_per_run: null argument");
	}
	if (b->graph) {
		size_t n = 0u;
		STPGB_CUDA_TRY(cudaGraphGetNodes(b->graph, nullptr, &n));
		std::vector<cudaGraphNode_t> nodes(n);
		STPGB_CUDA_TRY(cudaGraphGetNodes(b->graph, nodes.data(), &n));
		uint32_t k = 0u;
		for (size_t i = 0u; i < n; i++) {
			cudaGraphNodeType t;
			STPGB_CUDA_TRY(cudaGraphNodeGetType(nodes[i], &t));
			k += t == cudaGraphNodeTypeKernel ? 1u : 0u;
		}
		*kernels = k;
		return STPGB_OK;
	}
	// without a graph: the filter's nine launches, noise, one erosion launch per group, format
	*kernels = 9u + 1u + b->ngroups + 1u;
	return STPGB_OK;
}

int stpgb_batch_tuning_filter_path(const stpgb_batch* b, uint32_t* path, float* path_ms) {
	if (!b) {
		return inval("stpgb_batch_tuning_filter_path: null batch");
	}
	if (path) {
		*path = b->shf_path;
	}
	for (uint32_t c = 0u; c < stpgb_batch::kShfPathCands && path_ms; c++) {
		path_ms[c] = b->shf_path_ms[c];
	}
	return STPGB_OK;
}

int stpgb_batch_run_stage(stpgb_batch* b, uint32_t stage, void* stream) {
	if (!b) {
		return inval("stpgb_batch_run_stage: null batch");
	}
	return b->stage(stage, as_stream(stream));
}

int stpgb_batch_counters(stpgb_batch* b, uint64_t* realised_steps, uint64_t* erode_steps, int reset) {
	if (!b) {
		return inval("stpgb_batch_counters: null batch");
	}
	unsigned long long h[2] = { 0u, 0u };
	STPGB_CUDA_TRY(cudaDeviceSynchronize());
	STPGB_CUDA_TRY(cudaMemcpy(h, b->counters, sizeof(h), cudaMemcpyDeviceToHost));
	if (realised_steps) {
		*realised_steps = h[0];
	}
	if (erode_steps) {
		*erode_steps = h[1];
	}
	if (reset) {
		STPGB_CUDA_TRY(cudaMemset(b->counters, 0, sizeof(h)));
	}
	return STPGB_OK;
}

int stpgb_batch_download_inputs(stpgb_batch* b, uint16_t* const* biome_regions, float* const* starts_xy,
	void* stream) {
	if (!b) {
		return inval("stpgb_batch_download_inputs: null batch");
	}
	const cudaStream_t s = as_stream(stream);
	for (size_t n = 0; n < b->req.size(); n++) {
		const size_t S = b->req[n].MapSize;
		if (biome_regions && biome_regions[n]) {
			STPGB_CUDA_TRY(cudaMemcpyAsync(biome_regions[n], b->mem + b->layout[n].biome, 25u * S * S * sizeof(uint16_t),
				cudaMemcpyDeviceToHost, s));
		}
		if (starts_xy && starts_xy[n]) {
			STPGB_CUDA_TRY(cudaMemcpyAsync(starts_xy[n], b->mem + b->layout[n].starts,
				2u * sizeof(float) * b->req[n].DropletCount, cudaMemcpyDeviceToHost, s));
		}
	}
	return STPGB_OK;
}

int stpgb_batch_status(stpgb_batch* b, void* stream) {
	if (!b) {
		return inval("stpgb_batch_status: null batch");
	}
	return stpgb_status_check(b->status, stream);
}

} // extern "C"
