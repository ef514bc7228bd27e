// Free-slip particle hydraulic erosion: job descriptor and launch.
#pragma once

#include "internal.hpp"

namespace stpgb {

// Droplet parameters of STPRainDropSetting that the step loop reads.
struct RainParams {
	float Inertia, SedimentCapacityFactor, minSedimentCapacity, initWaterVolume, minWaterVolume, Friction,
		initSpeed, ErodeSpeed, DepositSpeed, EvaporateSpeed, Gravity;
	uint32_t BrushRadius;
	uint32_t MaxSteps; // hard cap on the droplet loop
};

// One merged free-slip map eroded by `count` droplets.
struct ErosionJob {
	float* map;
	uint32_t dim_x, dim_y;
	uint64_t pitch; // floats per row of `map`
	const float* starts; // count (x, y) pairs, merged-map coordinates
	uint32_t count;
	const int32_t* brush_index; // relative to a row pitch of `pitch`
	const float* brush_weight;
	uint32_t brush_size;
	RainParams p;
	double* residual;
	uint32_t* status;
	uint16_t* fixed; // formatted output (optional, batched path)
	// optional counters: [0] realised steps, [1] steps that eroded over the brush
	unsigned long long* counters;
	// pixels of the area the starts cover (the centre chunk); with `count`
	// it gives the droplets in flight per pixel that bound the row kernel's
	// blocks per round trip (0: one block per trip)
	uint32_t start_area;
};

RainParams rain_params(const stpgb_raindrop_setting& s);

// lanes_per_droplet: 1, 2, 4, 8, 16 or 32 lanes carry one droplet;
// exact_clamp: brush updates by compare-and-swap (never more than a cell
// holds) instead of the reference's read-then-subtract order;
// droplets_per_group: 1, or 2 / 4 droplets advanced together by a group of
// 4, 8 or 16 lanes (reference order only);
// vector_rows: with 2 or 4 lanes and 1 or 2 droplets per group, update the
// brush run by run in 16-byte blocks (every map 16-byte aligned, pitch a
// multiple of four floats);
// wide_trips: with vector_rows, let every job that keeps at most
// kWideConcurrency droplets in flight per pixel of its start area read up to
// three blocks of a run per round trip (one droplet per group) or two (two
// droplets);
// atomic_brush: with vector_rows, take each block's brush amounts with one
// returning vector atomic and give back what a cell lacked;
// interleave: the warp-cooperative kernel (lanes_per_droplet 1 with
// vector_rows) alternates the blocks of that many consecutive jobs
int erosion_launch(const ErosionJob* jobs, const ErosionJob& single, uint32_t njobs, uint32_t max_count,
	uint32_t max_brush, cudaStream_t stream, uint32_t lanes_per_droplet, bool exact_clamp = false,
	uint32_t droplets_per_group = 1u, bool vector_rows = false, bool wide_trips = false, bool atomic_brush = false,
	uint32_t interleave = 1u);
// Jobs a warp-cooperative launch interleaves: enough that each keeps at most
// kCoopInterleaveInFlight droplets in flight per pixel, with the maps of the
// interleaved jobs together in half of the L2.
constexpr double kCoopInterleaveInFlight = 0.2;
uint32_t erosion_coop_interleave(const ErosionJob* jobs, uint32_t njobs);

// Largest lanes-per-droplet that keeps at least four brush points per lane,
// and the per-call default, min(8, max_lanes).
uint32_t max_lanes(uint32_t brush_size);
uint32_t default_lanes(uint32_t brush_size);

// Lanes per droplet (4 or 2) that keep four sequential 16-byte blocks per
// lane in the brush-row update of the circular brush of `radius`; 0 if none.
uint32_t rows_max_lanes(uint32_t radius);

// Racing droplets that share cells can dig a channel below its neighbours
// once they are packed densely enough; how densely depends on how compressed
// in time a droplet's brush update is.  Variants with several lanes per
// droplet are taken up to kDenseRows droplets per pixel of the start area and
// up to kDenseInFlight droplets in flight at once per pixel (min(droplets,
// resident droplets of the two-lane row kernel) / area); beyond either only
// one lane per droplet (the reference kernel) is used.  Ten-run tests on
// 64^2 chunks kept every variant in range up to 3 droplets per pixel, all in
// flight, but across many runs the two-lane row kernel fell below range
// twice with every droplet in flight: once at 3 per pixel (brush 4), once
// at 2.3 (a 128^2 chunk in a batch); the reference kernel never has, up to 7.
// The production chunk keeps 0.33 in flight per pixel, a 256^2 chunk at
// 2.3 per pixel 1.34.
constexpr double kDenseRows = 3.0;
constexpr double kDenseInFlight = 1.5;
// The warp-cooperative kernel (one droplet per lane, the warp's brush runs
// shared out over all lanes: lanes = 1 with rows) takes every run of a
// droplet's brush at once and keeps twice the droplets in flight; it is
// taken up to kCoopInFlight droplets in flight per pixel counted as for two
// lanes (0.75 of its own), where several blocks of a run per round trip were
// measured inside the reference kernel's RMS band.  The default prefers it
// to two lanes per droplet up to kCoopDefaultInFlight: brush 4 at 2.3
// droplets per pixel took 3.73 against 3.91 ms on one 3x3 x 512^2 map (0.33
// in flight), 13.1 against 14.9 on 3x3 x 1024^2 (0.08), 173 against 229 on a
// 4096^2 field, but 71.1 against 69.4 ms on the production batch of 16
// multi-biome 512^2 neighbourhoods, where the autotuner decides.
constexpr double kCoopInFlight = 0.375;
constexpr double kCoopDefaultInFlight = 0.2;
// Droplets in flight per pixel of `area` for `count` droplets.
double erosion_in_flight(uint32_t count, double area);
bool erosion_variant_stable(uint32_t lanes, uint32_t droplets_per_group, bool rows, double density, double in_flight);

// Several brush blocks per round trip compress a droplet's brush update
// further, which moves the racy result away from the serial one where many
// droplets share the map at once.  What counts is the droplets in flight per
// pixel of the start area (min(count, resident droplets) / area): measured
// against the one-thread-per-droplet kernel's band around the FP64 serial
// result, brush 4 at 0.67 in flight per pixel stays at 0.55 of the band with
// three blocks per trip, while at 2.26 two blocks already reach 1.34 (one
// block: 0.93).  Wide trips are therefore taken only up to kWideConcurrency
// droplets in flight per pixel, and from brush radius kWideMinRadius (brush 3
// on densely packed 64^2 chunks dug channels below range with them).
constexpr uint32_t kWideMinRadius = 4u;
constexpr double kWideConcurrency = 0.75;
// Droplets the row kernel keeps resident on this device with `lanes` lanes
// per droplet and `dpg` droplets per group.
uint32_t erosion_resident_droplets(uint32_t lanes, uint32_t dpg);
// Whether a launch whose smallest brush has `min_radius` may take wide trips
// (each job then decides by its own droplets in flight per pixel).
bool erosion_rows_wide(uint32_t min_radius);

// The brush update as one returning vector atomic per 16-byte block (the
// cell's value at the moment of the update, w subtracted, and the part of w
// the cell lacked given back) in place of a read and a later reduction: half
// the L2 requests, and no read-to-update window in which racing droplets see
// a stale height.  A cell waiting for its give-back is transiently w too low
// for other droplets' corner reads; with brush radius 3 and four lanes those
// dips fed on each other on densely packed 64^2 chunks (heights below range
// from 3 droplets per pixel, one run ran away at 7), while two lanes with
// brush 3, and brushes 4 and 5 in every variant, stayed in range up to 7
// droplets per pixel.  So it is taken from brush radius kAtomicMinRadius, and
// with two lanes per droplet.
constexpr uint32_t kAtomicMinRadius = 4u;
bool erosion_rows_atomic(uint32_t min_radius, uint32_t lanes);

// lanes == 1 with rows: the warp-cooperative kernel
struct ErosionChoice {
	uint32_t lanes, droplets_per_group;
	bool rows;
};
// Default kernel for a brush of `radius` (`brush_size` points) at `density`
// droplets per pixel of the start area, `in_flight` of them at once.
ErosionChoice erosion_choice(uint32_t radius, uint32_t brush_size, double density, double in_flight,
	bool rows_allowed);

int format_launch(const float* in, uint64_t in_pitch, uint16_t* out, uint64_t out_pitch, uint32_t W, uint32_t H,
	cudaStream_t stream);

// Formatting of many maps in one launch.
struct FormatJob {
	const float* in;
	uint64_t in_pitch;
	uint16_t* out;
	uint64_t out_pitch;
	uint32_t W, H;
};

int format_batch_launch(const FormatJob* jobs, uint32_t njobs, uint32_t max_W, uint32_t max_H, cudaStream_t stream);

} // namespace stpgb
