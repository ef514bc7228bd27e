#!/usr/bin/env python3
"""Eroded 512x512 chunks per second on one GB300: batched vs plain per-chunk.

Workload (production chunk): each eroded chunk is a 3x3 free-slip
neighbourhood of 512x512 float32 chunks (1536x1536).  For every one of the
nine chunks the single histogram filter (radius 32) runs over its own 3x3
neighbourhood of a seeded Voronoi biome map (8 biomes), then the multi-biome
fractal simplex heightfield (octaves 4-8, scale 64-512, amplitude 0.2-1.0)
is generated; then 600,000 droplets (brush radius 4, inertia 0.05, capacity 4,
min capacity 0.01, deposit 0.3, erode 0.3, evaporate 0.01, gravity 4,
lifetime 50) erode the neighbourhood and the result is formatted to uint16.

A step is one pass of that pipeline over a batch of B independent eroded
chunks (default 16) with inputs (biome regions, droplet starts) resident in
HBM.  `value` = eroded chunks per second of the batched path (one CUDA graph
of batched launches).  The plain per-chunk call sequence on the same data
and the end-to-end rate through the C ABI with host buffers are reported
beside it.  `--impl reference` times the path on the host cores through the
reference's own CPU code where it has one (its filter, built for the host by
oracle/build_ref.sh) and the CPU restatement elsewhere (noise, erosion,
format: the reference runs them on the GPU only), without loading the
library under test.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MAP = 512
BIOMES = 8
RADIUS = 32
DROPLETS = 600_000
BRUSH = 4
LIFETIME = 50
VORONOI_CELL = 192
SEED = 42
SIMPLEX = (SEED, 8, 0.2181661565)  # Distribution and Offset of the demo's Biome.ini
WORKLOAD = "production chunk: 3x3 neighbourhood of 512^2 float32 chunks, 8 biomes, filter radius 32, " \
           "600000 droplets, brush 4, lifetime 50"
METRIC = "512^2 eroded chunks/s (batched, 1 GB300)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--batch", type=int, default=16)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-large-field", action="store_true",
                   help="skip the 4096^2 large-field and the uneven-batch sections")
    p.add_argument("--serve-requests", type=int, default=600,
                   help="camera-walk requests replayed through the server (0 skips the serving section)")
    return p.parse_args()


def raindrop(m, count):
    return m.RaindropSetting(**raindrop_dict(count))


def biome_table(np, dtype):
    rng = np.random.default_rng(SEED)
    t = np.zeros(BIOMES, dtype)
    t["Scale"] = np.exp(rng.uniform(np.log(64.0), np.log(512.0), BIOMES)).astype(np.float32)
    t["Octave"] = rng.integers(4, 9, BIOMES)
    t["Persistence"] = 0.5
    t["Lacunarity"] = 2.0
    t["Depth"] = 0.0
    t["Variation"] = rng.uniform(0.2, 1.0, BIOMES).astype(np.float32)
    return t


def requests(batch, rank):
    # neighbourhoods 4 chunks apart: independent, no shared free-slip border
    return [dict(MapSize=MAP, ChunkX=4 * (rank * batch + n), ChunkY=-3 * rank, InterpolationRadius=RADIUS,
                 DropletCount=DROPLETS, BrushRadius=BRUSH, Lifetime=LIFETIME) for n in range(batch)]


# DRAM bytes and L2 atomic requests of the production batch's erosion launch (16 requests of a 3x3 x
# 512^2 merged map and 600,000 droplets each, all jobs interleaved) from a full ncu capture: 101.04 MB
# read + 25.90 MB written; 5.106 G atomic requests at the L2 (the brush's returning 16-byte atomics
# and the scalar deposits) and 0.272 G vector reductions (the deposits whose row pair shares a
# 16-byte block); the merged maps stay in L2, so all of it grows with the requests of a launch
EROSION_DRAM_BYTES_PER_REQUEST = (101.04e6 + 25.90e6) / 16
EROSION_L2_ATOMICS_PER_REQUEST = 5.106e9 / 16
EROSION_L2_REDUCTIONS_PER_REQUEST = 0.272e9 / 16


def erosion_traffic(requests_per_launch):
    """DRAM bytes per erosion launch of `requests_per_launch` production requests."""
    return EROSION_DRAM_BYTES_PER_REQUEST * requests_per_launch


def log(msg):
    """Progress of the run on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def max_over_ranks(value, dist, device):
    """The largest value over the ranks (the slowest replica's elapsed time); `dist` is
    torch.distributed after init_process_group, or None for one process."""
    if not dist:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measure_roofline_peaks(m, torch, reps=5):
    """The chip's rates for the kernels the HBM copy peak does not bound, from the library's
    measurement kernels (stpgb_roofline_launch) on an L2-resident 8 MiB map (the production merged
    map is 9.4 MB): random scalar and 16-byte float reductions, random 16-byte returning atomics,
    random 16-byte loads, the latency of one dependent L2 load, and the FP32 fused multiply-add
    rate.  Each kernel is timed with CUDA events on its stream after a warm-up launch; the best of
    `reps` launches is kept."""
    import ctypes as C
    L = m.lib()
    dev = torch.cuda.current_device()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    n = 1 << 21
    buf = torch.zeros(n, dtype=torch.float32, device="cuda")
    sink = torch.zeros(4, dtype=torch.int64, device="cuda")
    st = torch.cuda.current_stream()
    sh = C.c_void_p(st.cuda_stream)

    def timed(kind, buffer, elements, blocks, iters):
        m.check(L.stpgb_roofline_launch(kind, C.c_void_p(buffer.data_ptr()), elements, blocks, iters,
                                        C.c_void_p(sink.data_ptr()), sh))
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            m.check(L.stpgb_roofline_launch(kind, C.c_void_p(buffer.data_ptr()), elements, blocks, iters,
                                            C.c_void_p(sink.data_ptr()), sh))
            e1.record(st)
            torch.cuda.synchronize()
            t = e0.elapsed_time(e1) / 1000.0
            best = t if best is None else min(best, t)
        return best

    blocks, iters = sms * 16, 256
    ops = blocks * 256 * iters
    t_red = timed(0, buf, n, blocks, iters)
    t_red4 = timed(1, buf, n, blocks, iters)
    t_at4 = timed(5, buf, n, blocks, iters)
    buf.zero_()
    t_ld4 = timed(2, buf, n, blocks, iters)
    # dependent loads: one random cycle through 2^21 entries
    perm = torch.randperm(n, generator=torch.Generator().manual_seed(7))
    nxt = torch.empty(n, dtype=torch.int64)
    nxt[perm] = torch.roll(perm, -1)
    table = nxt.to(torch.int32).cuda()
    chase_steps = 1 << 16
    timed(3, table, n, 1, chase_steps)
    ticks = int(sink[0].item())
    fma_blocks, fma_iters = sms * 8, 1 << 14
    t_fma = timed(4, buf, 1, fma_blocks, fma_iters)
    return {"red_f32_gops": ops / t_red / 1e9, "red_f32_gbs": 4 * ops / t_red / 1e9,
            "red_v4_f32_gbs": 16 * ops / t_red4 / 1e9, "load_v4_gbs": 16 * ops / t_ld4 / 1e9,
            "atom_v4_f32_gbs": 16 * ops / t_at4 / 1e9,
            "dependent_l2_load_cycles": ticks / chase_steps,
            "fp32_fma_tflops": fma_blocks * 256 * fma_iters * 16 / t_fma / 1e12,
            "map_bytes": 4 * n, "sms": sms,
            "method": "stpgb_roofline_launch kernels, best of %d event-timed launches; random addresses over an "
                      "8 MiB L2-resident map" % reps}


def erosion_l2_roofline(peaks, steps_total, erode_steps, brush_size, stage_ms):
    """Roofline of an erosion launch against the measured L2 rates.  Per realised step the
    reference's algorithm gathers 32 B (two bilinear corner reads); an eroding step reads and then
    atomically updates its brush (4 B + 4 B per point), a depositing step updates four corners
    (16 B).  The launch can take no less than loads / load rate + reductions / reduction rate (the
    16-byte vector forms, the fastest the chip offers); frac = that time / the launch's time."""
    loads = steps_total * 32 + erode_steps * 4 * brush_size
    reds = erode_steps * 4 * brush_size + (steps_total - erode_steps) * 16
    t = stage_ms / 1000.0
    t_min = loads / (peaks["load_v4_gbs"] * 1e9) + reds / (peaks["red_v4_f32_gbs"] * 1e9)
    total = loads + reds
    return {"bound": "l2", "achieved": total / t / 1e9, "peak": total / t_min / 1e9, "unit": "GB/s",
            "frac": t_min / t, "load_bytes": loads, "reduction_bytes": reds,
            "peak_note": "mix-weighted: L2 loads at the measured random 16-byte load rate, reductions at the "
                         "measured random 16-byte vector reduction rate"}


def l2_atomic_roofline(peaks, requests, stage_ms):
    """The erosion launch's L2 atomic work against the measured random 16-byte rates: the
    captured returning-atomic and reduction requests (scaled by the requests per launch), each
    counted as a 16-byte operation; frac = their time at the measured returning-atomic and
    reduction rates / the launch's time."""
    atom = EROSION_L2_ATOMICS_PER_REQUEST * requests
    red = EROSION_L2_REDUCTIONS_PER_REQUEST * requests
    t = stage_ms / 1000.0
    t_min = 16 * atom / (peaks["atom_v4_f32_gbs"] * 1e9) + 16 * red / (peaks["red_v4_f32_gbs"] * 1e9)
    return {"atomic_requests_per_launch": atom, "reduction_requests_per_launch": red,
            "achieved_gbs": 16 * (atom + red) / t / 1e9, "peak_gbs": 16 * (atom + red) / t_min / 1e9,
            "frac": t_min / t,
            "source": "ncu capture of the 16-request launch, scaled by the requests per launch",
            "peak_note": "mix-weighted: returning atomics at the measured random 16-byte returning-atomic "
                         "rate (atom.global.add.v4.f32, the brush's operation), reductions at the measured "
                         "random 16-byte reduction rate; one request per 16-byte block"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device_index):
        self.idx = device_index
        self.samples = []
        self.stop_ev = threading.Event()
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        while not self.stop_ev.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self.stop_ev.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop_ev.set()
        self.t.join(timeout=10)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx = float(s[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ CPU leg


def raindrop_dict(count):
    """The workload's droplet settings; the lifetime is expressed through minWaterVolume: the next
    float above the volume left after LIFETIME evaporation steps in float32."""
    import numpy as np
    evap = 0.01
    v = np.float32(1.0)
    for _ in range(LIFETIME):
        v = np.float32(v * np.float32(1.0 - np.float32(evap)))
    return dict(Seed=SEED, RainDropCount=count, Inertia=0.05, SedimentCapacityFactor=4.0, minSedimentCapacity=0.01,
                initWaterVolume=1.0, minWaterVolume=float(np.nextafter(v, np.float32(np.inf))), Friction=0.1,
                initSpeed=1.0, ErodeSpeed=0.3, DepositSpeed=0.3, EvaporateSpeed=evap, Gravity=4.0,
                ErosionBrushRadius=BRUSH)


def reference_eroded_chunk(threads, droplets=DROPLETS):
    """One eroded chunk of the workload on the host cores, each stage through the reference's own CPU
    code where it has one:
      * filter: the reference's STPSingleHistogramFilter built for this host by oracle/build_ref.sh,
        with the shipped 4-thread Parallel buffer (STPSingleHistogramFilter.cpp:36, chosen by the demo
        for chunks of 100,000 pixels and more), the nine calls shared out over threads // 4 workers,
        as the reference's generator workers call one filter concurrently;
      * noise, erosion, format: the reference runs these on the GPU only; the CPU restatement of the
        multi-biome generator script (rows split over the threads), the serial FP32 droplet loop and
        the format loop stand in.  Each equals the reference's own device code run on the host bit
        for bit (the erosion on this very workload: 600,000 droplets on the 1536^2 map).
    Without the reference build the filter is the restatement too.  Nothing here loads the library
    under test.  Returns (seconds, threads, kind, sample, seconds per stage, kind per stage)."""
    import concurrent.futures as cf

    import numpy as np

    from oracle.oracle import BIOME_DTYPE, Oracle, Reference
    orc = Oracle()
    try:
        ref = Reference()
    except (FileNotFoundError, OSError):
        ref = None
    S = MAP
    region = orc.voronoi(5 * S, 5 * S, (-2 * S, -2 * S), VORONOI_CELL, BIOMES, SEED)
    table = biome_table(np, BIOME_DTYPE)
    rc, perm, grad = (ref or orc).permutation(*SIMPLEX)
    rd = raindrop_dict(droplets)
    starts = orc.droplet_starts(droplets, SEED, 0, (S, S), (3, 3))
    idx, w = orc.brush(3 * S, BRUSH)
    subs = [np.ascontiguousarray(region[(c // 3) * S:(c // 3) * S + 3 * S, (c % 3) * S:(c % 3) * S + 3 * S])
            for c in range(9)]
    t = [time.perf_counter()]
    if ref:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(9, threads // 4))) as ex:
            hists = list(ex.map(lambda a: ref.shf(a, (S, S), (3, 3), RADIUS, parallel=True, capacity=8 * S * S),
                                subs))
    else:
        with cf.ThreadPoolExecutor(max_workers=min(threads, 9)) as ex:
            hists = list(ex.map(lambda a: orc.shf(a, (S, S), (3, 3), RADIUS), subs))
    t.append(time.perf_counter())
    merged = np.zeros((3 * S, 3 * S), np.float32)
    for c, (rc, off, bins) in enumerate(hists):
        h = orc.multibiome(off, bins, table, perm, grad, (S, S), (float((c % 3 - 1) * S), float((c // 3 - 1) * S)),
                           threads=threads)
        merged[(c // 3) * S:(c // 3 + 1) * S, (c % 3) * S:(c % 3 + 1) * S] = h
    t.append(time.perf_counter())
    orc.erode(merged, rd, starts, idx, w, fp64=False)
    t.append(time.perf_counter())
    orc.format(merged)
    t.append(time.perf_counter())
    stages = dict(zip(["single_histogram_filter", "multibiome_noise", "hydraulic_erosion", "format"],
                      [t[k + 1] - t[k] for k in range(4)]))
    kinds = {k: "port" for k in stages}
    if ref:
        kinds["single_histogram_filter"] = "reference"
        sample = (f"1 eroded chunk of the workload ({droplets} droplets): the reference's own filter built for the "
                  f"host (4-thread buffer, {max(1, min(9, threads // 4))} concurrent calls); noise, serial FP32 "
                  f"erosion and format through the CPU restatement (the reference has no CPU code for them), "
                  f"{threads} threads")
    else:
        sample = f"1 eroded chunk of the workload ({droplets} droplets), CPU restatement, {threads} threads"
    return t[-1] - t[0], threads, "reference" if ref else "port", sample, stages, kinds


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        reference_eroded_chunk(threads)
    runs = [reference_eroded_chunk(threads) for _ in range(args.steps)]
    total = sum(r[0] for r in runs)
    kind, sample = runs[0][2], runs[0][3]
    value = args.steps / total
    stages = {k: statistics.median(r[4][k] for r in runs) * 1000.0 for k in runs[0][4]}
    kinds = runs[0][5]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "chunks/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": "1 eroded chunk per step", "impl": sample},
            "stage_ms": stages, "stage_kind": kinds,
            "cpu_baseline": {"value": value, "unit": "chunks/s", "cores": threads, "kind": kind,
                             "sample": "1 eroded chunk per step", "stage_kind": kinds},
            "e2e": {"value": value, "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ GPU leg


def run_ours(args):
    import numpy as np
    import torch

    import superterrainplus_gb300 as m

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    B = args.batch
    reqs = requests(B, rank)
    table = biome_table(np, m.BIOME_DTYPE)
    base = raindrop(m, DROPLETS)
    simplex = m.SimplexSetting(*SIMPLEX)
    log("production batch: create, synthesize, tune")
    batch = m.Batch(reqs, base, simplex, table, graph=True)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    batch.synthesize(VORONOI_CELL, SEED, sh)
    stream.synchronize()
    # the autotuner times the filter's segment counts, the noise block sizes and the erosion
    # variants on these inputs, then the graph is re-captured
    batch.tune()
    lanes, tune_ms = batch.tuning()
    stage_tune = batch.tuning_stages()
    filter_path = batch.tuning_filter_path()
    kernels_per_step = batch.kernels_per_run()

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    log("production batch: warm-up and timed steps")
    for _ in range(max(args.warmup, 3)):
        batch.run(sh)
    barrier()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        torch.cuda.nvtx.range_push("timed_region")
        evs[0].record(stream)
        for k in range(args.steps):
            batch.run(sh)
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    batch.status(sh)
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    elapsed = evs[0].elapsed_time(evs[-1]) / 1000.0
    elapsed = max_over_ranks(elapsed, dist, "cuda")
    value = world * B * args.steps / elapsed

    # per-stage device time (stage kernels launched alone, CUDA events on the launching stream)
    stage_names = ["single_histogram_filter", "multibiome_noise", "hydraulic_erosion", "format"]
    stage_ms = []
    for st in range(4):
        batch.run_stage(st, sh)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 3
        e0.record(stream)
        for _ in range(reps):
            batch.run_stage(st, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        stage_ms.append(e0.elapsed_time(e1) / reps)
    # droplet step counts of one batch (algorithmic bytes of the erosion kernel)
    batch.counters(reset=True)
    batch.run(sh)
    steps_total, erode_steps = batch.counters(reset=True)
    brush_size = len(m.erosion_brush(3 * MAP, BRUSH)[0])

    # plain per-chunk call sequence on the same resident data
    log("plain per-chunk calls")
    batch.run_plain(sh)
    t0 = time.perf_counter()
    batch.run_plain(sh)
    plain_s = time.perf_counter() - t0
    plain_value = B / plain_s

    # end to end through the C ABI with host buffers: inputs H2D, outputs D2H, every step
    log("end to end")
    S = MAP
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    # host inputs of the same kind (Voronoi regions, central-chunk starts), made by the library's
    # own kernels and kept in pinned memory
    dev = m.DeviceOps()
    host_biome, host_starts = [], []
    for n, r in enumerate(reqs):
        tb = torch.empty((5 * S, 5 * S), dtype=torch.int16, device="cuda")
        dev.voronoi_biomemap(tb, 5 * S, 5 * S, 5 * S, ((r["ChunkX"] - 2) * S, (r["ChunkY"] - 2) * S), VORONOI_CELL,
                             BIOMES, SEED)
        ts = torch.empty(2 * DROPLETS, dtype=torch.float32, device="cuda")
        dev.droplet_starts(ts, DROPLETS, SEED, n * DROPLETS, (S, S), (3, 3))
        host_biome.append(tb.cpu().pin_memory().numpy().view(np.uint16))
        host_starts.append(ts.cpu().pin_memory().numpy())
    torch.cuda.synchronize()
    h2d = B * (25 * S * S * 2 + 2 * DROPLETS * 4)
    d2h = B * 9 * S * S * (4 + 2) + B * 8
    # as many end-to-end steps as timed device steps: a host-side stall in one of a few steps
    # moved the figure by up to 15 %
    e2e_steps = max(3, args.steps)

    def host_outputs():
        return ([pin((3 * S, 3 * S), torch.float32) for _ in range(B)],
                [pin((3 * S, 3 * S), torch.int16).view(np.uint16) for _ in range(B)], pin(B, torch.float64))

    # one batch, each step's copies and kernels one after the other
    out0 = host_outputs()
    for _ in range(2):
        batch.upload(host_biome, host_starts, sh)
        batch.run(sh)
        batch.download(*out0, sh)
        stream.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        batch.upload(host_biome, host_starts, sh)
        batch.run(sh)
        batch.download(*out0, sh)
        stream.synchronize()
    e2e_serial_value = B / ((time.perf_counter() - t0) / e2e_steps)
    batch.status(sh)
    # double-buffered, as a serving caller runs it: two batches alternate on two streams, so one
    # step's input upload and result download overlap the other step's kernels
    batch2 = m.Batch(reqs, base, simplex, table, graph=True)
    stream2 = torch.cuda.Stream()
    batch2.upload(host_biome, host_starts, stream2.cuda_stream)
    stream2.synchronize()
    batch2.tune()
    pipes = [(batch, stream, out0), (batch2, stream2, host_outputs())]
    # the kernels of one step wait for the other stream's kernels (an event after each run): only
    # copies overlap kernels, two erosions never share the L2
    ran = [None]

    def pipe_step(k):
        b_, st_, out_ = pipes[k % 2]
        st_.synchronize()  # this batch's previous step, and its host outputs, are done
        b_.upload(host_biome, host_starts, st_.cuda_stream)
        if ran[0] is not None:
            st_.wait_event(ran[0])
        b_.run(st_.cuda_stream)
        ran[0] = torch.cuda.Event()
        ran[0].record(st_)
        b_.download(*out_, st_.cuda_stream)

    for k in range(4):
        pipe_step(k)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        pipe_step(k)
    torch.cuda.synchronize()
    e2e_value = B * e2e_steps / (time.perf_counter() - t0)
    batch.status(sh)
    batch2.status(stream2.cuda_stream)
    del batch2

    peak, peak_kind = load_peaks()
    log("roofline peaks")
    peaks = measure_roofline_peaks(m, torch)
    dom = int(np.argmax(stage_ms))
    roof_stage = stage_names[dom]
    roof = None
    if roof_stage == "hydraulic_erosion":
        roof = erosion_l2_roofline(peaks, steps_total, erode_steps, brush_size, stage_ms[dom])
        alg_bytes = roof["load_bytes"] + roof["reduction_bytes"]
        roof.update({
            "kernel": roof_stage, "traffic": erosion_traffic(B),
            "traffic_source": "DRAM read + write of the 16-request production erosion launch (ncu capture), "
                              "scaled by the requests per launch: the merged maps stay in L2",
            "algorithmic_bytes_per_launch": alg_bytes,
            "hbm": {"achieved": alg_bytes / (stage_ms[dom] / 1000.0) / 1e9, "peak": peak, "peak_source": peak_kind,
                    "frac": alg_bytes / (stage_ms[dom] / 1000.0) / 1e9 / peak},
            "l2_atomics": l2_atomic_roofline(peaks, B, stage_ms[dom]),
            "dependent_l2_load_cycles": peaks["dependent_l2_load_cycles"],
            "note": "per realised step: 32 B corner gathers, then 4 B read + 4 B reduction per brush point "
                    "(eroding) or 16 B of reductions (depositing); more droplets in flight, fewer round trips "
                    "and fewer instructions per step measured no faster: the L2's atomic throughput under "
                    "this access pattern bounds the kernel"})
    elif roof_stage == "format":
        fb = B * 9 * S * S * (4 + 2)
        achieved = fb / (stage_ms[dom] / 1000.0) / 1e9
        roof = {"bound": "hbm", "kernel": roof_stage, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": fb}

    stage_roof = stage_rooflines(m, np, torch, dev, host_biome, table, stage_ms, stage_names, peak, peak_kind,
                                 peaks)

    serving = None
    if rank == 0 and args.serve_requests > 0:
        log("serving")
        serving = serve_section(m, np, torch, args.serve_requests)
        serving["at_120_per_s"] = serve_section(m, np, torch, args.serve_requests, rate=120.0, plain=False)
        serving["layer_chain_biomes"] = serve_section(m, np, torch, args.serve_requests, layer=True, plain=False)

    biomemap = splatmap = large = uneven = None
    if rank == 0:
        if not args.no_large_field:
            log("large field")
            large = large_field_section(m, np, torch)
            log("uneven batch")
            uneven = uneven_batch_section(m, np, torch)
        log("biome layer chain")
        biomemap = biomemap_section(m, np, torch, B, cpu=world == 1 and not args.no_cpu_baseline)
        log("splatmap")
        splatmap = splatmap_section(m, np, torch, batch, reqs, cpu=world == 1 and not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        log("CPU baseline")
        dt, cores, kind, sample, stages, kinds = reference_eroded_chunk(os.cpu_count() or 1)
        cpu = {"value": 1.0 / dt, "unit": "chunks/s", "cores": cores, "kind": kind, "sample": sample,
               "stage_ms": {k: 1000.0 * v for k, v in stages.items()}, "stage_kind": kinds}

    if rank == 0:
        cs = clocks.summary()
        line = {
            "metric": METRIC, "value": value, "unit": "chunks/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "batch_per_gpu": B, "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (biome regions %.0f MB, merged maps %.0f MB per step)"
                             % (B * 25 * S * S * 2 / 1e6, B * 9 * S * S * 4 / 1e6)},
            "plain_per_chunk": {"value": plain_value, "unit": "chunks/s",
                                "note": "same resident data, per-chunk calls, stream synchronised per call"},
            "batched_vs_plain": value / world / plain_value,
            "p50_chunk_latency_ms": statistics.median(step_ms), "p99_chunk_latency_ms": float(
                np.percentile(step_ms, 99)),
            "e2e": {"value": e2e_value, "unit": "chunks/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "pipelining": "two batches alternate on two streams: one step's uploads and downloads overlap "
                                  "the other step's kernels; the kernels of the two run one after the other",
                    "serial_value": e2e_serial_value, "steps": e2e_steps},
            "stage_ms": dict(zip(stage_names, stage_ms)),
            "droplet_steps_per_batch": steps_total, "erode_steps_per_batch": erode_steps,
            "roofline": roof, "stage_roofline": stage_roof, "cpu_baseline": cpu, "clocks": cs,
            "measured_peaks": peaks,
            "serving": serving,
            "biomemap": biomemap,
            "splatmap": splatmap,
            "large_field": large,
            "uneven_batch": uneven,
            "autotune": {"filter_path": filter_path[0],
                         "filter_ms_by_path": {str(k): v for k, v in filter_path[1].items()},
                         "filter_path_names": "0 by launch size, 1 few-values packed slides, 2 few-values "
                                              "row bands, 3 general slides",
                         "filter_segments": stage_tune[0],
                         "filter_ms_by_segments": {str(k): v for k, v in stage_tune[1].items()},
                         "noise_block": stage_tune[2],
                         "noise_ms_by_block": {str(k): v for k, v in stage_tune[3].items()},
                         "erosion_coop_jobs_interleaved": stage_tune[4],
                         "erosion_lanes_per_droplet": lanes[0], "erosion_droplets_per_group": lanes[1],
                         "erosion_brush_rows": bool(lanes[2]),
                         "erosion_ms_by_lanes_x_droplets": {f"{a}x{b}" + ("-rows" if r else ""): v
                                                            for (a, b, r), v in tune_ms.items()}},
            "gpu_launches": kernels_per_step * args.steps,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def biomemap_section(m, np, torch, batch, cpu=True, reps=3):
    """The demo's biome layer chain (14 layers, STPLayerChainBuilder) on the GPU: the 5x5-chunk
    biome region of each of `batch` requests (2560^2 uint16 each, 210 MB per pass for 16, more
    than L2), one stpgb_layer_biomemap call per region; beside it the CPU restatement of the
    reference's layer chain on one 512^2 chunk (one thread, as the reference's factory runs)."""
    dev = m.DeviceOps()
    chain, ids = m.layer_chain_demo()
    S = MAP
    regions = [torch.empty((5 * S, 5 * S), dtype=torch.int16, device="cuda") for _ in range(batch)]
    origins = [((4 * n - 2) * S, -2 * S) for n in range(batch)]

    def one_pass():
        for reg, (ox, oz) in zip(regions, origins):
            dev.layer_biomemap(chain, ids, SEED, reg, 5 * S, 5 * S, 5 * S, (ox, oz))

    for _ in range(3):
        one_pass()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        one_pass()
    e1.record(st)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1000.0 / reps
    px = batch * 25 * S * S
    out = {"workload": f"demo layer chain, 14 layers, 5x5 chunks of {S}^2 per request, {batch} requests",
           "value": batch * 25 / sec, "unit": f"{S}^2 biomemap chunks/s", "gpx_per_s": px / sec / 1e9,
           "ms_per_pass": 1000.0 * sec, "launches_per_pass": batch, "l2": "output larger than L2 per pass"}
    if cpu:
        from oracle.oracle import Oracle
        oc = Oracle()
        chain_t = [(c.Kind, c.Param, c.Salt) for c in chain]
        idv = np.array([ids.Ocean, ids.Plains, ids.Forest, *ids.ShallowOcean], np.uint16)
        t0 = time.perf_counter()
        oc.layer_biomemap(chain_t, idv, SEED, S, S, (0, 0))
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": f"{S}^2 biomemap chunks/s", "cores": 1, "kind": "port",
                               "sample": f"one {S}^2 chunk through the CPU restatement of the layer chain"}
    return out


def uneven_requests(np, seed=31, count=64, table_biomes=16):
    """64 independent eroded chunks: sides log-uniform 128-1024 (multiples of 32), an even filter
    radius of 8-48, 2.3 droplets/px, brush radius 2-5, lifetime 30, 1-16 biomes each."""
    rng = np.random.default_rng(seed)
    reqs, biomes = [], []
    for n in range(count):
        side = int(np.exp(rng.uniform(np.log(128.0), np.log(1024.0))))
        side = min(1024, max(128, 32 * int(round(side / 32.0))))
        reqs.append(dict(MapSize=side, ChunkX=40 * n - 1000, ChunkY=7 * n - 200,
                         InterpolationRadius=2 * int(rng.integers(4, 25)),
                         DropletCount=int(round(2.3 * side * side)), BrushRadius=int(rng.integers(2, 6)),
                         Lifetime=30))
        biomes.append(int(rng.integers(1, table_biomes + 1)))
    return reqs, biomes


def uneven_batch_section(m, np, torch, reps=3):
    """The uneven batch: 64 chunks of the shapes above in one autotuned CUDA graph of batched
    launches, against the 64 plain per-chunk call sequences on the same resident data."""

    class Ptr:
        def __init__(self, p):
            self.p = p

        def data_ptr(self):
            return self.p

    reqs, biomes = uneven_requests(np)
    rng = np.random.default_rng(31)
    table = np.zeros(16, m.BIOME_DTYPE)
    table["Scale"] = np.exp(rng.uniform(np.log(64.0), np.log(512.0), 16)).astype(np.float32)
    table["Octave"] = rng.integers(4, 9, 16)
    table["Persistence"] = 0.5
    table["Lacunarity"] = 2.0
    table["Variation"] = rng.uniform(0.2, 1.0, 16).astype(np.float32)
    evap = 0.01
    base = m.RaindropSetting(Seed=31, RainDropCount=1000, Inertia=0.05, SedimentCapacityFactor=4.0,
                             minSedimentCapacity=0.01, initWaterVolume=1.0,
                             minWaterVolume=m.lifetime_min_water_volume(1.0, evap, 30), Friction=0.1, initSpeed=1.0,
                             ErodeSpeed=0.3, DepositSpeed=0.3, EvaporateSpeed=evap, Gravity=4.0, ErosionBrushRadius=3)
    b = m.Batch(reqs, base, m.SimplexSetting(31, 8, 0.2181661565), table, graph=True)
    b.synthesize(96, 31)
    dev = m.DeviceOps()
    for n, r in enumerate(reqs):
        S = r["MapSize"]
        dev.voronoi_biomemap(Ptr(b.buffers(n)[0]), 5 * S, 5 * S, 5 * S,
                             ((r["ChunkX"] - 2) * S, (r["ChunkY"] - 2) * S), 96, biomes[n], 31)
    torch.cuda.synchronize()
    b.tune()
    choice, tune_ms = b.tuning()
    stage_tune = b.tuning_stages()
    filter_path = b.tuning_filter_path()
    st = torch.cuda.current_stream()
    for _ in range(3):
        b.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        b.run()
    e1.record(st)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1) / reps
    stage_ms = []
    for stage in range(4):
        b.run_stage(stage)
        e0.record(st)
        b.run_stage(stage)
        e1.record(st)
        torch.cuda.synchronize()
        stage_ms.append(e0.elapsed_time(e1))
    b.run_plain()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run_plain()
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1000.0
    b.status()
    px = sum(r["MapSize"] ** 2 for r in reqs)
    return {"workload": "64 chunks, sides log-uniform 128-1024 (x32), 1-16 biomes, filter radius 8-48, "
                        "2.3 droplets/px, brush 2-5, lifetime 30; %.1f M centre-chunk pixels, %.1f M droplets"
                        % (px / 1e6, sum(r["DropletCount"] for r in reqs) / 1e6),
            "batched_ms": batched_ms, "plain_ms": plain_ms, "batched_vs_plain": plain_ms / batched_ms,
            "chunks_per_s": 64 * 1000.0 / batched_ms, "plain_chunks_per_s": 64 * 1000.0 / plain_ms,
            "stage_ms": dict(zip(["single_histogram_filter", "multibiome_noise", "hydraulic_erosion", "format"],
                                 stage_ms)),
            "autotune_dominant_group": {"lanes_per_droplet": choice[0], "droplets_per_group": choice[1],
                                        "brush_rows": bool(choice[2])},
            "autotune_stages": {"filter_path": filter_path[0],
                                "filter_ms_by_path": {str(k): v for k, v in filter_path[1].items()},
                                "filter_segments": stage_tune[0],
                                "filter_ms_by_segments": {str(k): v for k, v in stage_tune[1].items()},
                                "noise_block": stage_tune[2],
                                "noise_ms_by_block": {str(k): v for k, v in stage_tune[3].items()}}}


def stage_rooflines(m, np, torch, dev, host_biome, table, stage_ms, stage_names, peak, peak_kind, peaks):
    """The batch's filter and noise stages against their own bounds, from the stage times of the
    timed region.  Filter (HBM): per chunk 2 (W+2r)(H+2r) bytes of samples read, 4 (WH+1) bytes of
    offsets and 8 bytes per bin written.  Noise (FP32 pipe): per bin 60 flops per octave of its
    biome + 4, and 8 per pixel (an FMA counts two).  The bins are counted by the library's filter
    on the same 3x3 chunk neighbourhoods of each request's biome region, outside the timed region."""
    S, r = MAP, RADIUS
    octave = torch.from_numpy(table["Octave"].astype(np.int64)).cuda()
    ws = dev.shf_workspace((S, S), (3, 3), r, BIOMES)
    nbins = 0
    noise_flops = 0
    for region in host_biome:
        reg = torch.from_numpy(region.view(np.int16)).cuda()
        for c in range(9):
            cx, cy = c % 3, c // 3
            sub = reg[cy * S:cy * S + 3 * S, cx * S:cx * S + 3 * S].contiguous()
            off, bins, st = dev.shf_filter(sub, (S, S), (3, 3), r, max_items=BIOMES, workspace=ws)
            n = int(off[-1].item())
            items = (bins[:n] & 0xFFFF).long()
            nbins += n
            noise_flops += int((60 * octave[items] + 4).sum().item()) + 8 * S * S
    dev.status_check(st)
    chunks = len(host_biome) * 9
    shf_bytes = chunks * (2 * (S + 2 * r) ** 2 + 4 * (S * S + 1)) + 8 * nbins
    ms = dict(zip(stage_names, stage_ms))
    shf_gbs = shf_bytes / (ms["single_histogram_filter"] / 1000.0) / 1e9
    noise_tf = noise_flops / (ms["multibiome_noise"] / 1000.0) / 1e12
    fp32 = peaks["fp32_fma_tflops"]
    return {
        "single_histogram_filter": {"bound": "hbm", "achieved": shf_gbs, "peak": peak, "unit": "GB/s",
                                    "frac": shf_gbs / peak, "peak_source": peak_kind,
                                    "algorithmic_bytes_per_launch": shf_bytes, "bins_per_launch": nbins},
        "multibiome_noise": {"bound": "fp32", "achieved": noise_tf, "peak": fp32, "unit": "TFLOP/s",
                             "frac": noise_tf / fp32, "peak_source": "measured FP32 FMA rate (measured_peaks)",
                             "algorithmic_flops_per_launch": noise_flops}}


def large_field_section(m, np, torch, reps=3):
    """The large single field: a 4096^2 float32 heightfield from 8-octave fractal simplex noise,
    32 biomes from a seeded Voronoi uint16 map (the filter's window of its 3x3 neighbourhood),
    filter radius 64, then 16,000,000 droplets with brush 5 and lifetime 64 eroding the field as its
    own free-slip neighbourhood, formatted to uint16.  Kernel-level calls on one stream, each stage
    timed alone with CUDA events; the erosion restarts from the same heights every repetition."""
    S, r, nb, cell, seed, count, brush, life = 4096, 64, 32, 512, 7, 16_000_000, 5, 64
    dev = m.DeviceOps()
    st = torch.cuda.current_stream()
    rng = np.random.default_rng(seed)
    table = np.zeros(nb, m.BIOME_DTYPE)
    table["Scale"] = np.exp(rng.uniform(np.log(64.0), np.log(512.0), nb)).astype(np.float32)
    table["Octave"] = 8
    table["Persistence"] = 0.5
    table["Lacunarity"] = 2.0
    table["Variation"] = rng.uniform(0.2, 1.0, nb).astype(np.float32)
    perm, grad = m.permutation_generate(seed, 8, 0.2181661565)
    d_perm, d_grad = torch.from_numpy(perm).cuda(), torch.from_numpy(grad).cuda()
    d_table = torch.from_numpy(table.view(np.float32)).cuda()
    biomes = torch.zeros((3 * S, 3 * S), dtype=torch.int16, device="cuda")
    w = S + 2 * r
    dev.voronoi_biomemap(biomes[S - r:, S - r:], 3 * S, w, w, (-r, -r), cell, nb, seed)
    starts = torch.empty(2 * count, dtype=torch.float32, device="cuda")
    dev.droplet_starts(starts, count, seed, 0, (S, S), (1, 1))
    evap = 0.01
    rd = m.RaindropSetting(Seed=seed, RainDropCount=count, Inertia=0.05, SedimentCapacityFactor=4.0,
                           minSedimentCapacity=0.01, initWaterVolume=1.0,
                           minWaterVolume=m.lifetime_min_water_volume(1.0, evap, life), Friction=0.1, initSpeed=1.0,
                           ErodeSpeed=0.3, DepositSpeed=0.3, EvaporateSpeed=evap, Gravity=4.0,
                           ErosionBrushRadius=brush)
    idx, wgt = m.erosion_brush(S, brush)
    d_idx, d_wgt = torch.from_numpy(idx).cuda(), torch.from_numpy(wgt).cuda()
    h0 = torch.empty((S, S), dtype=torch.float32, device="cuda")
    h = torch.empty_like(h0)
    fixed = torch.empty((S, S), dtype=torch.int16, device="cuda")
    residual = torch.zeros(1, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    ms = {"single_histogram_filter": [], "multibiome_noise": [], "hydraulic_erosion": [], "format": []}
    nbins = 0
    for k in range(1 + reps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(8)]
        ev[0].record(st)
        off, bins, fstatus = dev.shf_filter(biomes, (S, S), (3, 3), r, max_items=nb, bins_capacity=8 * S * S)
        ev[1].record(st)
        ev[2].record(st)
        dev.multibiome_heightmap(h0, S, off, bins, (S, S), (0.0, 0.0), d_perm, d_grad, d_table)
        ev[3].record(st)
        h.copy_(h0)
        residual.zero_()
        ev[4].record(st)
        dev.hydraulic_erosion(h, (S, S), (1, 1), rd, starts, count, d_idx, d_wgt, residual, status)
        ev[5].record(st)
        ev[6].record(st)
        dev.format_heightmap(h, fixed, S, S)
        ev[7].record(st)
        torch.cuda.synchronize()
        dev.status_check(fstatus)
        dev.status_check(status)
        if k == 0:
            nbins = int(off[-1].item())
            continue
        for j, name in enumerate(ms):
            ms[name].append(ev[2 * j].elapsed_time(ev[2 * j + 1]))
        del off, bins, fstatus
    med = {k: statistics.median(v) for k, v in ms.items()}
    total = sum(med.values())
    shf_bytes = 2 * w * w + 4 * (S * S + 1) + 8 * nbins
    noise_flops = nbins * (60 * 8 + 4) + 8 * S * S
    peak, peak_kind = load_peaks()
    fp32 = measure_roofline_peaks(m, torch)["fp32_fma_tflops"]
    shf_gbs = shf_bytes / (med["single_histogram_filter"] / 1000.0) / 1e9
    noise_tflops = noise_flops / (med["multibiome_noise"] / 1000.0) / 1e12
    return {"workload": "4096^2 float32 field, 8-octave noise, 32 Voronoi biomes, filter radius 64, 16,000,000 "
                        "droplets, brush 5, lifetime 64, free-slip 1x1",
            "ms_per_field": total, "fields_per_s": 1000.0 / total, "stage_ms": med,
            "droplets_per_s": count / (med["hydraulic_erosion"] / 1000.0),
            "filter_bins": nbins, "filter_algorithmic_gb_per_s": shf_gbs, "filter_frac_of_hbm": shf_gbs / peak,
            "noise_algorithmic_tflop_per_s": noise_tflops, "fp32_fma_tflops_measured": fp32,
            "noise_frac_of_fp32": noise_tflops / fp32,
            "peak_source": peak_kind, "launches_per_field": 7}


def splat_rules(m):
    """The demo's splat rules (STPBiomeSplatRule.tdl, written for samples 0 and 1) repeated for the
    workload's 8 biomes: even biomes take sample 0's rules, odd ones sample 1's."""
    alt, gra = m.splat_rules_demo()
    a = [(b, r.UpperBound, r.RegionIndex) for b in range(BIOMES) for r in alt if r.Sample == b % 2]
    g = [(b, r.minGradient, r.maxGradient, r.LowerBound, r.UpperBound, r.RegionIndex)
         for b in range(BIOMES) for r in gra if r.Sample == b % 2]
    return a, g


def splatmap_section(m, np, torch, batch, reqs, cpu=True, reps=3):
    """Splatmaps of the eroded neighbourhoods the batch just produced: per request the 3x3 chunks
    of its fixed heightmap (uint16, 1536^2) with the centre 3x3 of its biome region, one
    stpgb_splatmap call of 9 chunks per request; beside it the CPU restatement on one chunk."""
    S = MAP
    alt_rules, gra_rules = splat_rules(m)
    gen = m.STPSplatmapGenerator(alt_rules, gra_rules, m.SimplexSetting(*SIMPLEX), (S, S))
    outs = [torch.empty((3 * S, 3 * S), dtype=torch.uint8, device="cuda") for _ in reqs]
    calls = []
    for n, r in enumerate(reqs):
        biome, _, fixed, _ = batch.buffers(n)
        centre = biome + (S * 5 * S + S) * 2  # chunk (1, 1) of the 5x5 region
        chunks = [(c % 3, c // 3, float((r["ChunkX"] + c % 3 - 1) * S), float((r["ChunkY"] + c // 3 - 1) * S))
                  for c in range(9)]
        calls.append((centre, fixed, outs[n], chunks))

    def one_pass():
        for centre, fixed, out, chunks in calls:
            gen(centre, fixed, (5 * S, 3 * S), out, 3 * S, 3 * S, 3 * S, chunks)

    for _ in range(3):
        one_pass()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        one_pass()
    e1.record(st)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1000.0 / reps
    nchunks = 9 * len(reqs)
    regions = np.bincount(outs[0].cpu().numpy().ravel(), minlength=256)
    out = {"workload": f"demo splat rules over 8 biomes, 3x3 chunks of {S}^2 per request, {len(reqs)} requests",
           "value": nchunks / sec, "unit": f"{S}^2 splatmap chunks/s", "gpx_per_s": nchunks * S * S / sec / 1e9,
           "ms_per_pass": 1000.0 * sec, "launches_per_pass": len(reqs),
           "regions_of_request0": {int(k): int(v) for k, v in enumerate(regions) if v}}
    if cpu:
        from oracle.oracle import Oracle
        oc = Oracle()
        region = [np.empty((5 * S, 5 * S), np.uint16) for _ in reqs]
        fixed_h = [np.empty((3 * S, 3 * S), np.uint16) for _ in reqs]
        batch.download_inputs(biome_regions=region)
        batch.download(fixed=fixed_h)
        torch.cuda.synchronize()
        perm, grad = m.permutation_generate(*SIMPLEX)
        t0 = time.perf_counter()
        oc.splatmap(np.ascontiguousarray(region[0][S:4 * S, S:4 * S]), fixed_h[0], calls[0][3][4:5], (S, S),
                    alt_rules, gra_rules, perm, grad)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": f"{S}^2 splatmap chunks/s", "cores": 1, "kind": "port",
                               "sample": f"the centre {S}^2 chunk of request 0 through the CPU restatement"}
    return out


def serve_section(m, np, torch, n, rate=200.0, layer=False, plain=True):
    """Camera walk (1 chunk/s, new heading every 5 s), Poisson arrivals at `rate`/s (200 in the
    workload), LOD sides 256/512/1024 with p 0.5/0.35/0.15, 3x3 neighbourhoods, 8 biomes (or the
    demo's biome layer chain with `layer`), radius 32, 2.3 droplets/px, brush 4, lifetime 50,
    through the continuous-batching server on a 40 GB pool; with `plain`, beside it the plain
    per-request call sequence (9 generate + 1 erode through the drop-in generator API, host
    buffers) on a sample of the same requests."""
    from superterrainplus_gb300.serve import Server, camera_walk
    reqs, times = camera_walk(n, SEED, rate=rate)
    base = raindrop(m, 1)
    simplex = m.SimplexSetting(*SIMPLEX)
    table = biome_table(np, m.BIOME_DTYPE)
    sv = Server(base, simplex, table, hbm_budget=40 << 30, max_in_flight=64, max_batch=16, streams=3,
                voronoi_cell=VORONOI_CELL, biome_seed=SEED, layer_chain_biomes=layer)
    warm, wt = camera_walk(16, SEED + 1, rate=1e6)
    for w in warm:  # warm-up far from the measured walk, so it leaves no resident chunk behind for it
        w["ChunkX"] += 100000
    sv.replay(warm, wt)
    lat, wall = sv.replay(reqs, times)
    stats = sv.stats()
    sv.close()
    px512 = sum((r["MapSize"] / 512.0) ** 2 for r in reqs)
    out = {"requests": n, "arrival_rate_per_s": rate, "wall_s": wall, "chunks_per_s": n / wall,
           "chunks_512_equivalent_per_s": px512 / wall, "p50_latency_ms": float(np.percentile(lat, 50)),
           "p99_latency_ms": float(np.percentile(lat, 99)), "chunks_generated": stats["ChunksGenerated"],
           "launch_sequences": stats["Launches"], "hbm_pool_gb": 40,
           "biomes": "demo layer chain" if layer else "synthetic Voronoi, 8 biomes"}
    if not plain:
        return out
    # plain per-request calls on a sample of the same requests
    dev = m.DeviceOps()
    gens, sample = {}, reqs[: min(12, n)]
    plain_lat = []
    for r in sample:
        S = r["MapSize"]
        if S not in gens:
            cs = m.ChunkSetting()
            cs.MapSize[:] = [S, S]
            cs.DiversityNearestNeighbour[:] = [3, 3]
            cs.ErosionNearestNeighbour[:] = [3, 3]
            rd = raindrop(m, int(round(2.3 * S * S)))
            gens[S] = m.STPHeightfieldGenerator(cs, rd, simplex, table, RADIUS)
        region = torch.empty((5 * S, 5 * S), dtype=torch.int16, device="cuda")
        cell = max(1, VORONOI_CELL * S // 512)
        dev.voronoi_biomemap(region, 5 * S, 5 * S, 5 * S, ((r["ChunkX"] - 2) * S, (r["ChunkY"] - 2) * S), cell,
                             BIOMES, SEED)
        reg = region.cpu().numpy().view(np.uint16)
        chunk = lambda bx, by: np.ascontiguousarray(reg[by * S:(by + 1) * S, bx * S:(bx + 1) * S])
        heights = [np.zeros((S, S), np.float32) for _ in range(9)]
        fixed = [np.zeros((S, S), np.uint16) for _ in range(9)]
        t0 = time.perf_counter()
        for c in range(9):
            cx, cy = c % 3 + 1, c // 3 + 1  # in the 5x5 region
            biomes = [chunk(cx + (k % 3) - 1, cy + (k // 3) - 1) for k in range(9)]
            gens[S].generate(heights[c], biomes, (float((r["ChunkX"] + c % 3 - 1) * S),
                                                  float((r["ChunkY"] + c // 3 - 1) * S)))
        gens[S].erode(heights, fixed)
        plain_lat.append((time.perf_counter() - t0) * 1000.0)
    out["plain_per_request"] = {"sample": len(sample), "chunks_per_s": len(sample) / (sum(plain_lat) / 1000.0),
                                "p50_latency_ms": float(np.percentile(plain_lat, 50)),
                                "note": "drop-in generator API, host buffers, one request at a time, no queueing"}
    return out


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
