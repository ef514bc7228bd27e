"""Shared helpers of the test suite: fixture loading and seeded inputs."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_shf_kat():
    return dict(np.load(os.path.join(GOLDEN, "shf_kat.npz")))


def shf_small_cases(oracle):
    """Yields (name, samplemap, map_size, nn, radius, offsets, items, weights) from the reference fixtures."""
    z = np.load(os.path.join(GOLDEN, "shf_cases.npz"))
    for i in range(int(z["count"])):
        mx, my, nx, ny, r, seed = (int(v) for v in z[f"c{i}_meta"])
        kind = str(z[f"c{i}_kind"])
        param = tuple(int(v) for v in z[f"c{i}_param"])
        sm = sample_map(kind, mx, my, nx, ny, param, seed, oracle, stored=z.get(f"c{i}_input"))
        yield (f"{kind}-{mx}x{my}-r{r}", sm, (mx, my), (nx, ny), r, z[f"c{i}_offsets"], z[f"c{i}_items"],
               z[f"c{i}_weights"])


def shf_large_cases(oracle):
    z = np.load(os.path.join(GOLDEN, "shf_cases.npz"))
    with open(os.path.join(GOLDEN, "shf_digests.json")) as f:
        cases = json.load(f)
    for j, c in enumerate(cases):
        mx, my = c["map"]
        nx, ny = c["nn"]
        sm = sample_map(c["kind"], mx, my, nx, ny, tuple(c["param"]), c["seed"], oracle,
                        stored=z.get(f"large{j}_input"))
        yield c, sm


def sample_map(kind, mx, my, nx, ny, param, seed, oracle, stored=None):
    w, h = mx * nx, my * ny
    if stored is not None:
        return np.asarray(stored, np.uint16).reshape(h, w)
    if kind == "constant":
        return np.full((h, w), seed % 7, np.uint16)
    if kind == "voronoi":
        cell, biomes = param
        return oracle.voronoi(w, h, (-mx * (nx // 2), -my * (ny // 2)), cell, biomes, seed)
    raise ValueError(kind)


def digest(offsets, items, weights):
    import hashlib
    m = hashlib.sha256()
    m.update(np.ascontiguousarray(offsets, np.uint32).tobytes())
    m.update(np.ascontiguousarray(items, np.uint16).tobytes())
    m.update(np.ascontiguousarray(weights, np.float32).tobytes())
    return m.hexdigest()


def load_permutations():
    z = np.load(os.path.join(GOLDEN, "permutation.npz"))
    for i in range(int(z["count"])):
        seed, n = (int(v) for v in z[f"p{i}_setting"])
        yield seed, n, float(z[f"p{i}_offset"]), z[f"p{i}_perm"], z[f"p{i}_grad"]


def biome_table(n, seed):
    """Seeded multi-biome parameters (octaves 4-8, Scale log-uniform 64-512,
    Variation 0.2-1.0, Depth 0, persistence 0.5, lacunarity 2)."""
    from superterrainplus_gb300 import BIOME_DTYPE
    rng = np.random.default_rng(seed)
    t = np.zeros(n, BIOME_DTYPE)
    t["Scale"] = np.exp(rng.uniform(np.log(64.0), np.log(512.0), n)).astype(np.float32)
    t["Octave"] = rng.integers(4, 9, n)
    t["Persistence"] = 0.5
    t["Lacunarity"] = 2.0
    t["Depth"] = 0.0
    t["Variation"] = rng.uniform(0.2, 1.0, n).astype(np.float32)
    return t


def multibiome_terrain(oracle, stpgb, S, nbiomes, cell, seed):
    """A 3x3 neighbourhood of S^2 chunks from the oracle pipeline (Voronoi biome map, filter
    radius 16, multi-biome fractal noise)."""
    table = biome_table(nbiomes, seed)
    perm, grad = stpgb.permutation_generate(seed, 8, 0.2181661565)
    out = np.zeros((3 * S, 3 * S), np.float32)
    for c in range(9):
        kx, ky = c % 3 - 1, c // 3 - 1
        region = oracle.voronoi(3 * S, 3 * S, ((kx - 1) * S, (ky - 1) * S), cell, nbiomes, seed)
        rc, off, bins = oracle.shf(region, (S, S), (3, 3), 16)
        h = oracle.multibiome(off, bins, table, perm, grad, (S, S), (float(kx * S), float(ky * S)))
        out[(c // 3) * S:(c // 3 + 1) * S, (c % 3) * S:(c % 3 + 1) * S] = h
    return out


def raindrop_dict(count, radius=3, lifetime=30, seed=42):
    """Droplet settings of the small plain-method workload (inertia 0.05,
    capacity 4, min capacity 0.01, deposit 0.3, erode 0.3, evaporate 0.01,
    gravity 4); initWaterVolume 1, initSpeed 1, Friction 0.1 as the demo's
    Engine.ini; the lifetime is set through minWaterVolume."""
    evap = 0.01
    v = np.float32(1.0)
    for _ in range(lifetime):
        v = np.float32(v * np.float32(1.0 - np.float32(evap)))
    minv = float(np.nextafter(v, np.float32(np.inf)))
    return dict(Seed=seed, RainDropCount=count, Inertia=0.05, SedimentCapacityFactor=4.0, minSedimentCapacity=0.01,
                initWaterVolume=1.0, minWaterVolume=minv, Friction=0.1, initSpeed=1.0, ErodeSpeed=0.3,
                DepositSpeed=0.3, EvaporateSpeed=evap, Gravity=4.0, ErosionBrushRadius=radius)


# ------------------------------------------------------------------ erosion tolerance

BAND_FILE = os.path.join(GOLDEN, "erosion_band.json")


def spawn_draws(starts, map_size, nn, guess=None):
    from oracle.oracle import spawn_draws as f
    return f(starts, map_size, nn, guess)


def droplet_uniforms(oracle, count, seed, counter_base, map_size, nn):
    from oracle.oracle import droplet_draws
    return droplet_draws(oracle, count, seed, counter_base, map_size, nn)


def _reference_gpu():
    try:
        from oracle.oracle import ReferenceGPU
        return ReferenceGPU()
    except (FileNotFoundError, OSError):
        return None


def reference_band(case, oracle, h, map_size, nn, setting, seed, counter_base, ref64, runs=5):
    """The erosion tolerance of one case: the reference's own erosion kernel (hydraulicErosionKERNEL with
    STPRainDrop, built for sm_103a by oracle/build_ref.sh) run `runs` times on `h` with the droplets of
    (seed, counter_base); returns (RMS of each run against the FP64 serial result `ref64`, run-to-run
    spread = the largest RMS between two runs, source).  Where the reference build is absent, the
    figures recorded for `case` in tests/golden/erosion_band.json by the same runs on a GB300
    (tests/golden/make_erosion_band.py).  With STPGB_RECORD_BAND set to a file name, live figures are
    added to that file."""
    import json

    import pytest
    ref = _reference_gpu()
    if ref is None:
        rec = None
        if os.path.exists(BAND_FILE):
            with open(BAND_FILE) as f:
                rec = json.load(f).get(case)
        if rec is None:
            pytest.skip(f"reference GPU build absent and no recorded band for {case}")
        return rec["rms"], rec["spread"], "recorded"
    import torch
    count = setting["RainDropCount"]
    idx, w = oracle.brush(h.shape[1], setting["ErosionBrushRadius"])
    # The reference kernel copies the brush into shared memory with the block's live droplet threads
    # only (STPRainDrop.cu:63-71): a last block with fewer live droplets than brush points would erode
    # with unwritten brush entries, so no tolerance case may have one.
    block = ref.block_size(len(idx))
    assert count % block == 0 or count % block >= len(idx), \
        f"{case}: the reference kernel's last block would hold {count % block} droplets for {len(idx)} brush points"
    draws, exact = droplet_uniforms(oracle, count, seed, counter_base, map_size, nn)
    u = torch.from_numpy(draws).cuda()
    d_idx, d_w = torch.from_numpy(idx).cuda(), torch.from_numpy(w).cuda()
    outs = []
    for _ in range(runs):
        d = torch.from_numpy(np.ascontiguousarray(h, np.float32).copy()).cuda()
        torch.cuda.synchronize()
        ref.erode(d.data_ptr(), map_size, nn, setting, u.data_ptr(), count, d_idx.data_ptr(), d_w.data_ptr(),
                  len(idx))
        outs.append(d.cpu().numpy().astype(np.float64))
    # a run that left the finite range has an unbounded distance
    dist = lambda a, b: float(np.sqrt(np.mean((a - b) ** 2))) if np.isfinite(a).all() and np.isfinite(b).all() \
        else float("inf")
    rms = [dist(o, ref64) for o in outs]
    spread = max(dist(a, b) for i, a in enumerate(outs) for b in outs[i + 1:])
    record = os.environ.get("STPGB_RECORD_BAND")
    if record:
        data = {}
        if os.path.exists(record):
            with open(record) as f:
                data = json.load(f)
        data[case] = {"rms": rms, "spread": spread, "runs": runs, "block": ref.block_size(len(idx)),
                      "droplets_spawned_exactly": exact,
                      "finite": bool(all(np.isfinite(o).all() for o in outs))}
        with open(record, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
    return rms, spread, "live"
