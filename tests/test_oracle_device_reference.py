"""Pins the oracle's noise, multi-biome blend, droplet, brush, format and
splatmap restatements against the reference's own device code compiled as
host C++ (oracle/build_ref.sh: STPSimplexNoise.cu, STPRainDrop.cu, the demo's
STPMultiHeightGenerator.cu and STPSplatmapGenerator.cu scripts,
STPTextureSplatRuleWrapper.cu, the brush generator of
STPHeightfieldGenerator.cpp and the format kernel of STPHeightfieldKernel.cu),
run one thread at a time with no fused multiply-adds.  For the splatmap the
texture fetches and rnormf are host stand-ins, so that pin covers the
script's sampling positions, noise, altitude and rule lookups.  The oracle must agree
bit for bit: with the committed fixtures that build produced
(tests/golden/device_reference.npz) everywhere, and with the live build on
random inputs where the reference tree is present.  CPU only."""
import os

import numpy as np
import pytest

import helpers

INT_FIELDS = ("Seed", "RainDropCount", "ErosionBrushRadius")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def fix():
    return np.load(os.path.join(helpers.GOLDEN, "device_reference.npz"))


@pytest.fixture(scope="module")
def device_reference():
    from oracle.oracle import DeviceReference
    try:
        return DeviceReference()
    except Exception as e:  # no reference tree, or it could not be compiled here
        pytest.skip(f"reference device build unavailable: {e}")


def oracle_simplex(oracle, perm, grad, pts):
    f = oracle.lib.orc_simplex2d
    return np.array([f(perm.ctypes.data, grad.ctypes.data, len(grad) // 2, x, y) for x, y in pts], np.float32)


def oracle_fractal(oracle, perm, grad, pts, pers, lacu, oct, scale, off, half):
    f = oracle.lib.orc_fractal
    return np.array([f(perm.ctypes.data, grad.ctypes.data, len(grad) // 2, x, y, pers, lacu, int(oct), scale, off[0],
                       off[1], half[0], half[1]) for x, y in pts], np.float32)


def setting_from(row):
    from oracle.oracle import RAINDROP_FIELDS
    return {k: (int(v) if k in INT_FIELDS else float(v)) for (k, _), v in zip(RAINDROP_FIELDS, row)}


# ---------------------------------------------------------------- fixtures


def test_simplex_and_fractal_match_reference_fixtures(oracle, fix):
    """simplex2D at 2,305 points per table (|x| up to 1e4, near-integer lattice points, the origin)
    and simplex2DFractal for 5 parameter sets (1-10 octaves, offsets up to 1e5) at 256 points, for
    3 permutation tables."""
    for t in range(3):
        perm, grad = fix[f"t{t}_perm"], fix[f"t{t}_grad"]
        assert np.array_equal(bits(oracle_simplex(oracle, perm, grad, fix[f"t{t}_simplex_xy"])),
                              bits(fix[f"t{t}_simplex"]))
        for k, (p, lacu, o, sc, ox, oy, hx, hy) in enumerate(fix["fractal_sets"]):
            got = oracle_fractal(oracle, perm, grad, fix[f"t{t}_fractal_xy"], p, lacu, o, sc, (ox, oy), (hx, hy))
            assert np.array_equal(bits(got), bits(fix[f"t{t}_fractal"][k])), (t, k)


def test_multibiome_matches_reference_script_fixtures(oracle, fix):
    """The demo's generateMultiBiomeHeightmap (two biomes) over filtered two-ID sample maps."""
    perm, grad = fix["t0_perm"], fix["t0_grad"]
    for i in range(int(fix["multibiome_count"])):
        mx, my, nx, ny, r = (int(v) for v in fix[f"m{i}_meta"])
        rc, offsets, bins = oracle.shf(fix[f"m{i}_samplemap"], (mx, my), (nx, ny), r)
        assert rc == 0
        got = oracle.multibiome(offsets, bins, fix["two_biomes"], perm, grad, (mx, my), tuple(fix[f"m{i}_offset"]))
        assert np.array_equal(bits(got), bits(fix[f"m{i}_height"])), i


def test_droplets_match_reference_fixtures(oracle, fix):
    """STPRainDrop run droplet after droplet (3 maps, brush radii 2-5, 1,500-4,000 droplets,
    lifetimes 20-64, inertia 0-0.3): the oracle's FP32 serial erosion gives the same map bit for
    bit."""
    for i in range(int(fix["erosion_count"])):
        n, radius, count, lifetime, seed = (int(v) for v in fix[f"e{i}_meta"])
        s = setting_from(fix[f"e{i}_setting"])
        starts = oracle.droplet_starts(count, seed, 0, (n // 3, n // 3), (3, 3))
        idx, w = oracle.brush(n, radius)
        h = fix[f"e{i}_input"].astype(np.float32)
        got, _, steps = oracle.erode(h, s, starts, idx, w, fp64=False)
        assert steps > count
        assert np.array_equal(bits(got), bits(fix[f"e{i}_output"])), i


def test_brush_and_format_match_reference_fixtures(oracle, fix):
    at = 0
    for dim_x, radius, size in fix["brush_meta"]:
        idx, w = oracle.brush(int(dim_x), int(radius))
        assert len(idx) == size
        assert np.array_equal(idx, fix["brush_index"][at:at + size])
        assert np.array_equal(bits(w), bits(fix["brush_weight"][at:at + size]))
        at += size
    assert np.array_equal(oracle.format(fix["format_input"]), fix["format_output"])


def test_splatmap_matches_reference_script_fixtures(oracle, fix):
    """The demo's splatmap script: the demo's rules over the 9 chunks of a 3x3 buffer, and random
    rules (a sample without rules, empty gradient lists) over 4 of them."""
    rc, perm, grad = oracle.permutation(42, 8, 0.2181661565)
    for i in range(int(fix["splat_count"])):
        alt = [(int(a), float(b), int(c)) for a, b, c in fix[f"s{i}_altitude_rules"]]
        gra = [(int(r[0]), *(float(v) for v in r[1:5]), int(r[5])) for r in fix[f"s{i}_gradient_rules"]]
        chunks = [(int(a), int(b), float(c), float(d)) for a, b, c, d in fix[f"s{i}_chunks"]]
        got, _, _ = oracle.splatmap(fix[f"s{i}_biomemap"], fix[f"s{i}_heightmap"], chunks, (32, 32), alt, gra,
                                    perm, grad)
        assert np.array_equal(got, fix[f"s{i}_regions"]), i


# ------------------------------------------------------------ live builds

SAFE_DISTRIBUTIONS = [(8, 0.2181661565), (10, 0.11344640137963143), (16, 0.0), (32, 6.0), (7, 3.1)]


@pytest.mark.parametrize("seed", range(4))
def test_noise_matches_live_reference(oracle, device_reference, seed):
    rng = np.random.default_rng(100 + seed)
    n, off = SAFE_DISTRIBUTIONS[seed % len(SAFE_DISTRIBUTIONS)]
    rc, perm, grad = oracle.permutation(int(rng.integers(0, 2**63)), n, off)
    assert rc == 0
    scale = 10.0 ** rng.uniform(-1, 5, 3000)
    pts = (rng.uniform(-1, 1, (3000, 2)) * scale[:, None]).astype(np.float32)
    want = np.array([device_reference.simplex2d(perm, grad, x, y) for x, y in pts], np.float32)
    assert np.array_equal(bits(oracle_simplex(oracle, perm, grad, pts)), bits(want))
    for _ in range(6):
        args = (float(rng.uniform(0.1, 0.9)), float(rng.uniform(1.5, 3.5)), int(rng.integers(1, 13)),
                float(10 ** rng.uniform(0, 3.7)), tuple(float(v) for v in rng.uniform(-1e5, 1e5, 2)),
                tuple(float(v) for v in rng.integers(0, 1024, 2) / 2))
        fpts = rng.uniform(-4096, 4096, (200, 2)).astype(np.float32)
        want = np.array([device_reference.fractal(perm, grad, x, y, *args) for x, y in fpts], np.float32)
        assert np.array_equal(bits(oracle_fractal(oracle, perm, grad, fpts, *args)), bits(want)), args


@pytest.mark.parametrize("seed", range(3))
def test_multibiome_matches_live_reference(oracle, device_reference, seed):
    from oracle.oracle import BIOME_DTYPE
    rng = np.random.default_rng(200 + seed)
    ms = tuple(int(v) for v in rng.integers(2, 9, 2) * 8)
    r = int(rng.integers(1, min(ms) // 2 + 1)) * 2
    sm = (rng.random((ms[1] * 3, ms[0] * 3)) < rng.uniform(0.2, 0.8)).astype(np.uint16)
    rc, offsets, bins = oracle.shf(sm, ms, (3, 3), r)
    assert rc == 0
    table = np.zeros(2, BIOME_DTYPE)
    for b in range(2):
        table[b] = (10 ** rng.uniform(1, 3), rng.integers(1, 11), rng.uniform(0.2, 0.8), rng.uniform(1.5, 3.0),
                    rng.uniform(-0.2, 0.4), rng.uniform(0.05, 1.0))
    rc, perm, grad = oracle.permutation(seed, 8, 0.2181661565)
    off = tuple(float(v) for v in rng.uniform(-5e4, 5e4, 2))
    want = device_reference.multibiome(offsets, bins, table, perm, grad, ms, off)
    assert np.array_equal(bits(oracle.multibiome(offsets, bins, table, perm, grad, ms, off)), bits(want))


@pytest.mark.parametrize("seed", range(6))
def test_droplets_match_live_reference(oracle, device_reference, seed):
    """Random settings (inertia 0-0.9, capacity, deposit, erode, evaporation, gravity, friction),
    brush radii 1-7, maps 48-120 px, 500-5,000 droplets started in the central chunk: the oracle's
    FP32 serial erosion equals the reference droplet's map bit for bit."""
    rng = np.random.default_rng(300 + seed)
    n = int(rng.integers(16, 41)) * 3
    radius = int(rng.integers(1, min(8, n // 6)))
    count = int(rng.integers(500, 5001))
    s = helpers.raindrop_dict(count, radius=radius, lifetime=int(rng.integers(5, 80)))
    s.update(Inertia=float(rng.uniform(0, 0.9)), SedimentCapacityFactor=float(rng.uniform(1, 8)),
             minSedimentCapacity=float(rng.uniform(0.001, 0.05)), DepositSpeed=float(rng.uniform(0.05, 0.6)),
             ErodeSpeed=float(rng.uniform(0.05, 0.6)), Gravity=float(rng.uniform(1, 10)),
             Friction=float(rng.uniform(0, 0.3)), initSpeed=float(rng.uniform(0.5, 2)))
    y, x = np.mgrid[0:n, 0:n]
    h = (0.5 + 0.3 * np.sin(x / rng.uniform(4, 15)) * np.cos(y / rng.uniform(4, 15))
         + 0.05 * rng.random((n, n))).astype(np.float32)
    if seed == 5:
        h[:, : n // 2] = 0.5  # a flat half: droplets there stop at once (zero direction)
    starts = oracle.droplet_starts(count, seed, 0, (n // 3, n // 3), (3, 3))
    idx, w = device_reference.brush(n, radius)
    want = device_reference.erode(h, s, starts, idx, w)
    got, _, steps = oracle.erode(h, s, starts, idx, w, fp64=False)
    assert steps >= count and not np.array_equal(want, h)
    assert np.array_equal(bits(got), bits(want))


@pytest.mark.parametrize("seed", range(3))
def test_erosion_kernel_spawn_matches_live_reference(oracle, device_reference, seed):
    """The reference's hydraulicErosionKERNEL, spawn included: fed the oracle's Philox uniforms in
    place of curand's (the oracle's starts for a 1x1 neighbourhood of 2^2 chunks are the uniforms
    themselves: u * 1 + 0), it gives the map of the oracle's FP32 serial erosion from the oracle's
    starts for the real neighbourhood, bit for bit: same spawn range, same arithmetic."""
    rng = np.random.default_rng(500 + seed)
    ms = (int(rng.integers(12, 40)), int(rng.integers(12, 40)))
    nn = (3, 3) if seed < 2 else (5, 3)
    count = int(rng.integers(500, 4000))
    s = helpers.raindrop_dict(count, radius=int(rng.integers(1, 5)), lifetime=int(rng.integers(10, 60)))
    total = (ms[0] * nn[0], ms[1] * nn[1])
    y, x = np.mgrid[0:total[1], 0:total[0]]
    h = (0.5 + 0.3 * np.sin(x / rng.uniform(4, 12)) * np.cos(y / rng.uniform(4, 12))
         + 0.05 * rng.random(x.shape)).astype(np.float32)
    uniforms = oracle.droplet_starts(count, seed, 0, (2, 2), (1, 1))
    assert uniforms.min() > 0.0 and uniforms.max() <= 1.0
    starts = oracle.droplet_starts(count, seed, 0, ms, nn)
    idx, w = oracle.brush(total[0], s["ErosionBrushRadius"])
    want = device_reference.erosion_kernel(h, ms, nn, s, uniforms, idx, w)
    got, _, _ = oracle.erode(h, s, starts, idx, w, fp64=False)
    assert not np.array_equal(want, h)
    assert np.array_equal(bits(got), bits(want))


def test_brush_and_format_match_live_reference(oracle, device_reference):
    for dim_x in (7, 64, 513, 4096):
        for radius in range(1, 16):
            a, b = oracle.brush(dim_x, radius), device_reference.brush(dim_x, radius)
            assert np.array_equal(a[0], b[0]) and np.array_equal(bits(a[1]), bits(b[1]))
    rng = np.random.default_rng(5)
    v = np.concatenate([rng.uniform(-1, 2, 100000), rng.standard_normal(1000) * 1e-6,
                        np.arange(65536) / 65535.0 + 0.5 / 65535]).astype(np.float32)
    assert np.array_equal(oracle.format(v), device_reference.format(v))


@pytest.mark.parametrize("seed", range(3))
def test_splatmap_matches_live_reference(oracle, device_reference, seed):
    rng = np.random.default_rng(400 + seed)
    S = int(rng.integers(2, 7)) * 8
    y, x = np.mgrid[0:3 * S, 0:3 * S]
    hm = ((0.5 + 0.45 * np.sin(x / rng.uniform(3, 12)) * np.cos(y / rng.uniform(3, 12))
           + 0.05 * rng.random(x.shape)) * 65535).clip(0, 65535).astype(np.uint16)
    bm = rng.integers(0, 6, x.shape).astype(np.uint16)
    alt, gra = [], []
    for smp in range(5):
        for ub in sorted(rng.uniform(0.1, 1.0, int(rng.integers(1, 4)))):
            alt.append((smp, float(ub), int(rng.integers(0, 8))))
        for _ in range(int(rng.integers(0, 3))):
            g0, g1 = sorted(rng.uniform(0, 1, 2))
            a0, a1 = sorted(rng.uniform(0, 1, 2))
            gra.append((smp, float(g0), float(g1), float(a0), float(a1), int(rng.integers(0, 8))))
    chunks = [(c % 3, c // 3, float(rng.uniform(-1e5, 1e5)), float(rng.uniform(-1e5, 1e5))) for c in range(9)
              if rng.random() < 0.7]
    rc, perm, grad = oracle.permutation(seed, 8, 0.2181661565)
    want = device_reference.splatmap(bm, hm, chunks, (S, S), alt, gra, perm, grad)
    got, _, _ = oracle.splatmap(bm, hm, chunks, (S, S), alt, gra, perm, grad)
    assert np.array_equal(got, want)


def test_production_size_outputs_match_reference_digests(oracle):
    """A 512^2 chunk of the two-biome script (filter radius 32) and 600,000 droplets (brush 5,
    lifetime 50) on a 1536^2 merged map: the oracle reproduces the SHA-256 of the reference
    build's float32 outputs (tests/golden/device_digests.json)."""
    import hashlib
    import json
    import sys
    sys.path.insert(0, helpers.GOLDEN)
    import make_golden as g
    with open(os.path.join(helpers.GOLDEN, "device_digests.json")) as f:
        want = json.load(f)

    def digest(a):
        return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()

    m = want["multibiome_512"]
    rc, perm, grad = oracle.permutation(*g.DEVICE_PERMS[0])
    sm = g.two_id_samplemap((1536, 1536), tuple(m["samplemap_cell"]), m["samplemap_seed"])
    rc, offsets, bins = oracle.shf(sm, (512, 512), (3, 3), m["radius"])
    assert rc == 0
    table = np.array(g.TWO_BIOMES, g.BIOME_DTYPE)
    assert digest(oracle.multibiome(offsets, bins, table, perm, grad, (512, 512), tuple(m["offset"]),
                                    threads=4)) == m["sha256"]
    e = want["erosion_1536"]
    h = g.erosion_input(1536, e["input_seed"]).astype(np.float32)
    s = g.raindrop_setting(e["droplets"], e["brush"], e["lifetime"], e["inertia"])
    starts = oracle.droplet_starts(e["droplets"], e["start_seed"], 0, (512, 512), (3, 3))
    idx, w = oracle.brush(1536, e["brush"])
    out, _, _ = oracle.erode(h, s, starts, idx, w, fp64=False)
    assert digest(out) == e["sha256"]
