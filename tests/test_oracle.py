"""Pins the CPU oracle against the reference's own golden vectors and the
fixtures produced by the reference's compiled sources (CPU only)."""
import math

import numpy as np
import pytest

import helpers

FLT_EPS = np.finfo(np.float32).eps


def test_shf_reference_kat(oracle):
    """SuperTest+/SuperAlgorithm+/STPTestHistogram.cpp:77-105: ordered (item, weight) for pixels 0, 8, 15."""
    kat = helpers.load_shf_kat()
    rc, off, bins = oracle.shf(kat["texture"], (4, 4), (3, 3), 2)
    assert rc == 0
    expected = {0: [(0, .24), (3, .24), (2, .28), (1, .24)], 8: [(0, .36), (3, .24), (1, .16), (2, .24)],
                15: [(0, .32), (3, .2), (1, .12), (2, .36)]}
    for px, exp in expected.items():
        got = bins[off[px]:off[px + 1]]
        assert len(got) == len(exp)
        for b, (item, w) in zip(got, exp):
            assert b["Item"] == item
            assert math.isclose(b["Weight"], w, rel_tol=5 * FLT_EPS)
    # size() invariants (:156-162)
    assert len(off) == 17 and off[-1] == len(bins)
    assert np.array_equal(off, kat["offsets"])
    assert np.array_equal(bins["Item"], kat["items"])
    assert np.array_equal(bins["Weight"].view(np.uint32), kat["weights"].view(np.uint32))


@pytest.mark.parametrize("radius", [0, 3, 128])
def test_shf_reference_errors(oracle, radius):
    """STPTestHistogram.cpp:121-130: radius 0, odd radius and a radius past the neighbourhood are rejected."""
    kat = helpers.load_shf_kat()
    assert oracle.shf(kat["texture"], (4, 4), (3, 3), radius)[0] == 1


def test_shf_reference_fixtures(oracle):
    for name, sm, ms, nn, r, off, items, weights in helpers.shf_small_cases(oracle):
        rc, o, b = oracle.shf(sm, ms, nn, r)
        assert rc == 0, name
        assert np.array_equal(o, off), name
        assert np.array_equal(b["Item"], items), name
        assert np.array_equal(b["Weight"].view(np.uint32), weights.view(np.uint32)), name


def test_shf_reference_digests(oracle):
    for case, sm in helpers.shf_large_cases(oracle):
        rc, o, b = oracle.shf(sm, tuple(case["map"]), tuple(case["nn"]), case["radius"])
        assert rc == 0
        assert len(b) == case["nbins"]
        assert helpers.digest(o, b["Item"], b["Weight"]) == case["sha256"], case


def test_permutation_reference_kat(oracle):
    """STPTestPermutation.cpp:37-41,108-115: seed 6666, 10 gradients, offset 6.5 degrees."""
    rc, perm, grad = oracle.permutation(6666, 10, math.radians(6.5))
    assert rc == 0
    for i, deg in ((0, 6.5), (6, 114.5), (14, 258.5)):
        assert math.isclose(grad[i], math.cos(math.radians(deg)), rel_tol=10 * FLT_EPS)
        assert math.isclose(grad[i + 1], math.sin(math.radians(deg)), rel_tol=10 * FLT_EPS)
    assert np.array_equal(perm[:256], perm[256:])
    assert sorted(perm[:256]) == list(range(256))
    _, perm2, _ = oracle.permutation(6666, 10, math.radians(6.5))
    assert np.array_equal(perm, perm2)
    _, perm3, _ = oracle.permutation(183457092, 10, math.radians(6.5))
    assert not np.array_equal(perm, perm3)
    assert oracle.permutation(0, 0, 0.0)[0] == 1          # Distribution 0 -> STPInvalidEnvironment
    assert oracle.permutation(0, 8, -0.1)[0] == 1
    assert oracle.permutation(0, 8, 2 * math.pi)[0] == 1


def test_permutation_reference_fixtures(oracle):
    for seed, n, offset, perm, grad in helpers.load_permutations():
        rc, p, g = oracle.permutation(seed, n, offset)
        assert rc in (0, 2)
        assert np.array_equal(p, perm)
        assert np.array_equal(g.view(np.uint32), grad.view(np.uint32))


@pytest.mark.parametrize("radius,size", [(1, 1), (2, 9), (3, 25), (4, 45), (5, 69)])
def test_brush(oracle, radius, size):
    """generateErosionBrush (STPHeightfieldGenerator.cpp:44-77): sizes and normalised weights."""
    idx, w = oracle.brush(1536, radius)
    assert len(idx) == size
    assert abs(float(np.sum(w, dtype=np.float64)) - 1.0) < 1e-6
    dy, dx = np.divmod(idx + 1536 * radius + radius, 1536)
    assert np.all((dx - radius) ** 2 + (dy - radius) ** 2 < radius * radius)
    assert np.all(np.diff(idx) > 0)  # y-major, x-minor order


def test_philox_known_answers(oracle):
    """Philox4x32-10 against the published known-answer vectors of the Random123 distribution."""
    import ctypes as C
    lib = oracle.lib
    # drive the generator through the start mapping with MapSize - 1 = 2^24 would lose bits; instead
    # recompute the raw block via starts at counter 0, key 0 and compare the high 24 bits
    xy = oracle.droplet_starts(1, 0, 0, (2, 2), (1, 1))
    # with map 2x2 and nn 1: pos = u * 1 + 0 = u = ((x >> 8) + 1) / 2^24
    raw0 = int(round(float(xy[0]) * 16777216.0)) - 1
    raw1 = int(round(float(xy[1]) * 16777216.0)) - 1
    assert raw0 == 0x6627e8d5 >> 8
    assert raw1 == 0xe169c58d >> 8
    del lib, C


def test_voronoi_properties(oracle):
    a = oracle.voronoi(64, 48, (-64, -48), 16, 5, 9)
    b = oracle.voronoi(64, 48, (-64, -48), 16, 5, 9)
    assert np.array_equal(a, b)
    assert a.max() < 5
    # tiles agree with a larger map (the map is a function of global coordinates)
    big = oracle.voronoi(128, 96, (-64, -48), 16, 5, 9)
    assert np.array_equal(big[:48, :64], a)


def test_erosion_oracle_mass_balance(oracle):
    """FP64 serial oracle: sum(h0) - sum(h1) equals the sediment carried away by dying droplets."""
    rng = np.random.default_rng(3)
    n = 96
    y, x = np.mgrid[0:n, 0:n]
    h = (0.5 + 0.3 * np.sin(x / 9.0) * np.cos(y / 7.0) + 0.01 * rng.random((n, n))).astype(np.float32)
    s = helpers.raindrop_dict(500, radius=3, lifetime=30)
    starts = oracle.droplet_starts(500, 7, 0, (32, 32), (3, 3))
    idx, w = oracle.brush(n, 3)
    m, res, steps = oracle.erode(h, s, starts, idx, w, fp64=True)
    assert steps > 500
    assert abs((h.astype(np.float64).sum() - m.sum()) - res) < 1e-9 * h.sum()
    m32, res32, _ = oracle.erode(h, s, starts, idx, w, fp64=False)
    assert abs((h.astype(np.float64).sum() - m32.astype(np.float64).sum()) - res32) < 1e-5 * h.sum()


@pytest.fixture(scope="module")
def reference():
    """The reference's own filter and permutation sources compiled here (absent where the reference
    tree is not available: then these tests skip)."""
    from oracle.oracle import Reference
    try:
        return Reference()
    except Exception as e:  # no reference tree, or it could not be compiled here
        pytest.skip(f"reference build unavailable: {e}")


@pytest.mark.parametrize("seed", range(12))
def test_shf_oracle_matches_live_reference(oracle, reference, seed):
    """Random neighbourhoods (sides 3-40, 1-40 IDs, clustered or scattered, every legal even radius
    drawn at random): the oracle's filter equals the reference's serial and 4-thread parallel
    buffers, offsets and (item, weight) bins bit for bit, in bin order."""
    rng = np.random.default_rng(1000 + seed)
    mx, my = (int(v) for v in rng.integers(3, 41, 2))
    nx, ny = 3, 3
    ids = int(rng.integers(1, 41))
    if seed % 2:
        sm = rng.integers(0, ids, (ny * my, nx * mx)).astype(np.uint16)
    else:
        cell = int(rng.integers(2, 12))
        sm = oracle.voronoi(nx * mx, ny * my, (int(rng.integers(-500, 500)), int(rng.integers(-500, 500))), cell,
                            ids, seed)
    r = 2 * int(rng.integers(1, min(mx, my) // 2 + 1))
    rc, off, bins = oracle.shf(sm, (mx, my), (nx, ny), r)
    assert rc == 0
    for parallel in (False, True):
        rrc, roff, rbins = reference.shf(sm, (mx, my), (nx, ny), r, parallel=parallel)
        assert rrc == 0
        assert np.array_equal(off, roff), (mx, my, r, parallel)
        assert np.array_equal(bins["Item"], rbins["Item"])
        assert np.array_equal(bins["Weight"].view(np.uint32), rbins["Weight"].view(np.uint32))


@pytest.mark.parametrize("seed", [0, 1, 42, 6666, 2**40 + 7, 2**64 - 1])
def test_permutation_oracle_matches_live_reference(oracle, reference, seed):
    """Distributions whose gradient loop stays inside the reference's table (for 6, 11, 13, ... the
    reference writes one gradient past it, which the oracle reports instead of repeating)."""
    for distribution, offset in ((8, 0.2181661565), (10, 0.11344640137963143), (16, 0.0), (32, 6.0), (7, 3.1)):
        rc, perm, grad = oracle.permutation(seed, distribution, offset)
        rrc, rperm, rgrad = reference.permutation(seed, distribution, offset)
        assert rc == rrc == 0
        assert np.array_equal(perm, rperm)
        assert np.array_equal(grad.view(np.uint32), rgrad.view(np.uint32))


@pytest.mark.parametrize("params", [(64, 9400, 4, 50), (128, 37500, 3, 30)])
def test_droplet_order_spread_exceeds_fp64_distance(oracle, params):
    """The reference's droplet arithmetic (the FP32 serial oracle, equal to the reference's
    STPRainDrop bit for bit) depends on the order the droplets run in: a shuffled order moves the
    map by an RMS of about 1e-3 to 2e-3.  The FP64 oracle is closer to the index-order run than any
    reordered run is, so an RMS band measured against it bounds order effects, not a bias of the
    oracle."""
    S, count, brush, life = params
    rng = np.random.default_rng(S)
    y, x = np.mgrid[0:3 * S, 0:3 * S]
    h = (0.5 + 0.25 * np.sin(x / 23.0) * np.cos(y / 17.0) + 0.15 * np.sin((x + 2 * y) / 41.0)
         + 0.02 * rng.random(x.shape)).astype(np.float32)
    s = helpers.raindrop_dict(count, radius=brush, lifetime=life)
    starts = oracle.droplet_starts(count, 9, 0, (S, S), (3, 3))
    idx, w = oracle.brush(3 * S, brush)

    def rms(a, b):
        return float(np.sqrt(((a.astype(np.float64) - b.astype(np.float64)) ** 2).mean()))

    f64, _, _ = oracle.erode(h, s, starts, idx, w, fp64=True)
    f32, _, _ = oracle.erode(h, s, starts, idx, w, fp64=False)
    shuffled = [oracle.erode(h, s, starts.reshape(-1, 2)[rng.permutation(count)].ravel(), idx, w, fp64=False)[0]
                for _ in range(3)]
    order_spread = [rms(f32, m) for m in shuffled]
    assert min(order_spread) > 5e-4
    assert rms(f32, f64) < min(order_spread)
