"""Single histogram filter on the GPU, through the C ABI, against the oracle
and the reference's fixtures: offsets, items and weights bit-exact,
including the order of the bins."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def run_gpu(dev, sm, map_size, nn, radius, max_items=0):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(sm).view(np.int16)).cuda()
    off, bins, status = dev.shf_filter(t, map_size, nn, radius, max_items=max_items)
    dev.status_check(status)
    off = off.cpu().numpy().view(np.uint32)
    n = int(off[-1])
    raw = bins[:n].cpu().numpy().view(np.uint64)
    items = (raw & 0xFFFF).astype(np.uint16)
    weights = (raw >> 32).astype(np.uint32).view(np.float32)
    return off, items, weights


def assert_same(a, b, name=""):
    off, items, weights = a
    o2, i2, w2 = b
    assert np.array_equal(off, o2), name
    assert np.array_equal(items, i2), name
    assert np.array_equal(weights.view(np.uint32), np.asarray(w2, np.float32).view(np.uint32)), name


def test_shf_reference_kat(dev):
    kat = helpers.load_shf_kat()
    got = run_gpu(dev, kat["texture"], (4, 4), (3, 3), 2)
    assert_same(got, (kat["offsets"], kat["items"], kat["weights"]), "kat")


def test_shf_reference_fixtures(dev, oracle):
    for name, sm, ms, nn, r, off, items, weights in helpers.shf_small_cases(oracle):
        assert_same(run_gpu(dev, sm, ms, nn, r), (off, items, weights), name)


def test_shf_reference_digests(dev, oracle):
    for case, sm in helpers.shf_large_cases(oracle):
        off, items, weights = run_gpu(dev, sm, tuple(case["map"]), tuple(case["nn"]), case["radius"])
        assert len(items) == case["nbins"]
        assert helpers.digest(off, items, weights) == case["sha256"], case


@pytest.mark.parametrize("seed", range(6))
def test_shf_random_vs_oracle(dev, oracle, seed):
    rng = np.random.default_rng(100 + seed)
    mx, my = (int(v) for v in rng.integers(5, 70, 2))
    r = 2 * int(rng.integers(1, min(mx, my) // 2 + 1))
    ids = int(rng.integers(1, 40))
    sm = rng.integers(0, ids, (3 * my, 3 * mx)).astype(np.uint16)
    rc, off, b = oracle.shf(sm, (mx, my), (3, 3), r)
    assert rc == 0
    assert_same(run_gpu(dev, sm, (mx, my), (3, 3), r), (off, b["Item"], b["Weight"]), (mx, my, r, ids))


def test_shf_large_ids_and_uneven_neighbourhood(dev, oracle):
    rng = np.random.default_rng(5)
    sm = (rng.integers(0, 5, (3 * 20, 5 * 24)) * 9000 + 7).astype(np.uint16)  # ids up to 36007
    rc, off, b = oracle.shf(sm, (24, 20), (5, 3), 10)
    assert rc == 0
    assert_same(run_gpu(dev, sm, (24, 20), (5, 3), 10), (off, b["Item"], b["Weight"]))


def test_shf_item_bound_reported(dev):
    """More distinct values in a window than max_items is reported, not written out of bounds."""
    import superterrainplus_gb300 as m
    rng = np.random.default_rng(1)
    sm = rng.integers(0, 50, (48, 48)).astype(np.uint16)
    with pytest.raises(m.STPCapacityError):
        run_gpu(dev, sm, (16, 16), (3, 3), 8, max_items=4)


def test_shf_max_radius_edge(dev, oracle):
    """Radius equal to the central chunk's start coordinate is the largest legal one."""
    rng = np.random.default_rng(9)
    sm = rng.integers(0, 3, (3 * 6, 3 * 8)).astype(np.uint16)
    rc, off, b = oracle.shf(sm, (8, 6), (3, 3), 6)
    assert rc == 0
    assert_same(run_gpu(dev, sm, (8, 6), (3, 3), 6), (off, b["Item"], b["Weight"]))


def test_shf_host_api_matches(stpgb, dev, oracle):
    """The reference-style class API (host arrays in/out) gives the same histogram."""
    kat = helpers.load_shf_kat()
    f = stpgb.STPSingleHistogramFilter()
    for t in (stpgb.STPFilterBuffer.Serial, stpgb.STPFilterBuffer.Parallel):
        buf = stpgb.STPFilterBuffer(t)
        bins, off = f(kat["texture"], stpgb.NNInfo.make((4, 4), (3, 3)), buf, 2)
        assert buf.type() == t
        assert buf.size() == (len(kat["items"]), 17)
        assert np.array_equal(off, kat["offsets"])
        assert np.array_equal(bins["Item"], kat["items"])
        assert np.array_equal(bins["Weight"].view(np.uint32), kat["weights"].view(np.uint32))


@pytest.mark.parametrize("radius", [2, 4, 8])
def test_shf_run_boundaries_across_segments(dev, oracle, radius):
    """One chunk filtered alone runs in segments that rebuild their starting order from the rule that
    occurrences at most 2r+1 apart keep an item present.  Here items recur exactly 2r+1 and 2r+2
    rows / columns apart (joined and split runs), several interleaved with phase shifts, over a
    64x96 chunk, so segment starts fall inside both kinds of gap; the result must be the oracle's."""
    S_x, S_y = 64, 96
    H, W = 3 * S_y, 3 * S_x
    y, x = np.mgrid[0:H, 0:W]
    sm = np.zeros((H, W), np.uint16)
    for item, (period, phase) in enumerate([(2 * radius + 1, 0), (2 * radius + 2, 3), (2 * radius + 1, 5),
                                            (4 * radius + 3, 1), (2 * radius + 2, 7)], start=1):
        sm[(y + phase) % period == 0] = item
        sm[((x + 2 * phase) % (period + 1) == 0) & (y % 3 == item % 3)] = item + 10
    got = run_gpu(dev, sm, (S_x, S_y), (3, 3), radius)
    rc, off, bins = oracle.shf(sm, (S_x, S_y), (3, 3), radius)
    assert rc == 0
    assert_same(got, (off, bins["Item"], bins["Weight"]), f"r={radius}")
