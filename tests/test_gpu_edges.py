"""Edge cases of the hot path on the GPU, each against the oracle or the
reference's defined behaviour: no droplets, droplets that start off the map,
a map of one biome, a biome with no octaves, a one-step lifetime and the
smallest batch request."""
import numpy as np
import pytest

import helpers
from test_gpu_erosion import gpu_erode, terrain

pytestmark = pytest.mark.gpu


def test_no_droplets_leave_the_map_untouched(dev, stpgb):
    h = terrain(96, 96, 4)
    s = helpers.raindrop_dict(1, radius=3, lifetime=30)  # a valid setting; the call erodes none
    out, res = gpu_erode(dev, stpgb, h, (32, 32), (3, 3), s, np.zeros(0, np.float32))
    assert np.array_equal(out, h) and res == 0.0


def test_starts_off_the_map_die_at_once(dev, stpgb):
    """A start whose 2x2 bilinear footprint is not inside the map (negative, past the last cell,
    NaN) dies before its first step: the map is unchanged and nothing is carried away."""
    h = terrain(96, 96, 5)
    starts = np.array([-5.0, 40.0, 95.5, 40.0, 40.0, -0.25, 40.0, 95.0, np.nan, 40.0, 40.0, np.inf],
                      np.float32)
    s = helpers.raindrop_dict(len(starts) // 2, radius=3, lifetime=30)
    out, res = gpu_erode(dev, stpgb, h, (32, 32), (3, 3), s, starts)
    assert np.array_equal(out, h) and res == 0.0


def test_one_step_lifetime_follows_the_oracle(dev, stpgb, oracle):
    """Lifetime 1: every droplet takes exactly one step; sparse starts never meet, so the result is
    the serial oracle's."""
    h = terrain(160, 160, 6)
    g = np.arange(20, 140, 12, dtype=np.float32) + 0.3
    xs, ys = np.meshgrid(g, g)
    starts = np.stack([xs.ravel(), ys.ravel()], 1).ravel().astype(np.float32)
    s = helpers.raindrop_dict(len(starts) // 2, radius=3, lifetime=1)
    out, res = gpu_erode(dev, stpgb, h, (160, 160), (1, 1), s, starts)
    idx, w = oracle.brush(160, 3)
    ref, ref_res, steps = oracle.erode(h, s, starts, idx, w, fp64=False)
    assert steps == len(starts) // 2
    assert np.abs(out - ref).max() <= 1e-6 and abs(res - ref_res) <= 1e-6 * max(ref_res, 1.0)


def test_one_biome_map_gives_one_bin_per_pixel(dev, oracle):
    from test_gpu_shf import run_gpu
    for r in (2, 16):
        sm = np.full((3 * 40, 3 * 40), 7, np.uint16)
        off, items, weights = run_gpu(dev, sm, (40, 40), (3, 3), r)
        rc, ref_off, ref_bins = oracle.shf(sm, (40, 40), (3, 3), r)
        assert rc == 0
        assert np.array_equal(off, np.arange(40 * 40 + 1, dtype=np.uint32))
        assert np.array_equal(off, ref_off) and np.array_equal(items, ref_bins["Item"])
        assert np.array_equal(weights.view(np.uint32), np.ascontiguousarray(ref_bins["Weight"]).view(np.uint32))


def test_biome_without_octaves_matches_the_oracle(dev, oracle, stpgb):
    """A biome of zero octaves has no amplitude: the reference's (sum + R) / (2R) is 0/0 and
    __saturatef maps the NaN to 0, so the biome contributes Depth only."""
    import torch
    mx = my = 64
    perm, grad = stpgb.permutation_generate(9, 8, 0.2181661565)
    table = helpers.biome_table(2, 9)
    table["Octave"][1] = 0
    table["Depth"][1] = 0.25
    sm = oracle.voronoi(3 * mx, 3 * my, (-mx, -my), 24, 2, 9)
    rc, off, bins = oracle.shf(sm, (mx, my), (3, 3), 8)
    assert rc == 0 and (bins["Item"] == 1).any()
    ref = oracle.multibiome(off, bins, table, perm, grad, (mx, my), (128.0, -64.0))
    out = torch.full((my, mx), float("nan"), device="cuda")
    dev.multibiome_heightmap(out, mx, torch.from_numpy(off.view(np.int32)).cuda(),
                             torch.from_numpy(np.ascontiguousarray(bins).view(np.int64)).cuda(), (mx, my),
                             (128.0, -64.0), torch.from_numpy(perm).cuda(), torch.from_numpy(grad).cuda(),
                             torch.from_numpy(table.view(np.float32)).cuda())
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.isfinite(got).all() and np.abs(got - ref).max() <= 2e-6


def test_smallest_batch_request(stpgb, oracle):
    """One request of 8^2 chunks with filter radius 2 and brush radius 1 (a one-point brush)."""
    req = [dict(MapSize=8, ChunkX=1, ChunkY=-1, InterpolationRadius=2, DropletCount=100, BrushRadius=1,
                Lifetime=10)]
    base = stpgb.RaindropSetting(**helpers.raindrop_dict(100, radius=1, lifetime=10, seed=3))
    b = stpgb.Batch(req, base, stpgb.SimplexSetting(3, 8, 0.2181661565), helpers.biome_table(3, 3), graph=True)
    b.synthesize(5, 3)
    b.run_stage(0)
    b.run_stage(1)
    before = [np.zeros((24, 24), np.float32)]
    b.download(before)
    b.status()
    b.run()
    after, fixed, res = [np.zeros((24, 24), np.float32)], [np.zeros((24, 24), np.uint16)], np.zeros(1)
    b.download(after, fixed, res)
    b.status()
    t0 = before[0].astype(np.float64).sum()
    assert abs((t0 - after[0].astype(np.float64).sum()) - res[0]) <= 1e-5 * t0
    assert np.array_equal(fixed[0], oracle.format(after[0]))


def test_droplets_that_never_dry_stop_at_the_step_cap(dev, stpgb):
    """EvaporateSpeed 0 is a legal setting (the reference accepts [0, 1], STPEnvironment.cpp:62), and
    with it the reference's loop (while Volume >= minWaterVolume) never ends for a droplet that stays
    on the map.  Four droplets in a steep bowl whose lowest point lies inside a cell (no inertia, so
    each step turns them back towards it; no erosion or deposition, so the bowl keeps its shape) roll
    about its bottom for ever; the library's loop stops each at 2^20 steps and the call reports
    STPGB_ETIMEOUT instead of hanging.  The map is unchanged."""
    import torch
    n = 64
    y, x = np.mgrid[0:n, 0:n].astype(np.float32)
    h = (((x - 31.3) ** 2 + (y - 31.7) ** 2) * 0.01).astype(np.float32)
    s = helpers.raindrop_dict(4, radius=2, lifetime=30)
    s.update(EvaporateSpeed=0.0, minWaterVolume=0.5, Inertia=0.0, ErodeSpeed=0.0, DepositSpeed=0.0)
    starts = np.array([20.3, 22.7, 41.2, 25.1, 30.6, 44.4, 27.9, 31.2], np.float32)
    d = torch.from_numpy(h.copy()).cuda()
    st = torch.from_numpy(starts).cuda()
    idx, w = stpgb.erosion_brush(n, 2)
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    dev.hydraulic_erosion(d, (n, n), (1, 1), stpgb.RaindropSetting(**s), st, 4, torch.from_numpy(idx).cuda(),
                          torch.from_numpy(w).cuda(), res, status)
    with pytest.raises(stpgb.STPTimeout):
        dev.status_check(status)
    assert np.array_equal(d.cpu().numpy(), h)
