"""Hydraulic erosion, height formatting and droplet starts on the GPU.

Erosion is racy by design (droplets share the map through float atomics, as
in the reference's release build), so parity is stated as
  * mass balance: sum(h0) - sum(h1) == carried-away sediment, within 1e-5
    relative to sum(h0);
  * droplets that never meet follow the FP64 serial oracle (per-pixel RMS
    below 1e-5 of the height range);
  * for dense droplets, the per-pixel RMS against the FP64 serial oracle,
    measured over several runs, stays within the runs' own spread of each
    other (the run-to-run RMS).
"""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def terrain(n_x, n_y, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:n_y, 0:n_x]
    h = 0.5 + 0.25 * np.sin(x / 23.0) * np.cos(y / 17.0) + 0.15 * np.sin((x + 2 * y) / 41.0)
    h += 0.02 * rng.random((n_y, n_x))
    return h.astype(np.float32)


def gpu_erode(dev, stpgb, h, map_size, nn, setting, starts):
    import torch
    d = torch.from_numpy(h.copy()).cuda()
    st = torch.from_numpy(np.ascontiguousarray(starts, np.float32)).cuda()
    idx, w = stpgb.erosion_brush(h.shape[1], setting["ErosionBrushRadius"])
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    dev.hydraulic_erosion(d, map_size, nn, stpgb.RaindropSetting(**setting), st, len(starts) // 2,
                          torch.from_numpy(idx).cuda(), torch.from_numpy(w).cuda(), res, status)
    dev.status_check(status)
    return d.cpu().numpy(), float(res.item())


def test_droplet_starts_match_oracle(dev, oracle):
    import torch
    for ms, nn, count, seed, base in (((256, 256), (1, 1), 32768, 42, 0), ((512, 512), (3, 3), 100000, 7, 12345),
                                      ((100, 60), (3, 5), 999, 2**40 + 3, 2**33)):
        out = torch.empty(2 * count, dtype=torch.float32, device="cuda")
        dev.droplet_starts(out, count, seed, base, ms, nn)
        ref = oracle.droplet_starts(count, seed, base, ms, nn)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))
        x, y = ref[0::2], ref[1::2]
        assert x.min() > (nn[0] // 2) * ms[0] and x.max() <= (nn[0] // 2) * ms[0] + ms[0] - 1
        assert y.min() > (nn[1] // 2) * ms[1] and y.max() <= (nn[1] // 2) * ms[1] + ms[1] - 1


def test_format_matches_oracle(dev, oracle):
    import torch
    rng = np.random.default_rng(0)
    for w, h in ((256, 256), (1536, 1536), (37, 11)):
        a = rng.uniform(-0.2, 1.2, (h, w)).astype(np.float32)
        a[0, :3] = [np.nan, np.inf, -np.inf]
        a[1, :4] = [0.5 / 65535, 1.5 / 65535, 2.5 / 65535, 1.0]
        out = torch.empty((h, w), dtype=torch.int16, device="cuda")
        dev.format_heightmap(torch.from_numpy(a).cuda(), out, w, h)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.uint16), oracle.format(a))


def test_voronoi_matches_oracle(dev, oracle):
    import torch
    for (w, h, ox, oy, cell, nb, seed) in ((768, 768, -256, -256, 128, 4, 42), (300, 200, 10**9, -5 * 10**8, 37, 13, 5)):
        out = torch.empty((h, w), dtype=torch.int16, device="cuda")
        dev.voronoi_biomemap(out, w, w, h, (ox, oy), cell, nb, seed)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.uint16), oracle.voronoi(w, h, (ox, oy), cell, nb, seed))


@pytest.mark.parametrize("map_size,nn,count,radius,lifetime", [
    ((256, 256), (1, 1), 32768, 3, 30),
    ((128, 128), (3, 3), 60000, 4, 50),
    ((96, 64), (3, 3), 20000, 2, 40),
    ((64, 64), (3, 3), 9000, 5, 64),
])
def test_erosion_mass_balance(dev, oracle, stpgb, map_size, nn, count, radius, lifetime):
    mx, my = map_size
    h = terrain(mx * nn[0], my * nn[1], 1)
    s = helpers.raindrop_dict(count, radius=radius, lifetime=lifetime)
    starts = oracle.droplet_starts(count, 42, 0, map_size, nn)
    out, residual = gpu_erode(dev, stpgb, h, map_size, nn, s, starts)
    assert np.isfinite(out).all()
    assert not np.array_equal(out, h)
    total = h.astype(np.float64).sum()
    balance = (total - out.astype(np.float64).sum()) - residual
    assert abs(balance) <= 1e-5 * total, f"mass balance off by {balance:.3g} of {total:.3g}"


def test_erosion_sparse_droplets_follow_fp64_oracle(dev, oracle, stpgb):
    """Droplets whose paths cannot meet (starts 80 px apart, 30 steps, brush 3) run as the serial oracle."""
    mx = my = 320
    h = terrain(mx, my, 2)
    g = np.arange(40, 300, 80, dtype=np.float32) + 0.37
    xs, ys = np.meshgrid(g, g)
    starts = np.stack([xs.ravel(), ys.ravel()], 1).ravel().astype(np.float32)
    s = helpers.raindrop_dict(len(starts) // 2, radius=3, lifetime=30)
    out, res = gpu_erode(dev, stpgb, h, (mx, my), (1, 1), s, starts)
    idx, w = oracle.brush(mx, 3)
    ref, ref_res, _ = oracle.erode(h, s, starts, idx, w, fp64=True)
    rms = float(np.sqrt(np.mean((out.astype(np.float64) - ref) ** 2)))
    assert rms <= 1e-5 * float(h.max() - h.min()), rms
    assert abs(res - ref_res) <= 1e-4 * max(ref_res, 1e-6) + 1e-6


def test_erosion_rms_within_run_to_run_spread(dev, oracle, stpgb):
    """Dense droplets: the GPU runs' RMS against the FP64 serial oracle agree to within their own spread."""
    mx = my = 96
    nn = (3, 3)
    h = terrain(mx * 3, my * 3, 3)
    count = 20000
    s = helpers.raindrop_dict(count, radius=3, lifetime=30)
    starts = oracle.droplet_starts(count, 9, 0, (mx, my), nn)
    idx, w = oracle.brush(mx * 3, 3)
    ref, _, _ = oracle.erode(h, s, starts, idx, w, fp64=True)
    runs = [gpu_erode(dev, stpgb, h, (mx, my), nn, s, starts)[0].astype(np.float64) for _ in range(5)]
    rms_vs_oracle = [float(np.sqrt(np.mean((r - ref) ** 2))) for r in runs]
    spread = max(float(np.sqrt(np.mean((a - b) ** 2))) for i, a in enumerate(runs) for b in runs[i + 1:])
    print(f"RMS vs FP64 serial oracle: {rms_vs_oracle}; run-to-run spread (max pairwise RMS): {spread:.3g}")
    assert max(rms_vs_oracle) - min(rms_vs_oracle) <= spread + 1e-7
