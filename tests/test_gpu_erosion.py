"""Hydraulic erosion, height formatting and droplet starts on the GPU.

Erosion is racy by design (droplets share the map through float atomics, as
in the reference's release build), so parity is stated as
  * mass balance: sum(h0) - sum(h1) == carried-away sediment, within 1e-5
    relative to sum(h0);
  * droplets that never meet follow the FP64 serial oracle (per-pixel RMS
    below 1e-5 of the height range);
  * for dense droplets, the per-pixel RMS against the FP64 serial oracle
    stays within the band of the reference's own erosion kernel built for
    sm_103a (oracle/build_ref.sh), fed the same droplets: its worst RMS plus
    its own run-to-run spread over five runs.
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


@pytest.mark.parametrize("brush", [3, 4, 5])
def test_erosion_sparse_droplets_follow_fp64_oracle(dev, oracle, stpgb, brush):
    """Droplets whose paths cannot meet (starts 80 px apart, 30 steps, brush reach below 5) run as
    the serial oracle: brush 3 reads then reduces each 16-byte block, brushes 4 and 5 take the
    amounts with one returning atomic per block and give back what a cell lacked."""
    mx = my = 320
    h = terrain(mx, my, 2)
    g = np.arange(40, 300, 80, dtype=np.float32) + 0.37
    xs, ys = np.meshgrid(g, g)
    starts = np.stack([xs.ravel(), ys.ravel()], 1).ravel().astype(np.float32)
    s = helpers.raindrop_dict(len(starts) // 2, radius=brush, lifetime=30)
    out, res = gpu_erode(dev, stpgb, h, (mx, my), (1, 1), s, starts)
    idx, w = oracle.brush(mx, brush)
    ref, ref_res, _ = oracle.erode(h, s, starts, idx, w, fp64=True)
    rms = float(np.sqrt(np.mean((out.astype(np.float64) - ref) ** 2)))
    assert rms <= 1e-5 * float(h.max() - h.min()), rms
    assert abs(res - ref_res) <= 1e-4 * max(ref_res, 1e-6) + 1e-6


def erode_runs(dev, stpgb, h, map_size, nn, s, starts, runs, **kw):
    import torch
    idx, w = stpgb.erosion_brush(h.shape[1], s["ErosionBrushRadius"])
    out = []
    for _ in range(runs):
        d = torch.from_numpy(h.copy()).cuda()
        res = torch.zeros(1, dtype=torch.float64, device="cuda")
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        dev.hydraulic_erosion(d, map_size, nn, stpgb.RaindropSetting(**s),
                              torch.from_numpy(np.ascontiguousarray(starts)).cuda(), len(starts) // 2,
                              torch.from_numpy(idx).cuda(), torch.from_numpy(w).cuda(), res, status, **kw)
        dev.status_check(status)
        out.append((d.cpu().numpy().astype(np.float64), float(res.item())))
    return out


def rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)))


EROSION_CASES = {
    # smooth terrain, 96^2 chunks in a 3x3 neighbourhood
    "smooth-96": (96, 20000, 3, 30),
    # densely packed droplets: 9,000 droplets start inside one 64^2 chunk
    "dense-64": (64, 9000, 3, 30),
    "brush5-128": (128, 37000, 5, 50),
}


@pytest.mark.parametrize("lanes,droplets_per_group,pointwise", [
    (1, 1, True), (2, 1, True), (2, 1, False), (2, 2, False), (4, 1, False), (4, 1, True), (4, 2, False),
    (4, 2, True), (8, 2, True), (4, 4, True)])
def test_erosion_stays_physical_where_droplets_channel(dev, oracle, stpgb, lanes, droplets_per_group, pointwise):
    """Multi-biome terrain with many biome borders gathers densely packed droplets into shared
    channels; at 1.5 droplets per pixel of a 64^2 chunk, all in flight (the most the library runs
    several lanes per droplet at), in no variant (point by point, or brush rows in 16-byte blocks)
    may the heights leave their range.  Denser loads run the one-lane kernel
    (test_default_choice_stays_physical_when_densely_packed)."""
    S = 64
    h = helpers.multibiome_terrain(oracle, stpgb, S, 6, 20, 11)
    count = int(round(1.5 * S * S))
    s = helpers.raindrop_dict(count, radius=3, lifetime=30, seed=11)
    starts = oracle.droplet_starts(count, 11, 0, (S, S), (3, 3))
    total = h.astype(np.float64).sum()
    for out, res in erode_runs(dev, stpgb, h, (S, S), (3, 3), s, starts, 10, lanes=lanes,
                               droplets_per_group=droplets_per_group, pointwise=pointwise):
        assert np.isfinite(out).all() and out.min() >= h.min() - 1e-3 and out.max() <= h.max() + 1e-3
        assert abs((total - out.sum()) - res) <= 1e-5 * total


@pytest.mark.parametrize("brush,density", [(3, 2.3), (4, 3.0), (3, 4.9), (4, 4.9), (3, 7.0), (4, 7.0)])
def test_default_choice_stays_physical_when_densely_packed(dev, oracle, stpgb, brush, density):
    """Above 1.5 droplets in flight per pixel (here every droplet of a 64^2 chunk is in flight) the
    default runs one lane per droplet (the reference kernel's layout): from 2.3 to 7 droplets per pixel the
    heights stay in range."""
    S = 64
    h = helpers.multibiome_terrain(oracle, stpgb, S, 6, 20, 11)
    count = int(round(density * S * S))
    s = helpers.raindrop_dict(count, radius=brush, lifetime=30, seed=11)
    starts = oracle.droplet_starts(count, 11, 0, (S, S), (3, 3))
    total = h.astype(np.float64).sum()
    for out, res in erode_runs(dev, stpgb, h, (S, S), (3, 3), s, starts, 3):
        assert np.isfinite(out).all() and out.min() >= h.min() - 1e-3 and out.max() <= h.max() + 1e-3
        assert abs((total - out.sum()) - res) <= 1e-5 * total


@pytest.mark.parametrize("brush,lanes,droplets_per_group", [(3, 0, 1), (4, 0, 1), (5, 0, 1), (3, 4, 2), (4, 2, 2)])
def test_rows_stay_physical_at_the_dense_limit(dev, oracle, stpgb, brush, lanes, droplets_per_group):
    """At 1.5 droplets in flight per pixel, the densest load for which the default takes the brush-row
    kernels (the default choice and explicit row variants, one brush block per round trip at this many
    droplets in flight), the heights stay in range in every run.  Without the brush amount clamped at
    zero, brush 3 drove heights to -10^5 at 3 droplets per pixel: racing readers of one cell took it
    below zero, and every reader then added the negative height's magnitude back."""
    S = 64
    h = helpers.multibiome_terrain(oracle, stpgb, S, 6, 20, 11)
    count = int(round(1.5 * S * S))
    s = helpers.raindrop_dict(count, radius=brush, lifetime=30, seed=11)
    starts = oracle.droplet_starts(count, 11, 0, (S, S), (3, 3))
    total = h.astype(np.float64).sum()
    for out, res in erode_runs(dev, stpgb, h, (S, S), (3, 3), s, starts, 10, lanes=lanes,
                               droplets_per_group=droplets_per_group):
        assert np.isfinite(out).all() and out.min() >= h.min() - 1e-3 and out.max() <= h.max() + 1e-3
        assert abs((total - out.sum()) - res) <= 1e-5 * total


# The cases below keep every droplet in flight at about 2.2 per pixel, where the
# default is the one-lane kernel (one thread per droplet); "rows-2-lanes" and the other row
# variants update the brush in 16-byte row blocks (the maps here are aligned
# and a multiple of four wide); "pointwise" keeps the point-by-point kernels.
VARIANTS = {
    "default": {},
    "rows-2-lanes": {"lanes": 2},
    "pointwise": {"pointwise": True},
    "exact-clamp": {"exact_clamp": True},
    "rows-2-lanes-2-droplets": {"droplets_per_group": 2, "lanes": 2},
    "2-droplets-per-group": {"droplets_per_group": 2},
    "2-droplets-pointwise": {"droplets_per_group": 2, "pointwise": True},
    "8-lanes-2-droplets-pointwise": {"droplets_per_group": 2, "lanes": 8, "pointwise": True},
    "4-droplets-per-group": {"droplets_per_group": 4},
}


@pytest.mark.parametrize("case", sorted(EROSION_CASES))
@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_erosion_rms_within_reference_spread(dev, oracle, stpgb, case, variant):
    erosion_rms_within_reference_spread(dev, oracle, stpgb, EROSION_CASES[case], variant, case)


@pytest.mark.parametrize("params,variant", [((512, 600000, 4, 50), "default"), ((256, 150000, 4, 50), "default"),
                                            ((512, 600000, 4, 50), "warp-cooperative")],
                         ids=["512", "256", "512-warp-cooperative"])
def test_production_brush_rms_within_reference_spread(dev, oracle, stpgb, params, variant):
    """The production chunk (3x3 x 512^2, 600,000 droplets, brush 4, lifetime 50) and the same
    density on 256^2 chunks: the default choice (brush rows with two lanes, the brush taken by
    returning atomics, several blocks per round trip on the production chunk) and, on the production
    chunk, the warp-cooperative kernel (one droplet per lane, every run of the brush in flight at
    once) stay within the reference GPU build's band around the FP64 serial result."""
    erosion_rms_within_reference_spread(dev, oracle, stpgb, params, variant, f"brush4-{params[0]}",
                                        {"warp-cooperative": {"lanes": 1}}.get(variant))


_FP64 = {}


def fp64_serial(oracle, case, h, s, starts):
    """The FP64 serial oracle's result for a case (computed once per case and session)."""
    if case not in _FP64:
        idx, w = oracle.brush(h.shape[1], s["ErosionBrushRadius"])
        _FP64[case] = oracle.erode(h, s, starts, idx, w, fp64=True)[0]
    return _FP64[case]


def erosion_rms_within_reference_spread(dev, oracle, stpgb, params, variant, case, kw=None):
    """Per-pixel RMS against the FP64 serial oracle stays within the reference GPU build's own band.

    The reference's erosion kernel (hydraulicErosionKERNEL + STPRainDrop compiled by nvcc for sm_103a
    with its release flags, oracle/build_ref.sh) runs five times on the same map with the same
    droplets; its RMS against the FP64 serial oracle per run and its run-to-run spread (the largest
    RMS between two of its runs) make the band.  Every run of the library's kernel must satisfy
    RMS <= max(RMS_ref) + spread_ref, and conserve mass within 1e-5."""
    S, count, brush, life = params
    nn = (3, 3)
    h = terrain(3 * S, 3 * S, S)
    s = helpers.raindrop_dict(count, radius=brush, lifetime=life)
    starts = oracle.droplet_starts(count, 9, 0, (S, S), nn)
    ref = fp64_serial(oracle, case, h, s, starts)
    ref_rms, spread, source = helpers.reference_band(case, oracle, h, (S, S), nn, s, 9, 0, ref)
    kw = dict(VARIANTS[variant] if kw is None else kw)
    if kw.get("droplets_per_group", 1) > 1:
        kw.setdefault("lanes", 4)  # several droplets per group need >= 4 lanes; every brush here allows 4
    prod = erode_runs(dev, stpgb, h, (S, S), nn, s, starts, 3, **kw)
    prod_rms = [rms(r, ref) for r, _ in prod]
    print(f"{case} {variant}: reference GPU build ({source}) RMS vs FP64 {min(ref_rms):.3g}..{max(ref_rms):.3g}, "
          f"spread {spread:.3g}; library RMS {prod_rms}")
    assert max(prod_rms) <= max(ref_rms) + spread
    total = h.astype(np.float64).sum()
    for out, res in prod:
        assert abs((total - out.sum()) - res) <= 1e-5 * total
