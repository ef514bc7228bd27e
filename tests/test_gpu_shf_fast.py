"""The filter's few-values path (a chunk whose read region holds at most 8 distinct sample
values), in both formulations (packed sequential slides, row bands) and as chosen by launch
size, against the oracle: offsets, items, weights and bin order bit-exact, the path the chunk
took checked through stpgb_shf_filter_path, and the general slides taking over at 9 values, at a
max_items below the palette, past the row bands' column bound and when chosen."""
import zlib

import numpy as np
import pytest

from test_gpu_shf import assert_same

pytestmark = pytest.mark.gpu


def palette_map(rng, shape, k, kind, oracle=None):
    """A sample map of `k` values spread over the 16-bit range (noise, 3x3 blocks, Voronoi cells
    or one value)."""
    values = np.sort(rng.choice(np.arange(65536, dtype=np.uint32), k, replace=False)).astype(np.uint16)
    h, w = shape
    if kind == "noise":
        idx = rng.integers(0, k, shape)
    elif kind == "blocks":
        idx = np.repeat(np.repeat(rng.integers(0, k, (h // 3 + 1, w // 3 + 1)), 3, 0), 3, 1)[:h, :w]
    elif kind == "voronoi":
        idx = oracle.voronoi(w, h, (0, 0), max(4, min(h, w) // 6), k, int(rng.integers(0, 1000))).astype(np.int64)
    else:
        idx = np.zeros(shape, np.int64)
    return values[idx]


def run(dev, sm, map_size, nn, r, max_items=0, cap=None):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(sm).view(np.int16)).cuda()
    ws = dev.shf_workspace(map_size, nn, r, max_items)
    off, bins, status = dev.shf_filter(t, map_size, nn, r, max_items=max_items, bins_capacity=cap, workspace=ws)
    path = dev.shf_filter_path(ws, map_size, nn, r, max_items)
    return off, bins, status, path


def unpack(off, bins, n=None):
    off = off.cpu().numpy().view(np.uint32)
    n = int(off[-1]) if n is None else n
    raw = bins[:n].cpu().numpy().view(np.uint64)
    return off, (raw & 0xFFFF).astype(np.uint16), (raw >> 32).astype(np.uint32).view(np.float32)


def distinct_in_read_region(sm, map_size, nn, r):
    sx, sy = map_size[0] * (nn[0] // 2), map_size[1] * (nn[1] // 2)
    return len(np.unique(sm[sy - r:sy + map_size[1] + r, sx - r:sx + map_size[0] + r]))


CASES = [
    # name, map size, nn, radius, distinct values, map kind
    ("uniform", (64, 64), (3, 3), 8, 1, "uniform"),
    ("noise-8", (48, 40), (3, 3), 4, 8, "noise"),
    ("blocks-8-small", (12, 20), (3, 3), 2, 8, "blocks"),
    ("noise-3-odd-rows", (33, 37), (3, 3), 6, 3, "noise"),
    ("voronoi-8-production", (512, 512), (3, 3), 32, 8, "voronoi"),
    ("nn-5x3-radius-above-map", (8, 16), (5, 3), 16, 5, "noise"),
    ("two-columns-per-thread", (1000, 24), (3, 3), 16, 6, "blocks"),
    ("four-columns-per-thread", (2068, 8), (3, 3), 8, 7, "noise"),
    ("wider-than-bands", (4100, 4), (3, 3), 2, 5, "blocks"),
    ("nine-values-slides", (40, 40), (3, 3), 4, 9, "noise"),
]
# stpgb_shf_set_path: 0 by launch size (one chunk: row bands), 1 packed slides, 2 row bands
FORMS = [0, 1, 2]


def expected_path(form, k_read, ms, r):
    if k_read > 8:
        return 0
    bands = form in (0, 2)
    if bands and ms[0] + 2 * r > 4096:
        return 0
    return 2 if bands else 1


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("name,ms,nn,r,k,kind", CASES, ids=[c[0] for c in CASES])
def test_fast_path_vs_oracle(dev, oracle, shf_path, form, name, ms, nn, r, k, kind):
    shf_path(form)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    sm = palette_map(rng, (ms[1] * nn[1], ms[0] * nn[0]), k, kind, oracle)
    k_read = distinct_in_read_region(sm, ms, nn, r)
    rc, off_ref, b = oracle.shf(np.ascontiguousarray(sm), ms, nn, r)
    assert rc == 0
    off, bins, status, path = run(dev, sm, ms, nn, r)
    dev.status_check(status)
    assert_same(unpack(off, bins), (off_ref, b["Item"], b["Weight"]), name)
    assert path == expected_path(form, k_read, ms, r), (name, form, k_read)


def test_general_slides_when_chosen(dev, oracle, shf_path):
    """Path 3 sends a chunk of few values through the general slides: same output."""
    shf_path(3)
    rng = np.random.default_rng(3)
    sm = palette_map(rng, (96, 96), 4, "noise")
    rc, off_ref, b = oracle.shf(np.ascontiguousarray(sm), (32, 32), (3, 3), 6)
    off, bins, status, path = run(dev, sm, (32, 32), (3, 3), 6)
    dev.status_check(status)
    assert path == 0
    assert_same(unpack(off, bins), (off_ref, b["Item"], b["Weight"]))


def test_set_path_rejects_unknown(stpgb, dev):
    with pytest.raises(stpgb.STPNumericDomainError):
        dev.shf_set_path(4)


@pytest.mark.parametrize("form", [1, 2])
def test_fast_path_max_items_below_palette_takes_the_slides(stpgb, dev, oracle, shf_path, form):
    """Five values, max_items 4: the palette does not fit the accumulator bound, so the general
    slides run and report the window that overflows it, as they always did."""
    shf_path(form)
    rng = np.random.default_rng(5)
    sm = palette_map(rng, (60, 60), 5, "noise")
    off, bins, status, path = run(dev, sm, (20, 20), (3, 3), 4, max_items=4)
    assert path == 0
    with pytest.raises(stpgb.STPCapacityError):
        dev.status_check(status)
    # max_items 5 fits the palette: the few-values path, and the oracle's result
    rc, off_ref, b = oracle.shf(np.ascontiguousarray(sm), (20, 20), (3, 3), 4)
    off, bins, status, path = run(dev, sm, (20, 20), (3, 3), 4, max_items=5)
    dev.status_check(status)
    assert path == form
    assert_same(unpack(off, bins), (off_ref, b["Item"], b["Weight"]))


@pytest.mark.parametrize("form", [1, 2])
def test_fast_path_short_bins_capacity(stpgb, dev, oracle, shf_path, form):
    """A bins capacity 5 short of the total: ECAPACITY on the status, every offset still written and
    the bins that fit equal to the oracle's."""
    shf_path(form)
    rng = np.random.default_rng(9)
    ms, r = (64, 48), 6
    sm = palette_map(rng, (3 * ms[1], 3 * ms[0]), 6, "noise")
    rc, off_ref, b = oracle.shf(np.ascontiguousarray(sm), ms, (3, 3), r)
    total = int(off_ref[-1])
    off, bins, status, path = run(dev, sm, ms, (3, 3), r, cap=total - 5)
    assert path == form
    with pytest.raises(stpgb.STPCapacityError):
        dev.status_check(status)
    got_off, items, weights = unpack(off, bins, total - 5)
    assert np.array_equal(got_off, off_ref)
    assert np.array_equal(items, b["Item"][:total - 5])
    assert np.array_equal(weights.view(np.uint32), b["Weight"][:total - 5].view(np.uint32))


@pytest.mark.parametrize("form", [1, 2])
def test_fast_path_repeated_calls_same_workspace(dev, oracle, shf_path, form):
    """The path's packed histograms overlay the general slides' vertical buffer: a chunk of 9
    values, then one of 4, then the 9 again through one workspace give the oracle's result each
    time."""
    import torch
    shf_path(form)
    rng = np.random.default_rng(13)
    ms, r = (48, 48), 8
    maps = [palette_map(rng, (144, 144), k, "noise") for k in (9, 4)]
    maps.append(maps[0])
    ws = dev.shf_workspace(ms, (3, 3), r)
    for n, sm in enumerate(maps):
        rc, off_ref, b = oracle.shf(np.ascontiguousarray(sm), ms, (3, 3), r)
        t = torch.from_numpy(np.ascontiguousarray(sm).view(np.int16)).cuda()
        off, bins, status = dev.shf_filter(t, ms, (3, 3), r, workspace=ws)
        dev.status_check(status)
        assert dev.shf_filter_path(ws, ms, (3, 3), r) == (0 if n != 1 else form)
        assert_same(unpack(off, bins), (off_ref, b["Item"], b["Weight"]), n)
