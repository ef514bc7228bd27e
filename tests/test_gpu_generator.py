"""The plain per-chunk drop-in (STPHeightfieldGenerator::generate / erode over
host arrays) against the oracle."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def make_generator(stpgb, map_size, nbiomes, radius, count, brush, lifetime=30, seed=42):
    cs = stpgb.ChunkSetting()
    cs.MapSize[:] = list(map_size)
    cs.DiversityNearestNeighbour[:] = [3, 3]
    cs.ErosionNearestNeighbour[:] = [3, 3]
    rd = stpgb.RaindropSetting(**helpers.raindrop_dict(count, radius=brush, lifetime=lifetime, seed=seed))
    sx = stpgb.SimplexSetting(seed, 8, 0.2181661565)
    table = helpers.biome_table(nbiomes, seed)
    return stpgb.STPHeightfieldGenerator(cs, rd, sx, table, radius), table


def test_generate_matches_oracle(stpgb, dev, oracle):
    mx, my, nb, r = 128, 96, 6, 16
    gen, table = make_generator(stpgb, (mx, my), nb, r, 1000, 3)
    merged = oracle.voronoi(3 * mx, 3 * my, (0, 0), 50, nb, 5)
    chunks = [np.ascontiguousarray(merged[(i // 3) * my:(i // 3 + 1) * my, (i % 3) * mx:(i % 3 + 1) * mx])
              for i in range(9)]
    out = np.zeros((my, mx), np.float32)
    offset = (mx * 1.0, -2.0 * my)
    gen.generate(out, chunks, offset)
    rc, off, bins = oracle.shf(merged, (mx, my), (3, 3), r)
    perm, grad = stpgb.permutation_generate(42, 8, 0.2181661565)
    ref = oracle.multibiome(off, bins, table, perm, grad, (mx, my), offset)
    assert np.abs(out - ref).max() <= 2e-6


def test_erode_neighbour_pack_unpack(stpgb, dev, oracle):
    """STPTestNearestNeighbour.cpp: chunk i filled with i merges to the right place and unmerges back
    (zero droplets, so erosion leaves the map as it is); fixed-point output is the formatted map."""
    mx = my = 8
    gen, _ = make_generator(stpgb, (mx, my), 2, 2, 1, 1)
    chunks = [np.full((my, mx), i / 9.0, np.float32) for i in range(9)]
    fixed = [np.zeros((my, mx), np.uint16) for _ in range(9)]
    res = gen.erode(chunks, fixed, starts=np.zeros(0, np.float32))
    assert res == 0.0
    for i in range(9):
        assert np.all(chunks[i] == np.float32(i / 9.0))
        assert np.all(fixed[i] == oracle.format(chunks[i]))


def test_erode_mass_balance_and_format(stpgb, dev, oracle):
    mx = my = 128
    count = 30000
    gen, _ = make_generator(stpgb, (mx, my), 2, 2, count, 4, lifetime=50)
    rng = np.random.default_rng(4)
    y, x = np.mgrid[0:3 * my, 0:3 * mx]
    merged = (0.5 + 0.3 * np.sin(x / 31.0) * np.cos(y / 19.0) + 0.01 * rng.random(x.shape)).astype(np.float32)
    chunks = [np.ascontiguousarray(merged[(i // 3) * my:(i // 3 + 1) * my, (i % 3) * mx:(i % 3 + 1) * mx])
              for i in range(9)]
    fixed = [np.zeros((my, mx), np.uint16) for _ in range(9)]
    starts = oracle.droplet_starts(count, 11, 0, (mx, my), (3, 3))
    res = gen.erode(chunks, fixed, starts=starts)
    after = np.block([[chunks[3 * r + c] for c in range(3)] for r in range(3)])
    total = merged.astype(np.float64).sum()
    assert abs((total - after.astype(np.float64).sum()) - res) <= 1e-5 * total
    for i in range(9):
        assert np.array_equal(fixed[i], oracle.format(chunks[i]))
    # the default droplet source (Philox keyed by the raindrop seed) also runs
    gen.erode(chunks, fixed)
