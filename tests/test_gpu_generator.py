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


def _chunks(S, seed):
    rng = np.random.default_rng(seed)
    return [rng.integers(0, 4, (S, S)).astype(np.uint16) for _ in range(9)]


def test_setup_with_the_demo_plugin_equals_the_folded_constructor(stpgb):
    """STPHeightfieldGenerator(STPGeneratorSetup) with the demo's multi-biome plugin as its diversity
    generator gives the heightmap of the constructor that folds the plugin in, bit for bit."""
    S = 64
    cs = stpgb.ChunkSetting()
    cs.MapSize[:] = [S, S]
    cs.DiversityNearestNeighbour[:] = [3, 3]
    cs.ErosionNearestNeighbour[:] = [3, 3]
    rd = stpgb.RaindropSetting(**helpers.raindrop_dict(1000))
    simplex = stpgb.SimplexSetting(42, 8, 0.2181661565)
    table = helpers.biome_table(4, 3)
    plugin = stpgb.STPBiomefieldGenerator(simplex, table, 8)
    a = stpgb.STPHeightfieldGenerator.setup(cs, rd, plugin)
    b = stpgb.STPHeightfieldGenerator(cs, rd, simplex, table, 8)
    chunks = _chunks(S, 1)
    ha, hb = np.zeros((S, S), np.float32), np.zeros((S, S), np.float32)
    a.generate(ha, chunks, (64.0, -128.0))
    b.generate(hb, chunks, (64.0, -128.0))
    assert np.array_equal(ha, hb) and ha.max() > 0.0


def test_user_plugin_writes_the_heightmap_and_its_errors_reach_the_caller(stpgb):
    """A diversity plugin written by the caller: it reads the merged biome neighbourhood off the device
    and writes its own function of it into the chunk's heightmap (stpgb_copy on the call's stream).
    An exception it raises comes back out of generate unchanged."""
    S = 48

    class Terrace(stpgb.STPDiversityGenerator):
        calls = 0

        def __call__(self, heightmap, biomemap, offset, call):
            nn = call.biomemap_nn
            tw, th = nn.TotalMapSize[0], nn.TotalMapSize[1]
            merged = np.zeros((th, tw), np.uint16)
            stpgb.check(stpgb.lib().stpgb_copy(merged.ctypes.data, biomemap, merged.nbytes, call.stream, 1))
            centre = merged[S:2 * S, S:2 * S].astype(np.float32)
            out = np.ascontiguousarray(0.1 * centre + np.float32(1e-3) * np.float32(offset[0]), np.float32)
            stpgb.check(stpgb.lib().stpgb_copy(heightmap, out.ctypes.data, out.nbytes, call.stream, 1))
            Terrace.calls += 1

    class Refuse(stpgb.STPDiversityGenerator):
        def __call__(self, heightmap, biomemap, offset, call):
            raise KeyError("no heightmap for this chunk")

    cs = stpgb.ChunkSetting()
    cs.MapSize[:] = [S, S]
    cs.DiversityNearestNeighbour[:] = [3, 3]
    cs.ErosionNearestNeighbour[:] = [3, 3]
    rd = stpgb.RaindropSetting(**helpers.raindrop_dict(1000))
    gen = stpgb.STPHeightfieldGenerator.setup(cs, rd, Terrace())
    chunks = _chunks(S, 2)
    h = np.full((S, S), -1.0, np.float32)
    gen.generate(h, chunks, (96.0, 0.0))
    assert Terrace.calls == 1
    assert np.array_equal(h, (0.1 * chunks[4].astype(np.float32) + np.float32(1e-3) * np.float32(96.0)).astype(np.float32))
    bad = stpgb.STPHeightfieldGenerator.setup(cs, rd, Refuse())
    with pytest.raises(KeyError):
        bad.generate(h, chunks, (0.0, 0.0))
