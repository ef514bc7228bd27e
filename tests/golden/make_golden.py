"""Generates the committed golden fixtures from the reference's own compiled
host sources (oracle/_ref/libstpref.so, built by oracle/build_ref.sh from the
reference tree).  Run in the development container, where the reference
tree exists:

    python tests/golden/make_golden.py

Fixtures:
  shf_kat.npz          the 12x12 test texture of the reference's
                       SuperTest+/SuperAlgorithm+/STPTestHistogram.cpp:44-57, r = 2
  shf_cases.npz        seeded random and Voronoi sample maps (random inputs
                       stored, Voronoi inputs regenerated from their seeds by
                       the integer-only generator), reference output stored
                       in full for small cases
  shf_digests.json     SHA-256 of the reference output for large cases
                       (512x512 chunk, r = 32; 256x256, r = 16, ...)
  permutation.npz      reference permutation/gradient tables for several seeds
  layer_biomemap.npz   the demo's biome layer chain (STPLayerChainBuilder through
                       STPBiomeFactory::operator()) for several seeds, offsets and
                       biome-ID assignments, stored in full; STPLayer seed
                       arithmetic (mixSeed, seedLayer, seedLocal) known answers
  layer_digests.json   SHA-256 of the layer chain's output for large maps
  device_reference.npz the reference's device code compiled as host C++
                       (oracle/_ref/libstpref_device.so): simplex2D and
                       simplex2DFractal values, the demo's two-biome generator
                       script over filtered sample maps, droplets run one after
                       another (STPRainDrop), the demo's splatmap script with
                       the rule lookups, erosion brushes and the format kernel,
                       with their inputs
  device_digests.json  SHA-256 of that build's production-size outputs (a 512^2
                       two-biome chunk, 600,000 droplets on a 1536^2 map)

`python tests/golden/make_golden.py layers` rewrites only the layer fixtures,
`python tests/golden/make_golden.py device` only device_reference.npz.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import (RAINDROP_FIELDS, BIOME_DTYPE, DeviceReference, Oracle, Reference,  # noqa: E402
                           splat_rule_tables)

KAT_TEXTURE = np.array([
    2, 0, 2, 0, 1, 1, 0, 3, 3, 2, 1, 2,
    0, 1, 2, 1, 1, 1, 3, 2, 2, 0, 0, 1,
    0, 1, 0, 2, 1, 3, 1, 1, 1, 2, 1, 0,
    3, 3, 0, 1, 1, 2, 2, 2, 2, 0, 0, 3,
    3, 2, 3, 3, 0, 3, 2, 2, 1, 0, 0, 3,
    2, 0, 0, 1, 2, 0, 2, 2, 0, 2, 0, 3,
    1, 2, 3, 0, 3, 2, 1, 2, 2, 3, 0, 2,
    1, 1, 0, 3, 0, 2, 1, 0, 3, 2, 2, 1,
    2, 2, 0, 1, 0, 2, 0, 0, 0, 0, 1, 1,
    0, 1, 3, 3, 0, 3, 3, 3, 1, 0, 1, 1,
    3, 1, 3, 0, 2, 1, 1, 0, 2, 2, 2, 0,
    2, 0, 1, 1, 2, 3, 1, 2, 3, 2, 0, 1], np.uint16)

# (kind, map_x, map_y, nn_x, nn_y, radius, id_range or (cell, biomes), seed)
SMALL_CASES = [
    ("random", 4, 4, 3, 3, 2, 4, 1),
    ("random", 16, 12, 3, 3, 4, 6, 2),
    ("random", 23, 17, 3, 3, 8, 15, 3),
    ("random", 32, 32, 3, 3, 16, 15, 4),
    ("random", 20, 20, 5, 3, 20, 3, 5),
    ("random", 8, 8, 3, 3, 8, 2, 6),
    ("random", 40, 9, 3, 3, 6, 300, 7),
    ("constant", 16, 16, 3, 3, 6, 1, 8),
    ("voronoi", 64, 64, 3, 3, 16, (32, 4), 9),
    ("voronoi", 48, 40, 3, 3, 12, (20, 8), 10),
]

LARGE_CASES = [
    ("voronoi", 256, 256, 3, 3, 16, (128, 4), 42),
    ("voronoi", 512, 512, 3, 3, 32, (256, 8), 7),
    ("random", 128, 128, 3, 3, 32, 15, 11),
]

PERM_CASES = [(6666, 10, float(np.radians(6.5))), (42, 8, 0.2181661565), (183457092, 12, 1.0), (0, 1, 0.0),
              (2**63 + 12345, 16, 6.0)]


# (seed, width, height, offset_x, offset_z, (ocean, plains, desert, forest))
LAYER_CASES = [
    (42, 256, 256, 0, 0, (0, 1, 2, 3)),
    (7, 300, 200, -5000, 3000, (0, 1, 2, 3)),
    (2**63 + 12345, 128, 512, -70000, -90000, (0, 1, 2, 3)),
    (123, 77, 333, -3, -7, (0, 1, 2, 3)),
    (11, 1024, 1024, -512, -512, (0, 1, 2, 3)),
    (99, 640, 480, 2048, -4096, (4, 7, 0, 4)),
    (5, 600, 600, -100000, 100, (1, 0, 2, 1)),
    (0, 512, 512, 1000000, -2000000, (0, 1, 2, 3)),
    (3, 700, 700, -300, -300, (5, 2, 9, 1)),
]
LAYER_LARGE_CASES = [
    (7, 2048, 2048, -1024, -1024, (0, 1, 2, 3)),
    (2024, 1536, 1536, -768, 4096, (0, 1, 2, 3)),
]


def layer_digest(out):
    return hashlib.sha256(np.ascontiguousarray(out, np.uint16).tobytes()).hexdigest()


def make_layers(ref):
    out = {}
    for i, (seed, w, h, ox, oz, ids) in enumerate(LAYER_CASES):
        m = ref.layer_biomemap(seed, w, h, (ox, oz), *ids)
        out[f"l{i}_meta"] = np.array([w, h, ox, oz], np.int64)
        out[f"l{i}_seed"] = np.array(seed, np.uint64)
        out[f"l{i}_ids"] = np.array(ids, np.uint16)
        out[f"l{i}_map"] = m
    out["count"] = np.array(len(LAYER_CASES))
    rng = np.random.default_rng(2024)
    kat = []
    for _ in range(64):
        s = int(rng.integers(0, 2**64, dtype=np.uint64))
        fac = int(rng.integers(-2**63, 2**63 - 1))
        salt = int(rng.integers(0, 2**63))
        x, z = (int(v) for v in rng.integers(-2**31, 2**31 - 1, 2))
        kat.append((s, fac, salt, x, z, ref.mix_seed(s, fac), ref.layer_seed(s, salt), ref.local_seed(s, salt, x, z)))
    out["seed_kat"] = np.array([[k[0], k[1] & (2**64 - 1), k[2], k[3] & (2**64 - 1), k[4] & (2**64 - 1), k[5], k[6],
                                 k[7]] for k in kat], np.uint64)
    np.savez_compressed(os.path.join(HERE, "layer_biomemap.npz"), **out)
    digests = []
    for seed, w, h, ox, oz, ids in LAYER_LARGE_CASES:
        m = ref.layer_biomemap(seed, w, h, (ox, oz), *ids)
        values, counts = np.unique(m, return_counts=True)
        digests.append({"seed": seed, "size": [w, h], "offset": [ox, oz], "ids": list(ids), "sha256": layer_digest(m),
                        "histogram": {int(v): int(c) for v, c in zip(values, counts)}})
    with open(os.path.join(HERE, "layer_digests.json"), "w") as f:
        json.dump(digests, f, indent=1)


def make_samplemap(kind, mx, my, nx, ny, param, seed, oracle):
    w, h = mx * nx, my * ny
    if kind == "random":
        return np.random.default_rng(seed).integers(0, param, (h, w)).astype(np.uint16)
    if kind == "constant":
        return np.full((h, w), seed % 7, np.uint16)
    cell, biomes = param
    return oracle.voronoi(w, h, (-mx * (nx // 2), -my * (ny // 2)), cell, biomes, seed)


def digest(offsets, bins):
    m = hashlib.sha256()
    m.update(np.ascontiguousarray(offsets, np.uint32).tobytes())
    m.update(np.ascontiguousarray(bins["Item"], np.uint16).tobytes())
    m.update(np.ascontiguousarray(bins["Weight"], np.float32).tobytes())
    return m.hexdigest()


# (seed, distribution, offset) of the permutation tables the noise fixtures use
DEVICE_PERMS = [(42, 8, 0.2181661565), (6666, 16, 0.0), (2**63 + 5, 32, 6.0)]
# fractal parameter sets: persistence, lacunarity, octaves, scale, offset, half dimension
FRACTAL_SETS = [(0.5, 2.0, 8, 300.0, (0.0, 0.0), (256.0, 256.0)),
                (0.4, 2.5, 6, 123.5, (12.5, -40.25), (64.0, 32.0)),
                (0.7, 1.88, 3, 91.5, (-5120.0, 9216.0), (512.0, 512.0)),
                (0.25, 3.1, 10, 2048.0, (1.0e5, -3.3e4), (16.0, 16.0)),
                (0.6, 2.2, 1, 17.0, (0.5, 0.5), (0.0, 0.0))]
# two-biome generator cases: map size, neighbourhood, filter radius, cell size, seed, map offset
MULTIBIOME_CASES = [((32, 32), (3, 3), 8, (20, 17), 1, (512.25, -96.5)),
                    ((48, 40), (3, 3), 16, (13, 29), 2, (-7168.0, 2048.0)),
                    ((16, 24), (3, 3), 2, (5, 3), 3, (0.0, 0.0))]
TWO_BIOMES = [(160.0, 8, 0.4, 2.5, 0.2, 0.1), (330.0, 6, 0.5, 2.0, 0.0, 0.6)]
# the demo's splat rules (SuperDemo+/Script/STPBiomeSplatRule.tdl): (sample, upper bound, region) and
# (sample, min gradient, max gradient, lower bound, upper bound, region)
DEMO_ALTITUDE = [(0, 1.0, 4), (1, 0.5, 3), (1, 0.72, 2), (1, 1.0, 1)]
DEMO_GRADIENT = [(0, 0.0, 0.2, 0.0, 0.27, 3), (1, 0.4, 0.65, 0.58, 0.8, 5), (1, 0.625, 1.0, 0.65, 1.0, 0)]


def splat_random_rules(rng, samples):
    alt, gra = [], []
    for smp in samples:
        for ub in sorted(rng.uniform(0.1, 1.0, int(rng.integers(1, 4)))):
            alt.append((smp, float(ub), int(rng.integers(0, 8))))
        for _ in range(int(rng.integers(0, 3))):
            g0, g1 = sorted(rng.uniform(0, 1, 2))
            a0, a1 = sorted(rng.uniform(0, 1, 2))
            gra.append((smp, float(g0), float(g1), float(a0), float(a1), int(rng.integers(0, 8))))
    return alt, gra


# droplet cases: merged map side, brush radius, droplets, lifetime, inertia, seed
EROSION_CASES = [(96, 3, 3000, 30, 0.05, 7), (96, 5, 1500, 64, 0.3, 8), (72, 2, 4000, 20, 0.0, 9)]


def raindrop_setting(count, radius, lifetime, inertia):
    """The small workload's droplet setting; the lifetime is set through minWaterVolume."""
    evap = np.float32(0.01)
    v = np.float32(1.0)
    for _ in range(lifetime):
        v = np.float32(v * np.float32(np.float32(1.0) - evap))
    d = dict(Seed=42, RainDropCount=count, Inertia=inertia, SedimentCapacityFactor=4.0, minSedimentCapacity=0.01,
             initWaterVolume=1.0, minWaterVolume=float(np.nextafter(v, np.float32(np.inf))), Friction=0.1,
             initSpeed=1.0, ErodeSpeed=0.3, DepositSpeed=0.3, EvaporateSpeed=float(evap), Gravity=4.0,
             ErosionBrushRadius=radius)
    return d


def erosion_input(n, seed):
    """A smooth seeded relief with fine noise, in [0.1, 0.95], rounded to float16 values so that the
    stored input is half the size."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:n, 0:n].astype(np.float64)
    h = 0.5 + 0.3 * np.sin(x / 9.0 + seed) * np.cos(y / 7.0) + 0.1 * np.sin((x + 2 * y) / 23.0) \
        + 0.05 * rng.random((n, n))
    return h.astype(np.float16)


def two_id_samplemap(total, cell, seed):
    """Checkerboard of two biome IDs with cell sides `cell`, shifted by the seed."""
    y, x = np.mgrid[0:total[1], 0:total[0]]
    return np.where(((x + 3 * seed) // cell[0] + (y + 5 * seed) // cell[1]) % 2 == 0, 0, 1).astype(np.uint16)


def float_digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def make_device(orc):
    dev = DeviceReference()
    out = {}
    rng = np.random.default_rng(2024)
    for t, (seed, n, off) in enumerate(DEVICE_PERMS):
        rc, perm, grad = orc.permutation(seed, n, off)
        assert rc == 0
        out[f"t{t}_perm"], out[f"t{t}_grad"] = perm, grad
        # large, negative, near-integer and zero coordinates
        pts = np.concatenate([rng.uniform(-1e4, 1e4, (1024, 2)), rng.uniform(-8, 8, (1024, 2)),
                              np.round(rng.uniform(-300, 300, (256, 2))) + rng.choice([0.0, 1e-4, -1e-4], (256, 2)),
                              np.zeros((1, 2))]).astype(np.float32)
        out[f"t{t}_simplex_xy"] = pts
        out[f"t{t}_simplex"] = np.array([dev.simplex2d(perm, grad, x, y) for x, y in pts], np.float32)
        fpts = rng.uniform(-2000, 2000, (256, 2)).astype(np.float32)
        out[f"t{t}_fractal_xy"] = fpts
        out[f"t{t}_fractal"] = np.array([[dev.fractal(perm, grad, x, y, *fs) for x, y in fpts]
                                         for fs in FRACTAL_SETS], np.float32)
    out["fractal_sets"] = np.array([(p, l, o, sc, ox, oy, hx, hy) for p, l, o, sc, (ox, oy), (hx, hy)
                                    in FRACTAL_SETS], np.float64)
    table = np.array(TWO_BIOMES, BIOME_DTYPE)
    out["two_biomes"] = table
    rc, perm, grad = orc.permutation(*DEVICE_PERMS[0])
    for i, (ms, nn, r, cell, seed, off) in enumerate(MULTIBIOME_CASES):
        sm = two_id_samplemap((ms[0] * nn[0], ms[1] * nn[1]), cell, seed)
        rc, offsets, bins = orc.shf(sm, ms, nn, r)
        assert rc == 0
        out[f"m{i}_samplemap"] = sm
        out[f"m{i}_meta"] = np.array([*ms, *nn, r], np.int64)
        out[f"m{i}_offset"] = np.array(off, np.float32)
        out[f"m{i}_height"] = dev.multibiome(offsets, bins, table, perm, grad, ms, off)
    out["multibiome_count"] = np.array(len(MULTIBIOME_CASES))
    for i, (n, radius, count, lifetime, inertia, seed) in enumerate(EROSION_CASES):
        s = raindrop_setting(count, radius, lifetime, inertia)
        h = erosion_input(n, seed)
        # starts in the central chunk of a 3x3 neighbourhood, as the reference spawns them (the
        # oracle's Philox stream, pinned by its known answers, regenerates them from the seed)
        starts = orc.droplet_starts(count, seed, 0, (n // 3, n // 3), (3, 3))
        idx, w = dev.brush(n, radius)
        out[f"e{i}_setting"] = np.array([s[k] for k, _ in RAINDROP_FIELDS], np.float64)
        out[f"e{i}_meta"] = np.array([n, radius, count, lifetime, seed], np.int64)
        out[f"e{i}_input"] = h
        out[f"e{i}_output"] = dev.erode(h.astype(np.float32), s, starts, idx, w)
    out["erosion_count"] = np.array(len(EROSION_CASES))
    # splatmaps of a 3x3 rendering buffer of 32^2 chunks: the demo's rules over all 9 chunks, then
    # random rules for samples 0-4 (sample 5 has none) over 4 chunks
    S = 32
    y, x = np.mgrid[0:3 * S, 0:3 * S]
    for i, seed in enumerate((11, 12)):
        srng = np.random.default_rng(seed)
        hm = ((0.5 + 0.4 * np.sin(x / srng.uniform(5, 15)) * np.cos(y / srng.uniform(5, 15))
               + 0.05 * srng.random(x.shape)) * 65535).clip(0, 65535).astype(np.uint16)
        if i == 0:
            bm = ((x // 37 + y // 29) % 3).astype(np.uint16)
            alt, gra = DEMO_ALTITUDE, DEMO_GRADIENT
            chunks = [(c % 3, c // 3, float(c * 512.0 - 2048.0), float(1024.0 - c * 256.0)) for c in range(9)]
        else:
            bm = ((x // 11 + 2 * (y // 17)) % 6).astype(np.uint16)
            alt, gra = splat_random_rules(srng, range(5))
            chunks = [(c % 3, c // 3, float(srng.uniform(-1e4, 1e4)), float(srng.uniform(-1e4, 1e4)))
                      for c in (0, 4, 5, 7)]
        d, reg, an, gn = splat_rule_tables(alt, gra)
        out[f"s{i}_biomemap"], out[f"s{i}_heightmap"] = bm, hm
        out[f"s{i}_chunks"] = np.array(chunks, np.float64)
        out[f"s{i}_altitude_rules"] = np.array(alt, np.float64).reshape(-1, 3)
        out[f"s{i}_gradient_rules"] = np.array(gra, np.float64).reshape(-1, 6)
        out[f"s{i}_regions"] = dev.splatmap(bm, hm, chunks, (S, S), alt, gra, perm, grad)
    out["splat_count"] = np.array(2)
    # production size, stored as SHA-256 digests of the float32 bits: a 512^2 chunk of the two-biome
    # script (filter radius 32 over its 3x3 neighbourhood), and 600,000 droplets (brush 5,
    # lifetime 50) on a 1536^2 merged map
    rc, perm, grad = orc.permutation(*DEVICE_PERMS[0])
    sm = two_id_samplemap((1536, 1536), (97, 131), 4)
    rc, offsets, bins = orc.shf(sm, (512, 512), (3, 3), 32)
    assert rc == 0
    hm = dev.multibiome(offsets, bins, table, perm, grad, (512, 512), (-1536.0, 2560.5))
    h = erosion_input(1536, 5).astype(np.float32)
    s = raindrop_setting(600000, 5, 50, 0.05)
    starts = orc.droplet_starts(600000, 5, 0, (512, 512), (3, 3))
    idx, w = dev.brush(1536, 5)
    eroded = dev.erode(h, s, starts, idx, w)
    with open(os.path.join(HERE, "device_digests.json"), "w") as f:
        json.dump({"multibiome_512": {"samplemap_cell": [97, 131], "samplemap_seed": 4, "radius": 32,
                                      "offset": [-1536.0, 2560.5], "sha256": float_digest(hm)},
                   "erosion_1536": {"input_seed": 5, "droplets": 600000, "brush": 5, "lifetime": 50,
                                    "inertia": 0.05, "start_seed": 5, "sha256": float_digest(eroded)}}, f, indent=1)
    brushes = []
    for dim_x in (300, 1000):
        for radius in range(1, 11):
            idx, w = dev.brush(dim_x, radius)
            brushes.append((dim_x, radius, idx, w))
    out["brush_meta"] = np.array([(d, r, len(i)) for d, r, i, _ in brushes], np.int64)
    out["brush_index"] = np.concatenate([i for _, _, i, _ in brushes])
    out["brush_weight"] = np.concatenate([w for _, _, _, w in brushes])
    vals = np.concatenate([rng.uniform(-0.5, 1.5, 2048),
                           np.arange(0, 65536, 97) / 65535.0 + rng.choice([0.0, 3e-8, -3e-8, 7.6e-6], 676),
                           [np.nan, np.inf, -np.inf, -0.0, 0.0, 1.0, 0.5 / 65535, 1.5 / 65535]]).astype(np.float32)
    out["format_input"] = vals
    out["format_output"] = dev.format(vals)
    np.savez_compressed(os.path.join(HERE, "device_reference.npz"), **out)


def main():
    orc = Oracle()
    if sys.argv[1:] == ["device"]:
        make_device(orc)
        print("device fixtures written to", HERE)
        return
    ref = Reference()
    make_layers(ref)
    if sys.argv[1:] == ["layers"]:
        print("layer fixtures written to", HERE)
        return
    rc, off, bins = ref.shf(KAT_TEXTURE, (4, 4), (3, 3), 2)
    assert rc == 0
    np.savez_compressed(os.path.join(HERE, "shf_kat.npz"), texture=KAT_TEXTURE, offsets=off,
                        items=bins["Item"], weights=bins["Weight"])

    out = {}
    for i, (kind, mx, my, nx, ny, r, param, seed) in enumerate(SMALL_CASES):
        sm = make_samplemap(kind, mx, my, nx, ny, param, seed, orc)
        rc, off, bins = ref.shf(sm, (mx, my), (nx, ny), r)
        assert rc == 0, (kind, mx, my, r, rc)
        rc2, off2, bins2 = ref.shf(sm, (mx, my), (nx, ny), r, parallel=True)
        assert rc2 == 0 and np.array_equal(off, off2) and np.array_equal(bins, bins2)
        out[f"c{i}_meta"] = np.array([mx, my, nx, ny, r, seed], np.int64)
        out[f"c{i}_kind"] = np.array(kind)
        out[f"c{i}_param"] = np.array(param if isinstance(param, tuple) else (param,), np.int64)
        if kind == "random":
            out[f"c{i}_input"] = sm  # stored: numpy's generator streams may change between versions
        out[f"c{i}_offsets"] = off
        out[f"c{i}_items"] = bins["Item"]
        out[f"c{i}_weights"] = bins["Weight"]
    out["count"] = np.array(len(SMALL_CASES))

    digests = []
    for j, (kind, mx, my, nx, ny, r, param, seed) in enumerate(LARGE_CASES):
        sm = make_samplemap(kind, mx, my, nx, ny, param, seed, orc)
        if kind == "random":
            out[f"large{j}_input"] = sm
        rc, off, bins = ref.shf(sm, (mx, my), (nx, ny), r, parallel=True)
        assert rc == 0
        digests.append({"kind": kind, "map": [mx, my], "nn": [nx, ny], "radius": r,
                        "param": list(param) if isinstance(param, tuple) else [param], "seed": seed,
                        "nbins": int(len(bins)), "sha256": digest(off, bins)})
    np.savez_compressed(os.path.join(HERE, "shf_cases.npz"), **out)
    with open(os.path.join(HERE, "shf_digests.json"), "w") as f:
        json.dump(digests, f, indent=1)

    perm = {}
    for i, (seed, n, offset) in enumerate(PERM_CASES):
        rc, p, g = ref.permutation(seed, n, offset)
        assert rc == 0
        perm[f"p{i}_setting"] = np.array([seed, n], np.uint64)
        perm[f"p{i}_offset"] = np.array(offset, np.float64)
        perm[f"p{i}_perm"] = p
        perm[f"p{i}_grad"] = g
    perm["count"] = np.array(len(PERM_CASES))
    np.savez_compressed(os.path.join(HERE, "permutation.npz"), **perm)
    make_device(orc)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
