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

`python tests/golden/make_golden.py layers` rewrites only the layer fixtures.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, Reference  # noqa: E402

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


def main():
    orc, ref = Oracle(), Reference()
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
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
