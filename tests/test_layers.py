"""Biome layer chain, CPU side: the oracle restatement against the reference's
own layer chain (golden fixtures from tests/golden/make_golden.py, and the
compiled reference itself where it exists), the STPLayer seed arithmetic,
the STPLayer/STPBiomeFactory properties the reference's
SuperTest+/SuperTerrain+/STPTest2DBiome.cpp checks, and the C ABI's
argument handling (no device work)."""
import ctypes as C
import hashlib
import json
import os
import platform

import numpy as np
import pytest

from helpers import GOLDEN

DEMO_CHAIN = [(1, 0, 23457829), (2, 1, 875944), (3, 0, 5748329), (2, 0, 8947358941), (3, 0, 361249673),
              (3, 0, 8769575), (3, 0, 43562783426564), (4, 0, 74368), (2, 0, 1), (2, 0, 2), (2, 0, 3),
              (5, 0, 4), (5, 0, 5), (5, 0, 6)]


def demo_ids(ocean=0, plains=1, forest=3):
    # the demo registry: the four shallow oceans it never loads keep ID 0
    return np.array([ocean, plains, forest, ocean, 0, 0, 0, 0], np.uint16)


def layer_fixture():
    return np.load(os.path.join(GOLDEN, "layer_biomemap.npz"))


def test_seed_arithmetic_known_answers(oracle):
    kat = layer_fixture()["seed_kat"]
    for s, fac, salt, x, z, mix, layer, local in kat.tolist():
        fac = fac - (1 << 64) if fac >= 1 << 63 else fac
        x = x - (1 << 64) if x >= 1 << 63 else x
        z = z - (1 << 64) if z >= 1 << 63 else z
        assert oracle.mix_seed(s, fac) == mix
        assert oracle.layer_seed(s, salt) == layer
        assert oracle.local_seed(s, salt, x, z) == local


def test_oracle_matches_reference_fixtures(oracle):
    f = layer_fixture()
    for i in range(int(f["count"])):
        w, h, ox, oz = (int(v) for v in f[f"l{i}_meta"])
        ocean, plains, _desert, forest = (int(v) for v in f[f"l{i}_ids"])
        got = oracle.layer_biomemap(DEMO_CHAIN, demo_ids(ocean, plains, forest), int(f[f"l{i}_seed"]), w, h, (ox, oz))
        np.testing.assert_array_equal(got, f[f"l{i}_map"], err_msg=f"case {i}")


def test_oracle_matches_reference_digests(oracle):
    with open(os.path.join(GOLDEN, "layer_digests.json")) as fh:
        cases = json.load(fh)
    for c in cases:
        ocean, plains, _desert, forest = c["ids"]
        got = oracle.layer_biomemap(DEMO_CHAIN, demo_ids(ocean, plains, forest), c["seed"], *c["size"], c["offset"])
        assert hashlib.sha256(got.tobytes()).hexdigest() == c["sha256"]


def test_oracle_matches_live_reference(oracle):
    from oracle.oracle import Reference
    try:
        ref = Reference()
    except (FileNotFoundError, OSError):
        pytest.skip("reference build not available on this host")
    rng = np.random.default_rng(77)
    for _ in range(6):
        seed = int(rng.integers(0, 2**64, dtype=np.uint64))
        w, h = (int(v) for v in rng.integers(1, 400, 2))
        ox, oz = (int(v) for v in rng.integers(-10**6, 10**6, 2))
        np.testing.assert_array_equal(oracle.layer_biomemap(DEMO_CHAIN, demo_ids(), seed, w, h, (ox, oz)),
                                      ref.layer_biomemap(seed, w, h, (ox, oz)))


def test_biome_factory_properties(oracle):
    """STPTest2DBiome.cpp: same input, same output; the factory's map is the
    layer sampled at offset + (x, z); different seeds give different maps."""
    a = oracle.layer_biomemap(DEMO_CHAIN, demo_ids(), 9, 96, 64, (-4000, 2500))
    b = oracle.layer_biomemap(DEMO_CHAIN, demo_ids(), 9, 96, 64, (-4000, 2500))
    np.testing.assert_array_equal(a, b)
    inner = oracle.layer_biomemap(DEMO_CHAIN, demo_ids(), 9, 40, 30, (-4000 + 17, 2500 + 11))
    np.testing.assert_array_equal(inner, a[11:41, 17:57])
    # the chain emits only the IDs it is given
    big = oracle.layer_biomemap(DEMO_CHAIN, demo_ids(6, 8, 9), 12345, 512, 512, (-256, -256))
    assert set(np.unique(big).tolist()) <= {6, 8, 9, 1}


def test_local_seed_is_deterministic_and_coordinate_dependent(oracle):
    s1 = oracle.local_seed(19657483, 48321567, 1234, -5678)
    assert s1 == oracle.local_seed(19657483, 48321567, 1234, -5678)
    assert s1 != oracle.local_seed(19657483, 48321567, -1234, 5678)
    assert oracle.mix_seed(123456789, 987654321) != 123456789


def test_demo_chain_and_ids_from_the_library(stpgb):
    chain, ids = stpgb.layer_chain_demo()
    assert [(c.Kind, c.Param, c.Salt) for c in chain] == DEMO_CHAIN
    assert (ids.Ocean, ids.Plains, ids.Forest, list(ids.ShallowOcean)) == (0, 1, 3, [0] * 5)
    n = C.c_uint32(0)
    small = (stpgb.Layer * 4)()
    assert stpgb.lib().stpgb_layer_chain_demo(small, 4, C.byref(n)) == 1 and n.value == 14


@pytest.mark.parametrize("chain, what", [
    ([], "count"),
    ([(2, 0, 1)], "first layer"),
    ([(1, 0, 1), (1, 0, 2)], "first layer"),
    ([(1, 0, 1), (9, 0, 2)], "unknown"),
    ([(1, 0, 1), (2, 5, 2)], "scale type"),
    ([(1, 0, 1), (5, 1, 2)], "2-D"),
    ([(1, 0, 1)] + [(3, 0, 2)] * 32, "count"),
])
def test_layer_chain_validation_without_gpu(stpgb, chain, what):
    _, ids = stpgb.layer_chain_demo()
    arr = (stpgb.Layer * max(len(chain), 1))(*[stpgb.Layer(*c) for c in chain])
    out = np.zeros(16, np.uint16)
    rc = stpgb.lib().stpgb_layer_biomemap(arr, len(chain), 1, C.byref(ids), out.ctypes.data, 4, 4, 4, 0, 0, None)
    assert rc == 1
    assert what in stpgb.lib().stpgb_last_error().decode()


def test_factory_rejects_bad_dimension_and_array(stpgb):
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.STPLayerChainBuilder((0, 4), 1)
    f = stpgb.STPLayerChainBuilder((4, 4), 1)
    with pytest.raises(stpgb.STPNumericDomainError):
        f(np.zeros(15, np.uint16), (0, 0))
    with pytest.raises(stpgb.STPNumericDomainError):
        f(np.zeros(16, np.int32), (0, 0))


def test_coordinate_range_is_checked_without_gpu(stpgb):
    chain, ids = stpgb.layer_chain_demo()
    out = np.zeros(16, np.uint16)
    rc = stpgb.lib().stpgb_layer_biomemap(chain, len(chain), 1, C.byref(ids), out.ctypes.data, 4, 4, 4, 2**30 - 2,
                                          0, None)
    assert rc == 1 and "2^30" in stpgb.lib().stpgb_last_error().decode()


@pytest.mark.skipif(platform.machine() != "x86_64", reason="the compiled reference is an x86 build")
def test_reference_chain_is_linear_in_the_factory_offset():
    """STPBiomeFactory samples world pixels: a shifted request is a shifted crop."""
    from oracle.oracle import Reference
    try:
        ref = Reference()
    except (FileNotFoundError, OSError):
        pytest.skip("reference build not available")
    a = ref.layer_biomemap(31, 128, 128, (-64, -64))
    b = ref.layer_biomemap(31, 64, 64, (0, 0))
    np.testing.assert_array_equal(a[64:, 64:], b)
