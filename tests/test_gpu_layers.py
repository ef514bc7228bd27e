"""Biome layer chain on the GPU: bit-exact against the reference's own layer
chain (golden fixtures and digests made from the compiled reference) and
against the oracle on other chains, tile edges, pitches and offsets."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

from helpers import GOLDEN
from test_layers import DEMO_CHAIN, demo_ids, layer_fixture

pytestmark = pytest.mark.gpu


def ids_struct(stpgb, ids):
    s = stpgb.LayerBiomes()
    s.Ocean, s.Plains, s.Forest = (int(v) for v in ids[:3])
    s.ShallowOcean[:] = [int(v) for v in ids[3:]]
    return s


def gpu_map(dev, stpgb, chain, ids, seed, w, h, offset, pitch=None):
    import torch
    pitch = pitch or w
    out = torch.full((h, pitch), 0xBEEF, dtype=torch.int32, device="cuda").to(torch.int16)
    dev.layer_biomemap(chain, ids_struct(stpgb, ids), seed, out, pitch, w, h, offset)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint16)


def test_demo_chain_matches_reference_fixtures(dev, stpgb):
    f = layer_fixture()
    for i in range(int(f["count"])):
        w, h, ox, oz = (int(v) for v in f[f"l{i}_meta"])
        ocean, plains, _desert, forest = (int(v) for v in f[f"l{i}_ids"])
        got = gpu_map(dev, stpgb, DEMO_CHAIN, demo_ids(ocean, plains, forest), int(f[f"l{i}_seed"]), w, h, (ox, oz))
        np.testing.assert_array_equal(got, f[f"l{i}_map"], err_msg=f"case {i}")


def test_demo_chain_matches_reference_digests(dev, stpgb):
    with open(os.path.join(GOLDEN, "layer_digests.json")) as fh:
        cases = json.load(fh)
    for c in cases:
        ocean, plains, _desert, forest = c["ids"]
        got = gpu_map(dev, stpgb, DEMO_CHAIN, demo_ids(ocean, plains, forest), c["seed"], *c["size"], c["offset"])
        assert hashlib.sha256(np.ascontiguousarray(got).tobytes()).hexdigest() == c["sha256"]


# Chains that exercise every layer kind at full resolution, fuzzy scales,
# consecutive Voronoi zooms and land growth after zooms; IDs where forest
# and plains are shallow oceans too.
OTHER_CHAINS = [
    [(1, 0, 5), (5, 0, 1), (5, 0, 2)],
    [(1, 0, 9), (2, 1, 3), (2, 1, 4), (3, 0, 7), (4, 0, 8), (3, 0, 11)],
    [(1, 0, 1), (2, 0, 2), (3, 0, 3), (2, 0, 4), (3, 0, 5), (4, 0, 6), (5, 0, 7)],
    [(1, 0, 77)],
    [(1, 0, 3), (4, 0, 1), (4, 0, 2), (4, 0, 3), (2, 0, 5), (5, 0, 6), (3, 0, 8), (3, 0, 9)],
]
OTHER_IDS = [demo_ids(), np.array([2, 5, 7, 2, 7, 0, 0, 0], np.uint16), np.array([0, 1, 1, 0, 1, 9, 9, 9], np.uint16)]


@pytest.mark.parametrize("ci", range(len(OTHER_CHAINS)))
def test_other_chains_match_oracle(dev, stpgb, oracle, ci):
    chain = OTHER_CHAINS[ci]
    for k, ids in enumerate(OTHER_IDS):
        seed = 1000 * ci + k
        for w, h, off in [(131, 97, (-65, 33)), (64, 64, (0, 0)), (1, 1, (5, -5)), (300, 7, (-1000, 999))]:
            want = oracle.layer_biomemap(chain, ids, seed, w, h, off)
            got = gpu_map(dev, stpgb, chain, ids, seed, w, h, off)
            np.testing.assert_array_equal(got, want, err_msg=f"chain {ci} ids {k} size {w}x{h} offset {off}")


def test_pitch_leaves_padding_untouched(dev, stpgb, oracle):
    w, h, pitch = 200, 150, 256
    got = gpu_map(dev, stpgb, DEMO_CHAIN, demo_ids(), 17, w, h, (-100, 40), pitch=pitch)
    np.testing.assert_array_equal(got[:, :w], oracle.layer_biomemap(DEMO_CHAIN, demo_ids(), 17, w, h, (-100, 40)))
    assert np.all(got[:, w:] == 0xBEEF)


def test_tile_sizes_agree(dev, stpgb, oracle):
    """Requests of 2560^2, 1536^2, 700x600 and 37x29 pixels take 128, 64, 32
    and 16 pixel tiles; a crop of a large map equals a small map of the crop."""
    big = gpu_map(dev, stpgb, DEMO_CHAIN, demo_ids(), 2024, 2560, 2560, (-1280, -1280))
    large = gpu_map(dev, stpgb, DEMO_CHAIN, demo_ids(), 2024, 1536, 1536, (-1280 + 512, -1280 + 1000))
    np.testing.assert_array_equal(large, big[1000:2536, 512:2048])
    mid = gpu_map(dev, stpgb, DEMO_CHAIN, demo_ids(), 2024, 700, 600, (-1280 + 900, -1280 + 1300))
    small = gpu_map(dev, stpgb, DEMO_CHAIN, demo_ids(), 2024, 37, 29, (-1280 + 1999, -1280 + 7))
    np.testing.assert_array_equal(mid, big[1300:1900, 900:1600])
    np.testing.assert_array_equal(small, big[7:36, 1999:2036])
    np.testing.assert_array_equal(small, oracle.layer_biomemap(DEMO_CHAIN, demo_ids(), 2024, 37, 29,
                                                                (-1280 + 1999, -1280 + 7)))


def test_host_factory_matches_reference_fixture(stpgb):
    f = layer_fixture()
    w, h, ox, oz = (int(v) for v in f["l0_meta"])
    factory = stpgb.STPLayerChainBuilder((w, h), int(f["l0_seed"]))
    out = np.zeros(w * h, np.uint16)
    factory(out, (ox, oz))
    np.testing.assert_array_equal(out.reshape(h, w), f["l0_map"])
    again = np.zeros_like(out)
    factory(again, (ox, oz))
    np.testing.assert_array_equal(out, again)
