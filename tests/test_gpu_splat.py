"""Splatmap on the GPU against the oracle restatement, whose texture model
reproduces the texture unit's filtering bit for bit.  The kernel, like the
reference's NVRTC build (default -fmad=true), fuses `tap * HeightFactor -
other tap` into one multiply-add, the oracle rounds both: at most half an
ulp of 875.5 (3e-5) per gradient component, which moves the slope factor
1 - 5.5 / |g| by at most 0.07 * 2 * 3e-5 < 1e-5.  Altitudes differ by the
noise tolerance (2e-6 * 0.15).  Regions are equal except where the oracle's
slope or altitude lies within 1e-5 of a rule boundary."""
import numpy as np
import pytest

from test_splat import DEMO_ALTITUDE, DEMO_GRADIENT

pytestmark = pytest.mark.gpu

S = 64
SIMPLEX = (42, 8, 0.2181661565)


def rendering_buffer(seed, nx=3, ny=3, samples=(0, 1, 2)):
    rng = np.random.default_rng(seed)
    W, H = nx * S, ny * S
    y, x = np.mgrid[0:H, 0:W]
    h = 0.45 + 0.3 * np.sin(x / (9.0 + seed)) * np.cos(y / 13.0) + 0.12 * np.sin((x + 2 * y) / 5.0)
    h += 0.02 * rng.random((H, W))
    hm = np.round(np.clip(h, 0, 1) * 65535).astype(np.uint16)
    cells = rng.integers(0, len(samples), (ny * 4, nx * 4))
    bm = np.asarray(samples, np.uint16)[cells[(y // 16), (x // 16)]]
    return bm, hm


def near_boundary(slope, alt, rules_alt, rules_gra, eps=1e-4):
    bounds_s = {v for r in rules_gra for v in r[1:3]}
    bounds_a = {r[1] for r in rules_alt} | {v for r in rules_gra for v in r[3:5]}
    return (np.min([np.abs(slope - b) for b in bounds_s], axis=0) < eps) | \
        (np.min([np.abs(alt - b) for b in bounds_a], axis=0) < eps)


def run_gpu(stpgb, bm, hm, chunks, alt_rules=DEMO_ALTITUDE, gra_rules=DEMO_GRADIENT):
    import torch
    H, W = hm.shape
    gen = stpgb.STPSplatmapGenerator(alt_rules, gra_rules, stpgb.SimplexSetting(*SIMPLEX), (S, S))
    b = torch.from_numpy(bm.view(np.int16)).cuda()
    h = torch.from_numpy(hm.view(np.int16)).cuda()
    out = torch.full((H, W), 0x77, dtype=torch.uint8, device="cuda")
    slope = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    alt = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    gen(b, h, W, out, W, W, H, chunks, slope, alt)
    torch.cuda.synchronize()
    return out.cpu().numpy(), slope.cpu().numpy(), alt.cpu().numpy()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_splatmap_matches_oracle(stpgb, oracle, dev, seed):
    bm, hm = rendering_buffer(seed)
    chunks = [(cx, cy, float((cx - 1) * S + 1000 * seed), float((cy - 1) * S - 700)) for cy in range(3)
              for cx in range(3)]
    got, gs, ga = run_gpu(stpgb, bm, hm, chunks)
    perm, grad = stpgb.permutation_generate(*SIMPLEX)
    want, ws, wa = oracle.splatmap(bm, hm, chunks, (S, S), DEMO_ALTITUDE, DEMO_GRADIENT, perm, grad)
    assert np.abs(gs - ws).max() <= 1e-5, np.abs(gs - ws).max()
    assert np.abs(ga - wa).max() <= 1e-6, np.abs(ga - wa).max()
    diff = got != want
    assert not np.any(diff & ~near_boundary(ws, wa, DEMO_ALTITUDE, DEMO_GRADIENT, eps=1e-5)), int(diff.sum())
    assert diff.mean() < 1e-4
    # every rule fires somewhere, and sample 2 (not in the dictionary, above it) has no region
    assert set(np.unique(got[bm < 2]).tolist()) >= {0, 1, 2, 3, 4, 5}
    assert np.all(got[bm == 2] == 255)


def test_only_requested_chunks_are_written(stpgb, dev):
    bm, hm = rendering_buffer(4)
    got, _, _ = run_gpu(stpgb, bm, hm, [(1, 1, 0.0, 0.0), (2, 0, 64.0, -64.0)])
    mask = np.zeros_like(got, bool)
    mask[S:2 * S, S:2 * S] = True
    mask[0:S, 2 * S:3 * S] = True
    assert np.all(got[~mask] == 0x77) and not np.any(got[mask] == 0x77)


def test_missing_sample_takes_the_next_registry(stpgb, oracle, dev):
    """STPTextureSplatRuleWrapper::findSplatRegistry returns the lower bound without checking the
    sample: with rules for samples 0 and 5, sample 3 uses sample 5's rules."""
    alt = [(0, 1.0, 4), (5, 1.0, 7)]
    gra = [(5, -1.0, 2.0, -1.0, 2.0, 6)]
    bm, hm = rendering_buffer(5, samples=(0, 3, 5))
    got, _, _ = run_gpu(stpgb, bm, hm, [(c % 3, c // 3, 0.0, 0.0) for c in range(9)], alt, gra)
    assert np.all(got[bm == 3] == 6) and np.all(got[bm == 5] == 6)
    perm, grad = stpgb.permutation_generate(*SIMPLEX)
    want, ws, wa = oracle.splatmap(bm, hm, [(c % 3, c // 3, 0.0, 0.0) for c in range(9)], (S, S), alt, gra, perm, grad)
    assert np.array_equal(got, want)


def test_misaligned_buffer_is_refused(stpgb, dev):
    import torch
    gen = stpgb.STPSplatmapGenerator(DEMO_ALTITUDE, DEMO_GRADIENT, stpgb.SimplexSetting(*SIMPLEX), (S, S))
    base = torch.zeros(3 * S * 3 * S + 8, dtype=torch.int16, device="cuda")
    out = torch.zeros((3 * S, 3 * S), dtype=torch.uint8, device="cuda")
    with pytest.raises(stpgb.STPNumericDomainError):
        gen(base[1:], base[1:], 3 * S, out, 3 * S, 3 * S, 3 * S, [(0, 0, 0.0, 0.0)])
    with pytest.raises(stpgb.STPNumericDomainError):
        gen(base, base, 3 * S, out, 3 * S, 3 * S, 3 * S, [(3, 0, 0.0, 0.0)])
