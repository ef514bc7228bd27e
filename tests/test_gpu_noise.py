"""Multi-biome fractal simplex heightfield on the GPU against the FP32 CPU
oracle: |h_gpu - h_oracle| <= 2e-6 absolute (the stated noise tolerance)."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

NOISE_TOL = 2e-6


def noise_case(dev, oracle, stpgb, map_size, nbiomes, radius, seed, offset, cell):
    import torch
    mx, my = map_size
    sm = oracle.voronoi(3 * mx, 3 * my, (-mx, -my), cell, nbiomes, seed)
    rc, off, bins = oracle.shf(sm, map_size, (3, 3), radius)
    assert rc == 0
    perm, grad = stpgb.permutation_generate(seed, 8, 0.2181661565)
    table = helpers.biome_table(nbiomes, seed)
    ref = oracle.multibiome(off, bins, table, perm, grad, map_size, offset)
    d_off = torch.from_numpy(off.view(np.int32)).cuda()
    d_bins = torch.from_numpy(np.ascontiguousarray(bins).view(np.int64)).cuda()
    d_perm = torch.from_numpy(perm).cuda()
    d_grad = torch.from_numpy(grad).cuda()
    d_table = torch.from_numpy(table.view(np.float32)).cuda()
    out = torch.full((my, mx), float("nan"), device="cuda")
    dev.multibiome_heightmap(out, mx, d_off, d_bins, map_size, offset, d_perm, d_grad, d_table)
    torch.cuda.synchronize()
    return out.cpu().numpy(), ref


@pytest.mark.parametrize("map_size,nbiomes,radius,offset", [
    ((64, 64), 4, 16, (0.0, 0.0)),
    ((256, 256), 4, 16, (0.0, 0.0)),
    ((96, 80), 8, 20, (1234.0, -777.0)),
    ((128, 128), 16, 32, (-65536.0, 4096.0)),
])
def test_noise_vs_oracle(dev, oracle, stpgb, map_size, nbiomes, radius, offset):
    got, ref = noise_case(dev, oracle, stpgb, map_size, nbiomes, radius, 3, offset, max(map_size) // 2)
    err = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    assert np.isfinite(got).all()
    assert err.max() <= NOISE_TOL, f"max abs err {err.max():.3g} (tolerance {NOISE_TOL})"


def test_simplex_single_octave_grid(dev, oracle, stpgb):
    """One biome, one octave, weight 1: the heightmap is the normalised simplex itself at every pixel."""
    import torch
    mx = my = 64
    perm, grad = stpgb.permutation_generate(42, 8, 0.2181661565)
    table = np.zeros(1, stpgb.BIOME_DTYPE)
    table[0] = (7.5, 1, 0.5, 2.0, 0.0, 1.0)
    off = np.arange(mx * my + 1, dtype=np.uint32)
    bins = np.zeros(mx * my, stpgb.BIN_DTYPE)
    bins["Weight"] = 1.0
    ref = oracle.multibiome(off, bins, table, perm, grad, (mx, my), (3.0, -5.0))
    out = torch.zeros((my, mx), device="cuda")
    dev.multibiome_heightmap(out, mx, torch.from_numpy(off.view(np.int32)).cuda(),
                             torch.from_numpy(bins.view(np.int64)).cuda(), (mx, my), (3.0, -5.0),
                             torch.from_numpy(perm).cuda(), torch.from_numpy(grad).cuda(),
                             torch.from_numpy(table.view(np.float32)).cuda())
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy() - ref).max() <= NOISE_TOL
