"""The GPU against outputs of the reference's own device code (compiled as
host C++ and stored in tests/golden/device_reference.npz): the demo's
two-biome generator script within the noise tolerance, the format kernel bit
for bit."""
import os

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

NOISE_TOL = 2e-6


@pytest.fixture(scope="module")
def fix():
    return np.load(os.path.join(helpers.GOLDEN, "device_reference.npz"))


def test_multibiome_matches_reference_script_outputs(dev, oracle, fix):
    import torch
    perm, grad = np.array(fix["t0_perm"]), np.array(fix["t0_grad"])
    table = np.array(fix["two_biomes"])
    for i in range(int(fix["multibiome_count"])):
        mx, my, nx, ny, r = (int(v) for v in fix[f"m{i}_meta"])
        rc, off, bins = oracle.shf(fix[f"m{i}_samplemap"], (mx, my), (nx, ny), r)
        assert rc == 0
        offset = tuple(float(v) for v in fix[f"m{i}_offset"])
        out = torch.full((my, mx), float("nan"), device="cuda")
        dev.multibiome_heightmap(out, mx, torch.from_numpy(off.view(np.int32)).cuda(),
                                 torch.from_numpy(np.ascontiguousarray(bins).view(np.int64)).cuda(), (mx, my), offset,
                                 torch.from_numpy(perm).cuda(), torch.from_numpy(grad).cuda(),
                                 torch.from_numpy(table.view(np.float32)).cuda())
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        err = np.abs(got.astype(np.float64) - fix[f"m{i}_height"].astype(np.float64))
        assert err.max() <= NOISE_TOL, (i, err.max())


def test_format_matches_reference_kernel_outputs(dev, fix):
    import torch
    a = np.array(fix["format_input"], np.float32).reshape(2, -1)
    h, w = a.shape
    out = torch.empty((h, w), dtype=torch.int16, device="cuda")
    dev.format_heightmap(torch.from_numpy(a).cuda(), out, w, h)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint16).ravel(), fix["format_output"])
