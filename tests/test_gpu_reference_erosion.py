"""The reference's own erosion kernel built for sm_103a (oracle/_ref/libstpref_gpu.so), the build
whose run-to-run spread is the erosion tolerance of the RMS parity tests: its harness spawns exactly
the droplets the library's kernels are fed, and with droplets that never meet it follows the serial
algorithm."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def reference_gpu():
    ref = helpers._reference_gpu()
    if ref is None:
        pytest.skip("reference GPU build absent")
    return ref


def run_reference(ref, oracle, h, map_size, nn, s, draws):
    import torch
    count = len(draws) // 2
    idx, w = oracle.brush(h.shape[1], s["ErosionBrushRadius"])
    d_idx, d_w = torch.from_numpy(idx).cuda(), torch.from_numpy(w).cuda()
    u = torch.from_numpy(np.ascontiguousarray(draws, np.float32)).cuda()
    d = torch.from_numpy(np.ascontiguousarray(h, np.float32).copy()).cuda()
    torch.cuda.synchronize()
    ref.erode(d.data_ptr(), map_size, nn, s, u.data_ptr(), count, d_idx.data_ptr(), d_w.data_ptr(), len(idx))
    return d.cpu().numpy()


@pytest.mark.parametrize("brush", [3, 5])
def test_reference_build_with_sparse_droplets_follows_serial_oracle(reference_gpu, oracle, brush):
    """A 3x3 neighbourhood of 1024^2 chunks and a 12x12 grid of droplets 80 px apart in the centre
    chunk (30 steps and brush reach below 5 keep their paths apart), spawned by the reference kernel's
    own spawn from draws chosen to land on the grid: the kernel acts as the serial algorithm.  Each
    droplet's 80^2 tile is compared with the FP32 serial oracle (the reference's arithmetic without
    contracted multiply-adds); the kernel may differ from it on no more tiles than the FP32 and FP64
    oracles differ from each other.  (144 droplets fill one block with more live droplets than brush
    points: the reference kernel needs that, test_reference_brush_needs_live_droplets.)"""
    S = 1024
    n = 12
    rng = np.random.default_rng(brush)
    y, x = np.mgrid[0:3 * S, 0:3 * S]
    h = (0.5 + 0.3 * np.sin(x / 31.0) * np.cos(y / 23.0) + 0.01 * rng.random((3 * S, 3 * S))).astype(np.float32)
    g = S + 16 + 80 * np.arange(n, dtype=np.float32) + np.float32(40.375)
    xs, ys = np.meshgrid(g, g)
    starts = np.stack([xs.ravel(), ys.ravel()], 1).ravel().astype(np.float32)
    draws, exact = helpers.spawn_draws(starts, (S, S), (3, 3))
    assert exact == 1.0
    s = helpers.raindrop_dict(len(starts) // 2, radius=brush, lifetime=30, seed=1)
    out = run_reference(reference_gpu, oracle, h, (S, S), (3, 3), s, draws)
    idx, w = oracle.brush(3 * S, brush)
    ref32, _, _ = oracle.erode(h, s, starts, idx, w, fp64=False)
    ref64, _, _ = oracle.erode(h, s, starts, idx, w, fp64=True)
    assert not np.array_equal(out, h)
    tol = 1e-5 * float(h.max() - h.min())
    lo = S + 16

    def diverged(a, b):
        d = np.abs(a.astype(np.float64) - b.astype(np.float64))[lo:lo + 80 * n, lo:lo + 80 * n]
        return d.reshape(n, 80, n, 80).max(axis=(1, 3)) > tol

    ref_vs_f32, f32_vs_f64 = diverged(out, ref32), diverged(ref32, ref64)
    print(f"brush {brush}: tiles off the FP32 oracle {int(ref_vs_f32.sum())}, FP32 vs FP64 oracle "
          f"{int(f32_vs_f64.sum())} of {n * n}")
    assert ref_vs_f32.sum() <= max(2, f32_vs_f64.sum())
    # outside the droplets' tiles nothing changes
    outside = np.ones_like(h, bool)
    outside[lo:lo + 80 * n, lo:lo + 80 * n] = False
    assert np.array_equal(out[outside], h[outside])


def test_reference_build_runs_stay_finite_and_close(reference_gpu, oracle):
    """Five runs of the small plain-method density (3x3 x 96^2, 20,000 droplets, brush 3, lifetime
    30) stay finite and differ from run to run only by the order of their float atomics (well below
    the heights' range)."""
    S = 96
    rng = np.random.default_rng(5)
    y, x = np.mgrid[0:3 * S, 0:3 * S]
    h = (0.5 + 0.25 * np.sin(x / 23.0) * np.cos(y / 17.0) + 0.02 * rng.random((3 * S, 3 * S))).astype(np.float32)
    s = helpers.raindrop_dict(20000, radius=3, lifetime=30, seed=9)
    draws, exact = helpers.droplet_uniforms(oracle, 20000, 9, 0, (S, S), (3, 3))
    assert exact == 1.0
    outs = [run_reference(reference_gpu, oracle, h, (S, S), (3, 3), s, draws) for _ in range(5)]
    for o in outs:
        assert np.isfinite(o).all()
    spread = max(float(np.sqrt(np.mean((a.astype(np.float64) - b) ** 2))) for i, a in enumerate(outs)
                 for b in outs[i + 1:])
    assert spread < 0.01 * float(h.max() - h.min())


def test_reference_brush_needs_live_droplets(reference_gpu):
    """The reference kernel copies the erosion brush into shared memory with the block's droplet
    threads only (STPRainDrop.cu:63-71); threads past RainDropCount return before that
    (STPHeightfieldKernel.cu:86-88).  A block with fewer live droplets than brush points therefore
    erodes with brush entries nobody wrote.  Every tolerance case is sized so that the last block
    holds no droplets or at least a brush's worth (reference_band checks this for each case); this
    records the launch shape that rule is evaluated on."""
    for points in (9, 29, 45, 69):
        block = reference_gpu.block_size(points)
        assert block >= 69 and block % 32 == 0
