"""The roofline measurement kernels behind the bench's L2 and FP32 denominators: every random
reduction and returning atomic lands (the map's sum counts them exactly), the loads leave the map
and the sink alone, the chase walks its whole cycle and reports ticks."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,width", [(0, 1), (1, 4), (5, 4)], ids=["red", "red-v4", "atom-v4"])
def test_every_update_lands(stpgb, dev, kind, width):
    import torch
    lib = stpgb.lib()
    n, blocks, iters = 1 << 16, 8, 32
    buf = torch.zeros(n, dtype=torch.float32, device="cuda")
    sink = torch.zeros(4, dtype=torch.int64, device="cuda")
    stpgb.check(lib.stpgb_roofline_launch(kind, C.c_void_p(buf.data_ptr()), n, blocks, iters,
                                          C.c_void_p(sink.data_ptr()), None))
    torch.cuda.synchronize()
    counts = buf.cpu().numpy().astype(np.float64)
    assert counts.sum() == blocks * 256 * iters * width
    assert np.all(counts == np.round(counts))
    assert int(sink.abs().sum().item()) == 0


def test_loads_and_fma_write_nothing(stpgb, dev):
    import torch
    lib = stpgb.lib()
    n = 1 << 16
    buf = torch.zeros(n, dtype=torch.float32, device="cuda")
    sink = torch.zeros(4, dtype=torch.int64, device="cuda")
    for kind, elements, blocks, iters in ((2, n, 8, 32), (4, 1, 8, 64)):
        stpgb.check(lib.stpgb_roofline_launch(kind, C.c_void_p(buf.data_ptr()), elements, blocks, iters,
                                              C.c_void_p(sink.data_ptr()), None))
    torch.cuda.synchronize()
    assert int(torch.count_nonzero(buf).item()) == 0
    assert int(sink.abs().sum().item()) == 0


def test_chase_walks_the_cycle(stpgb, dev):
    import torch
    lib = stpgb.lib()
    n = 1 << 12
    perm = np.random.default_rng(3).permutation(n)
    nxt = np.empty(n, np.int32)
    nxt[perm] = np.roll(perm, -1)
    table = torch.from_numpy(nxt).cuda()
    sink = torch.zeros(4, dtype=torch.int64, device="cuda")
    stpgb.check(lib.stpgb_roofline_launch(3, C.c_void_p(table.data_ptr()), n, 1, n,
                                          C.c_void_p(sink.data_ptr()), None))
    torch.cuda.synchronize()
    ticks, last = (int(v) for v in sink[:2].cpu())
    assert ticks > 0
    j = 0
    for _ in range(n):
        j = int(nxt[j])
    assert last == j == 0
