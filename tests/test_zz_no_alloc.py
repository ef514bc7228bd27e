"""The allocation-free filter entry point (stpgb_shf_filter_noalloc).

It serves callers that may not allocate device memory themselves: a frame
loop where cudaFree would wait on the whole device, or an engine whose own
allocator owns its memory budget.  The entry point takes the filter's
scratch from a fixed array inside the library instead of a caller
workspace.  This file is collected last so that a run stopping at the first
failure has run every other test before it; it passes alone in a fresh
process as well.

Checks, through the C ABI: two calls in a row give output bit-identical to
stpgb_shf_filter with a caller workspace (the filter's tolerance is
exactness), also when consecutive calls lay the shared scratch out
differently; after the first call on the device, calls leave the device's
free memory unchanged; and a chunk whose scratch exceeds the array is
refused."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _outputs(info, cap):
    import torch
    npix = info.MapSize[0] * info.MapSize[1]
    return (torch.full((npix + 1,), -1, dtype=torch.int32, device="cuda"),
            torch.full((cap,), -1, dtype=torch.int64, device="cuda"), torch.full((1,), -1, dtype=torch.int32, device="cuda"))


def _filter(m, t, info, radius, max_items, cap, noalloc, outputs=None):
    import torch
    offsets, bins, status = outputs if outputs is not None else _outputs(info, cap)
    if outputs is not None:
        offsets.fill_(-1)
        bins.fill_(-1)
        status.fill_(-1)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = m.lib()
    if noalloc:
        rc = L.stpgb_shf_filter_noalloc(C.c_void_p(t.data_ptr()), C.byref(info), radius, max_items,
                                        C.c_void_p(offsets.data_ptr()), C.c_void_p(bins.data_ptr()), cap,
                                        C.c_void_p(status.data_ptr()), stream)
        m.check(rc)
    else:
        ws = C.c_size_t(0)
        m.check(L.stpgb_shf_workspace_size(C.byref(info), radius, max_items, C.byref(ws)))
        work = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
        m.check(L.stpgb_shf_filter(C.c_void_p(t.data_ptr()), C.byref(info), radius, max_items,
                                   C.c_void_p(work.data_ptr()), ws.value, C.c_void_p(offsets.data_ptr()),
                                   C.c_void_p(bins.data_ptr()), cap, C.c_void_p(status.data_ptr()), stream))
    m.check(L.stpgb_status_check(C.c_void_p(status.data_ptr()), stream))
    off = offsets.cpu().numpy().view(np.uint32)
    return off, bins[: int(off[-1])].cpu().numpy().view(np.uint64)


def test_noalloc_filter_matches_workspace_filter_twice():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import superterrainplus_gb300 as m
    S, radius, nb = 512, 32, 8
    info = m.NNInfo.make((S, S), (3, 3))
    # seeded Voronoi biome map over the 3x3 neighbourhood, made by the library on the device
    t = torch.empty((3 * S, 3 * S), dtype=torch.int16, device="cuda")
    m.DeviceOps().voronoi_biomemap(t, 3 * S, 3 * S, 3 * S, (-S, -S), 192, nb, 7)
    cap = S * S * nb
    ref_off, ref_bins = _filter(m, t, info, radius, nb, cap, noalloc=False)
    assert ref_off[-1] > S * S
    for _ in range(2):
        off, bins = _filter(m, t, info, radius, nb, cap, noalloc=True)
        assert np.array_equal(off, ref_off)
        assert np.array_equal(bins & 0xFFFFFFFF0000FFFF, ref_bins & 0xFFFFFFFF0000FFFF)
    # a second, smaller chunk through the same shared scratch, then the first again
    small = m.NNInfo.make((40, 24), (3, 3))
    ts = torch.randint(0, 5, (72, 120), dtype=torch.int16, device="cuda")
    s_ref = _filter(m, ts, small, 6, 5, 40 * 24 * 5, noalloc=False)
    s_got = _filter(m, ts, small, 6, 5, 40 * 24 * 5, noalloc=True)
    assert np.array_equal(s_ref[0], s_got[0]) and np.array_equal(s_ref[1], s_got[1])
    off, bins = _filter(m, t, info, radius, nb, cap, noalloc=True)
    assert np.array_equal(off, ref_off) and np.array_equal(bins, ref_bins)


def test_noalloc_filter_refuses_oversized_scratch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import superterrainplus_gb300 as m
    info = m.NNInfo.make((1024, 1024), (3, 3))
    t = torch.zeros((3072, 3072), dtype=torch.int16, device="cuda")
    with pytest.raises(m.STPCapacityError):
        _filter(m, t, info, 32, 64, 1024 * 1024, noalloc=True)


def test_noalloc_filter_allocates_nothing_and_follows_a_changed_layout():
    """Consecutive calls on the same 3x3 x 512^2 map with max_items 8, then 13, then 8 move the
    sub-arrays inside the shared scratch (their offsets grow with max_items); every call must still
    equal the workspace path bit for bit, so no call may read an entry an earlier call left behind.
    Once the first call on the device has looked up the array's address, two further calls leave
    the device's free memory (cudaMemGetInfo) exactly where it was."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import superterrainplus_gb300 as m
    S, radius, nb = 512, 32, 8
    info = m.NNInfo.make((S, S), (3, 3))
    t = torch.empty((3 * S, 3 * S), dtype=torch.int16, device="cuda")
    m.DeviceOps().voronoi_biomemap(t, 3 * S, 3 * S, 3 * S, (-S, -S), 192, nb, 11)
    cap = S * S * nb
    want = {k: _filter(m, t, info, radius, k, cap, noalloc=False) for k in (8, 13)}
    outs = _outputs(info, cap)
    for k in (8, 13, 8):
        off, bins = _filter(m, t, info, radius, k, cap, noalloc=True, outputs=outs)
        assert np.array_equal(off, want[k][0]) and np.array_equal(bins, want[k][1]), f"max_items {k}"
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for k in (13, 8):
        off, bins = _filter(m, t, info, radius, k, cap, noalloc=True, outputs=outs)
        assert np.array_equal(off, want[k][0]) and np.array_equal(bins, want[k][1])
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
