"""Argument checks of the batched pipeline, the server and the kernel-level
calls, each of which refuses a bad argument before any device work: these
run without a GPU and map onto the reference's exception types."""
import ctypes as C

import numpy as np
import pytest

import helpers


def base_setting(stpgb, **over):
    d = helpers.raindrop_dict(1000, radius=3, lifetime=30)
    d.update(over)
    return stpgb.RaindropSetting(**d)


def request(**over):
    r = dict(MapSize=64, ChunkX=0, ChunkY=0, InterpolationRadius=16, DropletCount=1000, BrushRadius=3,
             Lifetime=30)
    r.update(over)
    return r


@pytest.mark.parametrize("bad", [
    dict(MapSize=0), dict(MapSize=60), dict(MapSize=16392),       # a positive multiple of 8, at most 16384
    dict(InterpolationRadius=0), dict(InterpolationRadius=15),     # positive and even
    dict(InterpolationRadius=72),                                  # at most MapSize
    dict(BrushRadius=0), dict(BrushRadius=95),                     # inside the merged 3x3 map
])
def test_batch_refuses_bad_requests(stpgb, bad):
    simplex = stpgb.SimplexSetting(1, 8, 0.2)
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.Batch([request(), request(**bad)], base_setting(stpgb), simplex, helpers.biome_table(4, 1))


def test_batch_refuses_empty_batch_and_bad_settings(stpgb):
    simplex = stpgb.SimplexSetting(1, 8, 0.2)
    table = helpers.biome_table(4, 1)
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.Batch([], base_setting(stpgb), simplex, table)
    with pytest.raises(stpgb.STPException):
        stpgb.Batch([request()], base_setting(stpgb, Inertia=1.5), simplex, table)
    with pytest.raises(stpgb.STPException):
        stpgb.Batch([request()], base_setting(stpgb), stpgb.SimplexSetting(1, 0, 0.2), table)
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.Batch([request()], base_setting(stpgb), simplex, table[:0])


@pytest.mark.parametrize("kw", [dict(hbm_budget=0), dict(max_in_flight=0), dict(max_batch=0), dict(streams=0),
                                dict(voronoi_cell=0)])
def test_server_refuses_zero_limits(stpgb, kw):
    from superterrainplus_gb300.serve import Server
    with pytest.raises(stpgb.STPNumericDomainError):
        Server(base_setting(stpgb), stpgb.SimplexSetting(1, 8, 0.2), helpers.biome_table(4, 1), **kw)


def test_erosion_call_refuses_bad_arguments(stpgb):
    """stpgb_hydraulic_erosion_ex: the setting, null pointers, a map smaller than the brush, an
    oversized brush and a map of 2^32 cells are refused before a launch (the pointers are never
    read)."""
    L = stpgb.lib()
    fake = C.c_void_p(0x1000)
    good = base_setting(stpgb)

    def call(setting=good, nn=(64, 64, 3, 3), hm=fake, brush_size=25, count=10):
        info = stpgb.NNInfo.make(nn[:2], nn[2:])
        return L.stpgb_hydraulic_erosion_ex(hm, C.byref(info), C.byref(setting), fake, count, fake, fake, brush_size,
                                            None, None, 0, 1, 0, None)

    assert call(setting=base_setting(stpgb, ErodeSpeed=2.0)) == stpgb._capi.STPGB_EINVAL
    assert call(hm=None) == stpgb._capi.STPGB_EINVAL
    assert call(brush_size=0) == stpgb._capi.STPGB_EINVAL
    assert call(nn=(2, 2, 3, 3)) == stpgb._capi.STPGB_EINVAL        # 6x6 map, brush radius 3
    assert call(brush_size=8193) == stpgb._capi.STPGB_EINVAL
    assert call(nn=(65536, 65536, 1, 1)) == stpgb._capi.STPGB_EINVAL  # 2^32 cells
    assert b"cells" in L.stpgb_last_error()


def test_noise_call_refuses_bad_arguments(stpgb):
    L = stpgb.lib()
    fake = C.c_void_p(0x1000)
    perm = stpgb.Permutation(0x2000, 0x3000, 8)
    empty = stpgb.Permutation(0x2000, 0x3000, 0)
    assert L.stpgb_multibiome_heightmap(None, 64, fake, fake, 64, 64, 0.0, 0.0, C.byref(perm), fake, 2,
                                        None) == stpgb._capi.STPGB_EINVAL
    assert L.stpgb_multibiome_heightmap(fake, 63, fake, fake, 64, 64, 0.0, 0.0, C.byref(perm), fake, 2,
                                        None) == stpgb._capi.STPGB_EINVAL
    assert L.stpgb_multibiome_heightmap(fake, 64, fake, fake, 64, 64, 0.0, 0.0, C.byref(empty), fake, 2,
                                        None) == stpgb._capi.STPGB_EINVAL
    # an empty map is a valid call that does nothing
    assert L.stpgb_multibiome_heightmap(fake, 64, fake, fake, 0, 64, 0.0, 0.0, C.byref(perm), fake, 2,
                                        None) == stpgb._capi.STPGB_OK


def test_erosion_choice_refuses_empty_area(stpgb):
    got = C.c_uint32(0)
    assert stpgb.lib().stpgb_erosion_choice(4, 100, 0, C.byref(got), None) == stpgb._capi.STPGB_EINVAL
    assert stpgb.lib().stpgb_erosion_choice(0, 100, 64, C.byref(got), None) == stpgb._capi.STPGB_EINVAL
