"""C ABI checks that need no GPU: the library loads, exports every entry point
declared in include/stpgb.h, and its host-side paths (permutation table,
erosion brush, setting validation, argument checks) match the oracle and the
reference's error behaviour."""
import ctypes as C
import math
import os
import re
import subprocess

import numpy as np
import pytest

import helpers

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names += re.findall(r"STPGB_API\s+[\w\s\*]+?\b(stpgb_\w+)\s*\(", text)
    return names


def test_exports_every_declared_symbol(stpgb):
    from superterrainplus_gb300 import _capi
    names = declared_symbols()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", _capi.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (stpgb_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(stpgb.lib(), n)
    # nothing but the C ABI leaks out
    assert all(s.startswith("stpgb_") for s in exported)


def test_permutation_matches_oracle_and_reference(stpgb, oracle):
    for seed, n, offset, perm, grad in helpers.load_permutations():
        p, g = stpgb.permutation_generate(seed, n, offset)
        assert np.array_equal(p, perm)
        assert np.array_equal(g.view(np.uint32), grad.view(np.uint32))
    p, g = stpgb.permutation_generate(6666, 10, math.radians(6.5))
    _, po, go = oracle.permutation(6666, 10, math.radians(6.5))
    assert np.array_equal(p, po) and np.array_equal(g, go)


def test_permutation_invalid(stpgb):
    with pytest.raises(stpgb.STPInvalidEnvironment):
        stpgb.permutation_generate(1, 0, 0.0)
    with pytest.raises(stpgb.STPInvalidEnvironment):
        stpgb.permutation_generate(1, 8, 7.0)


def test_permutation_overflowing_distribution(stpgb, oracle):
    """Distributions whose angle loop runs once more in the reference still give N entries, no overrun."""
    for n in (6, 11, 13):
        p, g = stpgb.permutation_generate(5, n, 0.5)
        rc, po, go = oracle.permutation(5, n, 0.5)
        assert rc == 2
        assert np.array_equal(g, go)


@pytest.mark.parametrize("radius", [1, 2, 3, 4, 5, 8])
def test_brush_matches_oracle(stpgb, oracle, radius):
    for dim in (64, 1536, 3072):
        i1, w1 = stpgb.erosion_brush(dim, radius)
        i2, w2 = oracle.brush(dim, radius)
        assert np.array_equal(i1, i2)
        assert np.array_equal(w1.view(np.uint32), w2.view(np.uint32))


def test_brush_invalid(stpgb):
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.erosion_brush(64, 0)
    with pytest.raises(stpgb.STPNumericDomainError):
        stpgb.erosion_brush(0, 3)


def test_raindrop_validation(stpgb):
    L = stpgb.lib()
    good = stpgb.RaindropSetting(**helpers.raindrop_dict(100))
    assert L.stpgb_raindrop_setting_validate(C.byref(good)) == 0
    for field, bad in (("RainDropCount", 0), ("Inertia", 1.5), ("SedimentCapacityFactor", 0.0), ("Gravity", 0.0),
                       ("ErosionBrushRadius", 0), ("EvaporateSpeed", -0.1), ("Friction", 2.0)):
        s = stpgb.RaindropSetting(**helpers.raindrop_dict(100))
        setattr(s, field, bad)
        assert L.stpgb_raindrop_setting_validate(C.byref(s)) == 1, field


def test_lifetime_helper(stpgb):
    for life in (1, 30, 50, 64):
        v = stpgb.lifetime_min_water_volume(1.0, 0.01, life)
        vol, steps = np.float32(1.0), 0
        while vol >= np.float32(v):
            vol = np.float32(vol * np.float32(1.0 - np.float32(0.01)))
            steps += 1
        assert steps == life


def test_shf_argument_errors_without_gpu(stpgb):
    """Radius checks of STPSingleHistogramFilter.cpp:874-880 fire before any device work."""
    kat = helpers.load_shf_kat()
    f = stpgb.STPSingleHistogramFilter()
    buf = stpgb.STPFilterBuffer(stpgb.STPFilterBuffer.Serial)
    info = stpgb.NNInfo.make((4, 4), (3, 3))
    for r in (0, 3, 128):
        with pytest.raises(stpgb.STPNumericDomainError):
            f(kat["texture"], info, buf, r)
    with pytest.raises(stpgb.STPException):
        stpgb.STPFilterBuffer(7)


def test_generator_invalid_settings_without_gpu(stpgb):
    cs = stpgb.ChunkSetting()
    cs.MapSize[:] = [64, 64]
    cs.DiversityNearestNeighbour[:] = [3, 3]
    cs.ErosionNearestNeighbour[:] = [2, 3]  # must be odd
    rd = stpgb.RaindropSetting(**helpers.raindrop_dict(100))
    sx = stpgb.SimplexSetting(1, 8, 0.2)
    table = helpers.biome_table(2, 0)
    with pytest.raises(stpgb.STPInvalidEnvironment):
        stpgb.STPHeightfieldGenerator(cs, rd, sx, table, 8)
    cs.ErosionNearestNeighbour[:] = [3, 3]
    rd.Inertia = 2.0
    with pytest.raises(stpgb.STPInvalidEnvironment):
        stpgb.STPHeightfieldGenerator(cs, rd, sx, table, 8)


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from superterrainplus_gb300 import _capi
    monkeypatch.setattr(_capi, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(_capi, "_lib", None)
    with pytest.raises(ImportError):
        _capi.lib()


@pytest.mark.parametrize("radius,droplets,side,lanes,rows", [
    (4, 600000, 512, 2, 1),          # the production chunk (0.33 in flight per pixel): brush rows, two lanes
    (5, 2411725, 1024, 1, 1),        # 2.3 per pixel of a 1024^2 chunk, 0.08 in flight: warp-cooperative rows
    (5, 150733, 256, 2, 1),          # 2.3 per pixel of a 256^2 chunk, 1.34 in flight: rows, two lanes
    (3, 150733, 256, 2, 1),
    (2, 150733, 256, 2, 0),          # brush 2 is too small for row blocks
    (4, 9421, 64, 1, 0),             # 2.3 per pixel of a 64^2 chunk, all in flight: the reference kernel
    (3, 6144, 64, 2, 1),             # 1.5 in flight per pixel, the limit of the several-lane variants
    (4, 1048576, 512, 1, 0),         # above 3 droplets per pixel: one lane per droplet, the reference kernel
    (3, 20070, 64, 1, 0),
    (4, 28672, 64, 1, 0),
])
def test_erosion_choice_follows_density(stpgb, radius, droplets, side, lanes, rows):
    """Several lanes per droplet up to 3 droplets per pixel of the start area and 1.5 in flight at once
    (the two-lane row kernel keeps 152 SMs x 9 blocks x 64 droplets resident; no GPU here, so the SM
    count of the GB300 is taken); by default the warp-cooperative kernel (1 lane with rows) up to 0.2."""
    import ctypes as C
    area = side * side
    got_lanes, got_rows = C.c_uint32(0), C.c_uint32(0)
    stpgb.check(stpgb.lib().stpgb_erosion_choice(radius, droplets, area, C.byref(got_lanes), C.byref(got_rows)))
    assert (got_lanes.value, got_rows.value) == (lanes, rows)


def test_header_is_plain_c(tmp_path):
    """include/stpgb.h is the C boundary: it compiles as C11 with every warning, and a C program can
    call an entry point through it and link against the library."""
    from superterrainplus_gb300 import _capi
    src = tmp_path / "caller.c"
    src.write_text('#include "stpgb.h"\n#include <stdio.h>\n'
                   'int main(void) { uint32_t out[2]; const uint32_t range[2] = { 5u, 7u };\n'
                   '  int rc = stpgb_chunk_local_coordinate(7u, range, out);\n'
                   '  printf("%d %u %u %s\\n", rc, out[0], out[1], stpgb_version()); return rc; }\n')
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_capi.LIB_PATH)
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Wpedantic", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    str(src), "-L" + libdir, "-lstpgb", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out[:3] == ["0", "2", "1"]


def test_shf_set_path_range(stpgb):
    """The filter's process-wide path choice: 0..3 accepted, anything above refused (no GPU call)."""
    lib = stpgb.lib()
    for p in (1, 2, 3, 0):
        assert lib.stpgb_shf_set_path(p) == 0
    assert lib.stpgb_shf_set_path(4) != 0
    assert lib.stpgb_shf_set_path(0) == 0


def test_roofline_launch_argument_errors(stpgb):
    """The measurement kernels refuse an unknown kind, a missing sink and a map that is not a power
    of two before any device work (no GPU call)."""
    lib = stpgb.lib()
    fake = C.c_void_p(256)
    assert lib.stpgb_roofline_launch(6, fake, 1 << 10, 1, 1, fake, None) == stpgb._capi.STPGB_EINVAL
    for kind in (2, 5):  # 16-byte loads and returning atomics need a sink
        assert lib.stpgb_roofline_launch(kind, fake, 1 << 10, 1, 1, None, None) == stpgb._capi.STPGB_EINVAL
    for kind in (0, 1, 5):
        assert lib.stpgb_roofline_launch(kind, fake, 1000, 1, 1, fake, None) == stpgb._capi.STPGB_EINVAL
    assert lib.stpgb_roofline_launch(1, None, 1 << 10, 1, 1, fake, None) == stpgb._capi.STPGB_EINVAL
