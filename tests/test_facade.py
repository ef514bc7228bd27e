"""The C++ façade (include/stpgb.hpp) compiled against the library and run
with the reference's own test scenarios (tests/cpp/test_facade.cpp)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def facade_binary(tmp_path_factory, stpgb):
    from superterrainplus_gb300 import _capi
    out = str(tmp_path_factory.mktemp("facade") / "test_facade")
    libdir = os.path.dirname(_capi.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "test_facade.cpp"), "-L" + libdir, "-lstpgb",
                           "-Wl,-rpath," + libdir, "-o", out])
    return out


def test_facade_error_paths_and_permutation(facade_binary):
    r = subprocess.run([facade_binary, "--cpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_facade_reference_scenarios(facade_binary):
    r = subprocess.run([facade_binary], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
