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


def reference_chunk_test():
    """The reference's STPTest2DChunk.cpp: in the checkout named by STP_REFERENCE_ROOT, else in the copy
    of the reference's sources that oracle/build_ref.sh keeps in oracle/_ref/tree; None without either."""
    rel = os.path.join("SuperTest+", "SuperTerrain+", "STPTest2DChunk.cpp")
    root = os.environ.get("STP_REFERENCE_ROOT")
    for base in ([root] if root else []) + [os.path.join(ROOT, "oracle", "_ref", "tree")]:
        if os.path.exists(os.path.join(base, rel)):
            return os.path.join(base, rel)
    return None


def test_reference_chunk_scenario_compiles_against_the_facade(tmp_path, stpgb):
    """The reference's own STPChunk utility scenario (SuperTest+/SuperTerrain+/STPTest2DChunk.cpp, the
    part before its chunk-storage tests, copied unchanged into a scratch folder) compiles against
    the façade through the compatibility headers in tests/cpp/compat, with glm result types, and
    passes.  Skips where the reference's sources are absent."""
    path = reference_chunk_test()
    if path is None:
        pytest.skip("reference sources not present")
    from superterrainplus_gb300 import _capi
    with open(path) as f:
        text = f.read()
    cut = text.index("class ChunkTester")
    src = tmp_path / "chunk_scenario.cpp"
    src.write_text(text[:cut])
    libdir = os.path.dirname(_capi.LIB_PATH)
    exe = str(tmp_path / "chunk_scenario")
    subprocess.check_call(["g++", "-std=c++20", "-O1", "-DSTPGB_CATCH_MAIN",
                           "-I" + os.path.join(ROOT, "tests", "cpp", "compat"), "-I" + os.path.join(ROOT, "include"),
                           "-I" + os.path.join(ROOT, "oracle", "refshim"), str(src), "-L" + libdir, "-lstpgb",
                           "-Wl,-rpath," + libdir, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "1 scenarios, 0 failed checks" in r.stdout
