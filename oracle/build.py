"""Build recipe for the oracle (test infrastructure only).

`build()` compiles oracle/stp_oracle.cpp (the CPU restatement) into
oracle/liboracle.so.  `build_ref()` runs oracle/build_ref.sh, which compiles
the reference's own host sources into oracle/_ref/libstpref.so, its device
code as host C++ into oracle/_ref/libstpref_device.so and its erosion kernel
for sm_103a into oracle/_ref/libstpref_gpu.so, from a reference checkout
named by STP_REFERENCE_ROOT or from the copy of its sources that the recipe
keeps in the git-ignored oracle/_ref/tree.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libstpref.so")
REF_DEVICE_LIB = os.path.join(HERE, "_ref", "libstpref_device.so")
REF_GPU_LIB = os.path.join(HERE, "_ref", "libstpref_gpu.so")
REF_TREE = os.path.join(HERE, "_ref", "tree")
SRC = os.path.join(HERE, "stp_oracle.cpp")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    flags = ["-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread"]
    subprocess.check_call(["g++", *flags, SRC, "-o", LIB + ".tmp"])
    os.replace(LIB + ".tmp", LIB)
    return LIB


def _recipe_mtime():
    paths = [os.path.join(HERE, "build_ref.sh")]
    for d, _, files in os.walk(os.path.join(HERE, "refshim")):
        paths += [os.path.join(d, f) for f in files]
    return max(os.path.getmtime(q) for q in paths)


def _sources_present():
    root = os.environ.get("STP_REFERENCE_ROOT")
    if root:
        return os.path.isdir(os.path.join(root, "SuperTerrain+"))
    return os.path.isdir(os.path.join(REF_TREE, "SuperTerrain+"))


def build_ref(force=False, device=False, gpu=False):
    """Returns the path of oracle/_ref/libstpref.so (libstpref_device.so with `device`,
    libstpref_gpu.so with `gpu`), or None without reference sources.  The sources are a reference
    checkout named by STP_REFERENCE_ROOT (copied by the recipe into oracle/_ref/tree) or, without
    it, that copy.  The recipe reruns when a library is missing or older than the recipe, its shims
    or the copied tree."""
    lib = REF_GPU_LIB if gpu else REF_DEVICE_LIB if device else REF_LIB
    if not _sources_present():
        return lib if os.path.exists(lib) else None
    libs = (REF_LIB, REF_DEVICE_LIB, REF_GPU_LIB)
    newest = _recipe_mtime()
    if os.path.isdir(REF_TREE) and not os.environ.get("STP_REFERENCE_ROOT"):
        newest = max(newest, os.path.getmtime(REF_TREE))
    stale = any(not os.path.exists(q) or os.path.getmtime(q) < newest for q in libs)
    if force or stale:
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
    return lib if os.path.exists(lib) else None


if __name__ == "__main__":
    print(build(force=True))
    print(build_ref(force=True))
