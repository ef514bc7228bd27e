"""Build recipe for the oracle (test infrastructure only).

`build()` compiles oracle/stp_oracle.cpp (the CPU restatement) into
oracle/liboracle.so.  `build_ref()` runs oracle/build_ref.sh, which compiles
the reference's own host sources into oracle/_ref/libstpref.so and its
device code, as host C++, into oracle/_ref/libstpref_device.so when the
reference tree is present (development container only).
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libstpref.so")
REF_DEVICE_LIB = os.path.join(HERE, "_ref", "libstpref_device.so")
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


def build_ref(force=False, device=False):
    """Returns the path of oracle/_ref/libstpref.so (libstpref_device.so with `device`), or None
    without the reference tree.  The recipe reruns when a library is missing or older than the
    recipe or its shims."""
    root = os.environ.get("STP_REFERENCE_ROOT", "/root/reference")
    lib = REF_DEVICE_LIB if device else REF_LIB
    if not os.path.isdir(os.path.join(root, "SuperTerrain+")):
        return lib if os.path.exists(lib) and platform.machine() == "x86_64" else None
    stale = any(not os.path.exists(q) or os.path.getmtime(q) < _recipe_mtime() for q in (REF_LIB, REF_DEVICE_LIB))
    if force or stale:
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
    return lib


if __name__ == "__main__":
    print(build(force=True))
    print(build_ref(force=True))
