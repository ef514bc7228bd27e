"""Build recipe for the oracle (test infrastructure only).

`build()` compiles oracle/stp_oracle.cpp (the CPU restatement) into
oracle/liboracle.so.  `build_ref()` runs oracle/build_ref.sh, which compiles
the reference's own host sources into oracle/_ref/libstpref.so when the
reference tree is present (development container only).
"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libstpref.so")
SRC = os.path.join(HERE, "stp_oracle.cpp")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    flags = ["-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread"]
    subprocess.check_call(["g++", *flags, SRC, "-o", LIB + ".tmp"])
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_ref(force=False):
    """Returns the path of oracle/_ref/libstpref.so, or None without the reference tree."""
    root = os.environ.get("STP_REFERENCE_ROOT", "/root/reference")
    if not os.path.isdir(os.path.join(root, "SuperTerrain+")):
        return REF_LIB if os.path.exists(REF_LIB) and platform.machine() == "x86_64" else None
    if force or not os.path.exists(REF_LIB):
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
    return REF_LIB


if __name__ == "__main__":
    print(build(force=True))
    print(build_ref(force=True))
