"""Records the erosion tolerance of every RMS parity case into tests/golden/erosion_band.json.

For each case the reference's own erosion kernel (hydraulicErosionKERNEL with STPRainDrop, built for
sm_103a by oracle/build_ref.sh into oracle/_ref/libstpref_gpu.so) runs five times on the case's map
with the case's droplets; the file keeps, per case, the RMS of each run against the FP64 serial
oracle and the run-to-run spread (largest RMS between two runs).  The GPU parity tests compute the
same figures live wherever the reference GPU build exists and fall back to this file elsewhere.

Run on a machine with a GB300 and the reference GPU build:
    python tests/golden/make_erosion_band.py [output.json]
It runs the RMS parity tests with STPGB_RECORD_BAND naming the output file.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    out = os.path.abspath(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "erosion_band.json"))
    if os.path.exists(out):
        os.remove(out)
    env = dict(os.environ, STPGB_RECORD_BAND=out)
    rc = subprocess.call([sys.executable, "-m", "pytest", "tests", "-m", "gpu", "-q", "-k", "reference_spread",
                          "-p", "no:cacheprovider"], cwd=ROOT, env=env)
    print(f"wrote {out}" if os.path.exists(out) else "no band recorded (reference GPU build absent?)")
    return rc


if __name__ == "__main__":
    sys.exit(main())
