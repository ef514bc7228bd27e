"""The bench line's roofline arithmetic (no GPU): the erosion launch's algorithmic bytes and its
mix-weighted L2 bound, and the atomic-request roofline from the captured request counts."""
import math
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

import bench  # noqa: E402

PEAKS = {"load_v4_gbs": 4955.0, "red_v4_f32_gbs": 3670.0, "atom_v4_f32_gbs": 2206.0}


def test_erosion_l2_roofline_counts_the_algorithms_bytes():
    steps, erode, brush, ms = 480_000_000, 299_000_000, 45, 57.4
    r = bench.erosion_l2_roofline(PEAKS, steps, erode, brush, ms)
    loads = steps * 32 + erode * 4 * brush
    reds = erode * 4 * brush + (steps - erode) * 16
    assert r["load_bytes"] == loads and r["reduction_bytes"] == reds
    t_min = loads / (PEAKS["load_v4_gbs"] * 1e9) + reds / (PEAKS["red_v4_f32_gbs"] * 1e9)
    assert math.isclose(r["frac"], t_min / (ms / 1000.0))
    assert math.isclose(r["achieved"], (loads + reds) / (ms / 1000.0) / 1e9)
    # the peak is the mix-weighted rate: achieved / peak == frac
    assert math.isclose(r["achieved"] / r["peak"], r["frac"])
    assert r["bound"] == "l2" and r["unit"] == "GB/s"


def test_l2_atomic_roofline_scales_with_the_requests_per_launch():
    one = bench.l2_atomic_roofline(PEAKS, 16, 57.4)
    atom, red = bench.EROSION_L2_ATOMICS_PER_REQUEST * 16, bench.EROSION_L2_REDUCTIONS_PER_REQUEST * 16
    assert math.isclose(one["atomic_requests_per_launch"], atom)
    assert math.isclose(one["reduction_requests_per_launch"], red)
    t_min = 16 * atom / (PEAKS["atom_v4_f32_gbs"] * 1e9) + 16 * red / (PEAKS["red_v4_f32_gbs"] * 1e9)
    assert math.isclose(one["frac"], t_min / 0.0574)
    # twice the requests in twice the time: the same fraction
    two = bench.l2_atomic_roofline(PEAKS, 32, 2 * 57.4)
    assert math.isclose(two["frac"], one["frac"])
    assert math.isclose(bench.erosion_traffic(32), 2 * bench.erosion_traffic(16))
