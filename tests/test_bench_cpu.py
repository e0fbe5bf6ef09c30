"""bench.py's bookkeeping on the host: the algorithmic-byte counts the
roofline uses, the clock-sample summary and the JSON contract of the
reference arm's fixed fields."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_algorithmic_bytes_of_the_bench_workload():
    P, C, N, F, Ht, Wt = 8 * 1024 * 1024, 8, 35002, 70000, 1024, 1024
    step = bench.algorithmic_bytes(P, C, N, F, Ht, Wt, 1, 0)
    # 64 B per pixel + per view normals/faces/UVs + texture and its gradient + vertices + SH
    assert step == P * 64 + C * (12 * N + 12 * F + 24 * F + 12 * N) + 24 * Ht * Wt + 24 * N + 216 * C
    assert step == 589_758_896
    assert bench.kernel_bytes("k_raster", P, C, N, F, Ht, Wt, 1, 0) == 237_429_696
    # upstream gradient 12 + face id 4 + barycentrics 8 per pixel
    assert bench.kernel_bytes("k_bwd_pixels", P, C, N, F, Ht, Wt, 1, 0) == P * 24 + C * (12 * N + 36 * F) + 24 * Ht * Wt
    assert bench.kernel_bytes("k_cameras", P, C, N, F, Ht, Wt, 1, 0) is None


def test_clock_summary_flags_throttling(tmp_path):
    c = bench.ClockSampler(0)
    c.path = str(tmp_path / "clocks.csv")
    with open(c.path, "w") as fh:
        fh.write("0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active\n")
        fh.write("0, 2055, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active\n")
        fh.write("0, 300, 2070, 100.0, 0x0, Not Active, Not Active, Not Active, Not Active\n")
    out = c.stop()
    assert out["samples"] == 3 and out["sm_max_mhz"] == 2070.0
    assert out["sm_mhz"] == 2062.5            # median of the samples under load (>= half the max clock)
    assert out["reasons"] == ["sw_power_cap"]
