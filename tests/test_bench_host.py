"""Host-side logic of bench.py that needs no GPU: the clock record of the
timed region, the algorithmic-bytes formula, the GCP workload's CPU baseline and
reference line."""
import datetime

import bench

LINES = [
    "2026/12/03 15:57:11.000, 0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
    "2026/12/03 15:57:11.050, 0, 1800, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
    "2026/12/03 15:57:11.100, 0, 2040, 2070, 1200.0, 0x0, Not Active, Active, Not Active, Not Active",
    "2026/12/03 15:57:11.150, 0, 2070, 2070, 950.0, 0x0, Not Active, Not Active, Not Active, Not Active",
    "garbage line",
]


def t(ms):
    return datetime.datetime(2026, 12, 3, 15, 57, 11) + datetime.timedelta(milliseconds=ms)


def test_clock_samples_inside_the_region():
    sm, smax, reasons, n = bench.ClockSampler.summarise(LINES, t(40), t(110))
    assert n == 2
    assert sm == (1800 + 2040) / 2
    assert smax == 2070
    assert reasons == ["hw_thermal_slowdown", "sw_power_cap"]


def test_clock_nearest_sample_for_a_short_region():
    sm, _, reasons, n = bench.ClockSampler.summarise(LINES, t(120), t(125))
    assert n == 1 and sm == 2040 and reasons == ["hw_thermal_slowdown"]  # 100 ms is nearest to 122.5 ms


def test_clock_no_samples():
    assert bench.ClockSampler.summarise([], t(0), t(10)) == (None, None, [], 0)


def test_algorithmic_bytes_per_step():
    # J_u (N-1) 4 + J_u 8 + J_u R 8 + H (4 + 8) + 2 T R 8
    assert bench.algorithmic_bytes(4, 25, 1000, 5000, 300) == 1000 * 3 * 4 + 1000 * 8 + 1000 * 25 * 8 + 5000 * 12 + \
        2 * 300 * 25 * 8


def test_gcp_cpu_baseline_runs():
    """The GCP workload's CPU baseline (the GCP step restated with torch on the
    host) on a tiny tensor: it steps and reports a rate."""
    import numpy as np

    dims = (30, 20, 10)
    rng = np.random.default_rng(0)
    idx = np.stack([rng.integers(0, d, 200) for d in dims], axis=1).astype(np.int32)
    vals = rng.poisson(2.0, 200).astype(np.float32) + 1.0
    rate, threads = bench.gcp_cpu_sample(dims, idx, vals, 4, 64, 64, 1e-2, 2)
    assert rate > 0 and threads >= 1


def test_gcp_reference_arm_is_unavailable(capsys):
    import json
    import sys

    argv = sys.argv
    sys.argv = ["bench.py", "--impl", "reference", "--workload", "gcp4"]
    try:
        assert bench.main() == 0
    finally:
        sys.argv = argv
    line = json.loads(capsys.readouterr().out.strip())
    assert line["impl"] == "reference" and "unavailable" in line
