"""Host-side logic of bench.py that needs no GPU: the clock record of the
timed region and the algorithmic-bytes formula."""
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
