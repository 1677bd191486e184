"""Host-side helpers of bench.py (no GPU): the clock-sample filter and the
roofline arithmetic that the bench line reports."""
import datetime
import time

import pytest

import bench


def _stamp(t):
    return datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]


def _line(t, sm, reasons=("Not Active",) * 4):
    return f"{_stamp(t)}, {sm}, 2070, 900.0, " + ", ".join(reasons)


def test_clock_summary_keeps_samples_inside_the_timed_window():
    c = bench.Clocks(0)
    now = time.time()
    c.out = [_line(now - 0.5, 1200),                      # warm-up, outside the window
             _line(now + 0.01, 2070),
             _line(now + 0.03, 2060, ("Not Active", "Not Active", "Not Active", "Active")),
             "garbage line"]
    c.window(now, now + 0.05)
    s = c.summary()
    assert s["samples"] == 2 and s["span"] == "timed region"
    assert s["sm_mhz"] == pytest.approx(2065.0) and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_falls_back_to_the_whole_span():
    c = bench.Clocks(0)
    now = time.time()
    c.out = [_line(now - 0.2, 2070), _line(now - 0.1, 2070,
                                           ("Active", "Not Active", "Not Active", "Not Active"))]
    c.window(now, now + 0.001)              # shorter than the polling interval
    s = c.summary()
    assert s["samples"] == 2 and s["span"].startswith("warm-up and timed region")
    assert s["reasons"] == ["hw_slowdown"]


def test_mixed_roofline_arithmetic():
    r = bench.mixed_roofline(2.0, 70.0, {"bf16_tflops": 1900.0})
    f_cov = 8 * bench.M * bench.M * bench.T + 2 * bench.L * bench.L * bench.NS
    f_rest = (4.0 / 3.0) * bench.L ** 3 + 8 * bench.L * bench.L + 32 * bench.L + 8 * bench.M
    t = bench.NPIX * (f_cov / 950.0e12 + f_rest / 70.0e12) * 1e3
    assert r["t_roof_ms"] == pytest.approx(t) and r["frac"] == pytest.approx(t / 2.0)
    assert bench.mixed_roofline(2.0, 70.0, {}) is None


def test_headline_roofline_is_the_mixed_bound():
    h = bench.headline_roofline(2.0, 70.0, {"bf16_tflops": 1900.0})
    m = bench.mixed_roofline(2.0, 70.0, {"bf16_tflops": 1900.0})
    assert h["bound"] == "tensor" and h["frac"] == pytest.approx(m["frac"])
    assert h["achieved"] / h["peak"] == pytest.approx(h["frac"])
    assert bench.headline_roofline(2.0, 70.0, {}) is None


def test_workload_constants_are_config_1():
    assert (bench.M, bench.L, bench.K, bench.NX, bench.NY) == (64, 32, 2, 256, 2048)
    assert bench.NPIX == 256 * (2048 - 4) == 523264
    assert bench.FLOP_PER_PIXEL == pytest.approx(284842.67, rel=1e-6)
