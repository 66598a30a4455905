"""Host logic of the benchmark's clock record: nvidia-smi samples are kept
only when their own timestamp lies inside the timed region, throttle reasons
are collected from those samples, and a region shorter than the sampling
interval keeps the first sample after it started.  No GPU and no nvidia-smi:
the sampler is fed recorded lines."""
import datetime

import bench


def _line(t, sm, reasons=("Not Active",) * 4):
    ts = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return (t, f"{ts}, {sm}, 2070, 600.00, 0x0000000000000000, {', '.join(reasons)}\n")


def _sampler(lines, t0, t1):
    c = bench.ClockSampler(0)
    c.lines = lines
    c.t_start, c.t_stop = t0, t1
    return c


def test_only_samples_inside_the_region_count():
    base = 1.8e9
    lines = [_line(base + 0.02 * i, 1000 if i < 3 or i > 8 else 2070) for i in range(12)]
    s = _sampler(lines, base + 0.05, base + 0.17).summary()
    # samples 3..8 fall inside [0.05, 0.17]; the slow samples outside do not count
    assert s["samples"] == 6
    assert s["sm_mhz"] == 2070.0
    assert s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == []


def test_throttle_reasons_inside_the_region_are_reported():
    base = 1.8e9
    hot = ("Not Active", "Active", "Not Active", "Active")  # hw_thermal_slowdown, sw_power_cap
    lines = [_line(base + 0.02 * i, 1800, hot if i == 4 else ("Not Active",) * 4) for i in range(10)]
    s = _sampler(lines, base + 0.05, base + 0.15).summary()
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    # a reason outside the region is not reported
    s = _sampler(lines, base + 0.09, base + 0.15).summary()
    assert s["reasons"] == []


def test_short_region_keeps_the_next_sample():
    base = 1.8e9
    lines = [_line(base + 0.02 * i, 2000 + i) for i in range(5)]
    s = _sampler(lines, base + 0.021, base + 0.025).summary()
    assert s["samples"] == 1
    assert s["sm_mhz"] == 2002.0


def test_unparsable_lines_are_skipped():
    base = 1.8e9
    lines = [(base, "garbage\n"), _line(base + 0.01, 2070), (base + 0.02, "a, b, c, d, e, f, g, h, i\n")]
    s = _sampler(lines, base, base + 1.0).summary()
    assert s["samples"] == 1
