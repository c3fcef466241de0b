"""CPU checks of bench.py's host logic: the clock record that decides whether a
timed run saw throttling, the whole-job aggregate, and the roofline peaks."""
import os

import bench


def row(sm, hw="Not Active", hw_thermal="Not Active", sw_thermal="Not Active", power_cap="Not Active"):
    # the order of ClockSampler.Q: index, clocks.sm, clocks.max.sm, power.draw,
    # reasons.active, hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap
    return ["0", str(sm), "2070", "950.0", "0x0", hw, hw_thermal, sw_thermal, power_cap]


def test_clock_record_median_and_reasons():
    cs = bench.ClockSampler()
    cs.rows = [row(2070), row(2055), row(1980, power_cap="Active"), row(2070), row(2070)]
    rec = cs.stop()
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0 and rec["samples"] == 5
    assert rec["reasons"] == ["sw_power_cap"]


def test_clock_record_flags_each_slowdown():
    cs = bench.ClockSampler()
    cs.rows = [row(1500, hw="Active"), row(1400, hw_thermal="Active"), row(1600, sw_thermal="Active")]
    rec = cs.stop()
    assert rec["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert rec["sm_mhz"] == 1500.0


def test_clock_record_without_samples():
    rec = bench.ClockSampler().stop()
    assert rec["reasons"] == ["unsampled"] and rec["sm_mhz"] is None


def test_whole_job_aggregate():
    # N replicas, each one solve per step: the slowest rank's step sets the job's rate
    assert bench.aggregate(1, 64.0) == 1000.0 / 64.0
    assert bench.aggregate(4, 100.0) == 40.0


def test_peaks():
    pk = bench.peaks()
    assert pk["hbm_gbs"] > 0
    measured = os.path.exists(os.path.join(bench.ROOT, "MEASURED_PEAKS.json"))
    assert measured == ("fallback" not in pk)
