"""Host helpers of bench.py on CPU: the clock sampler's summary (median SM
clock under load, maximum, the throttle reasons seen) from nvidia-smi lines,
the Strouhal number of a probe trace, and the roofline inputs read from the
committed files."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_clock_summary_median_max_and_reasons():
    c = bench.Clocks(0)
    c.lines = [
        "2070, 2070, Not Active, Not Active, Not Active, Not Active",
        "2055, 2070, Not Active, Not Active, Not Active, Active",
        "2070, 2070, Not Active, Not Active, Not Active, Not Active",
        "[N/A], 2070, Not Active, Not Active, Not Active, Not Active",  # unreadable sample: skipped
        "garbage",
    ]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    c.lines = ["1500, 2070, Active, Not Active, Active, Not Active"]
    assert c.summary()["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    c.lines = []
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_strouhal_of_a_sine_trace():
    t = np.arange(20000)
    trace = 0.05 * np.sin(2 * np.pi * t / 400.0) + 0.01
    # frequency 1/400 per step, plate 40, inlet 0.1: St = 40 / (400 * 0.1) = 1
    assert abs(bench.strouhal(trace) - 1.0) < 0.01


def test_roofline_inputs_from_committed_files():
    peak, kind = bench.peaks()
    assert peak > 0 and kind in ("measured", "fallback")
    for st in ("fx64", "f64", "f16", "bf16"):
        tpn = bench.profile_traffic_per_node(st)
        assert tpn is not None and 0.5 * bench.BYTES_PER_NODE[st] < tpn < 2 * bench.BYTES_PER_NODE[st]


def test_phase_lag_of_shifted_cycles():
    t = np.arange(60000)
    ref = np.sin(2 * np.pi * t / 2600.0) + 0.3 * np.sin(4 * np.pi * t / 2600.0)
    for lag in (-700, -41, 0, 63, 1200):
        other = np.sin(2 * np.pi * (t + lag) / 2600.0) + 0.3 * np.sin(4 * np.pi * (t + lag) / 2600.0)
        assert bench.phase_lag(ref, other, 2600, 10400) == lag


def test_phase_lag_is_not_pulled_by_a_growing_amplitude():
    t = np.arange(100000)
    ref = (1 + t / 2e4) * np.sin(2 * np.pi * t / 2600.0)
    assert bench.phase_lag(ref, ref.copy(), 2600, 10400) == 0
    assert bench.phase_lag(ref, (1 + (t + 25) / 2e4) * np.sin(2 * np.pi * (t + 25) / 2600.0), 2600, 10400) == 25


def test_every_storage_has_a_bench_dtype():
    import bench
    from lattice_boltzmann_parallel_solver_gb300.lattice import BYTES_PER_NODE, STORAGES
    assert set(bench.DTYPES) == set(STORAGES) == set(BYTES_PER_NODE)
