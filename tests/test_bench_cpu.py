"""Host-side pieces of bench.py that run without a GPU: the clock-record summary (median SM
clock under load, throttle reasons) and the peak and traffic lookups."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import bench  # noqa: E402


def test_clock_summary_median_under_load_and_reasons(tmp_path):
    path = tmp_path / "clocks.csv"
    rows = ["0, 2070, 2070, 40.0, 0x0, Not Active, Not Active, Not Active, Not Active",   # idle
            "0, 2070, 2070, 560.0, 0x0, Not Active, Not Active, Not Active, Not Active",
            "0, 2055, 2070, 590.0, 0x4, Not Active, Not Active, Not Active, Active",
            "0, 2040, 2070, 600.0, 0x4, Not Active, Not Active, Not Active, Active"]
    path.write_text("\n".join(rows) + "\n")
    s = bench.ClockSampler(0)
    s.proc, s.path = object(), str(path)
    out = s.summary()
    assert out["samples"] == 4 and out["sm_max_mhz"] == 2070.0 and out["power_w_max"] == 600.0
    assert out["sm_mhz"] == 2055.0            # median over the three loaded samples
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_summary_flags_thermal_slowdown(tmp_path):
    path = tmp_path / "clocks.csv"
    path.write_text("0, 1500, 2070, 600.0, 0x40, Not Active, Active, Not Active, Not Active\n")
    s = bench.ClockSampler(0)
    s.proc, s.path = object(), str(path)
    assert s.summary()["reasons"] == ["hw_thermal_slowdown"]


def test_clock_summary_without_sampler():
    s = bench.ClockSampler(0)
    assert s.summary()["reasons"] == ["unavailable"]


def test_peak_and_traffic_lookups(monkeypatch, tmp_path):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.load_peak() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6787.6}))
    assert bench.load_peak() == (6787.6, "measured")
    assert bench.load_traffic("c2") is None
    os.makedirs(tmp_path / "profiles")
    (tmp_path / "profiles" / "k_element_c2_traffic.json").write_text(json.dumps({"dram_bytes_per_launch_full": 1.0}))
    assert bench.load_traffic("c2")["dram_bytes_per_launch_full"] == 1.0


def test_committed_traffic_summary_is_readable():
    tr = bench.load_traffic("c2")
    assert tr is not None and tr["lean"] is True and tr["dram_bytes_per_launch_full"] > tr["algorithmic_bytes_per_launch"]
