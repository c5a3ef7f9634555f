"""bench.py's host-side contract, without a GPU: the reference arm's JSON line
(the CPU implementation timed on the whole specimen) and the helpers that shape
the GPU arm's line (clock samples and their throttle reasons, percentiles)."""

import json
import os
import subprocess
import sys
import tempfile

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "plain128", "--steps", "1", "--warmup", "0"], capture_output=True, text=True, cwd=ROOT,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Gvoxel/s" and d["value"] > 0
    for key in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config"):
        assert key in d
    assert d["config"]["workload"].startswith("plain128")
    # the same config object as the GPU arm's line: the whole specimen every step
    assert d["config"] == bench.workload_config("plain128", (128, 128, 128), 1)
    assert "whole" in d["cpu_baseline"]["sample"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def _clock_summary(lines):
    fd, path = tempfile.mkstemp(suffix=".csv")
    with os.fdopen(fd, "w") as f:
        f.write("\n".join(lines) + "\n")
    s = bench.ClockSampler(0)
    s.path = path
    return s.summary()


def test_clock_summary_reports_throttle_reasons():
    ok = "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active"
    capped = "0, 1900, 2070, 1400.0, 0x4, Not Active, Not Active, Not Active, Active"
    hot = "0, 1500, 2070, 1300.0, 0x40, Not Active, Active, Not Active, Not Active"
    s = _clock_summary([ok, ok, capped])
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]
    assert s["samples"] == 3
    s = _clock_summary([ok, hot, "garbage line"])
    assert s["reasons"] == ["hw_thermal_slowdown"] and s["samples"] == 2
    assert _clock_summary([])["reasons"] == ["no samples"]


def test_percentile_is_numpy_linear():
    xs = [5.0, 1.0, 3.0, 2.0, 4.0]
    assert bench.percentile(xs, 0.5) == 3.0
    assert bench.percentile(xs, 0.99) == pytest.approx(4.96)
    assert bench.percentile([], 0.5) is None
