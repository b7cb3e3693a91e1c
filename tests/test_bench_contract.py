"""CPU: the JSON contract of ``bench.py --impl reference`` (the CPU implementation of the step timed
on the host cores) on the small configurations: one line with the arm's metric, unit, config and
the e2e / cpu_baseline objects the contract asks for; under torchrun only rank 0 prints. And the
clock record of the timed region (``bench.ClockSampler``) against an nvidia-smi stand-in."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, env_extra=None):
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    env.update(env_extra or {})
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    return [ln for ln in p.stdout.splitlines() if ln.strip()]


@pytest.mark.parametrize("config", ["burgers", "rayleigh_benard"])
def test_reference_arm_line(config):
    lines = _run(["--impl", "reference", "--config", config, "--steps", "2", "--warmup", "1"])
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert key in d, key
    assert d["unit"] == "steps/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] >= 3          # at least three warm-up steps, always
    assert d["n_gpus"] == 1 and d["dtype"] == "f64"
    assert d["value"] > 0 and abs(d["value"] * d["ms_per_step"] / 1e3 - 1.0) < 1e-9
    assert "workload" in d["config"] and "model" not in d["config"]
    # the same config dict as the GPU arm's line (bench.workload_config)
    assert set(d["config"]) == {"workload", "real_unknowns", "systems", "parallelism", "l2"}
    cb = d["cpu_baseline"]
    assert "full step" in cb["sample"] and "all" in cb["sample"]      # measured, not extrapolated
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_same_metric_as_gpu_arm():
    """The reference arm reports the plain FP64 metric string the GPU arm prints at FP64."""
    import bench
    d = json.loads(_run(["--impl", "reference", "--config", "burgers", "--steps", "2", "--warmup", "3"])[0])
    assert d["metric"] == bench.METRIC["burgers"] + " plain FP64"


def test_reference_arm_other_ranks_silent():
    lines = _run(["--impl", "reference", "--config", "burgers", "--gpus", "2", "--steps", "2",
                  "--warmup", "3"], {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert lines == []


def _fake_smi(tmp_path, reason_col=None):
    """An nvidia-smi stand-in: the first line after 0.3 s, then one every 50 ms, SM clock counting
    up from 1000; ``reason_col`` (0-3) marks one throttle reason Active."""
    flags = ["Not Active"] * 4
    if reason_col is not None:
        flags[reason_col] = "Active"
    p = tmp_path / "nvidia-smi"
    p.write_text("#!/bin/bash\nsleep 0.3\ni=0\nwhile true; do\n"
                 f'  echo "0, $((1000 + i)), 2070, 900.5, 0x0, {", ".join(flags)}"\n'
                 "  i=$((i+1))\n  sleep 0.05\ndone\n")
    p.chmod(0o755)
    return str(tmp_path)


def test_clock_sampler_keeps_the_region_samples(tmp_path, monkeypatch):
    import time
    import bench
    monkeypatch.setenv("PATH", _fake_smi(tmp_path) + os.pathsep + os.environ["PATH"])
    with bench.ClockSampler(0) as clk:
        assert clk.skip == 1                       # entering waited for the first sample
        time.sleep(0.4)
    s = clk.summary()
    assert s["samples"] >= 3 and s["sm_mhz"] > 1000.0       # the pre-region sample left out
    assert s["sm_max_mhz"] == 2070.0 and s["reasons"] == []


@pytest.mark.parametrize("col, name", [(0, "hw_slowdown"), (1, "hw_thermal_slowdown"),
                                       (2, "sw_thermal_slowdown"), (3, "sw_power_cap")])
def test_clock_sampler_reports_throttle_reasons(tmp_path, monkeypatch, col, name):
    import time
    import bench
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, col) + os.pathsep + os.environ["PATH"])
    with bench.ClockSampler(0) as clk:
        time.sleep(0.15)
    assert clk.summary()["reasons"] == [name]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    import bench
    monkeypatch.setenv("PATH", str(tmp_path))
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.summary()["reasons"] == ["nvidia-smi unavailable"]
