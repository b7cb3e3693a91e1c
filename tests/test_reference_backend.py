"""CPU: the reference's entry points after ``conatus_gb300.install()`` (needs the reference's
Python package: skipped where it is absent). ``backend="cuda"`` of ``Model.simulate`` reaches this
package's solver (which, without a CUDA device, stops there: no CPU fallback; on a GPU host it is
built), ``backend="cpu"`` stays the reference's own solver, and the layout maps of the route
round-trip exactly."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT, reference_python

REF = reference_python()
pytestmark = pytest.mark.skipif(REF is None, reason="the reference's Python package is not present")


def run_case(case, timeout=600):
    env = dict(os.environ)
    p = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "_reference_backend_case.py"), REF, case],
                       capture_output=True, text=True, timeout=timeout, env=env)
    assert p.returncode == 0, p.stderr[-3000:]
    return json.loads(p.stdout.strip().splitlines()[-1])


def test_backend_cuda_reaches_the_gb300_solver_and_cpu_stays_the_reference():
    out = run_case("cpu_routing")
    assert out["cpu_solver"] == "IVPSolver" and out["cpu_steps"] == 2
    if out["cuda_device"]:                        # a GPU host: the route builds the device solver
        assert out["cuda"] == "built GB300IVPSolver", out["cuda"]
    else:                                        # no device: this package refuses, never the CPU
        assert out["cuda"].startswith("CudaError") and "CUDA device" in out["cuda"], out["cuda"]
    assert out["state_roundtrip"] < 1e-15 and out["rows_roundtrip"] < 1e-15
