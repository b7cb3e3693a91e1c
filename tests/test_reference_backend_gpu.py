"""GPU: scripts written for the reference run unchanged on the GB300 step after
``conatus_gb300.install()`` (python/conatus/model/model.py:912-935, model/run.py:116-144,
timestep/integrator.py:161-218): ``m.simulate(..., backend="cuda")`` then ``sim.run(steps=n)``.
Each case runs in a fresh interpreter (installing patches the reference package) and needs the
reference's Python package (CONATUS_REFERENCE_PYTHON): skipped where it is absent.

* Burgers N = 128 (configuration 1), SBDF2, from ``sim.initial(u=lambda x: -sin(pi x))``: after
  1000 steps the GB300 route equals the reference's CPU path of the same script (its banded solves
  on this package's GPU core, ``conatus._core``) to 1e-11, and the reference's own run
  (tests/golden/traj_burgers128.npz, compiled core) to 1e-11; the FP32 form to 1e-6.
* Channel 8 x 17 x 8 (configuration 3 at a small size), SBDF3, 20 steps from a seeded state:
  the route against the reference's CPU path, per field (u 1e-10, p 2e-9: the pressure carries
  the systems' conditioning); a checkpoint written by one restarts the other (the reference's own
  file format), both ways.
* The Rayleigh-Benard configuration blows up (in the reference too): the route raises the
  reference's own NumericalError from its finite-state check at iteration 200."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, reference_python
from test_reference_backend import run_case

REF = reference_python()
pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(REF is None, reason="the reference's Python package is not present")]


def test_burgers_script_runs_on_the_gb300_step(cuda_lib):
    out = run_case("burgers")
    assert out["solver"] == "GB300IVPSolver" and out["iteration"] == 1000
    assert abs(out["t"] - 0.1) < 1e-12
    assert out["u0_same"] == 0.0
    assert out["cpu_core"].endswith("conatus_gb300.core")
    assert out["dev_vs_cpu"] < 1e-11, out["dev_vs_cpu"]
    g = golden("traj_burgers128.npz")
    u_ref = g["s1000_v0"]
    u = np.asarray(out["u1000"])
    assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) < 1e-11


def test_burgers_script_fp32_form(cuda_lib):
    fp64 = np.asarray(run_case("burgers")["u1000"])
    out = run_case("burgers_fp32")
    u = np.asarray(out["u1000"])
    err = np.linalg.norm(u - fp64) / np.linalg.norm(fp64)
    assert err < 1e-6
    # the run's own report (monitor_fp64, every 250 steps): its last entry is this error
    me = out["mixed_error"]
    assert sorted(int(k) for k in me) == [250, 500, 750, 1000]
    assert abs(me["1000"]["u"] - err) <= 1e-3 * err + 1e-15, (me["1000"], err)


def test_channel_script_and_checkpoints_both_ways(cuda_lib):
    out = run_case("channel")
    # the channel's pressure carries the conditioning of its (kx, kz) systems (about 6e5): the
    # reference's own rounding floor per step is 1.3e-10 in p (tests/golden/step_channel8x17x8.npz)
    tol = {"u": 1e-10, "p": 2e-9}
    for key in ("fields", "after_restart", "restart_from_reference"):
        for v, e in out[key].items():
            assert e < tol[v], (key, v, e)
    t1, i1, t2, i2 = out["clock"]
    assert i1 == i2 and abs(t1 - t2) < 1e-12


def test_blow_up_raises_the_reference_numerical_error(cuda_lib):
    out = run_case("blowup")
    assert out["raised"] is not None and "iteration 200" in out["raised"], out
