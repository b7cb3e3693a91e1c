"""GPU: whole trajectories of the configurations against the reference's own runs, with no teacher
forcing (golden fixtures ``traj_*.npz`` from the reference's IVPSolver, tests/golden/make_golden.py).

Each case starts from the benchmark's initial state (conatus_gb300.workloads), runs the plain FP64
drop-in for the configuration's length on the GPU and compares the coefficient arrays of every
variable with the reference's at the recorded steps (relative L2 per field). Over a trajectory the
two FP64 implementations drift apart by their rounding differences, amplified by the dynamics; the
tolerances below are the bound each case must keep (step-wise parity, teacher-forced to 1e-12, is
tests/test_step_gpu.py).

Tolerance per field: 1e-11 relative L2, raised to 10 times the reference's own spread (the
difference of its runs from X_0 perturbed by about one ulp, recorded in the fixture); each field's
norm is taken at least 1e-8 times the state's (the tau variables, zero up to rounding, are judged
against the state).

* Burgers N = 128, SBDF2, dt = 1e-4, 5000 steps, u0 = -sin(pi x) (field by field with the
  reference's NumPy path).
* Rayleigh-Benard 256 x 64, SBDF2, dt = 1e-4: at Ra = 1e6 (the configuration) the reference itself
  blows up between steps 150 and 200 (convection sets in with velocities of order sqrt(Ra), far
  beyond the advective limit of dt = 1e-4): compared at steps 50, 100 and 150, and the GPU run's
  finite-state check stops at step 200 exactly as the reference's does; the configured 2000 steps
  at Ra = 1e4, stable.
* Channel 16 x 17 x 16 (the configuration at a reduced resolution), SBDF3, dt = 5e-3, 500 steps.

The measured deviations are printed (``pytest -s``)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

CASES = {
    # fixture -> (template, template parameters, Fourier sizes, workload)
    "traj_burgers128.npz": ("burgers_n128", None, None, "burgers"),
    "traj_rb256x64_ra1e6.npz": ("rb_nz64", None, [256], "rayleigh_benard"),
    "traj_rb256x64_ra1e4.npz": ("rb_nz64_ra", {"Ra": 1e4}, [256], "rayleigh_benard"),
    "traj_channel16x17x16.npz": ("channel_ny17", None, [16, 16], "channel"),
}
BASE = 1e-11          # relative L2 per field
FACTOR = 10.0         # times the reference's own spread from a one-ulp perturbation of X_0
FLOOR = 1e-8          # a field's norm counts as at least this fraction of the state's norm


def _field_errors(arrs, g, step, floor=FLOOR):
    ref = [g[f"s{step}_v{v}"] for v in range(len(arrs))]
    tot = sum(float(np.sum(r ** 2)) for r in ref) ** 0.5
    return np.array([float(np.linalg.norm(a - r)) / max(float(np.linalg.norm(r)), floor * tot, 1e-300)
                     for a, r in zip(arrs, ref)])


@pytest.mark.parametrize("fixture", list(CASES))
def test_trajectory_matches_reference(fixture, cuda_lib):
    import torch
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import IVPSolver
    from oracle.ivp import OracleProblem
    tname, tparams, sizes, wl = CASES[fixture]
    g = golden(fixture)
    P = W.load_template(tname).instantiate(sizes, params=tparams)
    names = [str(x) for x in g["variables"]]
    assert names == [v["name"] for v in P.tpl.variables]
    solver = IVPSolver(P, scheme=str(g["scheme"]), dt=float(g["dt"]))
    solver.set_state(W.initial_state(wl, P, seed=0))
    op = OracleProblem(P)
    done = 0
    report = {}
    for step in (int(k) for k in g["steps"]):
        solver.run_graph(step - done)
        done = step
        torch.cuda.synchronize()
        errs = _field_errors(op.to_arrays(solver.state_to_host()), g, step)
        tols = np.maximum(BASE, FACTOR * g[f"spread_s{step}"])
        report[step] = {n: (f"{e:.2e}", f"{t:.1e}") for n, e, t in zip(names, errs, tols)}
        assert np.all(errs <= tols), (fixture, step, report[step])
    print(fixture, "error (tolerance) per field:", report)


def test_blow_up_stops_like_the_reference(cuda_lib):
    """The Rayleigh-Benard configuration blows up in the reference between steps 150 and 200; its
    finite-state check raises at iteration 200 (the first multiple of 100 after the blow-up), last
    checked finite at 100. The GPU run stops at the same check."""
    from conatus_gb300 import workloads as W
    from conatus_gb300.errors import NumericalError
    from conatus_gb300.ivp import IVPSolver
    P = W.problem("rayleigh_benard")
    solver = IVPSolver(P, scheme="SBDF2", dt=1e-4)
    solver.set_state(W.initial_state("rayleigh_benard", P, seed=0))
    solver.run_graph(100)                   # checked finite at 100
    with pytest.raises(NumericalError, match=r"at iteration 200.*last checked finite at iteration 100"):
        solver.run_graph(150)
    assert solver.finite_status() == 200


def test_finite_check_off_and_cadence(cuda_lib):
    """check_finite=False runs on through a blown-up state; check_finite=n checks every n steps."""
    from conatus_gb300 import workloads as W
    from conatus_gb300.errors import NumericalError
    from conatus_gb300.ivp import IVPSolver
    P = W.problem("rayleigh_benard")
    C0 = W.initial_state("rayleigh_benard", P, seed=0)
    off = IVPSolver(P, scheme="SBDF2", dt=1e-4, check_finite=False)
    off.set_state(C0)
    off.run_graph(250)
    assert off.finite_status() is None
    every = IVPSolver(P, scheme="SBDF2", dt=1e-4, check_finite=25, device_problem=off.dev)
    every.set_state(C0)
    with pytest.raises(NumericalError) as ei:
        every.run(250)
    bad = every.finite_status()
    assert bad is not None and bad % 25 == 0 and 150 < bad <= 200, str(ei.value)
    with pytest.raises(ValueError):
        IVPSolver(P, scheme="SBDF2", dt=1e-4, check_finite=0, device_problem=off.dev)
