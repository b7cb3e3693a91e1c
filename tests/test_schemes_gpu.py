"""GPU: the CN-family and IMEX Runge-Kutta steps of conatus_gb300.ivp.IVPSolver against the
reference's own trajectories (tests/golden/scheme_*.npz: three steps from a seeded state, lower-order
start-up, the reference's M and L values), per field and per step within 10x the reference's own
rounding floor (1e-12 relative L2 at least); graph replay equals plain steps bit for bit."""
from __future__ import annotations

import pytest

from _step_cases import SCHEME_FLOOR, field_errors, gather_state, load_scheme, scheme_fixtures, trajectory_tolerances

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fixture", scheme_fixtures())
def test_gpu_scheme_matches_reference(fixture, cuda_lib):
    import torch
    from conatus_gb300.ivp import IVPSolver
    P, g, maps, scheme = load_scheme(fixture)
    solver = IVPSolver(P, scheme=scheme, dt=float(g["dt"]))
    C0 = [gather_state(g["X0"], m) for m in maps]
    solver.set_state(C0)
    for k in range(g["Xs"].shape[0]):
        solver.step()
        C = solver.state_to_host()
        ref = [gather_state(g["Xs"][k], m) for m in maps]
        errs = field_errors(P, C, ref, floor=SCHEME_FLOOR)
        tols = trajectory_tolerances(P, g, maps, k)
        bad = {f: (errs[f], tols[f]) for f in errs if not errs[f] <= tols[f]}
        assert not bad, (k, bad)
    # the same steps as graph launches (start-up steps plain, then graphs)
    b = IVPSolver(P, scheme=scheme, dt=float(g["dt"]), device_problem=solver.dev)
    b.set_state(C0)
    b.run_graph(g["Xs"].shape[0])
    torch.cuda.synchronize()
    assert torch.equal(b.X, solver.X)


@pytest.mark.parametrize("scheme", ["RK443", "CNAB2"])
def test_gpu_scheme_fp32_form(scheme, cuda_lib):
    """The FP32 form (FP32 F and solves with FP64 refinement) of the RK and CN steps stays within
    the mixed-form budget of the FP64 form on a smooth RB state."""
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import IVPSolver
    P = W.load_template("rb_nz64").instantiate([64])
    C0 = W.rayleigh_benard_state(P, 0)
    out = {}
    for prec in ("fp64", "fp32"):
        s = IVPSolver(P, scheme=scheme, dt=1e-4, precision=prec)
        s.set_state(C0)
        s.run_graph(10)
        out[prec] = s.state_to_host()
    errs = field_errors(P, out["fp32"], out["fp64"])
    assert max(v for k, v in errs.items() if not k.startswith("tau")) < 1e-6, errs
