"""GPU: the explicit right-hand side F and the IMEX step on the device (conatus_gb300.ivp) against
the reference's own IVPSolver (golden fixtures, teacher-forced, the reference's own M and L values:
the drop-in case) and against the oracle at a medium size (template polynomials).

Tolerances: F to 1e-12 relative L2; X_{n+1} to 1e-12 relative L2 per field, raised per field to
10x the reference's own rounding floor (``field_tolerances``)."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import (STEP_CASES, field_errors, field_tolerances, gather_rows, gather_state,
                         load_step, template)

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.concatenate([np.ravel(x) for x in a])
    b = np.concatenate([np.ravel(x) for x in b])
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("fixture", list(STEP_CASES))
def test_gpu_F_matches_reference(fixture, cuda_lib):
    import torch
    from conatus_gb300.ivp import DeviceProblem
    P, g, maps = load_step(fixture)
    dev = DeviceProblem(P)
    C = [gather_state(g["Xn"], m) for m in maps]
    X = dev.to_device(C)
    out = dev.zeros()
    dev.F(X, out)
    torch.cuda.synchronize()
    R = dev.to_host(out)
    R_ref = [gather_rows(g["Fn"], m) for m in maps]
    assert _rel(R, R_ref) < 1e-12


@pytest.mark.parametrize("fixture", list(STEP_CASES))
def test_gpu_step_matches_reference(fixture, cuda_lib):
    import torch
    from conatus_gb300.ivp import IVPSolver
    P, g, maps = load_step(fixture)
    order = int(g["order"])
    solver = IVPSolver(P, scheme=f"SBDF{order}", dt=float(g["dt"]))
    dev = solver.dev
    solver.set_state([gather_state(g["Xn"], m) for m in maps])
    hist_mx = [dev.to_device([gather_rows(h, m) for m in maps]) for h in g["MXh"][:order - 1]]
    hist_f = [dev.to_device([gather_rows(h, m) for m in maps]) for h in g["Fh"][:order - 1]]
    solver.set_history(hist_mx, hist_f)
    solver.step()
    torch.cuda.synchronize()
    C1 = dev.to_host(solver.X)
    C1_ref = [gather_state(g["Xn1"], m) for m in maps]
    errs = field_errors(P, C1, C1_ref)
    tols = field_tolerances(P, g, maps)
    assert all(errs[k] <= tols[k] for k in errs), (errs, tols)


def _smooth_state(P, rng, amp=0.05):
    C = []
    for bi, b in enumerate(P.tpl.buckets):
        n_idx = np.maximum(b.col[:, 2], 0)
        z = rng.standard_normal((P.nsys[bi], b.n)).astype(np.complex128)
        if b.kind != "real":
            z = z + 1j * rng.standard_normal((P.nsys[bi], b.n))
        C.append(z * amp * np.exp(-0.35 * n_idx))
    return C


@pytest.mark.parametrize("tname,sizes,scheme,dt", [("rb_nz16", [64], "SBDF2", 1e-4),
                                                   ("channel_ny17", [16, 12], "SBDF3", 5e-3)])
def test_gpu_steps_match_oracle(tname, sizes, scheme, dt, rng, cuda_lib):
    """Three steps from a seeded state (lower-order start-up included) at a resolution the golden
    fixtures do not cover, template polynomials on both sides: GPU vs oracle."""
    import torch
    from conatus_gb300.ivp import IVPSolver
    from oracle.ivp import OracleProblem, SBDFStepper
    P = template(tname).instantiate(sizes)
    C0 = _smooth_state(P, rng)
    op = OracleProblem(P)
    st = SBDFStepper(op, int(scheme[-1]), dt)
    C = C0
    for _ in range(3):
        C = st.step(C)
    solver = IVPSolver(P, scheme=scheme, dt=dt)
    solver.set_state(C0)
    solver.run(3)
    torch.cuda.synchronize()
    Cg = solver.dev.to_host(solver.X)
    errs = field_errors(P, Cg, C)
    phys = {k: v for k, v in errs.items() if not k.startswith("tau")}
    assert max(phys.values()) < 1e-10, errs


def test_graph_replay_equals_steps(rng, cuda_lib):
    """run_graph(n) gives the same state as n plain steps, bit for bit (same kernels, same order)."""
    import torch
    from conatus_gb300.ivp import IVPSolver
    P = template("channel_ny17").instantiate([8, 8])
    C0 = _smooth_state(P, rng)
    a = IVPSolver(P, scheme="SBDF3", dt=5e-3)
    a.set_state(C0)
    a.run(7)
    b = IVPSolver(P, scheme="SBDF3", dt=5e-3, device_problem=a.dev)
    b.set_state(C0)
    b.run_graph(7)
    torch.cuda.synchronize()
    assert torch.equal(a.X, b.X)


@pytest.mark.parametrize("fixture", list(STEP_CASES))
def test_gpu_MX_matches_reference(fixture, cuda_lib):
    """M X_n on the device against the M X_n the reference's own step pushed on its history."""
    import torch
    from conatus_gb300.ivp import DeviceProblem
    P, g, maps = load_step(fixture)
    dev = DeviceProblem(P)
    X = dev.to_device([gather_state(g["Xn"], m) for m in maps])
    out = dev.zeros()
    dev.MX(X, out)
    torch.cuda.synchronize()
    assert _rel(dev.to_host(out), [gather_rows(g["MXn"], m) for m in maps]) < 1e-13


@pytest.mark.parametrize("config", ["rayleigh_benard", "burgers"])
def test_gpu_config_steps_match_oracle(config, rng, cuda_lib):
    """The configuration at its own size (RB 256 x 64, Burgers 128) from its benchmark state: F to
    1e-12 and three steps (lower-order start-up included) against the oracle, 1e-12 relative L2 per
    field raised to 10x the oracle's own spread from the state perturbed by about one ulp (two
    seeds); each field's norm taken at least 1e-8 times the state's (the tau variables)."""
    import torch
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import IVPSolver
    from oracle.ivp import OracleProblem, SBDFStepper
    cfg = W.CONFIGS[config]
    P = W.problem(config)
    C0 = W.initial_state(config, P, seed=0)
    op = OracleProblem(P)
    solver = IVPSolver(P, scheme=cfg["scheme"], dt=cfg["dt"])
    out = solver.dev.zeros()
    solver.dev.F(solver.dev.to_device(C0), out)
    torch.cuda.synchronize()
    assert _rel(solver.dev.to_host(out), op.F(C0)) < 1e-12

    def oracle_run(C):
        st = SBDFStepper(op, int(cfg["scheme"][-1]), cfg["dt"])
        for _ in range(3):
            C = st.step(C)
        return C

    C = oracle_run(C0)
    tol = {k: 1e-12 for k in (v["name"] for v in P.tpl.variables)}
    for _ in range(2):
        Cp = oracle_run([c * (1 + 2.0 ** -52 * rng.standard_normal(c.shape)) for c in C0])
        for k, e in field_errors(P, Cp, C, floor=1e-8).items():
            tol[k] = max(tol[k], 10 * e)
    solver.set_state(C0)
    solver.run(3)
    errs = field_errors(P, solver.state_to_host(), C, floor=1e-8)
    assert all(errs[k] <= tol[k] for k in errs), (errs, tol)
