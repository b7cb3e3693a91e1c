"""GPU: the mixed-precision form (FP32 transforms, products and banded solves; FP64 refinement
residual, solution update, state and history; FP64 factorization) against the plain FP64 form,
which is itself parity-checked against the reference. Bar: 1e-6 relative L2 per field after 20
steps (the mixed form's target against the FP64 oracle)."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import field_errors, template

pytestmark = pytest.mark.gpu


def _state(P, rng):
    C = []
    for bi, b in enumerate(P.tpl.buckets):
        n_idx = np.maximum(b.col[:, 2], 0)
        z = rng.standard_normal((P.nsys[bi], b.n)).astype(np.complex128)
        if b.kind != "real":
            z = z + 1j * rng.standard_normal((P.nsys[bi], b.n))
        C.append(z * 0.05 * np.exp(-0.35 * n_idx))
    return C


def _workload_state(tname, P, rng):
    """The configurations' own initial states (conatus_gb300.workloads) at test resolutions."""
    from conatus_gb300 import workloads as W
    if tname.startswith("channel"):
        return W.channel_state(P, 0)
    if tname.startswith("rb"):
        return W.rayleigh_benard_state(P, 0)
    return W.burgers_state(P)


@pytest.mark.parametrize("tname,sizes,scheme,dt", [("rb_nz64", [64], "SBDF2", 1e-4),
                                                   ("channel_ny129", [24, 24], "SBDF3", 5e-3),
                                                   ("burgers_n128", None, "SBDF2", 1e-4)])
def test_mixed_matches_fp64(tname, sizes, scheme, dt, rng, cuda_lib):
    import torch
    from conatus_gb300.ivp import IVPSolver
    P = template(tname).instantiate(sizes)
    C0 = _workload_state(tname, P, rng)
    out = {}
    for prec in ("fp64", "fp32"):
        s = IVPSolver(P, scheme=scheme, dt=dt, precision=prec)
        s.set_state(C0)
        s.run_graph(20)
        torch.cuda.synchronize()
        out[prec] = s.dev.to_host(s.X)
    errs = field_errors(P, out["fp32"], out["fp64"])
    phys = {k: v for k, v in errs.items() if not k.startswith("tau")}
    assert max(phys.values()) < 1e-6, errs


@pytest.mark.parametrize("tname,sizes", [("channel_ny17", [16, 12]), ("rb_nz16", [32])])
def test_fp32_F_error(tname, sizes, rng, cuda_lib):
    """F in FP32 against F in FP64 on the configuration's state: relative L2 per bucket below 1e-5
    (FP32 transforms and products)."""
    import torch
    from conatus_gb300.ivp import DeviceProblem
    P = template(tname).instantiate(sizes)
    C0 = _workload_state(tname, P, rng)
    outs = {}
    for prec in ("fp64", "fp32"):
        d = DeviceProblem(P, precision=prec)
        o = d.zeros()
        d.F(d.to_device(C0), o)
        torch.cuda.synchronize()
        outs[prec] = o.cpu().numpy()
    err = np.linalg.norm(outs["fp32"] - outs["fp64"]) / np.linalg.norm(outs["fp64"])
    assert err < 1e-5, err


def test_monitor_fp64_reports_the_error_of_every_run(rng, cuda_lib):
    """IVPSolver.monitor_fp64: the FP32 form records its error against an FP64 shadow every
    ``every`` steps and at the end of each call; the recorded error is the one against a separate
    FP64 run, the shadow leaves the FP32 trajectory unchanged, and an error above the bound warns."""
    import warnings
    import torch
    from conatus_gb300.ivp import IVPSolver
    P = template("channel_ny129").instantiate([16, 16])
    C0 = _workload_state("channel_ny129", P, rng)
    plain = IVPSolver(P, scheme="SBDF3", dt=5e-3, precision="fp32")
    plain.set_state(C0)
    plain.run_graph(12)
    ref = IVPSolver(P, scheme="SBDF3", dt=5e-3, precision="fp64")
    ref.set_state(C0)
    ref.run_graph(12)
    mon = IVPSolver(P, scheme="SBDF3", dt=5e-3, precision="fp32")
    mon.set_state(C0)
    mon.monitor_fp64(every=5)
    mon.run_graph(7)
    mon.run(3)
    mon.step()
    mon.step()
    torch.cuda.synchronize()
    assert sorted(mon.mixed_error) == [5, 7, 10, 11, 12]
    assert torch.equal(mon.X, plain.X)                      # the shadow does not touch the run
    got = mon.mixed_error[12]
    want = field_errors(P, mon.dev.to_host(mon.X), ref.dev.to_host(ref.X))
    for k, v in got.items():
        assert abs(v - want[k]) <= 1e-6 * want[k] + 1e-300, (k, v, want[k])
    assert max(got.values()) < 1e-6 and mon.mixed_error_last == got
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        mon._mon_bound = 1e-30
        mon.step()
    assert any(issubclass(x.category, RuntimeWarning) and "FP64 shadow" in str(x.message) for x in w)
    fp64 = IVPSolver(P, scheme="SBDF3", dt=5e-3, precision="fp64")
    with pytest.raises(ValueError):
        fp64.monitor_fp64()
