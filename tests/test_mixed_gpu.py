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
