"""GPU, the channel 192x129x192 at full size (the benchmark workload: 18241 systems, 19 M real
unknowns), checked through properties that need no reference step at this size:

* F on the GPU against the oracle's F on the host (the reference's polynomial form restated), on the
  same seeded state: 1e-12 relative L2 per bucket;
* one FP64 step solves its implicit equations: for sampled systems of every bucket, the GPU's
  X_{n+1} against the oracle's bordered-banded solve (banded.hpp restated, LAPACK) of the same
  a M + b L and the same right-hand side, within 1e-12 widened to 0.1 eps cond(A);
* the FP32 form stays within the 1e-6 budget of the FP64 form, per field, after 5 steps."""
from __future__ import annotations

import os

import numpy as np
import pytest

from _step_cases import field_errors

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def channel():
    from conatus_gb300 import workloads as W
    P = W.problem("channel", None)
    return P, W.CONFIGS["channel"], W.initial_state("channel", P, seed=0)


def test_full_channel_F_matches_oracle(channel, cuda_lib):
    import torch
    import oracle.ivp as O
    from conatus_gb300.ivp import DeviceProblem
    P, cfg, C0 = channel
    dev = DeviceProblem(P, "fp64")
    X = dev.to_device(C0)
    out = dev.zeros()
    dev.F(X, out)
    torch.cuda.synchronize()
    got = dev.to_host(out)
    del dev, X, out
    torch.cuda.empty_cache()
    O.WORKERS = os.cpu_count()
    try:
        ref = O.OracleProblem(P).F(C0)
    finally:
        O.WORKERS = None
    for bi, (g, r) in enumerate(zip(got, ref)):
        err = np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-300)
        assert err < 1e-12, (bi, err)


def test_full_channel_step_solves_its_equations(channel, cuda_lib, rng):
    import torch
    from conatus_gb300.ivp import IVPSolver
    from oracle.banded import BorderedBanded
    P, cfg, C0 = channel
    s = IVPSolver(P, scheme=cfg["scheme"], dt=cfg["dt"], precision="fp64")
    s.set_state(C0)
    (a, b_), = s._step_keys()
    s.step()
    torch.cuda.synchronize()
    X1, R = s.dev.to_host(s.X), s.dev.to_host(s.R)
    for bi, bk in enumerate(P.tpl.buckets):
        Mv, Lv = P.values(bi, "M"), P.values(bi, "L")
        for m in sorted({0, P.nsys[bi] - 1, int(rng.integers(P.nsys[bi]))}):
            vals = a * (Mv[m] if Mv.ndim == 2 else Mv) + b_ * Lv[m]
            ref = BorderedBanded(bk.n, bk.indptr, bk.indices, vals, list(range(bk.r))).solve(R[bi][m][None, :])[0]
            A = np.zeros((bk.n, bk.n), complex)
            np.add.at(A, (bk.coo_rows(), bk.indices), vals)
            tol = max(1e-12, 0.1 * np.finfo(float).eps * np.linalg.cond(A))
            err = np.linalg.norm(X1[bi][m] - ref) / np.linalg.norm(ref)
            assert err < tol, (bi, m, err, tol)


def test_full_channel_fp32_form_within_budget(channel, cuda_lib):
    import torch
    from conatus_gb300.ivp import IVPSolver
    P, cfg, C0 = channel
    out = {}
    for prec in ("fp64", "fp32"):
        s = IVPSolver(P, scheme=cfg["scheme"], dt=cfg["dt"], precision=prec)
        s.set_state(C0)
        s.run_graph(5)
        out[prec] = s.state_to_host()
        del s
        torch.cuda.empty_cache()
    errs = field_errors(P, out["fp32"], out["fp64"])
    assert max(v for k, v in errs.items() if not k.startswith("tau")) < 1e-6, errs
