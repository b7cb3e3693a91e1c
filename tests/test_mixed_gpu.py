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


@pytest.mark.parametrize("tname,sizes,scheme,dt", [("rb_nz16", [32], "SBDF2", 1e-4),
                                                   ("channel_ny17", [16, 12], "SBDF3", 5e-3),
                                                   ("burgers_n128", None, "SBDF2", 1e-4)])
def test_mixed_matches_fp64(tname, sizes, scheme, dt, rng, cuda_lib):
    import torch
    from conatus_gb300.ivp import IVPSolver
    P = template(tname).instantiate(sizes)
    C0 = _state(P, rng)
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
