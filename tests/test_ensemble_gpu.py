"""GPU: the fused ensemble step (cng_fourier_ensemble_step) for Kuramoto-Sivashinsky members of
different sizes and periods in one launch, against the oracle (oracle/ivp.py, itself pinned to the
reference's KS step) member by member; the FP32 form against the FP64 form; graph replay."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import template

pytestmark = pytest.mark.gpu


def _oracle_run(N, L, C0, steps, dt):
    from oracle.ivp import OracleProblem, SBDFStepper
    P = template("ks").instantiate([int(N)], [float(L)])
    st = SBDFStepper(OracleProblem(P), 2, dt)
    # mode layout of the template: bucket 0 = mean mode (1 system), bucket 1 = modes 1..K-1
    C = [np.array([[C0[0]]], np.complex128), np.asarray(C0[1:], np.complex128).reshape(-1, 1)]
    for _ in range(steps):
        C = st.step(C)
    return np.concatenate([C[0].ravel(), C[1].ravel()])


def test_ensemble_matches_oracle(cuda_lib):
    import torch
    from conatus_gb300.ensemble import FourierEnsemble
    tpl = template("ks")
    N = np.array([64, 128, 256, 64, 128])
    L = np.array([22.0, 45.5, 99.0, 30.0, 60.0])
    ens = FourierEnsemble(tpl, N, L, scheme="SBDF2", dt=0.01, precision="fp64")
    C0 = ens.random_state(seed=3)
    ens.set_state(C0)
    ens.run(6)
    torch.cuda.synchronize()
    got = ens.state()
    for m in range(len(N)):
        ref = _oracle_run(N[m], L[m], C0[m], 6, 0.01)
        err = np.linalg.norm(got[m] - ref) / np.linalg.norm(ref)
        assert err < 1e-12, (m, err)


def test_ensemble_fp32_and_graphs(cuda_lib):
    import torch
    from conatus_gb300.ensemble import FourierEnsemble, ks_members
    tpl = template("ks")
    N, L = ks_members(257, seed=1)
    out = {}
    for prec in ("fp64", "fp32"):
        ens = FourierEnsemble(tpl, N, L, scheme="SBDF2", dt=0.01, precision=prec)
        ens.set_state(ens.random_state(seed=5))
        ens.run_graph(40)
        torch.cuda.synchronize()
        out[prec] = np.concatenate(ens.state())
    err = np.linalg.norm(out["fp32"] - out["fp64"]) / np.linalg.norm(out["fp64"])
    print("KS ensemble FP32 form vs FP64 after 40 steps:", err)
    assert err < 1e-6, err
    a = FourierEnsemble(tpl, N, L, scheme="SBDF2", dt=0.01, precision="fp64")
    a.set_state(a.random_state(seed=5))
    a.run(40)
    torch.cuda.synchronize()
    assert np.array_equal(np.concatenate(a.state()), out["fp64"])
