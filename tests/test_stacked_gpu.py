"""GPU: an ensemble of Rayleigh-Benard cases stacked into one problem (conatus_gb300.template.
StackedProblem: one F pipeline pass and one solve launch for every case) gives each case's state of
the case run alone, FP64 and the FP32 form."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RAS = [2e4, 3e5, 4e6]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_stacked_equals_alone(precision, cuda_lib):
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import IVPSolver
    from conatus_gb300.template import StackedProblem
    tpl = W.load_template("rb_nz32_ra")
    S = StackedProblem(tpl, [32], [{"Ra": r} for r in RAS])
    dt = 2e-6
    alone, states = [], []
    for c, ra in enumerate(RAS):
        P = tpl.instantiate([32], None, {"Ra": ra})
        C0 = W.rayleigh_benard_state(P, seed=c)
        states.append(C0)
        s = IVPSolver(P, scheme="SBDF2", dt=dt, precision=precision)
        s.set_state(C0)
        s.run_graph(6)
        alone.append(s.state_to_host())
    st = IVPSolver(S, scheme="SBDF2", dt=dt, precision=precision)
    st.set_state(S.stack_states(states))
    st.run_graph(6)
    got = st.state_to_host()
    tol = 1e-13 if precision == "fp64" else 1e-12
    for c in range(len(RAS)):
        a = np.concatenate([x.ravel() for x in S.case_state(got, c)])
        b = np.concatenate([x.ravel() for x in alone[c]])
        assert np.all(np.isfinite(a))
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < tol, (c, np.linalg.norm(a - b) / np.linalg.norm(b))
