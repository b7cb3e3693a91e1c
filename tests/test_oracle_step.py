"""CPU: the oracle restatement of the IMEX step (oracle/ivp.py), on the mode layout of the problem
templates, against the reference's own IVPSolver step (golden fixtures), teacher-forced from the
reference's state and history: F(X_n) to 1e-12 relative L2, X_{n+1} to 1e-12 relative L2 per
field, raised per field to 10x the reference's own rounding floor where its implicit solve
amplifies rounding beyond that (``field_tolerances``)."""
from __future__ import annotations

from collections import deque

import numpy as np
import pytest

from _step_cases import (STEP_CASES, field_errors, field_tolerances, gather_rows, gather_state,
                         load_step, scatter_state)
from oracle.ivp import OracleProblem, SBDFStepper

TOL = 1e-12


def _rel(a, b):
    a, b = np.concatenate([np.ravel(x) for x in a]), np.concatenate([np.ravel(x) for x in b])
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("fixture", list(STEP_CASES))
def test_layout_round_trip(fixture):
    P, g, maps = load_step(fixture)
    C = [gather_state(g["Xn"], m) for m in maps]
    X = scatter_state(C, maps, g["Xn"].shape[0])
    assert np.array_equal(X, g["Xn"]) or _rel([X], [g["Xn"]]) < 1e-15


@pytest.mark.parametrize("fixture", list(STEP_CASES))
def test_oracle_F_matches_reference(fixture):
    P, g, maps = load_step(fixture)
    op = OracleProblem(P)
    C = [gather_state(g["Xn"], m) for m in maps]
    R = op.F(C)
    R_ref = [gather_rows(g["Fn"], m) for m in maps]
    assert _rel(R, R_ref) < TOL


@pytest.mark.parametrize("fixture", list(STEP_CASES))
def test_oracle_MX_matches_reference(fixture):
    P, g, maps = load_step(fixture)
    op = OracleProblem(P)
    C = [gather_state(g["Xn"], m) for m in maps]
    # MXn: the M X_n the reference's step pushed on its history (rows in the reference's layout)
    MX = op.MX(C)
    MX_ref = [gather_rows(g["MXn"], m) for m in maps]
    num = sum(float(np.sum(np.abs(a - b) ** 2)) for a, b in zip(MX, MX_ref))
    den = sum(float(np.sum(np.abs(b) ** 2)) for b in MX_ref)
    assert den > 0 and (num / den) ** 0.5 < 1e-14, (num / den) ** 0.5


@pytest.mark.parametrize("fixture", list(STEP_CASES))
def test_oracle_step_matches_reference(fixture):
    P, g, maps = load_step(fixture)
    op = OracleProblem(P)
    C = [gather_state(g["Xn"], m) for m in maps]
    st = SBDFStepper(op, int(g["order"]), float(g["dt"]))
    order = int(g["order"])
    st.MXh = deque([[gather_rows(h, m) for m in maps] for h in g["MXh"][:order - 1]])
    st.Fh = deque([[gather_rows(h, m) for m in maps] for h in g["Fh"][:order - 1]])
    C1 = st.step(C)
    C1_ref = [gather_state(g["Xn1"], m) for m in maps]
    errs = field_errors(P, C1, C1_ref)
    tols = field_tolerances(P, g, maps)
    assert all(errs[k] <= tols[k] for k in errs), (errs, tols)
