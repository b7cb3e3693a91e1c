"""CPU: the oracle's CN-family and IMEX Runge-Kutta steppers (oracle/ivp.py) against the
reference's own trajectories (tests/golden/scheme_*.npz, three steps from a seeded state with the
lower-order start-up), per field and per step, within 10x the reference's own rounding floor."""
from __future__ import annotations

import pytest

from _step_cases import SCHEME_FLOOR, field_errors, gather_state, load_scheme, scheme_fixtures, trajectory_tolerances


@pytest.mark.parametrize("fixture", scheme_fixtures())
def test_oracle_scheme_matches_reference(fixture):
    from oracle.ivp import CN, RK, CNStepper, OracleProblem, RKStepper
    P, g, maps, scheme = load_scheme(fixture)
    op = OracleProblem(P)
    st = RKStepper(op, scheme, float(g["dt"])) if scheme in RK else CNStepper(op, scheme, float(g["dt"]))
    assert scheme in RK or scheme in CN
    C = [gather_state(g["X0"], m) for m in maps]
    for k in range(g["Xs"].shape[0]):
        C = st.step(C)
        ref = [gather_state(g["Xs"][k], m) for m in maps]
        errs = field_errors(P, C, ref, floor=SCHEME_FLOOR)
        tols = trajectory_tolerances(P, g, maps, k)
        bad = {f: (errs[f], tols[f]) for f in errs if not errs[f] <= tols[f]}
        assert not bad, (k, bad)
