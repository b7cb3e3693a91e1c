"""CPU: stacked cases of a parameter-linear template (conatus_gb300.template.StackedProblem): the
systems of each case are those of the case alone, the refinement residual's split terms rebuild L
of every system, and the per-case state views round-trip."""
from __future__ import annotations

import numpy as np

from conatus_gb300 import workloads as W
from conatus_gb300.ivp import DeviceProblem
from conatus_gb300.template import StackedProblem

RAS = [1e4, 2.5e5, 3e6]


def _stack():
    tpl = W.load_template("rb_nz32_ra")
    return tpl, StackedProblem(tpl, [16], [{"Ra": r} for r in RAS])


def test_cases_are_the_problems_alone():
    tpl, S = _stack()
    for c, ra in enumerate(RAS):
        P = tpl.instantiate([16], None, {"Ra": ra})
        for bi in range(len(tpl.buckets)):
            ns = P.nsys[bi]
            for which in ("M", "L"):
                a = S.values(bi, which)[c * ns:(c + 1) * ns]
                b = P.values(bi, which)
                assert np.allclose(a, b, rtol=1e-15, atol=1e-12 * np.abs(b).max()), (bi, which)
            assert np.array_equal(S.modes[bi][c * ns:(c + 1) * ns], P.modes[bi])
            assert np.all(S.case_of[bi][c * ns:(c + 1) * ns] == c)
    assert S.n_total == sum(tpl.instantiate([16], None, {"Ra": r}).n_total for r in RAS)


def test_split_terms_rebuild_L():
    tpl, S = _stack()
    for bi, b in enumerate(tpl.buckets):
        terms = S.split_terms(bi)
        L = S.values(bi, "L")
        rebuilt = sum(np.outer(scale, row) for row, scale in terms)
        assert np.allclose(rebuilt, L, rtol=1e-14, atol=1e-12 * np.abs(L).max())
        split = DeviceProblem._split_operator(b, [row for row, _ in terms])
        assert split is not None                 # purely real or imaginary coefficients


def test_case_state_round_trip(rng=np.random.default_rng(0)):
    tpl, S = _stack()
    states = []
    for c in range(S.ncase):
        P = tpl.instantiate([16], None, {"Ra": RAS[c]})
        states.append([rng.standard_normal((ns, b.n)) + 0j for ns, b in zip(P.nsys, tpl.buckets)])
    st = S.stack_states(states)
    for c in range(S.ncase):
        for a, b in zip(S.case_state(st, c), states[c]):
            assert np.array_equal(a, b)
