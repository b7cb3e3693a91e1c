"""CPU: the host side of GroupedProblem (problems of different sizes in one mode layout, every kernel
of a step one launch for all of them): the joint bucket list and offsets, per-bucket dispatch to
the owning problem, the state round trip, shared-factor pairs carried with their offsets, the refusal
of problems with other variables, and the launch counts a grouped solver reports."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import template


def _groups():
    from conatus_gb300.template import StackedProblem
    a = StackedProblem(template("rb_nz32_ra"), [64], [{"Ra": 1e4}, {"Ra": 2e5}])
    b = StackedProblem(template("rb_nz48_ra"), [96], [{"Ra": 3e4}])
    return a, b


def test_joint_layout_and_dispatch():
    from conatus_gb300.template import GroupedProblem
    a, b = _groups()
    G = GroupedProblem([a, b])
    nba, nbb = len(a.tpl.buckets), len(b.tpl.buckets)
    assert G.group_buckets == [list(range(nba)), list(range(nba, nba + nbb))]
    assert G.nsys == list(a.nsys) + list(b.nsys)
    assert G.ncase == 3
    sizes = [ns * bk.n for ns, bk in zip(G.nsys, G.tpl.buckets)]
    assert G.offsets == list(np.concatenate([[0], np.cumsum(sizes)[:-1]]))
    assert G.n_total == sum(sizes) == a.n_total + b.n_total
    for bi in range(nbb):
        k = nba + bi
        assert G.tpl.buckets[k] is b.tpl.buckets[bi]
        assert np.array_equal(G.values(k, "L"), b.values(bi, "L"))
        assert np.array_equal(G.values(k, "M"), b.values(bi, "M"))
        assert np.array_equal(G.mono_values(k), b.mono_values(bi))
        assert G.d_active(k) == b.d_active(bi)
        ga = [(np.asarray(c), np.asarray(s)) for c, s in G.split_terms(k)]
        gb = [(np.asarray(c), np.asarray(s)) for c, s in b.split_terms(bi)]
        assert len(ga) == len(gb) and all(np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
                                          for x, y in zip(ga, gb))
    assert G.real_unknowns() == a.real_unknowns() + b.real_unknowns()
    assert len(G.b0_dense()) == nba + nbb
    rng = np.random.default_rng(0)
    sa = [rng.standard_normal((ns, bk.n)) for ns, bk in zip(a.nsys, a.tpl.buckets)]
    sb = [rng.standard_normal((ns, bk.n)) for ns, bk in zip(b.nsys, b.tpl.buckets)]
    C = G.stack_states([sa, sb])
    assert all(np.array_equal(x, y) for x, y in zip(G.group_state(C, 0), sa))
    assert all(np.array_equal(x, y) for x, y in zip(G.group_state(C, 1), sb))
    with pytest.raises(ValueError):
        G.stack_states([sa])


def test_sign_pairs_carry_offsets():
    from conatus_gb300.template import GroupedProblem
    t = template("channel_ny17")
    p1, p2 = t.instantiate([8, 8]), t.instantiate([12, 16])
    G = GroupedProblem([p1, p2])
    own = t.sign_pairs()
    nb = len(t.buckets)
    got = G.tpl.sign_pairs()
    assert set(got) == set(own) | {j + nb for j in own}
    for j, (i, dr, dc) in own.items():
        assert got[j + nb][0] == i + nb
        assert np.array_equal(got[j + nb][1], dr) and np.array_equal(got[j + nb][2], dc)


def test_planner_counts_every_group():
    """The memory planner of a grouped problem: one F evaluator per group, the joint vectors and
    every bucket's operators and factors; no more than the groups planned apart."""
    from conatus_gb300 import memory
    from conatus_gb300.template import GroupedProblem
    a, b = _groups()
    G = GroupedProblem([a, b])
    for prec in ("fp64", "fp32"):
        pg, pa, pb = (memory.plan_ivp(x, "SBDF2", prec) for x in (G, a, b))
        for part in ("rhs_work", "state", "history", "operators", "factors"):
            assert pg[part] == pa[part] + pb[part], (prec, part)
        assert max(pa["total"], pb["total"]) < pg["total"] <= pa["total"] + pb["total"]


def test_other_variables_refused():
    from conatus_gb300.template import GroupedProblem
    a, _ = _groups()
    with pytest.raises(ValueError, match="same variables"):
        GroupedProblem([a, template("burgers_n128").instantiate()])
    with pytest.raises(ValueError):
        GroupedProblem([])
