"""Serving (CPU): the seeded Poisson request stream, the pools' planned bytes and the
device-memory planner (no device work)."""
from __future__ import annotations

import numpy as np
import pytest

from conatus_gb300 import memory, serving
from conatus_gb300 import workloads as W


def test_stream_is_seeded_and_mixed():
    a = serving.poisson_stream(2000, seed=7)
    b = serving.poisson_stream(2000, seed=7)
    assert [(r.kind, r.params, r.steps, r.arrival) for r in a] == [(r.kind, r.params, r.steps, r.arrival) for r in b]
    kinds = np.array([r.kind for r in a])
    frac = {k: float(np.mean(kinds == k)) for k in ("burgers", "ks", "rb")}
    assert abs(frac["burgers"] - 0.5) < 0.04 and abs(frac["ks"] - 0.3) < 0.04 and abs(frac["rb"] - 0.2) < 0.04
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert abs(gaps.mean() - 1 / 200) < 0.1 / 200          # rate 200/s
    assert all(1000 <= r.steps <= 20000 for r in a)
    for r in a:
        p = r.params
        if r.kind == "burgers":
            assert p["N"] in serving.BURGERS_N and 1e-3 <= p["nu"] <= 1e-1
        elif r.kind == "ks":
            assert 22 <= p["L"] <= 100 and p["N"] >= 2 * p["L"] and p["N"] in (64, 128, 256)
        else:
            assert p["Nz"] in serving.RB_NZ and p["Nx"] == 4 * p["Nz"] and 1e4 <= p["Ra"] <= 1e7


@pytest.mark.parametrize("kind", ["burgers", "ks", "rb"])
def test_pool_plans_bytes(kind):
    """A pool's planned bytes: positive, growing with its slots, the FP32 form's copies on top of
    the FP64 factors; the problem of a Burgers / RB pool stacks one case per slot."""
    reqs = [r for r in serving.poisson_stream(200, seed=3) if r.kind == kind][:3]
    for r in reqs:
        key = serving.pool_key(r)
        a = serving.plan_pool(key, 2, "fp64")
        b = serving.plan_pool(key, 4, "fp64")
        assert 0 < a < b
        if kind != "ks":
            assert serving.plan_pool(key, 2, "fp32") > a
            _, S = serving._pool_problem(key, 3)
            assert S.ncase == 3 and S.n_total == 3 * sum(ns * bk.n for ns, bk in zip(S._nsys_case, S.tpl.buckets))


def test_ks_state_is_one_member_of_the_ensemble_state():
    """A KS request's initial state does not depend on its slot: one member of the ensemble's
    seeded state."""
    import types
    from conatus_gb300.ensemble import FourierEnsemble
    fake = types.SimpleNamespace(N=np.array([128]))
    ref = FourierEnsemble.random_state(fake, seed=17)[0]
    assert np.array_equal(serving.ks_state(128, 17), ref)


def test_plan_parts_scale():
    P = W.problem("rayleigh_benard")
    a = memory.plan_ivp(P, "SBDF2", "fp64")
    b = memory.plan_ivp(P, "SBDF2", "fp64", factor_sets=1)
    assert a["factors"] == 2 * b["factors"]
    assert a["total"] == sum(v for k, v in a.items() if k != "total")
    n_total = sum(ns * bk.n for ns, bk in zip(P.nsys, P.tpl.buckets))
    assert a["history"] == 2 * 2 * n_total * 16
    # band of the RB buckets as the factorization computes it
    assert [memory.bucket_band(bk) for bk in P.tpl.buckets] == [(12, 18), (12, 18)]
