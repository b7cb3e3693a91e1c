"""GPU: the serving loop (conatus_gb300.serving): requests share pools advanced by one set of
launches per step. A run served in the mix gives bit for bit the state of the same run served
alone, and follows a plain solver's trajectory; a diverged member is stopped at the next check while
the others finish; admission keeps the planned bytes of the pools in flight under the budget; the
memory planner bounds the device bytes a run actually holds."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_stream(count, seed, steps=(20, 90)):
    from conatus_gb300 import serving
    reqs = serving.poisson_stream(count, rate=2000.0, seed=seed, steps=steps)
    for r in reqs:           # keep the problems small enough for a quick test
        if r.kind == "rb":
            r.params.update(Nz=32, Nx=64, Ra=min(r.params["Ra"], 1e6))
        if r.kind == "burgers":
            r.params["N"] = min(r.params["N"], 192)
    return reqs


SLOTS = {"burgers": 4, "ks": 8, "rb": 2}


def _copy(r):
    from conatus_gb300 import serving
    return serving.Request(r.rid, r.kind, dict(r.params), r.steps, 0.0)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_alone_equals_mix(precision, cuda_lib):
    """Every request's final state is bit for bit the same served in the mix (sharing pools with
    others, joining at other boundaries) and served alone."""
    from conatus_gb300 import serving
    reqs = _small_stream(12, seed=11)
    assert {r.kind for r in reqs} == {"burgers", "ks", "rb"}
    eng = serving.ServingEngine(budget_bytes=150e9, precision=precision, chunk=25, unroll=5, slots=SLOTS,
                                keep_results=True)
    stats = eng.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs) and stats["nonfinite"] == 0
    assert stats["peak_members"] > stats["peak_pools"]              # pools do hold several members
    for r in reqs:
        alone = _copy(r)
        serving.ServingEngine(budget_bytes=150e9, precision=precision, chunk=25, unroll=5, slots=SLOTS,
                              keep_results=True).run([alone], realtime=False)
        a = np.concatenate([np.ravel(x) for x in r.result])
        b = np.concatenate([np.ravel(x) for x in alone.result])
        assert np.all(np.isfinite(b)) and np.linalg.norm(b) > 0
        assert np.array_equal(a, b), (r.kind, r.params, float(np.abs(a - b).max()))


def test_pool_member_matches_a_plain_run(cuda_lib):
    """A Burgers member of a pool follows the plain solver's trajectory (the reference's
    lower-order start-up, then SBDF2) to rounding: the pool changes where a run sits, not what it
    computes."""
    from conatus_gb300 import serving, workloads as W
    from conatus_gb300.ivp import IVPSolver
    req = serving.Request(3, "burgers", dict(N=128, nu=0.01 / np.pi), 200, 0.0)
    serving.ServingEngine(slots=SLOTS, keep_results=True, chunk=50, unroll=5).run([req], realtime=False)
    P = W.load_template("burgers_n128_nu").instantiate(None, None, {"nu": 0.01 / np.pi})
    s = IVPSolver(P, scheme="SBDF2", dt=1e-4)
    s.set_state(W.burgers_state(P))
    s.run(200)
    ref = s.state_to_host()[0]
    got = req.result[0]
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-13


def test_diverged_member_stops_and_the_others_finish(cuda_lib):
    """A member whose state holds a NaN is retired at the next check with status "nonfinite";
    the other members of its pool finish unchanged."""
    from conatus_gb300 import serving
    import time
    t0 = time.perf_counter()
    now = lambda: time.perf_counter() - t0
    pool = serving.Pool(("burgers", 96, 1e-4), 4, chunk=50, unroll=5)
    reqs = [serving.Request(i, "burgers", dict(N=96, nu=0.01), 300, 0.0) for i in range(2)]
    for r in reqs:
        pool.place(r)
    pool.boundary(now)
    pool.launch()
    while not pool.idle():
        time.sleep(1e-3)
    for sl in pool._slices(1):                 # plant a NaN in member 1's state (host write)
        pool.main.X[sl][0] = float("nan")
    left = []
    while not pool.empty():
        while not pool.idle():
            time.sleep(1e-3)
        left += pool.boundary(now)
        pool.launch()
    assert [r.status for r in reqs] == ["done", "nonfinite"]
    assert reqs[1].result is None and np.all(np.isfinite(reqs[0].result[0]))


def test_admission_respects_budget(cuda_lib):
    from conatus_gb300 import serving
    reqs = _small_stream(10, seed=5, steps=(30, 60))
    keys = {serving.pool_key(r) for r in reqs}
    plans = {k: serving.plan_pool(k, SLOTS[k[0]]) for k in keys}
    assert len(keys) >= 2
    budget = 1.001 * max(plans.values())         # the largest pool fits, not beside another one
    eng = serving.ServingEngine(budget_bytes=budget, precision="fp64", chunk=20, unroll=5, slots=SLOTS)
    stats = eng.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs) and stats["nonfinite"] == 0
    assert stats["peak_planned_bytes"] <= budget and stats["budget_waits"] > 0
    adm = [r.admitted for r in sorted(reqs, key=lambda r: r.rid)]
    assert adm == sorted(adm)                     # first come, first served


def test_planner_bounds_device_bytes(cuda_lib):
    """Device bytes held by a run (driver free-memory drop plus torch's allocations, measured after
    the steady state is reached) against the plan: never above it, and not far below."""
    import torch
    from conatus_gb300 import memory
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import IVPSolver
    from conatus_gb300._lib import lib
    import ctypes

    def free_bytes():
        f, t = ctypes.c_uint64(), ctypes.c_uint64()
        lib().cng_mem_info(ctypes.byref(f), ctypes.byref(t))
        return int(f.value)

    P = W.problem("rayleigh_benard")
    for precision in ("fp64", "fp32"):
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        f0, a0, r0 = free_bytes(), torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        s = IVPSolver(P, scheme="SBDF2", dt=1e-4, precision=precision, factor_sets=1)
        s.set_state(W.rayleigh_benard_state(P, 0))
        s.run(4)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        f1, a1, r1 = free_bytes(), torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        lib_bytes = (f0 - f1) - (r1 - r0)
        held = lib_bytes + (a1 - a0)
        plan = memory.plan_ivp(P, "SBDF2", precision, factor_sets=1)["total"]
        assert held <= plan + (8 << 20), (precision, held, plan)     # driver page rounding
        assert plan <= 2.5 * held, (precision, held, plan)
        del s
