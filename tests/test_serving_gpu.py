"""GPU: the serving loop (conatus_gb300.serving). A run served in the mix gives bit for bit the
state of the same run served alone; admission keeps the planned bytes of the runs in flight under
the budget; the memory planner bounds the device bytes a run actually holds."""
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


def _alone(req, precision, chunk, unroll):
    from conatus_gb300 import serving
    s = serving.Session(serving.prepare(req, precision), precision)
    while s.remaining:
        s.launch(chunk, unroll)
    return s.result()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_alone_equals_mix(precision, cuda_lib):
    from conatus_gb300 import serving
    reqs = _small_stream(9, seed=11)
    assert {r.kind for r in reqs} == {"burgers", "ks", "rb"}
    eng = serving.ServingEngine(budget_bytes=150e9, precision=precision, chunk=25, unroll=5, keep_results=True)
    stats = eng.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs) and stats["peak_active"] > 1 and stats["nonfinite"] == 0
    for r in reqs:
        got = r.result
        ref = _alone(serving.Request(r.rid, r.kind, dict(r.params), r.steps, 0.0), precision, 25, 5)
        a = np.concatenate([np.ravel(x) for x in got])
        b = np.concatenate([np.ravel(x) for x in ref])
        assert np.all(np.isfinite(b)) and np.linalg.norm(b) > 0
        assert np.array_equal(a, b), (r.kind, r.params, float(np.abs(a - b).max()))


def test_admission_respects_budget(cuda_lib):
    from conatus_gb300 import serving
    reqs = _small_stream(8, seed=5, steps=(30, 60))
    plans = [serving.prepare(r, "fp64").bytes for r in reqs]
    budget = 2.2 * max(plans)           # at most a few runs in flight at a time
    eng = serving.ServingEngine(budget_bytes=budget, precision="fp64", chunk=20, unroll=5)
    stats = eng.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs)
    assert stats["peak_planned_bytes"] <= budget
    assert stats["peak_active"] < len(reqs)
    # first come, first served
    adm = [r.admitted for r in sorted(reqs, key=lambda r: r.rid)]
    assert adm == sorted(adm)


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
