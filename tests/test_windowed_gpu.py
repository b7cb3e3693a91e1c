"""GPU: the windowed compact solve (schedules ``autotune.windowed_schedules()``: the two-systems
sweeps with only a window of each vector in shared memory, the finished rows in a per-handle
scratch) gives the bits of schedule 0: single solves in FP64 and in the FP32 form with its
refinement (shared pairs, the row-major copy of x, two refinement groups on two streams), system
ranges, and whole graph-replayed steps."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import template

pytestmark = pytest.mark.gpu

CASES = [("rb_nz64", [256], "fp64"), ("rb_nz64", [256], "fp32"), ("channel_ny17", [8, 8], "fp64"),
         ("channel_ny17", [8, 8], "fp32"), ("burgers_n128", None, "fp64"), ("rb_nz16", [32], "fp32")]


@pytest.mark.parametrize("tname,sizes,precision", CASES)
def test_windowed_solves_give_the_compact_bits(tname, sizes, precision, rng, cuda_lib):
    import torch
    from conatus_gb300 import autotune
    from conatus_gb300.ivp import DeviceProblem
    P = template(tname).instantiate(sizes)
    dev = DeviceProblem(P, precision)
    dev.autotune = False
    a, b = 1.5e3, 1.0
    fs = dev.factor(a, b)
    rhs = dev.zeros()
    rhs.copy_(torch.as_tensor(rng.standard_normal(dev.n_total) + 1j * rng.standard_normal(dev.n_total),
                              device=rhs.device))
    big = int(np.argmax([ns * bk.n for ns, bk in zip(dev.nsys, dev.tpl.buckets)]))
    if big in dev.shared:                              # a range of a pair: name its primary
        big = dev.shared[big]
    hi = min(dev.nsys[big], 6)
    fp32 = 1 if precision == "fp32" else 0
    # system ranges: several warp groups, and a single one (with 8 lanes per system a warp sweeps
    # two groups: the second half of its warp then has none)
    ranges = [(big, 2 if hi > 2 else 0, hi), (big, 2 if hi > 4 else 0, 4 if hi > 4 else hi)]
    ref = dev.zeros()
    ref_r = [dev.zeros() for _ in ranges]
    autotune.apply(fs, 0)
    dev.solve(a, b, rhs, ref)
    for rg, o in zip(ranges, ref_r):
        dev._batch_call(fs, [rg], rhs, o, None, fp32, 0, 0)
    torch.cuda.synchronize()
    wins = sorted(autotune.windowed_schedules())
    assert wins
    for s in wins:
        out = dev.zeros()
        autotune.apply(fs, s)
        dev.solve(a, b, rhs, out)
        torch.cuda.synchronize()
        assert torch.equal(out, ref), s
        for rg, o_ref in zip(ranges, ref_r):
            o = dev.zeros()
            dev._batch_call(fs, [rg], rhs, o, None, fp32, 0, 0)
            torch.cuda.synchronize()
            assert torch.equal(o, o_ref), (s, rg)


@pytest.mark.parametrize("config,fourier,precision", [("rayleigh_benard", None, "fp64"),
                                                      ("rayleigh_benard", None, "fp32"),
                                                      ("channel", [24, 24], "fp32")])
def test_windowed_steps_give_the_compact_bits(config, fourier, precision, cuda_lib):
    """Graph-replayed steps with a windowed schedule against schedule 0 from the same state: the
    same bits."""
    import torch
    from conatus_gb300 import autotune, workloads as W
    from conatus_gb300.ivp import DeviceProblem, IVPSolver
    P = W.problem(config, fourier)
    cfg = W.CONFIGS[config]
    C0 = W.initial_state(config, P, seed=0)
    out = []
    for sched in (0, min(autotune.windowed_schedules())):
        dev = DeviceProblem(P, precision)
        dev.autotune = False
        s = IVPSolver(P, scheme=cfg["scheme"], dt=cfg["dt"], device_problem=dev)
        s.set_state(C0)
        for _ in range(s.ring):                        # the start-up's factor sets
            s.step()
        for fs in dev._factors.values():
            autotune.apply(fs, sched)
        s.run_graph(10)
        torch.cuda.synchronize()
        out.append(s.X.clone())
    assert torch.equal(out[0], out[1])
