"""GPU: problems of different sizes advanced as one GroupedProblem (every kernel of a step one launch
for all of them: grouped F stages, grouped M X and residual, the multi-bucket solve) give each
problem the bits it has alone, FP64 and the FP32 form; F alone and grouped agree bit for bit; the
grouped entry point refuses handles it cannot run together."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [(32, [2e4, 3e5]), (48, [5e4]), (64, [1e4, 4e6])]


def _stacks(nx_factor=2):
    from conatus_gb300 import workloads as W
    from conatus_gb300.template import StackedProblem
    out = []
    for nz, ras in CASES:
        tpl = W.load_template(f"rb_nz{nz}_ra")
        S = StackedProblem(tpl, [nx_factor * nz], [{"Ra": r} for r in ras])
        states = [W.rayleigh_benard_state(tpl.instantiate([nx_factor * nz], None, {"Ra": r}), seed=c)
                  for c, r in enumerate(ras)]
        out.append((S, S.stack_states(states)))
    return out


def _device(P, precision):
    from conatus_gb300.ivp import DeviceProblem
    d = DeviceProblem(P, precision)
    d.autotune = False            # the default compact schedule on both sides
    return d


@pytest.mark.parametrize("precision,scheme", [("fp64", "SBDF2"), ("fp32", "SBDF2"), ("fp64", "RK443"),
                                              ("fp64", "CNAB2")])
def test_grouped_steps_are_each_problem_alone(precision, scheme, cuda_lib):
    import torch
    from conatus_gb300.ivp import IVPSolver
    from conatus_gb300.template import GroupedProblem
    dt = 2e-6
    stacks = _stacks()
    alone = []
    for S, C0 in stacks:
        s = IVPSolver(S, scheme=scheme, dt=dt, device_problem=_device(S, precision))
        s.set_state(C0)
        s.run_graph(6)
        torch.cuda.synchronize()
        alone.append([torch.as_tensor(x) for x in s.state_to_host()])
    G = GroupedProblem([S for S, _ in stacks])
    g = IVPSolver(G, scheme=scheme, dt=dt, device_problem=_device(G, precision))
    g.set_state(G.stack_states([C0 for _, C0 in stacks]))
    g.run_graph(6)
    torch.cuda.synchronize()
    got = g.state_to_host()
    for k, ref in enumerate(alone):
        mine = G.group_state(got, k)
        assert all(np.isfinite(x).all() for x in mine)
        assert all(torch.equal(torch.as_tensor(x), y) for x, y in zip(mine, ref)), (precision, scheme, k)
    # one launch per kernel for all groups: the grouped step launches no more kernels than one
    # group's step, and fewer than the groups' steps together
    one = IVPSolver(stacks[0][0], scheme=scheme, dt=dt, device_problem=_device(stacks[0][0], precision))
    one.set_state(stacks[0][1])
    one.run(2)
    assert g.launches_per_step() <= one.launches_per_step()


def test_grouped_F_is_F_alone(cuda_lib):
    import torch
    from conatus_gb300.template import GroupedProblem
    stacks = _stacks()
    G = GroupedProblem([S for S, _ in stacks])
    dg = _device(G, "fp64")
    X = dg.to_device(G.stack_states([C0 for _, C0 in stacks]))
    out = dg.zeros()
    dg.F(X, out)
    torch.cuda.synchronize()
    got = dg.to_host(out)
    for k, (S, C0) in enumerate(stacks):
        d = _device(S, "fp64")
        o = d.zeros()
        d.F(d.to_device(C0), o)
        torch.cuda.synchronize()
        ref = d.to_host(o)
        assert all(np.array_equal(x, y) for x, y in zip(G.group_state(got, k), ref)), k
    # unpack, Chebyshev backward, x backward, products, x forward, Chebyshev forward, pack, and the
    # constant part: one launch each for the three problems
    assert dg.f_launches() == 7 + (1 if dg.has_b0 else 0)


def test_grouped_entry_refuses(cuda_lib):
    from conatus_gb300._lib import call
    from conatus_gb300.template import GroupedProblem
    stacks = _stacks()
    G = GroupedProblem([S for S, _ in stacks[:2]])
    d64, d32 = _device(G, "fp64"), _device(stacks[0][0], "fp32")
    x, out = d64.zeros(), d64.zeros()
    h = d64._rhs_all
    dup = (ctypes.c_void_p * 2)(h[0].value, h[0].value)
    with pytest.raises(ValueError, match="twice"):
        call("cng_rhs_evaluate_group", 2, dup, x.data_ptr(), out.data_ptr(), None)
    mixed = (ctypes.c_void_p * 2)(h[0].value, d32._rhs.value)
    with pytest.raises(ValueError, match="precision"):
        call("cng_rhs_evaluate_group", 2, mixed, x.data_ptr(), out.data_ptr(), None)
    with pytest.raises(ValueError, match="alias"):
        call("cng_rhs_evaluate_group", 2, d64._rhs_arr, x.data_ptr(), x.data_ptr(), None)


def test_planned_bytes_bound_the_grouped_solver(cuda_lib):
    """The planner's prediction for a grouped problem bounds the device bytes its solver holds
    (driver free-memory drop plus torch's allocations, after the steady state)."""
    import gc
    import torch
    from conatus_gb300 import memory
    from conatus_gb300._lib import lib
    from conatus_gb300.ivp import IVPSolver
    from conatus_gb300.template import GroupedProblem

    def free_bytes():
        f, t = ctypes.c_uint64(), ctypes.c_uint64()
        lib().cng_mem_info(ctypes.byref(f), ctypes.byref(t))
        return int(f.value)

    stacks = _stacks(4)
    G = GroupedProblem([S for S, _ in stacks])
    for precision in ("fp64", "fp32"):
        gc.collect()
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        f0, a0, r0 = free_bytes(), torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        s = IVPSolver(G, scheme="SBDF2", dt=2e-6, precision=precision, factor_sets=1)
        s.set_state(G.stack_states([C0 for _, C0 in stacks]))
        s.run(4)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        f1, a1, r1 = free_bytes(), torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        held = (f0 - f1) - (r1 - r0) + (a1 - a0)
        plan = memory.plan_ivp(G, "SBDF2", precision, factor_sets=1)["total"]
        assert held <= plan + (8 << 20), (precision, held, plan)
        del s
