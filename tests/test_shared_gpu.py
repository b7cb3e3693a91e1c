"""GPU: shared factors of the channel's sign-similar buckets (the reference's SharedFactor,
python/conatus/timestep/shared_factors.py:1-40): the (kx, -kz) systems solved with the (kx, +kz)
factors in the same sweep give the bits of their own factorization's solve, in both precisions,
alone and inside whole steps; the shared set holds no factors for the partner."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import template

pytestmark = pytest.mark.gpu


def _devices(P, precision):
    from conatus_gb300.ivp import DeviceProblem
    out = []
    for share in (True, False):
        d = DeviceProblem(P, precision, share=share)
        d.autotune = False                  # the same compact schedule on both sides
        out.append(d)
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name,sizes", [("channel_ny17", [16, 12]), ("channel_ny129", [24, 24])])
def test_shared_solve_is_bitwise_the_unshared_solve(name, sizes, precision, rng, cuda_lib):
    import torch
    P = template(name).instantiate(sizes)
    sh, un = _devices(P, precision)
    a, b = 11 / 6 / 5e-3, 1.0
    fs = sh.factor(a, b)
    assert sh.shared == {4: 3} and fs[4].h is None
    assert un.shared == {} and all(h.h is not None for h in un.factor(a, b))
    rhs = sh.zeros()
    rhs.real.normal_()
    rhs.imag.normal_()
    xs, xu = sh.zeros(), un.zeros()
    sh.solve(a, b, rhs, xs)
    un.solve(a, b, rhs, xu)
    torch.cuda.synchronize()
    assert torch.equal(xs, xu)


def test_shared_steps_are_bitwise_the_unshared_steps(rng, cuda_lib):
    """Whole SBDF3 steps (graphs) with and without sharing: the same states bit for bit, FP64 and
    the FP32 form (FP32 solves with FP64 refinement)."""
    import torch
    from conatus_gb300 import workloads as W
    from conatus_gb300.ivp import IVPSolver
    P = template("channel_ny129").instantiate([16, 16])
    C0 = W.initial_state("channel", P, seed=3)
    for precision in ("fp64", "fp32"):
        sh, un = _devices(P, precision)
        out = []
        for dev in (sh, un):
            s = IVPSolver(P, scheme="SBDF3", dt=5e-3, device_problem=dev)
            s.set_state(C0)
            s.run_graph(6)
            torch.cuda.synchronize()
            out.append(s.X.clone())
        assert torch.equal(out[0], out[1]), precision


def test_shared_solve_matches_the_compiled_reference(cuda_lib):
    """The partner bucket's solve with shared factors against the reference's own BorderedBanded on
    the partner's matrices (oracle restatement pinned to the compiled reference)."""
    import torch
    from oracle.banded import BorderedBandedBatch
    P = template("channel_ny17").instantiate([8, 8])
    sh, _ = _devices(P, "fp64")
    a, b = 11 / 6 / 5e-3, 1.0
    sh.factor(a, b)
    rng = np.random.default_rng(5)
    bk = P.tpl.buckets[4]
    vals = a * P.values(4, "M") + b * P.values(4, "L")
    ref = BorderedBandedBatch([(bk.n, bk.indptr, bk.indices, v) for v in vals], list(range(bk.r)),
                              dtype=np.complex128)
    rhs_h = [np.zeros((ns, bb.n), np.complex128) for ns, bb in zip(P.nsys, P.tpl.buckets)]
    rhs_h[4] = rng.standard_normal((P.nsys[4], bk.n)) + 1j * rng.standard_normal((P.nsys[4], bk.n))
    x = sh.zeros()
    sh.solve(a, b, sh.to_device(rhs_h), x)
    torch.cuda.synchronize()
    xg = sh.to_host(x)[4]
    xr = ref.solve(rhs_h[4])
    import scipy.sparse as sp
    for m in range(P.nsys[4]):
        A = sp.csr_matrix((vals[m], bk.indices, bk.indptr), shape=(bk.n, bk.n)).toarray()
        tol = max(1e-12, 0.1 * np.finfo(float).eps * np.linalg.cond(A))    # the banded tests' bound
        assert np.linalg.norm(xg[m] - xr[m]) / np.linalg.norm(xr[m]) < tol, m


def test_band_kernel_and_split_schedules_refuse_partners(cuda_lib):
    """A shared pair needs a compact two-system schedule: the band kernel and the split-lane
    schedules refuse it at the solve, the partitioned solve already when it is set (the autotuner
    skips them all)."""
    from conatus_gb300 import autotune
    P = template("channel_ny17").instantiate([8, 8])
    sh, _ = _devices(P, "fp64")
    a, b = 11 / 6 / 5e-3, 1.0
    fs = sh.factor(a, b)
    rhs, x = sh.zeros(), sh.zeros()
    part = autotune.partitioned_schedules()
    for sched in [-1] + sorted(autotune.split_schedules()):
        with pytest.raises(ValueError):
            autotune.apply(fs, sched)
            assert sched not in part                     # refused where it is set
            sh.solve(a, b, rhs, x)
    autotune.apply(fs, 0)
    sh.solve(a, b, rhs, x)


def test_planned_bytes_bound_the_shared_solver(cuda_lib):
    """The planner's prediction with sharing still bounds the device bytes a solver holds (driver
    free-memory drop plus torch's allocations, after the steady state), and sharing lowers them."""
    import ctypes
    import gc
    import torch
    from conatus_gb300 import memory, workloads as W
    from conatus_gb300._lib import lib
    from conatus_gb300.ivp import IVPSolver

    def free_bytes():
        f, t = ctypes.c_uint64(), ctypes.c_uint64()
        lib().cng_mem_info(ctypes.byref(f), ctypes.byref(t))
        return int(f.value)

    P = template("channel_ny129").instantiate([32, 32])
    held = {}
    for share in (True, False):
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        f0, a0, r0 = free_bytes(), torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        from conatus_gb300.ivp import DeviceProblem
        s = IVPSolver(P, scheme="SBDF3", dt=5e-3, factor_sets=1,
                      device_problem=DeviceProblem(P, "fp64", factor_sets=1, share=share))
        s.set_state(W.initial_state("channel", P, seed=0))
        s.run(4)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        f1, a1, r1 = free_bytes(), torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
        held[share] = (f0 - f1) - (r1 - r0) + (a1 - a0)
        plan = memory.plan_ivp(P, "SBDF3", factor_sets=1, share=share)["total"]
        assert held[share] <= plan + (8 << 20), (share, held[share], plan)
        assert s.dev.shared == ({4: 3} if share else {})
        del s
        gc.collect()
    assert held[True] < held[False]


@pytest.mark.parametrize("share", [True, False])
def test_system_ranges_solve_alike(share, cuda_lib):
    """A bucket solved in two launches over system ranges (the FP32 refinement's two streams)
    gives the bits of one launch over the whole batch, and the ranged residual those of the whole."""
    import torch
    from conatus_gb300.ivp import DeviceProblem
    P = template("channel_ny129").instantiate([24, 24])
    dev = DeviceProblem(P, "fp32", share=share)
    dev.autotune = False
    a, b = 11 / 6 / 5e-3, 1.0
    fs = dev.factor(a, b)
    dev.ensure_residual(a, b)
    rhs = dev.zeros()
    rhs.real.normal_()
    rhs.imag.normal_()
    whole, parts = dev.zeros(), dev.zeros()
    nb = len(fs)
    dev._batch_call(fs, list(range(nb)), rhs, whole, None, 1, 0, 0)
    big = 3
    h = dev.nsys[big] // 2 & ~1
    # shared: bucket 4 follows bucket 3's ranges; unshared: solved whole in the first launch
    rest = [bi for bi in range(nb) if bi not in (big, 4)] + ([] if share else [4])
    dev._batch_call(fs, rest + [(big, 0, h)], rhs, parts, None, 1, 0, 0)
    dev._batch_call(fs, [(big, h, dev.nsys[big])], rhs, parts, None, 1, 0, 0)
    torch.cuda.synchronize()
    assert torch.equal(whole, parts)
    r1, r2 = dev.zeros(), dev.zeros()
    dev.residual(a, b, whole, rhs, r1)
    dev.residual(a, b, whole, rhs, r2, buckets=[(bi, 0, dev.nsys[bi]) for bi in range(nb) if bi != big]
                 + [(big, 0, h), (big, h, dev.nsys[big])])
    torch.cuda.synchronize()
    assert torch.equal(r1, r2)
