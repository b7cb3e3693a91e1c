"""GPU: the partitioned solve of small FP64 batches (schedule ``autotune.partitioned_schedules()``:
one block of warps per system, the blocks of 32 columns swept at once, their windows carried from
block to block by the responses built at factorization) solves the systems the compact schedules
solve: the same solutions to the systems' conditioning, residuals within a stated factor of the
sequential sweeps', whole steps within rounding of the default schedule; the tuner takes it only
when the problem opts into it; and it refuses what it does not do (shared pairs, the FP32 form,
system ranges)."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import template

pytestmark = pytest.mark.gpu

CASES = [("rb_nz64", [256]), ("burgers_n128", None), ("rb_nz16", [32]), ("channel_ny17", [8, 8])]


def _part():
    from conatus_gb300 import autotune
    (p,) = autotune.partitioned_schedules()
    return p


@pytest.mark.parametrize("tname,sizes", CASES)
def test_partitioned_solve_matches_the_compact_solve(tname, sizes, rng, cuda_lib):
    import torch
    from conatus_gb300 import autotune
    from conatus_gb300.ivp import DeviceProblem
    P = template(tname).instantiate(sizes)
    dev = DeviceProblem(P, "fp64", share=False)
    dev.autotune = False
    a, b = 1.5e3, 1.0
    fs = dev.factor(a, b)
    rhs = dev.zeros()
    rhs.copy_(torch.as_tensor(rng.standard_normal(dev.n_total) + 1j * rng.standard_normal(dev.n_total),
                              device=rhs.device))
    ref, out, res, res0 = dev.zeros(), dev.zeros(), dev.zeros(), dev.zeros()
    autotune.apply(fs, 0)
    dev.solve(a, b, rhs, ref)
    dev.residual(a, b, ref, rhs, res0)
    autotune.apply(fs, _part())
    dev.solve(a, b, rhs, out)
    dev.residual(a, b, out, rhs, res)
    torch.cuda.synchronize()
    assert torch.isfinite(torch.view_as_real(out)).all()
    nrm = lambda v: float(torch.linalg.vector_norm(v))
    err = nrm(out - ref) / nrm(ref)
    rres, rres0 = nrm(res) / nrm(rhs), nrm(res0) / nrm(rhs)
    # the same solution to the systems' conditioning (the bound every schedule meets against
    # schedule 0). The residual runs larger than the sequential sweeps': a block's sweep of its
    # right-hand side and its response to the carried window are summed after the fact, and they
    # cancel where the block's U is ill-conditioned (measured: RB 2.4x, Burgers 13x, the channel's
    # ny = 17 systems 9x schedule 0's residual)
    assert rres < max(1e-10, 16 * rres0), (rres, rres0)
    assert err < 1e-10, err
    # a second solve on the same responses gives the same bits
    out2 = dev.zeros()
    dev.solve(a, b, rhs, out2)
    torch.cuda.synchronize()
    assert torch.equal(out, out2)


def test_partitioned_steps_follow_the_default_schedule(cuda_lib):
    """RB 256x64 SBDF2, 30 graph-replayed steps with the partitioned solve against the default
    compact schedule: the states agree to rounding."""
    import torch
    from conatus_gb300 import autotune, workloads as W
    from conatus_gb300.ivp import DeviceProblem, IVPSolver
    P = W.problem("rayleigh_benard")
    C0 = W.initial_state("rayleigh_benard", P, seed=0)
    out = []
    for sched in (0, _part()):
        dev = DeviceProblem(P, "fp64")
        dev.autotune = False
        s = IVPSolver(P, scheme="SBDF2", dt=1e-4, device_problem=dev)
        s.set_state(C0)
        s.step()                                       # the lower-order start-up's factor set
        s.step()
        for fs in dev._factors.values():
            autotune.apply(fs, sched)
        s.run_graph(30)
        torch.cuda.synchronize()
        out.append(s.X.clone())
    err = float(torch.linalg.vector_norm(out[1] - out[0]) / torch.linalg.vector_norm(out[0]))
    assert err < 1e-12, err


def test_tuner_picks_it_only_when_opted_into(cuda_lib):
    """RB 256x64's factor set: without the opt-in the tuner never times the partitioned solve; with
    it the schedule is a candidate."""
    from conatus_gb300 import autotune, workloads as W
    from conatus_gb300.ivp import DeviceProblem
    P = W.problem("rayleigh_benard")
    p = _part()
    dev = DeviceProblem(P, "fp64")
    dev.autotune = False
    fs = dev.factor(1.5e3, 1.0)
    assert p not in autotune.tune_solve(dev, (1.5e3, 1.0), fs, reps=2)
    dev2 = DeviceProblem(P, "fp64")
    dev2.autotune = False
    dev2.partitioned = True
    fs2 = dev2.factor(1.5e3, 1.0)
    times = autotune.tune_solve(dev2, (1.5e3, 1.0), fs2, reps=5)
    assert p in times
    print(f"\nRB 256x64 solve schedules (ms): {times}")


def test_partitioned_refusals(cuda_lib):
    import torch
    from conatus_gb300 import autotune
    from conatus_gb300._lib import call
    from conatus_gb300.ivp import DeviceProblem
    p = _part()
    # shared pairs: refused when the schedule is set
    P = template("channel_ny17").instantiate([8, 8])
    sh = DeviceProblem(P, "fp64", share=True)
    sh.autotune = False
    fs = sh.factor(1.5e3, 1.0)
    assert sh.shared
    with pytest.raises(ValueError, match="shared pairs"):
        autotune.apply(fs, p)
    # the FP32 form: refused at the solve
    R = template("rb_nz16").instantiate([32])
    d32 = DeviceProblem(R, "fp32")
    d32.autotune = False
    f32 = d32.factor(1.5e3, 1.0)
    autotune.apply(f32, p)
    with pytest.raises(ValueError, match="FP64 only"):
        d32.solve(1.5e3, 1.0, d32.zeros(), d32.zeros())
    # a system range: refused
    d64 = DeviceProblem(R, "fp64")
    d64.autotune = False
    f64 = d64.factor(1.5e3, 1.0)
    autotune.apply(f64, p)
    big = int(np.argmax(d64.nsys))
    x, rhs = d64.zeros(), d64.zeros()
    with pytest.raises(ValueError, match="system range"):
        d64._batch_call(f64, [(big, 0, 2)], rhs, x, None, 0, 0, 0)
    torch.cuda.synchronize()
