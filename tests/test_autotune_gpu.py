"""GPU: the solve schedules picked by the autotuner (conatus_gb300.autotune) all solve the same
systems: every schedule (band kernel and compact-stream schedules) against schedule 0 on the step's
factor sets, FP64 and the FP32 form with refinement; the tuner keeps the fastest one it timed."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import template

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tname,sizes,share", [("rb_nz16", [32], True), ("channel_ny17", [8, 8], True),
                                               ("channel_ny17", [8, 8], False)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_every_schedule_solves_alike(tname, sizes, share, precision, rng, cuda_lib):
    import torch
    from conatus_gb300 import autotune
    from conatus_gb300.ivp import DeviceProblem
    P = template(tname).instantiate(sizes)
    dev = DeviceProblem(P, precision, share=share)
    dev.autotune = False
    a, b = 1.5e3, 1.0
    fs = dev.factor(a, b)
    rhs = dev.zeros()
    rhs.copy_(torch.as_tensor(rng.standard_normal(dev.n_total) + 1j * rng.standard_normal(dev.n_total),
                              device=rhs.device))
    ref = dev.zeros()
    autotune.apply(fs, 0)
    dev.solve(a, b, rhs, ref)
    torch.cuda.synchronize()
    ref_h = ref.cpu().numpy()
    # the two-systems-per-warp compact schedules share their arithmetic (only the staging differs);
    # the split-lane schedules sum the border correction in another order, the band kernel the
    # whole solve: FP64 solutions agree to the conditioning of the systems, and the FP32 form
    # (one refinement step) to its own error, about (cond eps32)^2
    tol = 1e-10 if precision == "fp64" else 1e-5
    r = dev.zeros()
    split = autotune.split_schedules()
    part = autotune.partitioned_schedules()
    refused = set()
    for sched in autotune.schedules():
        out = dev.zeros()
        if dev.shared and (sched < 0 or sched in split):
            # a shared pair needs a compact two-system schedule: refused, never run otherwise (the
            # partitioned schedule already when it is set)
            with pytest.raises(ValueError):
                autotune.apply(fs, sched)
                dev.solve(a, b, rhs, out)
            refused.add(sched)
            continue
        autotune.apply(fs, sched)
        if precision == "fp32" and sched in part:       # the partitioned solve is FP64 only
            with pytest.raises(ValueError):
                dev.solve(a, b, rhs, out)
            refused.add(sched)
            continue
        dev.solve(a, b, rhs, out)
        dev.residual(a, b, out, rhs, r)
        torch.cuda.synchronize()
        err = np.linalg.norm(out.cpu().numpy() - ref_h) / np.linalg.norm(ref_h)
        res = float(torch.linalg.vector_norm(r).item() / torch.linalg.vector_norm(rhs).item())
        assert err < tol, (sched, err)
        assert res < (1e-10 if precision == "fp64" else 1e-5), (sched, res)
        if sched >= 0 and sched not in split:            # same arithmetic as schedule 0
            assert np.array_equal(out.cpu().numpy(), ref_h), sched
    assert bool(dev.shared) == (share and tname.startswith("channel"))
    times = autotune.tune_solve(dev, (a, b), fs, reps=2)
    assert set(times) == set(autotune.schedules()) - refused - part     # partitioned: opted into
    assert autotune.cache()[autotune._signature(dev, fs)][0] == min(times, key=times.get)
