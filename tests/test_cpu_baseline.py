"""CPU: the reference arm's stepper (oracle.ivp.ParallelStepper: the oracle's SBDF step with the
solves spread over spawned worker processes and the transforms on scipy.fft threads) takes the
oracle's own steps: the same states as SBDFStepper from the same history, to rounding (the
threaded transforms and the vectorized M X may round differently from the defaults)."""
from __future__ import annotations

from collections import deque

import numpy as np
import pytest

from _step_cases import template

# a handful of systems (solved in this process) and 265 systems (two worker processes)
CASES = [("rb_nz16", [32], 2, 1e-3), ("channel_ny17", [8, 8], 3, 5e-3), ("channel_ny17", [24, 24], 3, 5e-3)]


@pytest.mark.parametrize("tname,sizes,order,dt", CASES)
def test_parallel_stepper_takes_the_oracle_steps(tname, sizes, order, dt):
    import oracle.ivp as OI
    from conatus_gb300 import workloads as W
    P = template(tname).instantiate(sizes)
    kind = "channel" if tname.startswith("channel") else "rayleigh_benard"
    C0 = [np.asarray(c, np.complex128) for c in W.initial_state(kind, P, seed=1)]
    try:
        st = OI.ParallelStepper(P, order, dt, workers=2)
        try:
            st.time_steps(C0, steps=2, warmup=0)
        finally:
            st.close()
        got = st.state
        OI.WORKERS = None
        op = OI.OracleProblem(P)
        ref = OI.SBDFStepper(op, order, dt)
        ref.MXh = deque([op.MX(C0)] * (order - 1))
        ref.Fh = deque([op.F(C0)] * (order - 1))
        C = C0
        for _ in range(2):
            C = ref.step(C)
    finally:
        OI.WORKERS = None
    for a, b in zip(got, C):
        assert np.linalg.norm(a - b) <= 1e-12 * max(np.linalg.norm(b), 1e-300)
