"""GPU: checkpoints of the device solver (IVPSolver.save_checkpoint / load_checkpoint, the
reference's npz payload on the mode layout): a run restarted from a checkpoint continues bit for bit
(SBDF3, CNAB2 and RK443; the restart mid-way through the multistep start-up too; the FP32 form), and
a checkpoint of other numerics is refused."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import template

pytestmark = pytest.mark.gpu


def _state(P, rng):
    C = []
    for bi, b in enumerate(P.tpl.buckets):
        n_idx = np.maximum(b.col[:, 2], 0)
        z = rng.standard_normal((P.nsys[bi], b.n)).astype(np.complex128)
        if b.kind != "real":
            z = z + 1j * rng.standard_normal((P.nsys[bi], b.n))
        C.append(0.05 * z * np.exp(-0.35 * n_idx))
    return C


@pytest.mark.parametrize("scheme,first,precision", [("SBDF3", 5, "fp64"), ("SBDF3", 1, "fp64"),
                                                    ("CNAB2", 4, "fp64"), ("RK443", 3, "fp64"),
                                                    ("SBDF3", 5, "fp32")])
def test_restart_is_bit_for_bit(scheme, first, precision, tmp_path, rng, cuda_lib):
    import torch
    from conatus_gb300.ivp import IVPSolver
    P = template("channel_ny17").instantiate([8, 8])
    a = IVPSolver(P, scheme=scheme, dt=5e-3, precision=precision)
    a.set_state(_state(P, rng))
    a.run(first)
    path = a.save_checkpoint(tmp_path / "chk")
    a.run_graph(4)
    b = IVPSolver(P, scheme=scheme, dt=5e-3, precision=precision, device_problem=a.dev)
    b.load_checkpoint(path)
    assert b.iteration == first
    b.run_graph(4)
    torch.cuda.synchronize()
    assert torch.equal(a.X, b.X)
    assert b.iteration == a.iteration


def test_checkpoint_of_other_numerics_refused(tmp_path, rng, cuda_lib):
    from conatus_gb300.ivp import IVPSolver
    P = template("channel_ny17").instantiate([8, 8])
    a = IVPSolver(P, scheme="SBDF2", dt=5e-3)
    a.set_state(_state(P, rng))
    a.run(2)
    path = a.save_checkpoint(tmp_path / "chk.npz")
    for kw in (dict(scheme="SBDF3", dt=5e-3), dict(scheme="SBDF2", dt=1e-3)):
        b = IVPSolver(P, device_problem=a.dev, **kw)
        with pytest.raises(ValueError, match="checkpoint mismatch"):
            b.load_checkpoint(path)
