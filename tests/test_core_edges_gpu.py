"""GPU: edge cases of the conatus._core surface (conatus_gb300.core), the behaviours the
reference's own core tests check (tests/core/test_core_banded.py, tests/core/
test_runtime_review_v011.py, tests/core/test_cuda_review_r05_gpu.py): random bordered banded
systems with border rows anywhere against dense solves (plain and transposed, real and complex,
1 to 4 border rows, no border), a batch against its systems one by one, an empty batch and
right-hand sides of the wrong shape refused, a band solve captured in a CUDA graph, and no device
memory left behind by many factorizations."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def _almost_banded(rng, n, kl, ku, border, dtype):
    """A band (kl, ku) made diagonally dominant, with full random rows at ``border``."""
    A = np.zeros((n, n), dtype=dtype)
    for d in range(-kl, ku + 1):
        v = rng.standard_normal(n - abs(d))
        if dtype == complex:
            v = v + 1j * rng.standard_normal(n - abs(d))
        A += np.diag(v, d)
    A += np.eye(n) * 4 * (kl + ku + 1)
    for i in border:
        A[i] = rng.standard_normal(n) + (1j * rng.standard_normal(n) if dtype == complex else 0)
    return A


@pytest.mark.parametrize("dtype", [float, complex])
@pytest.mark.parametrize("r", [0, 1, 2, 3, 4])
def test_bordered_solve_matches_dense(dtype, r, rng, cuda_lib):
    from conatus_gb300 import core
    n, kl, ku = int(rng.integers(20, 80)), int(rng.integers(0, 4)), int(rng.integers(0, 4))
    border = sorted(rng.choice(n, size=r, replace=False).tolist())
    # the band lies on the layout with the border rows first: build it there, then scatter back
    Ap = _almost_banded(rng, n, kl, ku, range(r), dtype)
    order = border + [i for i in range(n) if i not in border]
    A = np.empty_like(Ap)
    A[order] = Ap
    C = sp.csr_matrix(A)
    cls = core.BorderedBandedZ if dtype == complex else core.BorderedBandedD
    s = cls(n, C.indptr, C.indices, C.data, border)
    assert s.rank == r and s.kl <= kl + r and s.ku <= ku + r
    b = rng.standard_normal((3, n)) + (1j * rng.standard_normal((3, n)) if dtype == complex else 0)
    x = s.solve(b)
    assert np.max(abs(A @ x.T - b.T)) < 1e-12 * np.max(abs(b)) * n
    xt = s.solve(b, transpose=True)
    assert np.max(abs(A.T @ xt.T - b.T)) < 1e-12 * np.max(abs(b)) * n


def test_batch_matches_individual(rng, cuda_lib):
    from conatus_gb300 import core
    n, mats, dense, bs = 40, [], [], []
    for _ in range(6):
        A = _almost_banded(rng, n, 2, 2, [0, 1], complex)
        C = sp.csr_matrix(A)
        mats.append((n, C.indptr, C.indices, C.data))
        dense.append(A)
        bs.append(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    X = core.BorderedBandedBatchZ(mats, [0, 1]).solve(np.array(bs))
    for A, b_, x_ in zip(dense, bs, X):
        assert np.max(abs(A @ x_ - b_)) < 1e-11
    for (n_, ip, ix, d), b_, x_ in zip(mats, bs, X):
        one = core.BorderedBandedZ(n_, ip, ix, d, [0, 1]).solve(b_[None, :])[0]
        assert np.max(abs(one - x_)) <= 1e-14 * np.max(abs(x_))


def test_empty_batch_and_bad_shapes_refused(rng, cuda_lib):
    from conatus_gb300 import core
    with pytest.raises(ValueError):
        core.BorderedBandedBatchZ([], [0])
    n = 12
    C = sp.csr_matrix(_almost_banded(rng, n, 1, 1, [0], float))
    bt = core.BorderedBandedBatchD([(n, C.indptr, C.indices, C.data)] * 2, [0])
    for bad in (np.ones(24), np.ones((3, n)), np.ones((2, n - 1)), np.ones((2, n, 1))):
        with pytest.raises(ValueError):
            bt.solve(bad)
    with pytest.raises(TypeError):
        bt.solve(np.ones((2, n)) + 1j)                  # complex right-hand side, real factors


def test_band_solve_captured_in_a_cuda_graph(rng, cuda_lib):
    """The device solve on a caller stream inside a capture: the replay gives the direct result."""
    import torch
    from conatus_gb300 import core
    from conatus_gb300._lib import call
    n, batch = 64, 37
    mats = []
    for _ in range(batch):
        C = sp.csr_matrix(_almost_banded(rng, n, 3, 2, [0, 5], complex))
        mats.append((n, C.indptr, C.indices, C.data))
    B = core.BandedBatchZ(mats, [0, 5])
    b = torch.as_tensor(rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n)), device="cuda")
    direct = b.clone()
    B.solve_ptr(direct.data_ptr(), batch, n)
    work = torch.empty_like(b)
    s = torch.cuda.Stream()
    h = ctypes.c_void_p()
    torch.cuda.synchronize()
    call("cng_graph_begin", s.cuda_stream)
    try:
        B.solve_ptr(work.data_ptr(), batch, n, s.cuda_stream)
    finally:
        call("cng_graph_end", s.cuda_stream, ctypes.byref(h))
    for _ in range(2):
        work.copy_(b)
        torch.cuda.synchronize()
        call("cng_graph_launch", h, s.cuda_stream)
        s.synchronize()
        assert torch.equal(work, direct)
    call("cng_graph_destroy", h)


def test_factorizations_leave_no_device_memory(rng, cuda_lib):
    import torch
    from conatus_gb300 import core
    from conatus_gb300._lib import lib

    def free():
        f, t = ctypes.c_uint64(), ctypes.c_uint64()
        lib().cng_mem_info(ctypes.byref(f), ctypes.byref(t))
        return int(f.value)

    n = 96
    C = sp.csr_matrix(_almost_banded(rng, n, 4, 3, [0, 1, 2], complex))
    mats = [(n, C.indptr, C.indices, C.data)] * 500
    b = torch.ones((500, n), dtype=torch.complex128, device="cuda")
    core.BandedBatchZ(mats, [0, 1, 2]).solve_ptr(b.data_ptr(), 500, n)   # first-use allocations
    torch.cuda.synchronize()
    f0 = free()
    for _ in range(20):
        B = core.BandedBatchZ(mats, [0, 1, 2])
        B.solve_ptr(b.data_ptr(), 500, n)
        del B
    torch.cuda.synchronize()
    assert free() >= f0 - (2 << 20)                     # driver page granularity


def test_pool_counts_handle_memory(rng, cuda_lib):
    """cuda.pool_stats counts the device memory of live handles: a factored batch adds at least
    its LU band, and destroying it gives every byte back."""
    import gc
    from conatus_gb300 import core
    gc.collect()
    live0, _, nalloc0, _ = core.cuda.pool_stats()
    n, batch = 40, 3
    mats = []
    for _ in range(batch):
        C = sp.csr_matrix(_almost_banded(rng, n, 2, 3, [0, 1], float))
        mats.append((n, C.indptr, C.indices, C.data))
    B = core.cuda.BandedBatchD(mats, [0, 1])
    live1, _, nalloc1, _ = core.cuda.pool_stats()
    ldab = 2 * B.kl + B.ku + 1
    assert live1 - live0 >= batch * n * ldab * 8 and nalloc1 > nalloc0
    del B
    gc.collect()
    assert core.cuda.pool_stats()[0] == live0
