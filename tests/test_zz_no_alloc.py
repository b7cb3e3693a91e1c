"""GPU: cng_banded_solve_host_static (host-buffer solve staged in the library's fixed device array,
no device allocation) against cng_banded_solve_host on the same factors, two calls in a row, plain
and transposed; sizes above the array are refused before any device work.

Collected last so that it also runs after every other GPU test in the same process."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from _banded_cases import CASES, buckets, rel, tol_vs_reference

pytestmark = pytest.mark.gpu

STATIC_BYTES = 8 << 20


def _solve(fn, h, b, transpose):
    from conatus_gb300._lib import call
    b = np.ascontiguousarray(b)
    x = np.empty_like(b)
    call(fn, h, b.ctypes.data, x.ctypes.data, int(transpose))
    return x


@pytest.mark.parametrize("case", CASES)
def test_static_host_solve_matches_host_solve(case, cuda_lib):
    from conatus_gb300 import core
    from conatus_gb300._lib import call
    for label, dtype, mats, border, rhs, x, xt, band in buckets(case):
        B = (core.BandedBatchZ if np.dtype(dtype).kind == "c" else core.BandedBatchD)(mats, border)
        h = B._h.h
        b = rhs.astype(dtype)
        assert b.nbytes <= STATIC_BYTES
        tol = tol_vs_reference(case, label)
        ref = _solve("cng_banded_solve_host", h, b, False)
        for _ in range(2):                         # two calls in a row share the array
            got = _solve("cng_banded_solve_host_static", h, b, False)
            assert rel(got, ref) <= 1e-15, label
            assert rel(got, x) < tol, label
        call("cng_banded_prepare_transpose", h, None)
        ref_t = _solve("cng_banded_solve_host", h, b, True)
        for _ in range(2):
            got_t = _solve("cng_banded_solve_host_static", h, b, True)
            assert rel(got_t, ref_t) <= 1e-15, label
            assert rel(got_t, xt) < tol, label


def test_static_host_solve_refuses_oversize(cuda_lib):
    """batch * n * 16 bytes just above the array: status 1 (invalid argument) with a message, and
    the next in-range call still works."""
    import scipy.sparse as sp
    from conatus_gb300 import core
    from conatus_gb300._lib import lib
    rng = np.random.default_rng(0)
    n = 64
    batch = STATIC_BYTES // (16 * n) + 1
    A = sp.diags([np.full(n - 1, -1.0), np.full(n, 4.0), np.full(n - 1, -1.0)], [-1, 0, 1], format="csr")
    A = A.astype(np.complex128)
    mats = [(n, A.indptr, A.indices, A.data)] * batch
    B = core.BandedBatchZ(mats, [])
    b = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex128)
    assert b.nbytes > STATIC_BYTES
    x = np.zeros_like(b)
    L = lib()
    st = L.cng_banded_solve_host_static(B._h.h, b.ctypes.data_as(ctypes.c_void_p), x.ctypes.data_as(ctypes.c_void_p), 0)
    assert st == 1
    assert b"static staging buffer" in L.cng_last_error()
    assert not np.any(x)
    # transposed solve without prepare_transpose: refused too (preparing it would allocate)
    small = core.BandedBatchZ(mats[:4], [])
    bs = b[:4].copy()
    st = L.cng_banded_solve_host_static(small._h.h, bs.ctypes.data_as(ctypes.c_void_p), bs.ctypes.data_as(ctypes.c_void_p), 1)
    assert st == 1 and b"prepare_transpose" in L.cng_last_error()
    got = _solve("cng_banded_solve_host_static", small._h.h, b[:4], False)
    ref = _solve("cng_banded_solve_host", small._h.h, b[:4], False)
    assert rel(got, ref) <= 1e-15


def _batch(n=96, batch=24, seed=1):
    import scipy.sparse as sp
    from conatus_gb300 import core
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(batch):
        A = sp.diags([rng.standard_normal(n - 2), rng.standard_normal(n - 1), 6 + rng.standard_normal(n),
                      rng.standard_normal(n - 1)], [-2, -1, 0, 1], format="lil")
        A[0, :] = rng.standard_normal(n)               # a border row
        A = A.tocsr().astype(np.complex128)
        mats.append((n, A.indptr, A.indices, A.data))
    return core.BandedBatchZ(mats, [0]), rng


def test_static_host_solve_allocates_nothing(cuda_lib):
    """After the first call (which looks up the array's address), further calls leave the device's
    free memory and the library's allocation counters unchanged."""
    import torch
    from conatus_gb300 import core
    B, rng = _batch()
    b = rng.standard_normal((24, 96)) + 1j * rng.standard_normal((24, 96))
    _solve("cng_banded_solve_host_static", B._h.h, b, False)
    torch.cuda.synchronize()
    free0, stats0 = torch.cuda.mem_get_info()[0], core.pool_stats()
    for _ in range(20):
        _solve("cng_banded_solve_host_static", B._h.h, b, False)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert core.pool_stats() == stats0


def test_static_host_solve_from_two_threads(cuda_lib):
    """Two host threads solving different right-hand sides on one device take turns on the shared
    array: each result equals its own plain host solve."""
    import threading
    B, rng = _batch(seed=2)
    rhs = [rng.standard_normal((24, 96)) + 1j * rng.standard_normal((24, 96)) for _ in range(2)]
    refs = [_solve("cng_banded_solve_host", B._h.h, r, False) for r in rhs]
    errors = []

    def work(k):
        try:
            for _ in range(25):
                got = _solve("cng_banded_solve_host_static", B._h.h, rhs[k], False)
                if rel(got, refs[k]) > 1e-15:
                    errors.append((k, rel(got, refs[k])))
        except Exception as e:              # noqa: BLE001 -- reported below
            errors.append((k, repr(e)))

    ts = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
