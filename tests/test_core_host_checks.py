"""CPU: the ``conatus._core`` surface refuses invalid systems on the host, before any device work,
with the reference's error class and message (``ValueError`` from ``std::invalid_argument``,
core/include/conatus/banded.hpp:150-151,178) — the same on a host with or without a GPU. On a
host without a CUDA device a valid system raises ``CudaError``: there is no CPU fallback."""
from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp


def _system(n=10, dtype=float):
    A = 4.0 * np.eye(n) + np.eye(n, k=1) + np.eye(n, k=-1)
    A[0, :] = 1.0                                    # one dense border row
    C = sp.csr_matrix(A.astype(dtype))
    return n, C.indptr.astype(np.int32), C.indices.astype(np.int32), C.data


def _cases():
    n, ip, ix, d = _system()
    bad_col = ix.copy()
    bad_col[3] = n + 5
    nan = d.copy()
    nan[2] = np.nan
    inf = d.copy()
    inf[-1] = np.inf
    dec = ip.copy()
    dec[4], dec[5] = dec[5], dec[4]
    short = ip.copy()
    short[-1] -= 1
    return {
        "duplicate border row": ((n, ip, ix, d), [0, 0], "duplicate border row"),
        "border row out of range": ((n, ip, ix, d), [n], "border row out of range"),
        "negative border row": ((n, ip, ix, d), [-1], "border row out of range"),
        "NaN entry": ((n, ip, ix, nan), [0], "non-finite matrix entry"),
        "infinite entry": ((n, ip, ix, inf), [0], "non-finite matrix entry"),
        "column out of range": ((n, ip, bad_col, d), [0], "column index"),
        "indptr decreasing": ((n, dec, ix, d), [0], "indptr"),
        "indptr[n] != nnz": ((n, short, ix, d), [0], "inconsistent CSR"),
    }


REFERENCE_CHECKED = ("duplicate border row", "border row out of range", "negative border row",
                     "NaN entry", "infinite entry")


@pytest.mark.parametrize("name", list(_cases()))
def test_invalid_system_refused_on_host(name):
    from conatus_gb300 import core
    mat, border, msg = _cases()[name]
    with pytest.raises(ValueError, match=msg):
        core.BorderedBandedBatchD([mat], border)
    with pytest.raises(ValueError, match=msg):
        core.BorderedBandedD(*mat, border)
    n, ip, ix, d = mat
    with pytest.raises(ValueError, match=msg):
        core.BorderedBandedBatchZ([(n, ip, ix, d.astype(np.complex128))] * 2, border)


@pytest.mark.parametrize("name", REFERENCE_CHECKED)
def test_same_refusal_as_oracle_and_reference(name):
    """The oracle and the reference's own banded.hpp (compiled here) refuse the same input with
    the same message. Only the cases the reference itself checks are handed to it."""
    from oracle import banded as ob, ref
    from conatus_gb300 import core
    mat, border, msg = _cases()[name]
    with pytest.raises(ValueError) as ours:
        core.BorderedBandedBatchD([mat], border)
    with pytest.raises(ValueError) as theirs:
        ob.BorderedBandedBatch([mat], border, dtype=np.float64)
    assert msg in str(theirs.value) and msg in str(ours.value)
    if ref.available():
        with pytest.raises(ValueError) as compiled:
            ref.RefBatch([mat], border, np.float64)
        assert msg in str(compiled.value)


def test_no_device_means_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from conatus_gb300 import core
    from conatus_gb300.errors import CudaError
    with pytest.raises(CudaError):
        core.BorderedBandedBatchD([_system()], [0])
