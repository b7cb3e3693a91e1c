"""CPU: the oracle restatement of the bordered banded solver against the golden solutions of the
reference's own C++ core (banded.hpp), forward and transposed, and its refusals."""
from __future__ import annotations

import numpy as np
import pytest

from _banded_cases import CASES, buckets, rel
from oracle import banded as ob
from oracle import ref as oref


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_golden(case):
    for label, dtype, mats, border, rhs, x, xt, band in buckets(case):
        B = ob.BorderedBandedBatch(mats, border, dtype=dtype)
        assert (B.kl, B.ku) == band, label
        assert rel(B.solve(rhs), x) < 1e-13, label
        assert rel(B.solve(rhs, transpose=True), xt) < 1e-13, label


@pytest.mark.skipif(not oref.available(), reason="reference sources absent: oracle/_ref not built")
@pytest.mark.parametrize("case", CASES)
def test_compiled_reference_reproduces_golden(case):
    for label, dtype, mats, border, rhs, x, xt, band in buckets(case):
        R = oref.RefBatch(mats, border, dtype)
        assert np.array_equal(R.solve(rhs), x), label


def test_oracle_refusals():
    n = 6
    A = np.diag(np.arange(1.0, n + 1))
    import scipy.sparse as sp
    C = sp.csr_matrix(A)
    with pytest.raises(ValueError, match="duplicate border row"):
        ob.BorderedBanded(n, C.indptr, C.indices, C.data, [1, 1])
    bad = C.data.copy()
    bad[2] = np.nan
    with pytest.raises(ValueError, match="non-finite"):
        ob.BorderedBanded(n, C.indptr, C.indices, bad, [0])
    Z = C.copy()
    Z.data[3] = 0.0
    with pytest.raises(RuntimeError, match="singular"):
        ob.BorderedBanded(n, Z.indptr, Z.indices, Z.data, [0])
