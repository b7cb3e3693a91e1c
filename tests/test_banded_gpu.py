"""GPU: the bordered-banded batch kernels through the C-ABI against the golden solutions of the
reference's own banded.hpp, every solve variant of the reference's device surface
(core/bindings/module.cpp:281-440), and the errors.

Tolerances: against the reference's solution, 1e-12 relative L2, widened to 0.1 eps cond(A) for
ill-conditioned systems (random right-hand sides excite the worst directions; both solvers are
backward stable, so they may differ by up to eps cond(A)); and a backward error
||A x - b|| / (||A|| ||x|| + ||b||) below 1e-14."""
from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp

from _banded_cases import CASES, backward_error, buckets, rel, tol_vs_reference

pytestmark = pytest.mark.gpu
BWD = 1e-14


def _cls(dtype, device=True):
    from conatus_gb300 import core
    if device:
        return core.BandedBatchZ if np.dtype(dtype).kind == "c" else core.BandedBatchD
    return core.BorderedBandedBatchZ if np.dtype(dtype).kind == "c" else core.BorderedBandedBatchD


def _t(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("case", CASES)
def test_solve_ptr_matches_reference(case, cuda_lib):
    import torch
    for label, dtype, mats, border, rhs, x, xt, band in buckets(case):
        B = _cls(dtype)(mats, border)
        assert (B.kl, B.ku) == band, label
        b = _t(rhs.astype(dtype))
        B.solve_ptr(b.data_ptr(), b.shape[0], b.shape[1])
        torch.cuda.synchronize()
        xg = b.cpu().numpy()
        assert rel(xg, x) < tol_vs_reference(case, label), label
        assert backward_error(mats, xg, rhs) < BWD, label


@pytest.mark.parametrize("case", CASES)
def test_transpose_matches_reference(case, cuda_lib):
    import torch
    for label, dtype, mats, border, rhs, x, xt, band in buckets(case):
        B = _cls(dtype)(mats, border)
        B.prepare_transpose()
        b = _t(rhs.astype(dtype))
        B.solve_transpose_ptr(b.data_ptr(), b.shape[0], b.shape[1])
        torch.cuda.synchronize()
        xg = b.cpu().numpy()
        assert rel(xg, xt) < tol_vs_reference(case, label), label
        assert backward_error(mats, xg, rhs, transpose=True) < BWD, label


@pytest.mark.parametrize("case", CASES)
def test_host_batch_solve(case, cuda_lib):
    for label, dtype, mats, border, rhs, x, xt, band in buckets(case):
        B = _cls(dtype, device=False)(mats, border)
        assert len(B) == len(mats)
        assert rel(B.solve(rhs), x) < tol_vs_reference(case, label), label
        assert rel(B.solve(rhs, transpose=True), xt) < tol_vs_reference(case, label), label


def test_mapped_and_split(rng, cuda_lib):
    import torch
    for label, dtype, mats, border, rhs, x, xt, band in buckets("banded_rb32x16.npz"):
        Bn, n = rhs.shape
        B = _cls(dtype)(mats, border)
        # mapped: rhs scattered in a global vector through a random permutation
        tot = Bn * n
        rows = rng.permutation(tot).reshape(Bn, n)
        cols = rng.permutation(tot).reshape(Bn, n)
        glob = np.zeros(tot, dtype=dtype)
        glob[rows] = rhs
        xg = torch.zeros(tot, dtype=torch.complex128 if dtype.kind == "c" else torch.float64, device="cuda")
        g, r_, c_ = _t(glob), _t(rows.astype(np.int64)), _t(cols.astype(np.int64))
        B.solve_mapped_ptr(g.data_ptr(), r_.data_ptr(), xg.data_ptr(), c_.data_ptr())
        torch.cuda.synchronize()
        tol = tol_vs_reference("banded_rb32x16.npz", label)
        assert rel(xg.cpu().numpy()[cols], x) < tol, label
        # in place with one map for rows and cols (allowed, as in the reference); two maps refused
        gi = _t(glob)
        B.solve_mapped_ptr(gi.data_ptr(), r_.data_ptr(), gi.data_ptr(), r_.data_ptr())
        torch.cuda.synchronize()
        assert rel(gi.cpu().numpy()[rows], x) < tol, label
        gn = _t(glob[rows].reshape(-1))
        B.solve_mapped_ptr(gn.data_ptr(), 0, gn.data_ptr(), 0)
        torch.cuda.synchronize()
        assert rel(gn.cpu().numpy().reshape(Bn, n), x) < tol, label
        with pytest.raises(ValueError, match="alias"):
            B.solve_mapped_ptr(g.data_ptr(), r_.data_ptr(), g.data_ptr(), c_.data_ptr())
        if dtype.kind == "c":
            # split: real data vector, b = re[rows_c] + i re[rows_s]
            tot2 = 2 * tot
            perm_in = rng.permutation(tot2)
            rc, rs = perm_in[:tot].reshape(Bn, n), perm_in[tot:].reshape(Bn, n)
            perm_out = rng.permutation(tot2)
            cc, cs = perm_out[:tot].reshape(Bn, n), perm_out[tot:].reshape(Bn, n)
            re = np.zeros(tot2)
            re[rc] = rhs.real
            re[rs] = rhs.imag
            xo = torch.zeros(tot2, dtype=torch.float64, device="cuda")
            tr = [_t(v.astype(np.int64)) for v in (rc, rs, cc, cs)]
            rre = _t(re)
            B.solve_split_ptr(rre.data_ptr(), tr[0].data_ptr(), tr[1].data_ptr(), xo.data_ptr(),
                              tr[2].data_ptr(), tr[3].data_ptr())
            torch.cuda.synchronize()
            xs = xo.cpu().numpy()
            assert rel(xs[cc] + 1j * xs[cs], x) < tol, label


def test_shared_pattern_device_assembly(cuda_lib):
    """Values on the device, one CSR pattern: the device layout builder gives the same solves."""
    import torch
    from conatus_gb300 import core
    for label, dtype, mats, border, rhs, x, xt, band in buckets("banded_channel8x17x8.npz"):
        n = mats[0][0]
        dense = [sp.csr_matrix((d, ix, ip), shape=(n, n)) for (_, ip, ix, d) in mats]
        union = sum(abs(A) for A in dense)
        union = sp.csr_matrix(union)
        union.sort_indices()
        vals = []
        for A in dense:
            Ad = A.toarray()
            r_, c_ = np.repeat(np.arange(n), np.diff(union.indptr)), union.indices
            vals.append(Ad[r_, c_])
        V = _t(np.stack(vals).astype(dtype))
        H = core._Handle.shared(dtype, len(mats), n, union.indptr, union.indices, V, border)
        b = _t(rhs.astype(dtype))
        from conatus_gb300._lib import call
        call("cng_banded_solve", H.h, b.data_ptr(), None)
        torch.cuda.synchronize()
        assert rel(b.cpu().numpy(), x) < tol_vs_reference("banded_channel8x17x8.npz", label), label
        # refactor with the same values: same solutions, bit for bit
        H.refactor(V)
        b2 = _t(rhs.astype(dtype))
        call("cng_banded_solve", H.h, b2.data_ptr(), None)
        b3 = _t(rhs.astype(dtype))
        call("cng_banded_solve", H.h, b3.data_ptr(), None)
        torch.cuda.synchronize()
        assert torch.equal(b2, b3)


def test_errors(cuda_lib):
    from conatus_gb300 import core
    n = 8
    A = sp.csr_matrix(np.diag(np.arange(1.0, n + 1)) + np.diag(np.ones(n - 1), 1))
    with pytest.raises(ValueError, match="duplicate border row"):
        core.BandedBatchD([(n, A.indptr, A.indices, A.data)], [1, 1])
    bad = A.data.copy()
    bad[0] = np.inf
    with pytest.raises(ValueError, match="non-finite"):
        core.BandedBatchD([(n, A.indptr, A.indices, bad)], [0])
    Z = A.copy()
    Z.data[Z.indptr[4]] = 0.0          # zero diagonal with nothing below it: singular band
    with pytest.raises(RuntimeError, match="singular"):
        core.BandedBatchD([(n, Z.indptr, Z.indices, Z.data)], [0])
    with pytest.raises(ValueError):
        core.BandedBatchD([(n, A.indptr, A.indices, A.data)], [n])
    B = core.BandedBatchD([(n, A.indptr, A.indices, A.data)], [0])
    with pytest.raises(ValueError, match="matching the factorization"):
        B.solve_ptr(12345, 2, n)


@pytest.mark.parametrize("case", CASES)
def test_compact_solve_matches_dense(case, cuda_lib):
    """The compact bucket-union solve (4 systems per warp, union pattern of the factors) against
    the dense band solve of the same factors: same arithmetic up to the order of the sums."""
    import torch
    from conatus_gb300 import core
    from conatus_gb300._lib import call
    for label, dtype, mats, border, rhs, x, xt, band in buckets(case):
        if np.dtype(dtype).kind != "c":
            continue
        B = core.BandedBatchZ(mats, border)
        b = _t(rhs.astype(dtype))
        B.solve_ptr(b.data_ptr(), b.shape[0], b.shape[1])
        call("cng_banded_compact", B._h.h, None)
        b2 = _t(rhs.astype(dtype))
        B.solve_ptr(b2.data_ptr(), b2.shape[0], b2.shape[1])
        torch.cuda.synchronize()
        assert rel(b2.cpu().numpy(), b.cpu().numpy()) < tol_vs_reference(case, label), label
        assert rel(b2.cpu().numpy(), x) < tol_vs_reference(case, label), label
        # FP32 copies + refinement-free solve: FP32 accuracy against the FP64 solution
        call("cng_banded_make_fp32", B._h.h, None)
        out = torch.zeros_like(b2)
        call("cng_banded_solve_fp32", B._h.h, _t(rhs.astype(dtype)).data_ptr(), out.data_ptr(), 0, None)
        torch.cuda.synchronize()
        assert rel(out.cpu().numpy(), x) < 1e-2, label
