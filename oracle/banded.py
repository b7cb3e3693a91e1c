"""Oracle (test infrastructure only): CPU restatement of the reference's bordered banded solver.

This module is the checker for the GPU bordered-banded factor/solve. It is imported only by
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of
``bench.py``; the product path never calls it.

It follows ``core/include/conatus/banded.hpp`` of the reference:

* ``make_layout``            -> ``make_bordered_layout`` / ``measure_band`` (banded.hpp:135-251):
  border rows first, each border row replaced in B by ``s_i e_i`` with ``s_i = max |row|``
  (1 if the row is zero), ``V^T`` = border rows minus ``diag(s)``, LAPACK band storage with
  ``ldab = 2 kl + ku + 1``, non-finite entries refused.
* ``BorderedBanded``         -> ``BorderedBanded<T>`` (banded.hpp:253-478): ``gbtrf`` on B,
  ``W = B^{-1} U``, capacitance ``S = I + V^T W`` (LU + 1-norm condition), solve
  ``y = B^{-1} P b``, ``z = S^{-1} V^T y``, ``x = y - W z``; transposed solve with
  ``Wt = B^{-T} V``, ``St = I + U^T Wt``.
* ``BorderedBandedBatch``    -> the nanobind batch of ``core/bindings/module.cpp:157-206``.

The class surface (names, argument meaning, error messages containing "singular") mirrors the
reference's ``conatus._core`` so that the reference's own Python package runs on top of it
(``install_as_reference_core``). LAPACK comes from SciPy (``scipy.linalg.lapack``), which is the
third-party arithmetic the reference binds (banded.hpp:274,290,298,322,331,357,415,424).
The column-border variant (``col_border=True``, used only by spherical-shell plans) is not
restated and is refused.
"""
from __future__ import annotations

import sys
import types

import numpy as np
from scipy.linalg import lapack as _lp

__all__ = ["make_layout", "BorderedBanded", "BorderedBandedBatch", "install_as_reference_core"]


def _csr_checked(n, indptr, indices, data):
    """Structural checks of ``to_csr`` (core/bindings/module.cpp:75-98)."""
    indptr = np.asarray(indptr, dtype=np.int64)
    indices = np.asarray(indices, dtype=np.int64)
    data = np.asarray(data)
    if n < 0:
        raise ValueError(f"CSR: n must be >= 0, got {n}")
    if indptr.shape[0] != n + 1:
        raise ValueError("indptr must have n+1 entries")
    if indices.shape[0] != data.shape[0] or indptr[0] != 0 or indptr[-1] != data.shape[0]:
        raise ValueError("inconsistent CSR arrays (indptr[0] = 0, indptr[n] = nnz = "
                         "len(indices) = len(data) required)")
    if np.any(np.diff(indptr) < 0):
        raise ValueError("CSR: indptr decreases")
    if indices.size and (indices.min() < 0 or indices.max() >= n):
        raise ValueError(f"CSR: column index outside [0, {n})")
    return indptr, indices, data


class Layout:
    """Unfactored bordered-banded layout (banded.hpp:119-132): perm, band storage, V^T."""

    def __init__(self, n, r, kl, ku, perm, ab, Vt):
        self.n, self.r, self.kl, self.ku = n, r, kl, ku
        self.ldab = 2 * kl + ku + 1
        self.perm, self.ab, self.Vt = perm, ab, Vt


def make_layout(n, indptr, indices, data, border, dtype, kl_min=0, ku_min=0) -> Layout:
    """Bordered layout of a CSR matrix (banded.hpp:135-251, row border only)."""
    indptr, indices, data = _csr_checked(n, indptr, indices, data)
    data = data.astype(dtype, copy=False)
    if not np.all(np.isfinite(data)):
        k = int(np.flatnonzero(~np.isfinite(data))[0])
        row = int(np.searchsorted(indptr, k, side="right") - 1)
        raise ValueError(f"BorderedBanded: non-finite matrix entry at ({row}, {int(indices[k])}): "
                         "the operator must be finite")
    r = len(border)
    is_border = np.zeros(n, bool)
    for i in border:
        if i < 0 or i >= n:
            raise ValueError("border row out of range")
        if is_border[i]:
            raise ValueError("duplicate border row")
        is_border[i] = True
    perm = np.array(list(border) + [i for i in range(n) if not is_border[i]], dtype=np.int64)
    # band of the bulk rows (measure_band, banded.hpp:116-133): explicit zeros do not count
    kl = ku = 0
    for i in range(r, n):
        o = perm[i]
        for p in range(indptr[o], indptr[o + 1]):
            if data[p] == 0:
                continue
            j = int(indices[p])
            kl = max(kl, i - j)
            ku = max(ku, j - i)
    kl, ku = max(kl, kl_min), max(ku, ku_min)
    ldab = 2 * kl + ku + 1
    ab = np.zeros((ldab, n), dtype=dtype)           # ab[kl + ku + i - j, j] = B[i, j]
    Vt = np.zeros((r, n), dtype=dtype)
    for i in range(n):
        o = perm[i]
        lo, hi = indptr[o], indptr[o + 1]
        if i < r:
            s = 0.0
            for p in range(lo, hi):
                s = max(s, float(abs(data[p])))
                Vt[i, indices[p]] += data[p]
            if s == 0.0:
                s = 1.0
            ab[kl + ku, i] = s
            Vt[i, i] -= s
        else:
            for p in range(lo, hi):
                if data[p] == 0:
                    continue
                j = int(indices[p])
                ab[kl + ku + i - j, j] += data[p]
    return Layout(n, r, kl, ku, perm, ab, Vt)


def _lapack(dtype):
    z = np.dtype(dtype).kind == "c"
    return ((_lp.zgbtrf, _lp.zgbtrs, _lp.zgetrf, _lp.zgetrs) if z else
            (_lp.dgbtrf, _lp.dgbtrs, _lp.dgetrf, _lp.dgetrs))


def _check(info, routine, where):
    """``lapack_check`` (banded.hpp:41-50)."""
    if info < 0:
        raise RuntimeError(f"{where}: LAPACK {routine} rejected argument {-info} "
                           "(internal layout error, please report)")
    if info > 0:
        raise RuntimeError(f"{where}: LAPACK {routine} returned info = {info}")


class BorderedBanded:
    """One factored bordered-banded system (banded.hpp:253-478), row border only."""

    def __init__(self, n, indptr, indices, data, border, col_border=False, *, dtype=None):
        if col_border:
            raise NotImplementedError("oracle: the column border (spherical shells) is not restated")
        if dtype is None:
            dtype = np.complex128 if np.iscomplexobj(np.asarray(data)) else np.float64
        self.dtype = np.dtype(dtype)
        Lo = make_layout(n, indptr, indices, data, list(border), self.dtype)
        self._n, self._r, self._kl, self._ku = Lo.n, Lo.r, Lo.kl, Lo.ku
        self.perm, self.Vt = Lo.perm, Lo.Vt
        gbtrf, gbtrs, getrf, getrs = _lapack(self.dtype)
        self._gbtrs, self._getrs = gbtrs, getrs
        if n == 0:
            self.lu, self.ipiv = Lo.ab, np.zeros(0, np.int32)
        else:
            lu, ipiv, info = gbtrf(Lo.ab, Lo.kl, Lo.ku)
            if info < 0:
                raise RuntimeError(f"BorderedBanded: gbtrf rejected argument {-info}")
            if info > 0:
                raise RuntimeError(
                    f"BorderedBanded: banded part is singular at pivot {info}; the non-border rows "
                    "must form an invertible banded operator (check the row/column ordering of "
                    "the plan)")
            self.lu, self.ipiv = lu, ipiv
        self._cond = 1.0
        self._tr = None
        if self._r > 0:
            U = np.zeros((n, self._r), dtype=self.dtype)
            U[np.arange(self._r), np.arange(self._r)] = 1
            self.W = self._band_solve(U, 0)                          # W = B^{-1} U   (n, r)
            S = np.eye(self._r, dtype=self.dtype) + self.Vt @ self.W  # S = I + V^T W
            self.S_lu, self.S_piv, self._cond = self._factor_small(S)

    # -- helpers
    def _band_solve(self, b, trans):
        x, info = self._gbtrs(self.lu, self._kl, self._ku, b, self.ipiv, trans=trans)
        _check(info, "gbtrs", "BorderedBanded.solve")
        return x

    def _factor_small(self, S):
        """LU of the r x r capacitance and its 1-norm condition (banded.hpp:399-431)."""
        getrf, getrs = _lapack(self.dtype)[2:]
        nS = float(np.max(np.sum(np.abs(S), axis=0))) if S.size else 0.0
        lu, piv, info = getrf(S)
        if info < 0:
            raise RuntimeError(f"BorderedBanded: getrf rejected argument {-info}")
        if info > 0:
            raise RuntimeError(
                "BorderedBanded: capacitance matrix is singular: the boundary rows are not "
                "independent of the banded operator (ill-posed or rank-deficient BCs)")
        inv, info = getrs(lu, piv, np.eye(S.shape[0], dtype=self.dtype))
        _check(info, "getrs", "BorderedBanded (capacitance inverse)")
        c = nS * float(np.max(np.sum(np.abs(inv), axis=0)))
        if np.isnan(c):
            raise RuntimeError("BorderedBanded: capacitance condition number is NaN")
        return lu, piv, c

    def _ensure_transpose(self):
        """``ensure_transpose`` (banded.hpp:433-466): Wt = B^{-T} V, St = I + U^T Wt."""
        if self._tr is not None or self._r == 0:
            return
        Wt = self._band_solve(self.Vt.T.copy(), 1)              # (n, r)
        St = np.eye(self._r, dtype=self.dtype) + Wt[:self._r, :]
        lu, piv, _ = self._factor_small(St)
        self._tr = (Wt, lu, piv)

    # -- public surface of conatus._core.BorderedBanded{D,Z}
    n = property(lambda self: self._n)
    kl = property(lambda self: self._kl)
    ku = property(lambda self: self._ku)
    rank = property(lambda self: self._r)
    capacitance_cond = property(lambda self: self._cond)
    col_border = property(lambda self: False)
    col_border_nnz = property(lambda self: 0)

    def solve_columns(self, Y, transpose=False):
        """Solve for the columns of Y (n, nrhs); returns a new array."""
        Y = np.asarray(Y, dtype=self.dtype)
        if self._n == 0:
            return Y.copy()
        if not transpose:
            y = self._band_solve(Y[self.perm, :], 0)
            if self._r:
                z, info = self._getrs(self.S_lu, self.S_piv, self.Vt @ y)
                _check(info, "getrs", "BorderedBanded.solve")
                y = y - self.W @ z
            return y
        self._ensure_transpose()
        y = self._band_solve(Y.copy(), 1)
        if self._r:
            Wt, lu, piv = self._tr
            z, info = self._getrs(lu, piv, y[:self._r, :].copy())
            _check(info, "getrs", "BorderedBanded.solve_transpose")
            y = y - Wt @ z
        x = np.empty_like(y)
        x[self.perm, :] = y
        return x

    def solve(self, b, transpose=False):
        """b: (nrhs, n) row-major right-hand sides -> new (nrhs, n) array (module.cpp:144-154)."""
        b = np.asarray(b)
        if b.ndim != 2 or b.shape[1] != self._n:
            raise ValueError("rhs length != n")
        return np.ascontiguousarray(self.solve_columns(b.T, transpose).T)


class BorderedBandedBatch:
    """One factorization per system of equal size n (module.cpp:157-206)."""

    def __init__(self, mats, border, col_border=False, *, dtype=None):
        mats = list(mats)
        if dtype is None:
            dtype = (np.complex128 if any(np.iscomplexobj(np.asarray(m[3])) for m in mats)
                     else np.float64)
        self.sys = [BorderedBanded(n, ip, ix, d, border, col_border, dtype=dtype)
                    for (n, ip, ix, d) in mats]

    def __len__(self):
        return len(self.sys)

    kl = property(lambda self: max((s.kl for s in self.sys), default=0))
    ku = property(lambda self: max((s.ku for s in self.sys), default=0))

    def solve(self, b, transpose=False, threads=1):
        """b: (batch, n) -> x: (batch, n). ``threads`` is accepted and ignored (the reference's
        threaded loop gives the same bits as one thread)."""
        b = np.asarray(b)
        if b.ndim != 2 or b.shape[0] != len(self.sys):
            raise ValueError("batch size mismatch")
        out = np.empty(b.shape, dtype=np.result_type(b.dtype, self.sys[0].dtype if self.sys else b.dtype))
        for k, s in enumerate(self.sys):
            if b.shape[1] != s.n:
                raise ValueError("rhs length != n")
            out[k] = s.solve_columns(b[k][:, None], transpose)[:, 0]
        return out


def _typed(cls, dtype):
    class Typed(cls):
        def __init__(self, *a, **k):
            super().__init__(*a, dtype=dtype, **k)
    Typed.__name__ = cls.__name__ + ("Z" if np.dtype(dtype).kind == "c" else "D")
    return Typed


def install_as_reference_core(version: str = "0.5.0") -> types.ModuleType:
    """Insert this restatement as ``conatus._core`` so the reference package imports on a CPU-only
    host (the reference's loader accepts a preloaded module: python/conatus/runtime/__init__.py:55-59).
    Only the host surface used by the NumPy IVP path is provided."""
    m = types.ModuleType("conatus._core")
    m.__version__ = version
    m.BorderedBandedD = _typed(BorderedBanded, np.float64)
    m.BorderedBandedZ = _typed(BorderedBanded, np.complex128)
    m.BorderedBandedBatchD = _typed(BorderedBandedBatch, np.float64)
    m.BorderedBandedBatchZ = _typed(BorderedBandedBatch, np.complex128)
    m.cuda_compiled = lambda: False
    sys.modules["conatus._core"] = m
    return m
