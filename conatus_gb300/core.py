"""Drop-in face of the reference's compiled core ``conatus._core`` on the GB300 library.

The reference loads ``conatus._core`` (python/conatus/runtime/__init__.py:55-81) and binds it in
core/bindings/module.cpp. This module offers the same classes, argument meanings and errors, backed
by the CUDA kernels of ``libconatus_gb300.so``:

* ``BorderedBandedBatchD/Z(mats, border, col_border=False)`` with ``solve(b, transpose=False,
  threads=1)``, ``kl``, ``ku``, ``len()`` (module.cpp:157-206): factors on the GPU, host buffers
  copied in and out inside ``solve``.
* ``BorderedBandedD/Z(n, indptr, indices, data, border, col_border=False)`` with ``solve(b,
  transpose)``, ``n kl ku rank capacitance_cond col_border col_border_nnz`` (module.cpp:128-155).
* ``cuda.BandedBatchD/Z(mats, border_rows, pivot=True, ...)`` with ``solve_ptr``,
  ``solve_mapped_ptr``, ``solve_split_ptr``, ``prepare_transpose``, ``solve_transpose_ptr`` on
  caller-owned device memory (module.cpp:281-440), ``cuda.available()``, ``device_name()``,
  ``synchronize()``.

``install()`` inserts this module as ``conatus._core`` so that an unmodified reference package runs
its IVP path on these kernels. The column border (``col_border=True``) is refused (spherical
shells are outside this library).
"""
from __future__ import annotations

import ctypes
import sys
import types

import numpy as np

from . import _lib
from ._lib import call

__version__ = "0.5.0"

_F64, _C128 = 0, 1


def _kind(dtype) -> int:
    return _C128 if np.dtype(dtype).kind == "c" else _F64


def _ptr(a) -> int:
    """Device or host address of an array-like (torch tensor, numpy array, or an int)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    raise TypeError(f"cannot take the address of {type(a).__name__}")


def _pack_csr(mats, dtype):
    """(indptr (B, n+1) int32, indices int32, data, offsets int64, n) of a list of CSR tuples."""
    mats = list(mats)
    if not mats:
        raise ValueError("BandedBatch: no matrix given")
    n = int(mats[0][0])
    ips, ixs, ds, offs = [], [], [], []
    off = 0
    for k, (nk, ip, ix, d) in enumerate(mats):
        if int(nk) != n:
            raise ValueError(f"matrix {k}: size {nk} differs from {n} (a batch has one size)")
        ip = np.ascontiguousarray(ip, dtype=np.int32)
        ix = np.ascontiguousarray(ix, dtype=np.int32)
        d = np.asarray(d)
        if _kind(dtype) == _F64 and np.iscomplexobj(d):
            raise TypeError("complex matrix data for real (float64) factors")
        d = np.ascontiguousarray(d, dtype=np.complex128 if _kind(dtype) else np.float64)
        if ip.shape[0] != n + 1:
            raise ValueError("indptr must have n+1 entries")
        if ix.shape[0] != d.shape[0] or ip[0] != 0 or ip[-1] != d.shape[0]:
            raise ValueError("inconsistent CSR arrays (indptr[0] = 0, indptr[n] = nnz = "
                             "len(indices) = len(data) required)")
        ips.append(ip)
        ixs.append(ix)
        ds.append(d)
        offs.append(off)
        off += d.shape[0]
    return (np.concatenate(ips), np.concatenate(ixs), np.concatenate(ds),
            np.asarray(offs, dtype=np.int64), n)


class _Handle:
    """Owner of one ``cng_banded`` handle."""

    def __init__(self, dtype, mats, border, pivot=True, stream=0):
        self.kind = _kind(dtype)
        ip, ix, d, offs, n = _pack_csr(mats, dtype)
        bd = np.ascontiguousarray([int(i) for i in border], dtype=np.int32)
        h = ctypes.c_void_p()
        call("cng_banded_create_csr", self.kind, len(offs), n, ip.ctypes.data, ix.ctypes.data,
             d.ctypes.data, offs.ctypes.data, bd.ctypes.data if bd.size else None, int(bd.size),
             int(bool(pivot)), stream or None, ctypes.byref(h))
        self.h = h
        self._read_info()

    @classmethod
    def shared(cls, dtype, batch, n, indptr, indices, values_dev, border, pivot=True, stream=0):
        """Batch sharing one CSR pattern; ``values_dev`` (batch, nnz) on the device."""
        self = cls.__new__(cls)
        self.kind = _kind(dtype)
        ip = np.ascontiguousarray(indptr, dtype=np.int32)
        ix = np.ascontiguousarray(indices, dtype=np.int32)
        bd = np.ascontiguousarray([int(i) for i in border], dtype=np.int32)
        h = ctypes.c_void_p()
        call("cng_banded_create_shared", self.kind, int(batch), int(n), ip.ctypes.data,
             ix.ctypes.data if ix.size else None, int(ix.size), _ptr(values_dev),
             bd.ctypes.data if bd.size else None, int(bd.size), int(bool(pivot)), stream or None,
             ctypes.byref(h))
        self.h = h
        self._read_info()
        return self

    def refactor(self, values_dev, stream=0):
        call("cng_banded_refactor_shared", self.h, _ptr(values_dev), stream or None)
        self._read_info()

    def _read_info(self):
        dims = np.zeros(8, np.int32)
        stats = np.zeros(2, np.float64)
        call("cng_banded_info", self.h, dims.ctypes.data, stats.ctypes.data)
        (self.batch, self.n, self.rank, self.kl, self.ku, self.ldab, _, self.pivot) = map(int, dims)
        self.factor_ms, self.cond_max = float(stats[0]), float(stats[1])

    def cond(self) -> np.ndarray:
        c = np.zeros(self.batch, np.float64)
        call("cng_banded_capacitance_cond", self.h, c.ctypes.data)
        return c

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            try:
                _lib.lib().cng_banded_destroy(h)
            except Exception:
                pass
            self.h = None


def _check_col_border(col_border):
    if col_border:
        raise NotImplementedError("col_border=True (column border of spherical-shell plans) is not "
                                  "supported by the GB300 library")


# ------------------------------------------------------------------------------------------------
# host surface: BorderedBandedBatch{D,Z}, BorderedBanded{D,Z}

class _BorderedBandedBatch:
    _dtype = np.float64

    def __init__(self, mats, border, col_border=False):
        _check_col_border(col_border)
        self._h = _Handle(self._dtype, mats, border)

    def __len__(self):
        return self._h.batch

    kl = property(lambda self: self._h.kl)
    ku = property(lambda self: self._h.ku)

    def solve(self, b, transpose=False, threads=1):
        """b: (batch, n) C-contiguous -> new (batch, n) array. ``threads`` is accepted for the
        reference's signature; the GPU solve does not depend on it."""
        b = np.asarray(b)
        if b.ndim != 2 or b.shape[0] != self._h.batch:
            raise ValueError("batch size mismatch")
        if b.shape[1] != self._h.n:
            raise ValueError("rhs length != n")
        if np.dtype(self._dtype).kind != "c" and np.iscomplexobj(b):
            raise TypeError("complex right-hand side for real factors")
        b = np.ascontiguousarray(b, dtype=self._dtype)
        x = np.empty_like(b)
        call("cng_banded_solve_host", self._h.h, b.ctypes.data, x.ctypes.data, int(bool(transpose)))
        return x


class _BorderedBanded:
    _dtype = np.float64

    def __init__(self, n, indptr, indices, data, border, col_border=False):
        _check_col_border(col_border)
        self._h = _Handle(self._dtype, [(n, indptr, indices, data)], border)

    n = property(lambda self: self._h.n)
    kl = property(lambda self: self._h.kl)
    ku = property(lambda self: self._h.ku)
    rank = property(lambda self: self._h.rank)
    capacitance_cond = property(lambda self: self._h.cond_max)
    col_border = property(lambda self: False)
    col_border_nnz = property(lambda self: 0)

    def solve(self, b, transpose=False):
        """b: (nrhs, n) row-major -> new (nrhs, n) (one GPU solve per right-hand side)."""
        b = np.asarray(b)
        if b.ndim != 2 or b.shape[1] != self._h.n:
            raise ValueError("rhs length != n")
        b = np.ascontiguousarray(b, dtype=self._dtype)
        x = np.empty_like(b)
        for c in range(b.shape[0]):
            row_in, row_out = b[c:c + 1], x[c:c + 1]
            call("cng_banded_solve_host", self._h.h, row_in.ctypes.data, row_out.ctypes.data,
                 int(bool(transpose)))
        return x


class BorderedBandedBatchD(_BorderedBandedBatch):
    _dtype = np.float64


class BorderedBandedBatchZ(_BorderedBandedBatch):
    _dtype = np.complex128


class BorderedBandedD(_BorderedBanded):
    _dtype = np.float64


class BorderedBandedZ(_BorderedBanded):
    _dtype = np.complex128


# ------------------------------------------------------------------------------------------------
# device surface: cuda.BandedBatch{D,Z}

class _BandedBatch:
    _dtype = np.float64

    def __init__(self, mats, border_rows, pivot=True, level_schedule=True, level_merge=True,
                 col_border=False):
        _check_col_border(col_border)
        self._h = _Handle(self._dtype, mats, border_rows, pivot=pivot)
        self._level_schedule = bool(level_schedule)

    n = property(lambda self: self._h.n)
    kl = property(lambda self: self._h.kl)
    ku = property(lambda self: self._h.ku)
    rank = property(lambda self: self._h.rank)
    batch = property(lambda self: self._h.batch)
    pivot = property(lambda self: bool(self._h.pivot))
    factor_ms = property(lambda self: self._h.factor_ms)
    capacitance_cond_max = property(lambda self: self._h.cond_max)
    col_border = property(lambda self: False)
    col_border_nnz = property(lambda self: 0)
    # the GB300 solve reads the band directly (one warp per system); no level schedule is built,
    # so the reference's level-schedule diagnostics (module.cpp:356-373) report none
    level_scheduled = property(lambda self: False)
    level_transposed = property(lambda self: False)
    level_merged = property(lambda self: False)
    level_depth_forward = property(lambda self: 0)
    level_depth_backward = property(lambda self: 0)
    level_steps_forward = property(lambda self: 0)
    level_steps_backward = property(lambda self: 0)
    level_stream_bytes = property(lambda self: 0)
    level_t_stream_bytes = property(lambda self: 0)
    level_note = property(lambda self: "no level schedule: the GB300 solve sweeps the LU band, "
                                       "one warp per system")
    level_t_note = property(lambda self: "no level schedule: the transposed solve sweeps the LU band")
    level_t_steps = property(lambda self: (0, 0))
    band_released = property(lambda self: False)

    def _check_dims(self, batch, n, where):
        if batch != self._h.batch or n != self._h.n:
            raise ValueError(f"BandedBatch.{where}: expected (batch, n) matching the factorization")

    def solve_ptr(self, ptr, batch, n, stream=0):
        self._check_dims(batch, n, "solve_ptr")
        if not ptr:
            raise ValueError("BandedBatch.solve_ptr: null device pointer")
        call("cng_banded_solve", self._h.h, ptr, stream or None)

    def solve_mapped_ptr(self, rhs, rows, x, cols, stream=0):
        if not rhs or not x:
            raise ValueError("BandedBatch.solve_mapped_ptr: null device pointer")
        call("cng_banded_solve_mapped", self._h.h, rhs, rows or None, x, cols or None, stream or None)

    def solve_split_ptr(self, re, rows_c, rows_s, x, cols_c, cols_s, stream=0):
        call("cng_banded_solve_split", self._h.h, re, rows_c, rows_s, x, cols_c, cols_s, stream or None)

    def prepare_transpose(self):
        call("cng_banded_prepare_transpose", self._h.h, None)

    def build_transpose_schedule(self):
        self.prepare_transpose()

    def release_band(self):
        """The reference frees the LU band once its level schedules hold the factors
        (module.cpp:366-367). Every solve here reads the band, so it stays: nothing to release."""

    def solve_transpose_ptr(self, ptr, batch, n, stream=0):
        self._check_dims(batch, n, "solve_transpose_ptr")
        if not ptr:
            raise ValueError("BandedBatch.solve_transpose_ptr: null device pointer")
        call("cng_banded_solve_transpose", self._h.h, ptr, stream or None)

    def solve(self, b):
        """In-place solve of a (batch, n) device tensor."""
        self._check_dims(b.shape[0], b.shape[1], "solve")
        call("cng_banded_solve", self._h.h, _ptr(b), None)

    def solve_transpose(self, b):
        self._check_dims(b.shape[0], b.shape[1], "solve_transpose")
        self.prepare_transpose()
        call("cng_banded_solve_transpose", self._h.h, _ptr(b), None)


class BandedBatchD(_BandedBatch):
    _dtype = np.float64


class BandedBatchZ(_BandedBatch):
    _dtype = np.complex128


def available() -> bool:
    return bool(_lib.lib().cng_cuda_available())


def device_name(dev: int = 0) -> str:
    buf = ctypes.create_string_buffer(256)
    call("cng_device_name", int(dev), buf, 256)
    return buf.value.decode()


def synchronize() -> None:
    import torch
    torch.cuda.synchronize()


def pool_stats() -> tuple:
    """(live bytes, cached bytes, allocations, reuses) of the device memory the library's handles
    hold, as the reference core's cuda.pool_stats (core/bindings/module.cpp:450-453). Nothing is
    cached: a handle's memory goes back to the driver when the handle is destroyed."""
    v = [ctypes.c_uint64() for _ in range(4)]
    call("cng_pool_stats", *(ctypes.byref(x) for x in v))
    return tuple(int(x.value) for x in v)


def pool_trim() -> None:
    """The reference's cuda.pool_trim (module.cpp:454): no cached blocks here, so nothing to do."""
    call("cng_pool_trim")


def plan_cache_size() -> int:
    """The reference's count of cached cuFFT plans (module.cpp:455). The transforms here use
    compile-time plans inside the kernels and keep no runtime plans: 0."""
    return 0


cuda = types.SimpleNamespace(
    BandedBatchD=BandedBatchD, BandedBatchZ=BandedBatchZ, available=available,
    device_name=device_name, synchronize=synchronize, pool_stats=pool_stats, pool_trim=pool_trim,
    plan_cache_size=plan_cache_size)


def cuda_compiled() -> bool:
    return True


def install() -> types.ModuleType:
    """Insert this module as ``conatus._core`` (before the reference package is imported) so the
    reference's loader picks it up (python/conatus/runtime/__init__.py:55-59)."""
    sys.modules["conatus._core"] = sys.modules[__name__]
    return sys.modules[__name__]
