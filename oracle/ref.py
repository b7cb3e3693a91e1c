"""Oracle (test infrastructure only): ctypes face of ``oracle/_ref/libref_banded.so``, the
reference's own ``core/include/conatus/banded.hpp`` compiled unmodified (``oracle/Makefile``).

Available only where the reference sources were present at build time (``available()``).
LAPACK is SciPy's: the function pointers of ``scipy.linalg.cython_lapack`` are handed to the
library once (the reference binds the same routines, lapack.hpp:6-25).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_LIB = None
_HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(_HERE, "_ref", "libref_banded.so")


def available() -> bool:
    return os.path.exists(PATH)


def _capsule_ptr(cap) -> int:
    get = ctypes.pythonapi.PyCapsule_GetPointer
    get.restype = ctypes.c_void_p
    get.argtypes = [ctypes.py_object, ctypes.c_char_p]
    name = ctypes.pythonapi.PyCapsule_GetName
    name.restype = ctypes.c_char_p
    name.argtypes = [ctypes.py_object]
    return get(cap, name(cap))


def lib():
    global _LIB
    if _LIB is None:
        if not available():
            raise RuntimeError(f"{PATH} not built (make -C oracle, needs the reference sources)")
        L = ctypes.CDLL(PATH)
        import scipy.linalg.cython_lapack as cl
        names = ["dgbtrf", "dgbtrs", "zgbtrf", "zgbtrs", "dgetrf", "dgetrs", "zgetrf", "zgetrs"]
        ptrs = (ctypes.c_void_p * 8)(*[_capsule_ptr(cl.__pyx_capi__[n]) for n in names])
        L.ref_set_lapack(ptrs)
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_batch_create.restype = ctypes.c_void_p
        L.ref_batch_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int]
        L.ref_batch_info.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p]
        L.ref_batch_solve.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                      ctypes.c_int]
        L.ref_batch_destroy.argtypes = [ctypes.c_int, ctypes.c_void_p]
        _LIB = L
    return _LIB


class RefBatch:
    """The reference's ``BorderedBanded<T>`` over a batch of CSR matrices of equal size n."""

    def __init__(self, mats, border, dtype):
        L = lib()
        self.cplx = np.dtype(dtype).kind == "c"
        self.dtype = np.complex128 if self.cplx else np.float64
        mats = list(mats)
        self.batch = len(mats)
        self.n = n = int(mats[0][0])
        indptr = np.concatenate([np.asarray(m[1], np.int32) for m in mats])
        indices = np.concatenate([np.asarray(m[2], np.int32) for m in mats])
        data = np.concatenate([np.asarray(m[3], self.dtype) for m in mats])
        off = np.cumsum([0] + [len(m[3]) for m in mats[:-1]]).astype(np.int64)
        bd = np.asarray(list(border), np.int32)
        self._keep = (indptr, indices, data, off, bd)
        h = L.ref_batch_create(int(self.cplx), self.batch, n, indptr.ctypes.data, indices.ctypes.data,
                               data.ctypes.data, off.ctypes.data, bd.ctypes.data, len(bd))
        if not h:
            msg = L.ref_last_error().decode()
            raise (ValueError if "non-finite" in msg or "border" in msg else RuntimeError)(msg)
        self._h = h

    def info(self, k):
        v = np.zeros(4, np.int32)
        c = ctypes.c_double()
        lib().ref_batch_info(int(self.cplx), self._h, k, v.ctypes.data, ctypes.byref(c))
        return dict(n=int(v[0]), kl=int(v[1]), ku=int(v[2]), rank=int(v[3]), cond=c.value)

    def solve(self, b, transpose=False, threads=1):
        x = np.array(b, dtype=self.dtype, order="C", copy=True)
        if x.shape != (self.batch, self.n):
            raise ValueError("batch size mismatch")
        if lib().ref_batch_solve(int(self.cplx), self._h, x.ctypes.data, int(transpose), int(threads)):
            raise RuntimeError(lib().ref_last_error().decode())
        return x

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().ref_batch_destroy(int(self.cplx), h)
            self._h = None


def install_compiled_core(version: str = "0.5.0"):
    """Insert a ``conatus._core`` whose batched bordered-banded solver is the reference's own
    compiled ``BorderedBanded<T>`` (this library), so that the reference's Python package runs its
    CPU path on its own C++ solves (threaded as the reference threads them, core/bindings/
    module.cpp:181-206). Single systems use the oracle restatement. Test infrastructure only."""
    import sys
    import types
    from .banded import BorderedBanded

    class _Batch:
        def __init__(self, mats, border, col_border=False):
            if col_border:
                raise NotImplementedError("oracle: the column border is not bound")
            self._b = RefBatch(mats, border, self._dtype)
            info = [self._b.info(k) for k in range(self._b.batch)]
            self._kl = max((i["kl"] for i in info), default=0)
            self._ku = max((i["ku"] for i in info), default=0)

        kl = property(lambda self: self._kl)
        ku = property(lambda self: self._ku)

        def __len__(self):
            return self._b.batch

        def solve(self, b, transpose=False, threads=1):
            return self._b.solve(b, transpose, threads)

    def typed(base, dtype, suffix):
        return type(base.__name__ + suffix, (base,), {"_dtype": dtype})

    def single(dtype, suffix):
        class Typed(BorderedBanded):
            def __init__(self, *a, **k):
                super().__init__(*a, dtype=dtype, **k)
        Typed.__name__ = "BorderedBanded" + suffix
        return Typed

    m = types.ModuleType("conatus._core")
    m.__version__ = version
    m.BorderedBandedBatchD = typed(_Batch, np.float64, "D")
    m.BorderedBandedBatchZ = typed(_Batch, np.complex128, "Z")
    m.BorderedBandedD = single(np.float64, "D")
    m.BorderedBandedZ = single(np.complex128, "Z")
    m.cuda_compiled = lambda: False
    sys.modules["conatus._core"] = m
    return m
