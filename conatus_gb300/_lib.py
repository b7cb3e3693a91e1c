"""ctypes binding of ``libconatus_gb300.so`` (the C-ABI of ``include/conatus_gb300.h``).

The library is built in-tree (``conatus_gb300.build``). If it is missing or cannot be loaded,
every entry point raises: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

from .errors import CudaError, check_status

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libconatus_gb300.so")

_lib = None
_lock = threading.Lock()

c_int, c_void_p, c_double, c_char_p = ctypes.c_int, ctypes.c_void_p, ctypes.c_double, ctypes.c_char_p
P = ctypes.c_void_p


class MatvecPart(ctypes.Structure):
    """cng_matvec_part: one bucket of a grouped M X launch."""
    _fields_ = [("nsys", ctypes.c_int32), ("n", ctypes.c_int32), ("indptr", P), ("indices", P), ("values", P),
                ("x", P), ("y", P)]


class ResidualPart(ctypes.Structure):
    """cng_residual_part: systems s0 .. s1 - 1 of one bucket of a grouped residual launch."""
    _fields_ = [("nsys", ctypes.c_int32), ("s0", ctypes.c_int32), ("s1", ctypes.c_int32), ("n", ctypes.c_int32),
                ("ptr", P), ("col", P), ("val", P), ("code", P), ("mono", P), ("nmono", ctypes.c_int32),
                ("rowscale", P), ("x", P), ("xT", P), ("b", P), ("r", P)]

# name -> argtypes (all return int status unless listed in _RESTYPES)
_SIGS = {
    "cng_last_error": [],
    "cng_version": [],
    "cng_cuda_available": [],
    "cng_device_name": [c_int, c_char_p, c_int],
    "cng_mem_info": [P, P],
    "cng_pool_stats": [P, P, P, P],
    "cng_pool_trim": [],
    "cng_banded_create_csr": [c_int, c_int, c_int, P, P, P, P, P, c_int, c_int, P, P],
    "cng_banded_create_shared": [c_int, c_int, c_int, P, P, c_int, P, P, c_int, c_int, P, P],
    "cng_banded_refactor_shared": [P, P, P],
    "cng_banded_destroy": [P],
    "cng_banded_info": [P, P, P],
    "cng_banded_capacitance_cond": [P, P],
    "cng_banded_solve": [P, P, P],
    "cng_banded_solve_mapped": [P, P, P, P, P, P],
    "cng_banded_solve_split": [P, P, P, P, P, P, P, P],
    "cng_banded_prepare_transpose": [P, P],
    "cng_banded_solve_transpose": [P, P, P],
    "cng_banded_solve_host": [P, P, P, c_int],
    "cng_banded_solve_host_static": [P, P, P, c_int],
    "cng_banded_make_fp32": [P, P],
    "cng_banded_compact": [P, P],
    "cng_banded_solve_batch": [c_int, P, P, P, c_int, c_int, P],
    "cng_banded_schedules": [P, P, P, P],
    "cng_banded_set_schedule": [P, c_int],
    "cng_banded_solve_fp32": [P, P, P, c_int, P],
    "cng_poly_residual": [c_int, c_int, P, P, P, P, P, c_int, c_double, c_double, P, P, P, P],
    "cng_twiddle_table": [c_int, c_int, P],
    "cng_fourier_ensemble_step": [P, P, P, P, c_int, P, P, c_double, P],
    "cng_rhs_create": [P, P],
    "cng_rhs_destroy": [P],
    "cng_rhs_evaluate": [P, P, P, P],
    "cng_rhs_evaluate_group": [c_int, P, P, P, P],
    "cng_csr_matvec_real_group": [c_int, P, P],
    "cng_split_residual_group": [c_int, P, c_double, c_double, P],
    "cng_rhs_workspace_bytes": [P, P],
    "cng_rhs_set_tuning": [P, c_int, c_int],
    "cng_cheb_transform": [c_int, P, P, ctypes.c_int64, c_int, c_int, P],
    "cng_fft_axis": [c_int, P, P, ctypes.c_int64, c_int, c_int, c_int, P],
    "cng_rfft_axis": [c_int, P, P, ctypes.c_int64, c_int, c_int, c_int, P],
    "cng_csr_matvec": [c_int, c_int, P, P, P, c_int, P, P, P],
    "cng_csr_matvec_real": [c_int, c_int, P, P, P, P, P, P],
    "cng_sbdf_rhs": [c_int, P, P, P, P, P, ctypes.c_int64, P],
    "cng_sbdf_rhs_fused": [c_int, P, P, P, P, P, ctypes.c_int64, c_int, P],
    "cng_lincomb": [ctypes.c_int64, P, c_int, P, P, P, P, P],
    "cng_check_finite": [P, ctypes.c_int64, ctypes.c_int64, P, P],
    "cng_dfma_probe": [ctypes.c_int64, c_int, P, P, P],
    "cng_split_residual": [c_int, c_int, P, P, P, P, P, c_int, c_double, c_double, P, P, P, P, P, P],
    "cng_split_residual_range": [c_int, c_int, c_int, c_int, P, P, P, P, P, c_int, c_double, c_double, P, P, P,
                                 P, P, P],
    "cng_banded_solve_batch_xt": [c_int, P, P, P, P, c_int, P],
    "cng_banded_solve_batch2": [c_int, P, P, P, P, P, P, P, P, c_int, c_int, P],
    "cng_banded_share": [P, P, P, P],
    "cng_graph_begin": [P],
    "cng_graph_end": [P, P],
    "cng_graph_launch": [P, P],
    "cng_graph_destroy": [P],
}
_RESTYPES = {"cng_last_error": c_char_p, "cng_version": c_char_p}

#: names the header declares (the CPU test checks that the library exports each of them)
EXPORTS = tuple(_SIGS)


def lib():
    """The loaded library (raises if it is not built or not loadable)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise CudaError(f"{LIB_PATH} is not built: run `python -m conatus_gb300.build` "
                            "(nvcc, sm_103a). There is no CPU fallback.")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, c_int)
        _lib = L
    return _lib


def call(name: str, *args) -> None:
    """Call a status-returning entry point and raise the mapped Python error on failure."""
    L = lib()
    st = getattr(L, name)(*args)
    if st:
        check_status(st, L.cng_last_error().decode(errors="replace"), name)


def last_error() -> str:
    return lib().cng_last_error().decode(errors="replace")
