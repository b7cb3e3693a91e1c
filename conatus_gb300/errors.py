"""Errors of the C-ABI mapped to Python exceptions.

The reference maps C++ ``std::invalid_argument`` to ``ValueError`` and ``runtime_error`` /
``logic_error`` to ``RuntimeError`` (nanobind defaults; core/bindings/module.cpp), and refuses
rather than falls back (a GPU never silently becomes the CPU). The same mapping is kept here.
"""
from __future__ import annotations


class CudaError(RuntimeError):
    """A CUDA failure, or the CUDA library is missing (never a silent CPU fallback)."""


class NumericalError(RuntimeError):
    """A run has blown up: its state holds a NaN or an infinity (the reference's
    ``conatus.errors.NumericalError`` of the finite-state check, python/conatus/timestep/
    run_checks.py:67-99)."""


def check_status(status: int, message: str, where: str) -> None:
    if status == 1:
        raise ValueError(message)
    if status == 2:
        raise RuntimeError(message)
    if status == 3:
        raise CudaError(f"{where}: {message}")
    if status == 4:
        raise MemoryError(f"{where}: {message}")
    raise RuntimeError(f"{where}: status {status}: {message}")
