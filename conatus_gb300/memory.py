"""Device-memory planner: the bytes a run will hold on the device, predicted before anything is
allocated (the serving loop's admission oracle).

The reference predicts device bytes per solver from a liveness model of its buffers
(python/conatus/runtime/memory.py); the prediction here follows this library's own allocations
one by one:

* state and work vectors: X and R (plus the FP32 form's refinement residual and its copy of x
  row-major over the systems), the history ring of
  M X and F (q slots each), complex128 over the mode layout;
* per bucket: M values (one shared copy when M is constant, else per system), L values per system,
  the pattern, the per-(row, system) scales of the residual's merged entry lists (one table per
  factor set, plus one for -L X), and the factor set of ``cng_banded_create_shared`` (band LU ldab x n, pivots, the
  border blocks V^T and W (r x n each), the capacitance LU (r x r)), its FP32 copies in the FP32
  form, and the compact factor streams (bounded above by the band: at most kl entries of L and
  kl + ku + 1 of U per column, r x n of V) with the windowed schedules' scratch (one complex128
  vector per system slot); one transient copy of a M + b L while factoring;
* the F pipeline's work buffers (``cng_rhs_create``: the spectra S and two grid buffers).

A shared pair's partner (the (kx, -kz) systems solved with the (kx, +kz) factors) holds no factors;
its primary's compact streams hold one system per warp group.

Factor sets kept: one in the steady state when the solver keeps a single set (``IVPSolver(...,
factor_sets=1)``), else one per start-up order.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = ["bucket_band", "plan_ivp", "plan_fourier_ensemble"]

_Z = 16          # complex128
_C = 8           # complex64


def bucket_band(b) -> tuple:
    """(kl, ku) of the non-border rows of a bucket in solver order (border rows 0..r-1), as the
    factorization computes them."""
    kl = ku = 0
    for i in range(b.r, b.n):
        cols = b.indices[b.indptr[i]:b.indptr[i + 1]]
        if cols.size:
            kl = max(kl, int(i - cols.min()))
            ku = max(ku, int(cols.max() - i))
    return kl, ku


def _factor_bytes(b, nsys, precision, compact, shared=False):
    n, r = b.n, b.r
    kl, ku = bucket_band(b)
    ldab = 2 * kl + ku + 1
    nnz = int(b.indices.size)
    out = nsys * (n * ldab * _Z + n * 4 + 2 * r * n * _Z + r * r * _Z + r * 4 + 4 + 8) + n * 4 + nnz * 8
    if precision == "fp32":
        out += nsys * (n * ldab * _C + 2 * r * n * _C + r * r * _C)
    if shared:
        out += 2 * n                                   # the sign flags of the partner
    if compact:
        # two systems per warp group, one for a shared pair's primary
        slots = nsys if shared else int(math.ceil(nsys / 2)) * 2
        per = n * kl + n * (kl + ku + 1) + r * n
        out += slots * (per * _Z + n * 4) + 6 * (n + 1) * 4 + per * 5
        if precision == "fp32":
            out += slots * per * _C
        # the windowed schedules' scratch (two vectors per warp group), held when the tuner picks one
        out += (2 * nsys if shared else slots) * n * _Z
    return out


def _rhs_bytes(problem, precision):
    """Work buffers of the F pipeline (the sizes ``cng_rhs_create`` allocates; a grouped problem has
    one evaluator per group)."""
    from .ivp import smooth_size
    if hasattr(problem, "parts"):
        return sum(_rhs_bytes(p, precision) for p in problem.parts)
    tpl = problem.tpl
    cs = _C if precision == "fp32" else _Z
    rs = cs // 2
    d = len(tpl.fourier_axes)
    ax = tpl.axes
    if tpl.cheb_axis >= 0:
        ny = ax[tpl.cheb_axis]["N"]
        my = smooth_size(ax[tpl.cheb_axis]["M"], even=True)
    else:
        ny = my = 1
    Kx = problem.fourier_sizes[0] // 2 if d >= 1 else 1
    mx = smooth_size(int(math.floor(problem.fourier_sizes[0] * ax[tpl.fourier_axes[0]].get("dealias", 1.5)))) if d >= 1 else 1
    if d >= 2:
        Nzc = problem.fourier_sizes[1]
        mz = smooth_size(int(math.floor(problem.fourier_sizes[1] * ax[tpl.fourier_axes[1]].get("dealias", 1.5))))
    else:
        Nzc = mz = 1
    nc = int(getattr(problem, "ncase", 1))          # stacked cases: fields of every case
    nf, no = len(tpl.factors) * nc, len(tpl.outputs) * nc
    nfo = max(nf, no)
    P = mx * mz * my
    S = max(cs * nfo * Kx * Nzc * ny, rs * nf * P)
    W = max(cs * nfo * Kx * Nzc * my, cs * nfo * Kx * mz * my, rs * nfo * mx * mz * my, cs * nfo * P)
    nlam = max(tpl.conv) if tpl.conv else 0
    return S + 2 * W + nlam * ny * ny * 8


def plan_ivp(problem, scheme: str = "SBDF2", precision: str = "fp64", compact: bool = True,
             factor_sets: int | None = None, share: bool = True) -> dict:
    """Predicted device bytes of ``IVPSolver(problem, scheme, precision=precision)``, by part,
    with the total under ``"total"``."""
    tpl = problem.tpl
    q = int(scheme[-1])
    n_total = sum(ns * b.n for ns, b in zip(problem.nsys, tpl.buckets))
    vec = n_total * _Z
    parts = {"state": vec * (2 + (2 if precision == "fp32" else 0)), "history": 2 * q * vec,
             "rhs_work": _rhs_bytes(problem, precision)}
    ops = fac = trans = rows = 0
    # shared pairs (conatus_gb300.ivp: partners solved with their primary's factors)
    pairs = tpl.sign_pairs() if compact and share else {}
    primaries = {i for i, _, _ in pairs.values()}
    vals = 0
    for bi, (b, ns) in enumerate(zip(tpl.buckets, problem.nsys)):
        nnz = int(b.indices.size)
        const_m = b.m_is_constant() and b.exact is None
        ops += (nnz * (_Z + 8) if const_m else ns * nnz * _Z) + ns * nnz * _Z + (b.n + 1 + nnz) * 4
        if bi not in pairs:
            fac += _factor_bytes(b, ns, precision, compact, shared=bi in primaries)
        vals += ns * nnz * _Z                          # a M + b L of every bucket while factoring
        trans = max(trans, ns * nnz * _Z)
        if precision == "fp32":
            ops += 2 * b.n * 16 + ns * 16 * 8        # split-operator residual lists (bounded)
        if const_m:
            rows += ns * b.n * 8                     # per-(row, system) scales of merged residual lists
    sets = q if factor_sets is None else max(1, min(q, int(factor_sets)))
    parts["operators"] = ops + rows * (sets + 1)
    parts["factors"] = fac * sets
    # while factoring: the values of every bucket (the pairs are checked on them), plus one copy
    parts["factor_transient"] = vals + trans
    parts["total"] = int(sum(parts.values()))
    return parts


def plan_fourier_ensemble(sizes, scheme: str = "SBDF2") -> dict:
    """Predicted device bytes of ``FourierEnsemble(tpl, sizes, ...)``: X and the history ring of
    N/2 complex amplitudes per member, plus the per-member descriptors."""
    q = int(scheme[-1])
    K = int(np.sum(np.asarray(sizes) // 2))
    m = len(sizes)
    parts = {"state": K * _Z, "history": 2 * q * K * _Z, "descriptors": m * (4 + 4 + 8 + 8 + 4)}
    parts["total"] = int(sum(parts.values()))
    return parts
