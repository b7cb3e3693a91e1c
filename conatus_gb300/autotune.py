"""Autotuner of the batched banded solve: the schedule of the step's solve is picked by timing.

Candidates: the band kernel (one warp per system over the LU band, ``cng_banded_set_schedule(h,
-1)``) and the compact-stream schedules of ``cng_banded_schedules`` (two systems per warp over the
union pattern of the factors, with different staging chunks and ring depths, over whole vectors
or over windows of them with the rest in a scratch (more resident warps, the same bits); one
system per warp with the lanes split over entries and components for small batches; and the
partitioned solve of small FP64 batches, one block of warps per system sweeping its blocks of 32
columns at once). The
partitioned solve is a candidate only where the DeviceProblem opts into it (``dev.partitioned``,
or CONATUS_GB300_PARTITIONED=1): its residuals run up to about 15x those of the sequential sweeps.
Candidates a factor set cannot take (a shared pair, the FP32 form, a batch too large for the
partitioned solve's responses) are refused by the library and skipped. Each candidate solves
the step's systems (all buckets, one batched call, the FP32 form with its refinement residual) a
few times on the factors at hand; the fastest is kept for every handle of the factor set. Results
are cached per process by the shapes of the buckets (batch, n, border, band) and the precision, so
runs of the same resolution (a serving stream, an ensemble) are timed once. The environment variable
CONATUS_GB300_SOLVE_SCHEDULE fixes the schedule instead (-1, 0, 1, ...), e.g. for profiling.

The F evaluation's transforms are tuned the same way (``tune_rhs``: sequences and threads per
block of the shared-memory FFTs), once per problem shape and precision; CONATUS_GB300_RHS_TUNING
("sequences,threads") fixes them instead.

The reference chooses its solve kernel by constructor flags (python/conatus/runtime/cuda.py:140-152).
"""
from __future__ import annotations

import ctypes
import os

from ._lib import call

__all__ = ["schedules", "split_schedules", "partitioned_schedules", "windowed_schedules", "tune_solve", "tune_rhs",
           "cache"]

_CACHE: dict = {}


def schedules() -> list:
    """Candidate schedules: -1 (band kernel) and 0 .. count-1 (compact)."""
    n = ctypes.c_int32()
    call("cng_banded_schedules", ctypes.byref(n), None, None, None)
    return [-1] + list(range(int(n.value)))


def _flags() -> list:
    n = ctypes.c_int32()
    call("cng_banded_schedules", ctypes.byref(n), None, None, None)
    flags = (ctypes.c_int32 * n.value)()
    call("cng_banded_schedules", ctypes.byref(n), None, None, flags)
    return list(flags)


def split_schedules() -> set:
    """Compact schedules that do not sweep two systems per warp over whole vectors and refuse
    shared pairs: one system per warp with the lanes split over entries and components (the
    latency variant: the same sweeps, another order of sums in the border correction), and the
    partitioned solve."""
    return {k for k, f in enumerate(_flags()) if f in (1, 2)}


def partitioned_schedules() -> set:
    """Schedules of the partitioned solve (small batches, FP64: blocks of 32 columns swept at once
    with their responses to the blocks before them); refused for the FP32 form, shared pairs,
    system ranges and large batches."""
    return {k for k, f in enumerate(_flags()) if f == 2}


def windowed_schedules() -> set:
    """Schedules of the windowed compact solve: the two-systems sweeps with a window of each vector
    in shared memory and the rest in a per-handle scratch (more resident warps; the same bits as
    schedule 0)."""
    return {k for k, f in enumerate(_flags()) if f == 3}


def cache() -> dict:
    return dict(_CACHE)


def _signature(dev, fs):
    return (dev.precision, bool(getattr(dev, "partitioned", False)),
            tuple((h.batch, h.n, h.rank, h.kl, h.ku, getattr(h, "primary", -1)) for h in fs))


def apply(fs, sched: int) -> None:
    for h in fs:
        if h.h is None:                   # a shared pair's partner: solved with its primary's schedule
            continue
        call("cng_banded_set_schedule", h.h, int(sched))
        h.schedule = int(sched)


def tune_solve(dev, key, fs, stream=None, reps: int = 3, candidates=None) -> dict:
    """Time every candidate schedule on the factor set ``fs`` of ``dev`` (key = (a, b)) and keep
    the fastest. Returns {schedule: ms per solve}. Runs on ``stream`` (a torch stream or None for
    the current one); never inside a graph capture."""
    from .ivp import _torch
    torch = _torch()
    fixed = os.environ.get("CONATUS_GB300_SOLVE_SCHEDULE")
    if fixed is not None:                 # a fixed schedule instead of timing (reproducible runs)
        apply(fs, int(fixed))
        return {int(fixed): None}
    sig = _signature(dev, fs)
    if sig in _CACHE:
        apply(fs, _CACHE[sig][0])
        return _CACHE[sig][1]
    if candidates is None:
        candidates = schedules()
        if not getattr(dev, "partitioned", False):       # opted into (its residuals run larger)
            part = partitioned_schedules()
            candidates = [c for c in candidates if c not in part]
    if stream is None:
        st = torch.cuda.current_stream()
    elif isinstance(stream, int):
        st = torch.cuda.ExternalStream(stream)
    else:
        st = stream
    rhs = dev.zeros()
    out = dev.zeros()
    with torch.cuda.stream(st):
        rhs.fill_(1.0)
    times = {}
    for sched in candidates:
        try:
            apply(fs, sched)
            dev._solve_with(fs, key[0], key[1], rhs, out, st)          # warm-up (and first-use set-up)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(reps):
                dev._solve_with(fs, key[0], key[1], rhs, out, st)
            e1.record(st)
            e1.synchronize()
            times[sched] = e0.elapsed_time(e1) / reps
        except ValueError:
            continue                      # schedule does not fit (shared memory), or does not solve
                                          # shared pairs: not a candidate
    if not times:
        raise ValueError("no solve schedule fits these systems (shared memory)")
    best = min(times, key=times.get)
    apply(fs, best)
    _CACHE[sig] = (best, times)
    return times


_RHS_CACHE: dict = {}


def _set_rhs_tuning(dev, q, t) -> None:
    """One launch shape for every F evaluator of ``dev`` (a grouped problem's handles share it)."""
    for h in dev._rhs_all:
        call("cng_rhs_set_tuning", h, int(q), int(t))


def tune_rhs(dev, reps: int = 2, candidates=((1, 64), (2, 64), (1, 128), (2, 128), (4, 128), (8, 128), (2, 256),
                                               (4, 256), (8, 256), (16, 256))) -> dict:
    """Time the F evaluation of ``dev`` (a DeviceProblem) with each launch shape of its shared-memory
    transforms (sequences per block, threads per block) and keep the fastest
    (``cng_rhs_set_tuning``). Cached per precision, template, Fourier sizes and case count. Returns
    {"sequences x threads": ms per evaluation}."""
    from .ivp import _torch
    torch = _torch()
    P = dev.P
    fixed = os.environ.get("CONATUS_GB300_RHS_TUNING")
    if fixed is not None:                 # "sequences,threads" instead of timing (reproducible runs)
        q, t = (int(v) for v in fixed.split(","))
        _set_rhs_tuning(dev, q, t)
        return {f"{q}x{t}": None}
    key = (dev.precision, dev.tpl.name, tuple(P.fourier_sizes), int(getattr(P, "ncase", 1)),
           tuple(dev.nsys))
    if key in _RHS_CACHE:
        _set_rhs_tuning(dev, *_RHS_CACHE[key][0])
        return _RHS_CACHE[key][1]
    st = torch.cuda.Stream()
    x, out = dev.zeros(), dev.zeros()
    times = {}
    for q, t in candidates:
        _set_rhs_tuning(dev, int(q), int(t))
        dev.F(x, out, st)                                 # warm-up (first-use set-up)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            dev.F(x, out, st)
        e1.record(st)
        e1.synchronize()
        times[(q, t)] = e0.elapsed_time(e1) / reps
    best = min(times, key=times.get)
    _set_rhs_tuning(dev, *best)
    report = {f"{q}x{t}": v for (q, t), v in times.items()}
    _RHS_CACHE[key] = (best, report)
    return report
