"""CPU: the C-ABI library builds, loads without a GPU, and exports every function that
include/conatus_gb300.h declares (no compute calls)."""
from __future__ import annotations

import ctypes
import os
import re

from conftest import ROOT


def declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"\b(cng_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from conatus_gb300 import build, _lib
    path = build.build()
    L = ctypes.CDLL(path)
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding knows every declared symbol too
    assert set(declared()) <= set(_lib.EXPORTS), sorted(set(declared()) - set(_lib.EXPORTS))


def test_library_reports_no_device_on_cpu_host():
    import torch
    from conatus_gb300 import _lib
    if not torch.cuda.is_available():
        assert _lib.lib().cng_cuda_available() == 0


def test_solve_schedule_table():
    """The schedules the autotuner times: chunks of 2-16 columns, rings 2-4 deep, the split-lane
    (flag 1), partitioned (2) and windowed (3) variants flagged (a host-only query)."""
    from conatus_gb300 import autotune
    n = ctypes.c_int32()
    from conatus_gb300._lib import call
    call("cng_banded_schedules", ctypes.byref(n), None, None, None)
    chunk, stages, split = ((ctypes.c_int32 * n.value)() for _ in range(3))
    call("cng_banded_schedules", ctypes.byref(n), chunk, stages, split)
    assert n.value >= 8
    assert all(chunk[k] in (2, 4, 8, 16) and 2 <= stages[k] <= 4 for k in range(n.value))
    assert autotune.schedules() == [-1] + list(range(n.value))
    assert all(split[k] in (0, 1, 2, 3) for k in range(n.value))
    assert autotune.split_schedules() == {k for k in range(n.value) if split[k] in (1, 2)}
    assert autotune.partitioned_schedules() == {k for k in range(n.value) if split[k] == 2}
    assert autotune.windowed_schedules() == {k for k in range(n.value) if split[k] == 3}
    assert autotune.split_schedules()                     # the latency variant is offered
    assert autotune.windowed_schedules()


def test_pool_queries_and_device_surface_attributes():
    """Host-only queries of the reference core's device surface: the pool counters (nothing
    cached), pool_trim, plan_cache_size, and every member the reference's runtime wrapper reads
    from a device BandedBatch (python/conatus/runtime/cuda.py)."""
    from conatus_gb300 import core
    live, cached, n_alloc, n_reuse = core.cuda.pool_stats()
    assert live >= 0 and n_alloc >= 0 and cached == 0 and n_reuse == 0
    core.cuda.pool_trim()
    assert core.cuda.plan_cache_size() == 0
    for name in ("batch", "build_transpose_schedule", "capacitance_cond_max", "col_border",
                 "col_border_nnz", "factor_ms", "kl", "ku", "n", "pivot", "rank", "prepare_transpose",
                 "release_band", "solve", "solve_ptr", "solve_mapped_ptr", "solve_split_ptr",
                 "solve_transpose", "solve_transpose_ptr", "level_scheduled", "level_transposed",
                 "level_merged", "level_depth_forward", "level_depth_backward", "level_steps_forward",
                 "level_steps_backward", "level_stream_bytes", "level_t_stream_bytes", "level_note",
                 "level_t_note", "level_t_steps", "band_released"):
        for cls in (core.BandedBatchD, core.BandedBatchZ):
            assert hasattr(cls, name), (cls.__name__, name)


def test_product_path_does_not_use_the_oracle():
    """The package never imports the oracle (it is the checker, not a fallback), and bench.py
    touches it only in its CPU-baseline and reference-arm functions."""
    import ast
    pkg = os.path.join(ROOT, "conatus_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                tree = ast.parse(open(os.path.join(dirpath, f)).read())
                for node in ast.walk(tree):
                    if isinstance(node, ast.ImportFrom):
                        assert not (node.module or "").startswith("oracle"), (f, node.module)
                    elif isinstance(node, ast.Import):
                        assert not any(a.name.startswith("oracle") for a in node.names), f
    tree = ast.parse(open(os.path.join(ROOT, "bench.py")).read())
    users = set()
    for fn in [n for n in tree.body if isinstance(n, ast.FunctionDef)]:
        for node in ast.walk(fn):
            if isinstance(node, ast.ImportFrom) and (node.module or "").startswith("oracle"):
                users.add(fn.name)
    assert users <= {"cpu_baseline", "run_reference"}, users
    top = [n for n in tree.body if isinstance(n, (ast.Import, ast.ImportFrom))]
    assert not any(isinstance(n, ast.ImportFrom) and (n.module or "").startswith("oracle") for n in top)


def test_binding_argument_counts_match_the_header():
    """Every ctypes signature in the Python binding has the header declaration's arguments, in
    number and in type (a mismatch would pass wrong values across the C-ABI: a 32-bit int where
    the function takes a 64-bit one leaves the register's upper half undefined)."""
    from conatus_gb300 import _lib
    C = ctypes
    accepted = {"ptr": (C.c_void_p, C.c_char_p), "int": (C.c_int, C.c_int32), "int32_t": (C.c_int32, C.c_int),
                "int64_t": (C.c_int64, C.c_longlong), "long long": (C.c_longlong, C.c_int64),
                "double": (C.c_double,), "float": (C.c_float,), "size_t": (C.c_size_t,),
                "uint64_t": (C.c_uint64,)}
    txt = open(os.path.join(ROOT, "include", "conatus_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    decls = dict(re.findall(r"\b(cng_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt))
    checked = 0
    for name, argtypes in _lib._SIGS.items():
        if name not in decls:
            continue
        params = decls[name].strip()
        params = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
        assert len(params) == len(argtypes), (name, len(params), len(argtypes))
        for p, a in zip(params, argtypes):
            kind = "ptr" if "*" in p else " ".join(p.replace("const ", "").split()[:-1])
            assert a in accepted[kind], (name, p, a)
        checked += 1
    assert checked >= 40
