"""CPU: the split operator of the FP64 refinement residual (DeviceProblem._split_operator), with the
terms of a row that share their entry list merged under one per-(row, system) scale, reproduces
r = b - (a M + c L) x of the dense per-system operator (the arithmetic of k_split_residual restated
in NumPy, group by group)."""
from __future__ import annotations

import numpy as np
import pytest

from _step_cases import template


def _split_apply(split, mvh, rowscale, a, c, x, b):
    ptr, col, val, code, act, rowsets = split
    n = len(ptr) - 1
    r = np.array(b, dtype=complex)
    for i in range(n):
        e, e1 = ptr[i], ptr[i + 1]
        acc = 0j
        while e < e1:
            tt = code[e] >> 1
            g = 0j
            while e < e1 and (code[e] >> 1) == tt:
                g += (1j if code[e] & 1 else 1.0) * val[e] * x[col[e]]
                e += 1
            from conatus_gb300.ivp import SPLIT_MERGED
            sc = rowscale[i] if tt == SPLIT_MERGED else (a if tt < 0 else c * mvh[tt])
            acc += sc * g
        r[i] = b[i] - acc
    return r


@pytest.mark.parametrize("tname,sizes", [("channel_ny17", [8, 8]), ("rb_nz16", [32])])
def test_split_operator_matches_dense(tname, sizes, rng=np.random.default_rng(3)):
    from conatus_gb300.ivp import SPLIT_MERGED, DeviceProblem
    P = template(tname).instantiate(sizes)
    merged_seen = False
    for bi, b in enumerate(P.tpl.buckets):
        if not b.m_is_constant() or b.exact is not None:
            continue
        terms = [(b.Lc[t], P.mono_values(bi)[:, t]) for t in range(b.monos.shape[0]) if np.any(b.Lc[t] != 0)]
        split = DeviceProblem._split_operator(b, [row for row, _ in terms])
        assert split is not None
        ptr, col, val, code, act, rowsets = split
        merged_seen |= bool(np.any((code >> 1) == SPLIT_MERGED))
        mv = np.stack([terms[k][1] for k in act], axis=1)
        Mv, Lv = P.values(bi, "M"), P.values(bi, "L")
        rows = b.coo_rows()
        for a, c in ((366.7, 1.0), (0.0, 1.0), (1.0, 2.5e-3)):
            tab = DeviceProblem._rowscale_table(rowsets, mv, b.n, a, c)
            for m in sorted({0, P.nsys[bi] // 2, P.nsys[bi] - 1}):
                Mm = Mv[m] if Mv.ndim == 2 else Mv
                A = np.zeros((b.n, b.n), complex)
                np.add.at(A, (rows, b.indices), a * Mm + c * Lv[m])
                x = rng.standard_normal(b.n) + 1j * rng.standard_normal(b.n)
                rhs = rng.standard_normal(b.n) + 1j * rng.standard_normal(b.n)
                ref = rhs - A @ x
                got = _split_apply(split, mv[m], tab[:, m], a, c, x, rhs)
                scale = np.abs(A).max() * np.abs(x).max() * b.n
                assert np.abs(got - ref).max() <= 1e-13 * scale, (bi, a, c, m)
    if tname.startswith("channel"):
        assert merged_seen                         # M, kx^2 and kz^2 share the conversion rows
