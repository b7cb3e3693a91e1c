"""Readers of the banded golden fixtures (tests/golden/banded_*.npz)."""
from __future__ import annotations

import numpy as np

from conftest import golden

CASES = ["banded_burgers128.npz", "banded_rb32x16.npz", "banded_channel8x17x8.npz"]


def buckets(name):
    """[(label, dtype, mats (n, indptr, indices, data) list, border, rhs, x, xt, (kl, ku))]."""
    g = golden(name)
    out = []
    for bi, label in enumerate(g["labels"]):
        p = f"b{bi}_"
        ip, ix, d, nnz = g[p + "indptr"], g[p + "indices"], g[p + "data"], g[p + "nnz"]
        off = np.concatenate([[0], np.cumsum(nnz)])
        n = ip.shape[1] - 1
        mats = [(n, ip[k], ix[off[k]:off[k + 1]], d[off[k]:off[k + 1]]) for k in range(len(nnz))]
        out.append((str(label), d.dtype, mats, list(g[p + "border"]), g[p + "rhs"], g[p + "x"],
                    g[p + "xt"], tuple(g[p + "band"])))
    return out


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
