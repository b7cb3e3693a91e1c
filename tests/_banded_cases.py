"""Readers of the banded golden fixtures (tests/golden/banded_*.npz)."""
from __future__ import annotations

import numpy as np

from conftest import golden

COND = {}
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
        COND[(name, str(label))] = float(np.max(g[p + "cond"]))
    return out


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def tol_vs_reference(name, label):
    """Tolerance of a solve against the reference's solution on these (seeded, random) right-hand
    sides: 1e-12 relative, widened to a tenth of the forward-error bound eps * cond(A) of a
    backward-stable solver when the system is ill-conditioned (both solvers err by up to that)."""
    return max(1e-12, 0.1 * np.finfo(float).eps * COND[(name, label)])


def backward_error(mats, x, b, transpose=False):
    """max over systems of ||A x - b|| / (||A|| ||x|| + ||b||) (size-independent property)."""
    import scipy.sparse as sp
    worst = 0.0
    for k, (n, ip, ix, d) in enumerate(mats):
        A = sp.csr_matrix((d, ix, ip), shape=(n, n))
        if transpose:
            A = A.T
        r = A @ x[k] - b[k]
        worst = max(worst, np.linalg.norm(r) / (sp.linalg.norm(A) * np.linalg.norm(x[k]) + np.linalg.norm(b[k])))
    return worst
