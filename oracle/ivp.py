"""Oracle (test infrastructure only): CPU restatement of the reference's IMEX step on the mode
layout of a problem template (``conatus_gb300.template``).

Imported only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``. It
follows, in NumPy/SciPy:

* ``_to_arrays`` / ``_to_rows``: the reference's ``GlobalSystem.scatter`` / ``gather_rhs``
  (python/conatus/timestep/system.py:876-931) composed with its complex views of RealFourier pairs
  (system.py:600-726): a_p = 2^(1-d) sum_s Re(conj(w_s(p)) C_s), R_s = sum_p w_s(p) r_p,
  w_s(p) = prod_j (i s_j)^p_j; the C^(lambda) conversion of each equation (``zconv``).
* ``F``: ``FusedRHS.evaluate`` (python/conatus/timestep/fused.py:994-1085): factor derivatives in
  coefficient space (``SpectralEvaluator._diff``, spectral.py:199-223: Fourier pair swap times k,
  Chebyshev backward recurrence ``_cheb_diff_recurrence`` spectral.py:53-80 times 2/L), backward
  transforms Chebyshev first, the product sums, forward transforms Fourier first; transforms with
  the conventions of python/conatus/reference/transforms.py:103-187 (DCT-II/III on Gauss nodes,
  rfft with (cos, -sin) pairs); plus the constant part F(0).
* ``sbdf_step``: ``IVPSolver._sbdf_step`` (python/conatus/timestep/integrator.py:361-373) with
  ``sbdf_coefficients`` (schemes.py:106-116) and ``sbdf_rhs`` (lincomb.py:146-162), solves by
  the oracle bordered-banded restatement (oracle/banded.py), factorizations cached per (a, b).
* ``CNStepper`` / ``RKStepper``: ``IVPSolver._cn_step`` (integrator.py:567-603) and
  ``rk_stages`` (integrator.py:605-646) with ``cn_coefficients`` / ``rk_tableau``
  (schemes.py:91-143), lower-order start-up.
"""
from __future__ import annotations

import itertools
import os
from collections import deque

import numpy as np
import scipy.fft as sfft
import scipy.sparse as sp

from .banded import BorderedBandedBatch

SBDF = {1: ([1, -1], [0, 1]),
        2: ([1.5, -2, 0.5], [0, 2, -1]),
        3: ([11 / 6, -3, 1.5, -1 / 3], [0, 3, -3, 1]),
        4: ([25 / 12, -4, 3, -4 / 3, 0.25], [0, 4, -6, 4, -1])}

# CN family (a in units of 1/dt, b, c), schemes.py:91-103 (Wang & Ruuth 2008)
CN = {"CNAB1": ([1.0, -1.0], [0.5, 0.5], [0.0, 1.0]),
      "CNAB2": ([1.0, -1.0, 0.0], [0.5, 0.5, 0.0], [0.0, 1.5, -0.5]),
      "MCNAB2": ([1.0, -1.0, 0.0], [9 / 16, 6 / 16, 1 / 16], [0.0, 1.5, -0.5]),
      "CNLF2": ([0.5, 0.0, -0.5], [0.5, 0.0, 0.5], [0.0, 1.0, 0.0])}


def _rk_tables():
    """IMEX Runge-Kutta tableaux (A, H, c) in cumulative form, schemes.py:106-143."""
    g = (2 - np.sqrt(2)) / 2
    d = 1 - 1 / g / 2
    al, be = (29 / 96, -3 / 40, 1 / 6), (37 / 160, 5 / 24, 1 / 6)
    ga, ze = (8 / 15, 5 / 12, 3 / 4), (-17 / 60, -5 / 12)
    return {
        "RK111": ([[0, 0], [1, 0]], [[0, 0], [0, 1]], [0, 1]),
        "RK222": ([[0, 0, 0], [g, 0, 0], [d, 1 - d, 0]], [[0, 0, 0], [0, g, 0], [0, 1 - g, g]], [0, g, 1]),
        "RK443": ([[0, 0, 0, 0, 0], [1 / 2, 0, 0, 0, 0], [11 / 18, 1 / 18, 0, 0, 0],
                   [5 / 6, -5 / 6, 1 / 2, 0, 0], [1 / 4, 7 / 4, 3 / 4, -7 / 4, 0]],
                  [[0, 0, 0, 0, 0], [0, 1 / 2, 0, 0, 0], [0, 1 / 6, 1 / 2, 0, 0],
                   [0, -1 / 2, 1 / 2, 1 / 2, 0], [0, 3 / 2, -3 / 2, 1 / 2, 1 / 2]],
                  [0, 1 / 2, 2 / 3, 1 / 2, 1]),
        "RKSMR": ([[0, 0, 0, 0], [ga[0], 0, 0, 0], [ga[0] + ze[0], ga[1], 0, 0],
                   [ga[0] + ze[0], ga[1] + ze[1], ga[2], 0]],
                  [[0, 0, 0, 0], [al[0], be[0], 0, 0], [al[0], be[0] + al[1], be[1], 0],
                   [al[0], be[0] + al[1], be[1] + al[2], be[2]]], [0, 8 / 15, 2 / 3, 1]),
        "RKGFY": ([[0, 0, 0], [1, 0, 0], [1 / 2, 1 / 2, 0]], [[0, 0, 0], [1 / 2, 1 / 2, 0], [1 / 2, 0, 1 / 2]],
                  [0, 1, 1]),
    }


RK = _rk_tables()


# ------------------------------------------------------------------------------------------------
# reference transforms (reference/transforms.py:103-187), along axis 0

def _workers(a):
    """scipy.fft threads for array ``a``: the CPU baseline's WORKERS for large arrays, one for small
    ones (starting the threads costs more than they save); None (the default) outside it."""
    return WORKERS if (WORKERS is None or a.size >= 1 << 16) else 1


def cheb_forward(f, N):
    M = f.shape[0]
    y = sfft.dct(f, type=2, axis=0, workers=_workers(f)) / M
    y[0] /= 2
    sign = (-1.0) ** np.arange(M)
    return (y * sign.reshape((M,) + (1,) * (f.ndim - 1)))[:N]


def cheb_backward(c, M):
    N = c.shape[0]
    y = np.zeros((M,) + c.shape[1:], dtype=c.dtype)
    sign = (-1.0) ** np.arange(N)
    y[:N] = c * sign.reshape((N,) + (1,) * (c.ndim - 1))
    y[0] *= 2
    y *= M
    return sfft.idct(y, type=2, axis=0, workers=_workers(y))


WORKERS = None      # scipy.fft worker threads for the CPU baseline (None: NumPy's transforms)


def _rfft(f):
    return np.fft.rfft(f, axis=0) if WORKERS is None else sfft.rfft(f, axis=0, workers=_workers(f))


def _irfft(F, n):
    return np.fft.irfft(F, n=n, axis=0) if WORKERS is None else sfft.irfft(F, n=n, axis=0, workers=_workers(F))


def rf_forward(f, N):
    M = f.shape[0]
    F = _rfft(f) / M
    K = N // 2
    c = np.zeros((N,) + f.shape[1:])
    c[0] = F[0].real
    c[2:N:2] = 2 * F[1:K].real
    c[3:N:2] = 2 * F[1:K].imag
    return c


def rf_backward(c, M):
    N = c.shape[0]
    K = N // 2
    F = np.zeros((M // 2 + 1,) + c.shape[1:], dtype=complex)
    F[0] = c[0]
    F[1:K] = (c[2:N:2] + 1j * c[3:N:2]) / 2
    F *= M
    return _irfft(F, M)


def _along(fn, a, axis, *args):
    a = np.moveaxis(a, axis, 0)
    return np.moveaxis(fn(a, *args), 0, axis)


def cheb_diff(c, length):
    """Chebyshev derivative along axis 0 (spectral.py:53-80), times 2/L."""
    N = c.shape[0]
    out = np.zeros_like(c)
    if N >= 2:
        out[N - 2] = 2 * (N - 1) * c[N - 1]
        for n in range(N - 3, -1, -1):
            out[n] = out[n + 2] + 2 * (n + 1) * c[n + 1]
        out[0] = out[0] / 2
    return out * (2.0 / length)


def rf_diff(c, length):
    """RealFourier derivative along axis 0 on (cos, -sin) pairs (spectral.py:214-221)."""
    N = c.shape[0]
    k = 2 * np.pi * np.arange(N // 2) / length
    kk = k.reshape((N // 2,) + (1,) * (c.ndim - 1))
    out = np.zeros_like(c)
    out[0::2] = -kk * c[1::2]
    out[1::2] = kk * c[0::2]
    return out


# ------------------------------------------------------------------------------------------------

class OracleProblem:
    """A template instantiated on the CPU (``conatus_gb300.template.Problem``) with the maps
    between the mode layout and the reference's coefficient arrays."""

    def __init__(self, problem):
        self.P = problem
        self.tpl = tpl = problem.tpl
        self.d = len(tpl.fourier_axes)
        self.ax_sizes = []
        for i, ax in enumerate(tpl.axes):
            if ax["kind"] == "RealFourier":
                self.ax_sizes.append(problem.fourier_sizes[tpl.fourier_axes.index(i)])
            else:
                self.ax_sizes.append(ax["N"])
        # dealiased grids: floor(N * dealias) (the reference's Basis.grid_size)
        self.grid_sizes = [int(np.floor(s * tpl.axes[i].get("dealias", tpl.axes[i]["M"] / tpl.axes[i]["N"])))
                           for i, s in enumerate(self.ax_sizes)]
        self._factors = {}

    # ---- layout maps
    def _pos_index(self, bi, m, p):
        """Per-axis index into a coefficient array for Fourier positions p (cos 0 / msin 1) of
        system m of bucket bi (Chebyshev entry left as None)."""
        idx = []
        mode = self.P.modes[bi][m]
        for i, ax in enumerate(self.tpl.axes):
            if ax["kind"] == "RealFourier":
                j = self.tpl.fourier_axes.index(i)
                idx.append(2 * int(mode[j]) + int(p[j]) if mode[j] > 0 else 0)
            else:
                idx.append(None)
        return idx

    def _weights(self, bi):
        """[(p, w_s(p))] over the Fourier positions of bucket bi's active directions."""
        b = self.tpl.buckets[bi]
        act = [j for j in range(self.d) if b.active[j]]
        out = []
        for q in itertools.product((0, 1), repeat=len(act)):
            p = [0] * self.d
            w = 1.0 + 0j
            for jj, j in enumerate(act):
                p[j] = q[jj]
                s = b.sign if j == 1 else 1
                w *= (1j * s) ** q[jj]
            out.append((tuple(p), w))
        return out

    def _shape(self, obj):
        sh = list(obj["shape"])
        rank = obj["rank"]
        for i in range(len(self.tpl.axes)):
            if sh[rank + i] > 1:
                sh[rank + i] = self.ax_sizes[i]
        return tuple(sh)

    @staticmethod
    def _index(shape, rank, comp, base, n):
        """Index of (component, Fourier positions ``base``, Chebyshev index n) in an object's
        coefficient array (size-1 axes: the object does not depend on that coordinate)."""
        idx = list(comp)
        for a, bpos in enumerate(base):
            size = shape[rank + a]
            if bpos is None:                      # Chebyshev axis
                idx.append(n if (size > 1 and n >= 0) else 0)
            else:
                idx.append(bpos if size > 1 else 0)
        return tuple(idx)

    def _flat_maps(self, bi, kind):
        """Cached per bucket: for each Fourier position p (weight w) and each object k, the
        positions of the bucket's columns (kind "col") or rows ("row") that belong to k and their
        flat indices (nsys, count) into k's coefficient array."""
        key = ("maps", kind, bi)
        if key in self._factors:
            return self._factors[key]
        tpl = self.tpl
        b = tpl.buckets[bi]
        modes = self.P.modes[bi]
        ns = modes.shape[0]
        desc = b.col if kind == "col" else b.row
        objs = tpl.variables if kind == "col" else tpl.equations
        out = []
        for p, w in self._weights(bi):
            per = {}
            for k in np.unique(desc[:, 0]):
                k = int(k)
                obj = objs[k]
                rank = obj["rank"]
                shape = self._shape(obj)
                sel = np.nonzero(desc[:, 0] == k)[0]
                idx = []
                comp = [np.unravel_index(int(cf), tuple(obj["shape"][:rank])) if rank else ()
                        for cf in desc[sel, 1]]
                for r in range(rank):
                    idx.append(np.broadcast_to(np.array([c[r] for c in comp])[None, :], (ns, sel.size)))
                for a, axd in enumerate(tpl.axes):
                    size = shape[rank + a]
                    if axd["kind"] == "RealFourier":
                        j = tpl.fourier_axes.index(a)
                        base = np.where(modes[:, j] > 0, 2 * modes[:, j] + p[j], 0)
                        ia = base[:, None] if size > 1 else np.zeros((ns, 1), int)
                        idx.append(np.broadcast_to(ia, (ns, sel.size)))
                    else:
                        nn = desc[sel, 2]
                        ia = np.where((nn >= 0) & (size > 1), nn, 0)
                        idx.append(np.broadcast_to(ia[None, :], (ns, sel.size)))
                flat = np.ravel_multi_index(tuple(np.asarray(i) for i in idx), shape)
                per[k] = (sel, flat)
            out.append((p, w, per))
        self._factors[key] = out
        return out

    def to_arrays(self, C):
        """Mode layout -> coefficient arrays of the variables (system.scatter)."""
        tpl = self.tpl
        arrs = [np.zeros(self._shape(v)) for v in tpl.variables]
        for bi in range(len(tpl.buckets)):
            da = self.P.d_active(bi)
            scale = 2.0 ** (1 - da) if da >= 1 else 1.0
            Cb = np.asarray(C[bi])
            for p, w, per in self._flat_maps(bi, "col"):
                coef = scale * np.conj(w)
                for v, (sel, flat) in per.items():
                    np.add.at(arrs[v].reshape(-1), flat.ravel(), (coef * Cb[:, sel]).real.ravel())
        return arrs

    def to_rows(self, eq_arrays):
        """Equation coefficient arrays (Chebyshev T) -> mode-layout right-hand sides, each row
        converted to its equation's C^(lambda) space (system.gather_rhs + complex view)."""
        tpl = self.tpl
        ca = tpl.cheb_axis
        conv_cache = {}
        out = []
        for bi, b in enumerate(tpl.buckets):
            R = np.zeros((self.P.nsys[bi], b.n), np.complex128)
            for p, w, per in self._flat_maps(bi, "row"):
                for e, (sel, flat) in per.items():
                    arr = eq_arrays[e]
                    if arr is None:
                        continue
                    rank = tpl.equations[e]["rank"]
                    lams = np.unique(b.row[sel, 3])
                    for lam in lams:
                        sub = b.row[sel, 3] == lam
                        a = arr
                        if lam > 0 and ca >= 0 and arr.shape[rank + ca] > 1:
                            key = (e, int(lam))
                            if key not in conv_cache:
                                S = tpl.conv[int(lam)]
                                conv_cache[key] = np.moveaxis(
                                    np.tensordot(S, np.moveaxis(arr, rank + ca, 0), axes=(1, 0)), 0, rank + ca)
                            a = conv_cache[key]
                        R[:, sel[sub]] += w * a.reshape(-1)[flat[:, sub]]
            out.append(R)
        return out

    # ---- F
    def factor_arrays(self, C):
        tpl = self.tpl
        arrs = self.to_arrays(C)
        G = []
        for v, cf, orders in tpl.factors:
            var = tpl.variables[v]
            a = arrs[v]
            if var["rank"]:
                a = a.reshape((-1,) + a.shape[var["rank"]:])[cf]
            for ax, o in enumerate(orders):
                for _ in range(o):
                    if tpl.axes[ax]["kind"] == "Chebyshev":
                        a = _along(cheb_diff, a, ax, self.P.axis_length(ax))
                    else:
                        a = _along(rf_diff, a, ax, self.P.axis_length(ax))
            G.append(a)
        return G

    def F(self, C):
        """Nonlinear part (polynomial form) + constant part F(0), mode layout."""
        tpl = self.tpl
        G = self.factor_arrays(C)
        order = [i for i, ax in enumerate(tpl.axes) if ax["kind"] == "Chebyshev"] + \
                [i for i, ax in enumerate(tpl.axes) if ax["kind"] != "Chebyshev"]
        grids = []
        for g in G:
            for ax in order:
                fn = cheb_backward if tpl.axes[ax]["kind"] == "Chebyshev" else rf_backward
                g = _along(fn, g, ax, self.grid_sizes[ax])
            grids.append(g)
        eq_arrays = [None] * len(tpl.equations)
        for e, cf, monos in tpl.outputs:
            acc = np.zeros(grids[0].shape if grids else tuple(self.grid_sizes))
            for c, fs in monos:
                t = c.real if np.imag(c) == 0 else c
                for j in fs:
                    t = t * grids[j]
                acc = acc + t
            for ax in order[::-1]:
                fn = cheb_forward if tpl.axes[ax]["kind"] == "Chebyshev" else rf_forward
                acc = _along(fn, acc, ax, self.ax_sizes[ax])
            eqd = tpl.equations[e]
            if eq_arrays[e] is None:
                eq_arrays[e] = np.zeros(self._shape(eqd))
            rank = eqd["rank"]
            if rank:
                comp = np.unravel_index(cf, tuple(eqd["shape"][:rank]))
                eq_arrays[e][comp] = acc
            else:
                eq_arrays[e][...] = acc
        R = self.to_rows(eq_arrays)
        b0 = self.P.b0_dense()
        return [r + c for r, c in zip(R, b0)]

    # ---- linear algebra
    def csr(self, bi, which, m):
        b = self.tpl.buckets[bi]
        vals = self._vals(bi, which)[m]
        return sp.csr_matrix((vals, b.indices, b.indptr), shape=(b.n, b.n))

    def _vals(self, bi, which):
        key = ("vals", bi, which)
        if key not in self._factors:
            self._factors[key] = self.P.values(bi, which)
        return self._factors[key]

    def _apply(self, C, which):
        out = []
        for bi, b in enumerate(self.tpl.buckets):
            V = self._vals(bi, which)
            rows = b.coo_rows()
            Y = np.zeros_like(C[bi])
            for m in range(C[bi].shape[0]):
                np.add.at(Y[m], rows, V[m] * C[bi][m, b.indices])
            out.append(Y)
        return out

    def MX(self, C):
        return self._apply(C, "M")

    def LX(self, C):
        return self._apply(C, "L")

    def factor(self, a, b_):
        key = ("lu", float(a), float(b_))
        if key not in self._factors:
            fs = []
            for bi, b in enumerate(self.tpl.buckets):
                Vm, Vl = self._vals(bi, "M"), self._vals(bi, "L")
                mats = []
                for m in range(Vm.shape[0]):
                    vals = a * Vm[m] + b_ * Vl[m]
                    if b.kind == "real":
                        vals = vals.real
                    mats.append((b.n, b.indptr, b.indices, vals))
                dt = np.float64 if b.kind == "real" else np.complex128
                fs.append(BorderedBandedBatch(mats, list(range(b.r)), dtype=dt))
            self._factors[key] = fs
        return self._factors[key]

    def solve(self, a, b_, rhs):
        out = []
        for bi, (B, r) in enumerate(zip(self.factor(a, b_), rhs)):
            if self.tpl.buckets[bi].kind == "real":
                out.append(B.solve(r.real).astype(np.complex128))
            else:
                out.append(B.solve(r))
        return out


class SBDFStepper:
    """``IVPSolver`` SBDF-q stepping on the mode layout (integrator.py:361-373), lower-order
    start-up (q = 1, 2, .. while the history fills)."""

    def __init__(self, oproblem, order, dt):
        self.op, self.order, self.dt = oproblem, int(order), float(dt)
        self.MXh, self.Fh = deque(), deque()

    def step(self, C):
        op, dt = self.op, self.dt
        self.MXh.appendleft(op.MX(C))
        self.Fh.appendleft(op.F(C))
        while len(self.MXh) > self.order:
            self.MXh.pop()
            self.Fh.pop()
        q = min(self.order, len(self.MXh))
        a, c = SBDF[q]
        rhs = []
        for bi in range(len(C)):
            r = np.zeros_like(C[bi])
            for j in range(1, q + 1):
                r += c[j] * self.Fh[j - 1][bi] - (a[j] / dt) * self.MXh[j - 1][bi]
            rhs.append(r)
        return op.solve(a[0] / dt, 1.0, rhs)


class CNStepper:
    """``IVPSolver`` CN-family multistep stepping (integrator.py:567-603): history of M X, L X and
    F; rhs = sum_{j>=1} c_j F_j - (a_j/dt) M X_j - b_j L X_j accumulated from zero in that order
    (zero coefficients skipped); (a_0/dt M + b_0 L) X = rhs; CNAB1 until the history is full."""

    def __init__(self, oproblem, scheme, dt):
        self.op, self.dt = oproblem, float(dt)
        self.coefs = CN[scheme]
        self.nhist = len(self.coefs[0]) - 1
        self.MXh, self.LXh, self.Fh = deque(), deque(), deque()

    def step(self, C):
        op, dt = self.op, self.dt
        self.MXh.appendleft(op.MX(C))
        self.LXh.appendleft(op.LX(C))
        self.Fh.appendleft(op.F(C))
        while len(self.MXh) > self.nhist:
            self.MXh.pop()
            self.LXh.pop()
            self.Fh.pop()
        a, b, c = self.coefs if len(self.MXh) >= self.nhist else CN["CNAB1"]
        rhs = []
        for bi in range(len(C)):
            r = np.zeros_like(C[bi])
            for j in range(1, len(a)):
                if c[j] != 0:
                    r = r + c[j] * self.Fh[j - 1][bi]
                if a[j] != 0:
                    r = r - (a[j] / dt) * self.MXh[j - 1][bi]
                if b[j] != 0:
                    r = r - b[j] * self.LXh[j - 1][bi]
            rhs.append(r)
        return op.solve(a[0] / dt, b[0], rhs)


class RKStepper:
    """``IVPSolver`` IMEX Runge-Kutta step (integrator.py:605-646): M X_i = M X_0 + dt sum_k A_ik
    F_k - dt sum_k H_ik L X_k, the terms added in order k = 0.., F before L X;
    (M + dt H_ii L) X_i = rhs."""

    def __init__(self, oproblem, scheme, dt):
        self.op, self.dt = oproblem, float(dt)
        self.A, self.H, self.c = RK[scheme]

    def step(self, C):
        op, dt, A, H = self.op, self.dt, self.A, self.H
        S = len(self.c) - 1
        X = [C]
        Fs, LX = [None] * (S + 1), [None] * (S + 1)
        MX0 = op.MX(C)
        for i in range(1, S + 1):
            j = i - 1
            if any(A[m][j] != 0 for m in range(j + 1, S + 1)):
                Fs[j] = op.F(X[j])
            if any(H[m][j] != 0 for m in range(j + 1, S + 1)):
                LX[j] = op.LX(X[j])
            rhs = []
            for bi in range(len(C)):
                r = MX0[bi].copy()
                for k in range(i):
                    if A[i][k] != 0:
                        r = r + (dt * A[i][k]) * Fs[k][bi]
                    if H[i][k] != 0:
                        r = r - (dt * H[i][k]) * LX[k][bi]
                rhs.append(r)
            X.append(op.solve(1.0, dt * H[i][i], rhs))
        return X[-1]


def _factor_batches(jobs):
    """Factorizations (the oracle restatement of banded.hpp) of a share of every bucket's systems:
    one batch per bucket, None where the share is empty."""
    from .banded import BorderedBandedBatch
    batches = []
    for n, r, real, indptr, indices, monos_val, Mc, Lc, a, b_ in jobs:
        if monos_val.shape[0] == 0:
            batches.append(None)
            continue
        Vm = monos_val.astype(np.complex128) @ Mc
        Vl = monos_val.astype(np.complex128) @ Lc
        vals = a * Vm + b_ * Vl
        if real:
            vals = vals.real
        mats = [(n, indptr, indices, v) for v in vals]
        batches.append(BorderedBandedBatch(mats, list(range(r)), dtype=np.float64 if real else np.complex128))
    return batches


def _solve_batches(batches, rhs):
    out = []
    for B, b in zip(batches, rhs):
        if B is None:
            out.append(None)
        elif B.sys[0].dtype == np.float64:
            out.append(B.solve(b.real).astype(np.complex128))
        else:
            out.append(B.solve(b))
    return out


def _solve_worker(conn):
    """A worker process of ``ParallelStepper``: holds the factorizations of its share of the systems
    of every bucket and solves them on request."""
    batches = []
    while True:
        msg = conn.recv()
        if msg[0] == "factor":
            batches = _factor_batches(msg[1])
            conn.send("ok")
        elif msg[0] == "solve":
            conn.send(_solve_batches(batches, msg[1]))
        else:
            conn.close()
            return


class ParallelStepper:
    """The oracle's SBDF-q step on a whole workload, timed as the CPU baseline: F (transforms on
    ``workers`` scipy.fft threads), M X, the right-hand side of ``SBDFStepper.step`` and the solves
    of every system of every bucket, spread over up to ``workers`` processes (started with
    ``spawn``; at least 64 systems each, so a few dozen systems are solved in this process: the
    messages cost more than the solves of a small share), each
    holding the factorizations of its share (made before the timing: the reference times steps
    after a warm-up that factors, examples/benchmarks/cases.py:27-43)."""

    SYSTEMS_PER_PROCESS = 64

    def __init__(self, problem, order, dt, workers=None):
        import multiprocessing as mp
        global WORKERS
        workers = int(workers or os.cpu_count() or 1)
        WORKERS = workers
        self.op = OracleProblem(problem)
        self.P = problem
        self.order, self.dt = int(order), float(dt)
        self.workers = workers
        a0 = SBDF[self.order][0][0] / self.dt
        self._procs, self._conns, self._shares, self._local = [], [], [], None
        nb = len(problem.tpl.buckets)
        nproc = max(1, min(workers, -(-sum(problem.nsys) // self.SYSTEMS_PER_PROCESS)))
        self.processes = nproc if nproc > 1 else 0
        bounds = [np.linspace(0, ns, nproc + 1).round().astype(int) for ns in problem.nsys]

        def jobs_of(w):
            jobs, share = [], []
            for bi, b in enumerate(problem.tpl.buckets):
                lo, hi = int(bounds[bi][w]), int(bounds[bi][w + 1])
                mv = problem.mono_values(bi)[lo:hi]
                jobs.append((b.n, b.r, b.kind == "real", b.indptr, b.indices, mv, b.Mc, b.Lc, a0, 1.0))
                share.append((lo, hi))
            return jobs, share

        if nproc == 1:
            jobs, share = jobs_of(0)
            self._local = _factor_batches(jobs)
            self._shares.append(share)
        else:
            ctx = mp.get_context("spawn")
            for w in range(nproc):
                parent, child = ctx.Pipe()
                pr = ctx.Process(target=_solve_worker, args=(child,), daemon=True)
                pr.start()
                child.close()
                jobs, share = jobs_of(w)
                parent.send(("factor", jobs))
                self._procs.append(pr)
                self._conns.append(parent)
                self._shares.append(share)
            for c in self._conns:
                if c.recv() != "ok":
                    raise RuntimeError("oracle worker failed to factor")
        self._Mcsr = [self.op._vals(bi, "M") if not problem.tpl.buckets[bi].m_is_constant() else None
                      for bi in range(nb)]

    def close(self):
        for c in self._conns:
            try:
                c.send(("stop",))
            except (BrokenPipeError, OSError):
                pass
        for p in self._procs:
            p.join(timeout=10)
        self._conns, self._procs = [], []

    def __del__(self):
        if getattr(self, "_conns", None):
            self.close()

    def _mx(self, C):
        out = []
        for bi, b in enumerate(self.P.tpl.buckets):
            if self._Mcsr[bi] is None:               # one M for every system of the bucket
                mv = self.P.mono_values(bi)[:1].astype(np.complex128) @ b.Mc
                A = sp.csr_matrix((mv[0], b.indices, b.indptr), shape=(b.n, b.n))
                out.append(np.asarray(C[bi] @ A.T))
            else:                                    # per-system values on the bucket's pattern:
                V = self._Mcsr[bi]                   # row sums of the products, all systems at once
                prod = V * C[bi][:, b.indices]
                Y = np.zeros_like(C[bi])
                full = np.diff(b.indptr) > 0
                if prod.shape[1]:
                    Y[:, full] = np.add.reduceat(prod, b.indptr[:-1][full], axis=1)
                out.append(Y)
        return out

    def _solve(self, rhs):
        if self._local is not None:                  # a handful of systems: this process
            xs = _solve_batches(self._local, rhs)
            return [x if x is not None else np.empty_like(r) for x, r in zip(xs, rhs)]
        for c, share in zip(self._conns, self._shares):
            c.send(("solve", [np.ascontiguousarray(r[lo:hi]) for r, (lo, hi) in zip(rhs, share)]))
        out = [np.empty_like(r) for r in rhs]
        for c, share in zip(self._conns, self._shares):
            xs = c.recv()
            for bi, (x, (lo, hi)) in enumerate(zip(xs, share)):
                if x is not None:
                    out[bi][lo:hi] = x
        return out

    def time_steps(self, C0, steps=1, warmup=0):
        """Seconds per step (mean over ``steps`` steps after ``warmup`` untimed ones) from the
        state C0, and a description. Every step is of the full order: the history starts as
        ``order - 1`` copies of C0's M X and F (made before the timing), so that one factor set
        serves every step (the reference's lower-order start-up would need one set per order)."""
        import time
        C = [np.asarray(c, np.complex128) for c in C0]
        F0, MX0 = self.op.F(C), self._mx(C)
        hist_f = deque([F0] * (self.order - 1))
        hist_mx = deque([MX0] * (self.order - 1))
        a, c = SBDF[self.order]
        times = []
        for it in range(warmup + steps):
            t0 = time.perf_counter()
            hist_f.appendleft(self.op.F(C))
            hist_mx.appendleft(self._mx(C))
            while len(hist_f) > self.order:
                hist_f.pop()
                hist_mx.pop()
            rhs = []
            for bi in range(len(C)):
                r = np.zeros_like(C[bi])
                for j in range(1, self.order + 1):
                    r += c[j] * hist_f[j - 1][bi] - (a[j] / self.dt) * hist_mx[j - 1][bi]
                rhs.append(r)
            C = self._solve(rhs)
            if it >= warmup:
                times.append(time.perf_counter() - t0)
        self.state = C
        desc = (f"{steps} full step(s) after {warmup} untimed: F, M X, right-hand side and the "
                f"banded solves of all {sum(self.P.nsys)} systems ({self.P.real_unknowns()} unknowns) "
                + (f"on {self.processes} processes" if self.processes else "in one process")
                + f"; factorizations untimed; scipy.fft workers={WORKERS} (one thread for small arrays)")
        return float(np.mean(times)), desc
