"""IMEX time stepping on the GB300: the reference's ``IVPSolver`` SBDF path on the mode layout.

``DeviceProblem`` places a problem (``template.Problem``) on the device: the explicit right-hand
side F as one ``cng_rhs`` evaluator, M of every bucket for ``M X``, and the factorizations of
``a M + b L`` (one ``cng_banded`` handle per bucket and per (a, b), assembled on the device from the
wavenumber polynomials, or from the reference's own values when the problem carries them).

``IVPSolver`` mirrors python/conatus/timestep/integrator.py:129-771 for the SBDF family:
``step()`` is ``_sbdf_step`` (integrator.py:361-373) -- M X and F(X) of the current state pushed
on the history, ``rhs = sum_j c_j F_j - (a_j/dt) M X_j`` (lincomb.py:146-162) with the
lower-order start-up of ``startup="lower_order"``, then ``(a_0/dt M + L) X = rhs`` -- and
``run_graph(n)`` replays whole steps as CUDA graphs (integrator.py:781-920). State, history and
factors stay resident in HBM; nothing is copied to the host inside a step.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import _lib
from ._lib import call
from .core import _Handle
from .errors import CudaError, NumericalError

SBDF = {1: ([1, -1], [0, 1]),
        2: ([1.5, -2, 0.5], [0, 2, -1]),
        3: ([11 / 6, -3, 1.5, -1 / 3], [0, 3, -3, 1]),
        4: ([25 / 12, -4, 3, -4 / 3, 0.25], [0, 4, -6, 4, -1])}

P32 = ctypes.POINTER(ctypes.c_int32)


def smooth_size(m: int, even: bool = False) -> int:
    """Smallest n >= m whose prime factors are 2, 3 and 5 (even if requested)."""
    n = max(1, int(m))
    while True:
        k = n
        for p in (2, 3, 5):
            while k % p == 0:
                k //= p
        if k == 1 and (not even or n % 2 == 0):
            return n
        n += 1


class RhsDesc(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("ndir", ctypes.c_int32), ("nx", ctypes.c_int32),
                ("nz", ctypes.c_int32), ("mx", ctypes.c_int32), ("mz", ctypes.c_int32),
                ("ny", ctypes.c_int32), ("my", ctypes.c_int32),
                ("lx", ctypes.c_double), ("lz", ctypes.c_double), ("ly", ctypes.c_double),
                ("nfactors", ctypes.c_int32), ("noutputs", ctypes.c_int32),
                ("factors", ctypes.c_void_p), ("out_lam", ctypes.c_void_p),
                ("out_mono_ptr", ctypes.c_void_p), ("mono_coef", ctypes.c_void_p),
                ("mono_factors", ctypes.c_void_p), ("nbuckets", ctypes.c_int32),
                ("buckets", ctypes.c_void_p), ("bucket_offset", ctypes.c_void_p),
                ("modes", ctypes.c_void_p), ("colpos", ctypes.c_void_p), ("rowmap", ctypes.c_void_p),
                ("nlam", ctypes.c_int32), ("conv", ctypes.c_void_p), ("nb0", ctypes.c_int64),
                ("b0_index", ctypes.c_void_p), ("b0_value", ctypes.c_void_p),
                ("ncase", ctypes.c_int32), ("case_of", ctypes.c_void_p)]


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise CudaError("conatus_gb300 needs a CUDA device (there is no CPU fallback)")
    return torch


def _stream_handle(stream) -> int:
    if stream is None:
        return _torch().cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


SPLIT_MERGED = 63      # code >> 1 of a merged entry list of the split residual (scale per row, system)

#: finite-state check cadence in steps (the reference's FINITE_CHECK_EVERY,
#: python/conatus/timestep/run_checks.py:15-20)
FINITE_CHECK_EVERY = 100
_FLAG_CLEAR = 2 ** 63 - 1


def finite_cadence(check_finite, where: str = "IVPSolver") -> int:
    """Steps between two finite-state checks: True -> 100, False -> 0 (off), n > 0 -> n
    (run_checks.finite_cadence, python/conatus/timestep/run_checks.py:36-51)."""
    if check_finite is True:
        return FINITE_CHECK_EVERY
    if check_finite is False:
        return 0
    if isinstance(check_finite, (int, np.integer)) and not isinstance(check_finite, bool) and check_finite > 0:
        return int(check_finite)
    raise ValueError(f"{where}: check_finite={check_finite!r}: True (every {FINITE_CHECK_EVERY} steps), "
                     "False (off) or a positive number of steps")


class DeviceProblem:
    """A problem instance resident on the device (see module docstring)."""

    def __init__(self, problem, precision: str = "fp64", device: str = "cuda", compact: bool = True,
                 factor_sets: int | None = None, share: bool = True):
        torch = _torch()
        _lib.lib()
        self.factor_sets = factor_sets      # None: keep every (a, b) factorization, else at most this many
        self.autotune = True                # time the solve schedules on each new factor set
        # let the tuner pick the partitioned solve of small FP64 batches (blocks of 32 columns swept
        # at once): faster on small batches, but its residuals run up to about 15x those of the
        # sequential sweeps (the blocks' separate responses cancel), so it is opted into
        self.partitioned = os.environ.get("CONATUS_GB300_PARTITIONED", "0") == "1"
        self.refine = 1                     # FP32 form: refinement passes (FP64 residual + FP32 solve)
        self.overlap_refine = True          # FP32 form: two bucket groups refined on two streams
        self._aux = None
        self._groups = None
        self._XT = None                     # FP32 form: x row-major over each bucket's systems
        self.tuning = None
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.P = problem
        self.tpl = tpl = problem.tpl
        self.precision = precision
        self.compact = bool(compact)
        # buckets solved with another bucket's factors (the reference's SharedFactor): structural
        # candidates here, the values checked at every factorization
        self._pairs = tpl.sign_pairs() if (share and self.compact) else {}
        self.shared = {}                    # partner -> primary of the current factor set
        self.device = torch.device(device)
        self.d = len(tpl.fourier_axes)
        self.nsys = list(problem.nsys)
        self.offsets = []
        off = 0
        for b, ns in zip(tpl.buckets, self.nsys):
            self.offsets.append(off)
            off += ns * b.n
        self.n_total = off
        self._build_rhs()
        # M of every bucket (constant across the bucket when it does not depend on k)
        self._M, self._pat = [], []
        for bi, b in enumerate(tpl.buckets):
            ip = torch.as_tensor(b.indptr.astype(np.int32), device=self.device)
            ix = torch.as_tensor(b.indices.astype(np.int32), device=self.device)
            self._pat.append((ip, ix))
            if b.m_is_constant() and b.exact is None:
                t0 = int(np.nonzero(np.all(b.monos == 0, axis=1))[0][0])
                mc = b.Mc[t0].astype(np.complex128)
                if np.all(mc.imag == 0):       # real mass matrix: the real-valued kernel
                    # M X runs over M's own nonzeros (the bucket pattern is that of a M + b L: on
                    # the channel two thirds of it are zeros of M)
                    keep = mc.real != 0
                    rows = np.repeat(np.arange(b.n), np.diff(b.indptr))
                    ipM = np.concatenate([[0], np.cumsum(np.bincount(rows[keep], minlength=b.n))])
                    self._M.append((torch.as_tensor(mc, device=self.device),
                                    torch.as_tensor(np.ascontiguousarray(mc.real[keep]), device=self.device),
                                    torch.as_tensor(ipM.astype(np.int32), device=self.device),
                                    torch.as_tensor(b.indices[keep].astype(np.int32), device=self.device)))
                else:
                    self._M.append((torch.as_tensor(mc, device=self.device), 0))
            else:
                self._M.append((torch.as_tensor(problem.values(bi, "M"), device=self.device).contiguous(), 1))
        self._L = [None] * len(tpl.buckets)
        self._factors = {}
        self._resid = [None] * len(tpl.buckets)
        self._R2 = None
        self.rhs_tuning = None
        if self.autotune:
            from .autotune import tune_rhs
            self.rhs_tuning = tune_rhs(self)

    # ------------------------------------------------------------------ F
    def _build_rhs(self):
        """The F evaluator: one handle, or one per group of a GroupedProblem (each placed at its
        buckets' offsets in the joint layout, evaluated together by cng_rhs_evaluate_group)."""
        P = self.P
        parts = getattr(P, "parts", None)
        self._has_b0 = []
        if parts is None:
            self._rhs_all = [self._make_rhs(P, self.offsets)]
        else:
            self._rhs_all = [self._make_rhs(p, [self.offsets[k] for k in P.group_buckets[g]])
                             for g, p in enumerate(parts)]
        self._rhs = self._rhs_all[0]
        self._rhs_arr = (ctypes.c_void_p * len(self._rhs_all))(*[h.value for h in self._rhs_all])
        self.has_b0 = any(self._has_b0)

    def _make_rhs(self, P, offsets):
        tpl = P.tpl
        d = self.d
        ax = tpl.axes
        fa = tpl.fourier_axes
        ca = tpl.cheb_axis
        desc = RhsDesc()
        desc.precision = 0 if self.precision == "fp64" else 1
        desc.ndir = d
        keep = []

        def arr(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a.ctypes.data

        if d >= 1:
            desc.nx = P.fourier_sizes[0]
            desc.mx = smooth_size(int(math.floor(P.fourier_sizes[0] * ax[fa[0]].get("dealias", 1.5))))
            desc.lx = P.lengths[0]
        if d >= 2:
            desc.nz = P.fourier_sizes[1]
            desc.mz = smooth_size(int(math.floor(P.fourier_sizes[1] * ax[fa[1]].get("dealias", 1.5))))
            desc.lz = P.lengths[1]
        if ca >= 0:
            desc.ny = ax[ca]["N"]
            desc.my = smooth_size(ax[ca]["M"], even=True)
            desc.ly = ax[ca]["L"]
        else:
            desc.ny, desc.my, desc.ly = 1, 1, 1.0
        if not self._has_b0:               # the first (or only) problem's grids
            self.grid = dict(mx=desc.mx, mz=desc.mz, my=desc.my)

        def axis_orders(orders):
            ox = orders[fa[0]] if d >= 1 else 0
            oz = orders[fa[1]] if d >= 2 else 0
            oy = orders[ca] if ca >= 0 else 0
            return ox, oy, oz

        facs = np.array([[v, c, *axis_orders(a)] for v, c, a in tpl.factors], np.int32).reshape(-1, 5)
        desc.nfactors = facs.shape[0]
        desc.factors = arr(facs, np.int32)
        # outputs: lambda from the rows of their equation
        # without a Chebyshev axis every field has a single coefficient, marked n = -1: index 0
        cheb_n = (lambda n: int(n)) if ca >= 0 else (lambda n: 0 if int(n) == -1 else int(n))
        lam_of = {}
        for b in tpl.buckets:
            for e, c, n, lam in b.row:
                if cheb_n(n) >= 0:
                    lam_of[(int(e), int(c))] = max(int(lam), 0)
        outs = tpl.outputs
        desc.noutputs = len(outs)
        desc.out_lam = arr([lam_of.get((e, c), 0) for e, c, _ in outs], np.int32)
        ptr, coef, mf = [0], [], []
        for e, c, monos in outs:
            for co, fs in monos:
                if len(fs) > 4:
                    raise NotImplementedError("monomials of more than 4 factors")
                if complex(co).imag != 0:
                    raise NotImplementedError("complex monomial coefficients")
                coef.append(complex(co).real)
                mf.append(list(fs) + [-1] * (4 - len(fs)))
            ptr.append(len(coef))
        desc.out_mono_ptr = arr(ptr, np.int32)
        desc.mono_coef = arr(coef if coef else [0.0], np.float64)
        desc.mono_factors = arr(mf if mf else [[-1] * 4], np.int32)
        out_index = {(e, c): o for o, (e, c, _) in enumerate(outs)}
        nb = len(tpl.buckets)
        desc.nbuckets = nb
        bd, modes_p, col_p, row_p = [], [], [], []
        ny = desc.ny
        for bi, b in enumerate(tpl.buckets):
            bd.append([P.nsys[bi], b.n, P.d_active(bi), b.sign, 1 if b.kind == "real" else 0])
            md = np.zeros((P.nsys[bi], 2), np.int32)
            if d >= 1:
                md[:, 0] = P.modes[bi][:, 0]
            if d >= 2:
                md[:, 1] = P.modes[bi][:, 1]
            modes_p.append(arr(md, np.int32))
            cp = -np.ones((facs.shape[0], ny), np.int32)
            for f, (v, c, *_o) in enumerate(facs):
                for i, (cv, cc, cn) in enumerate(b.col):
                    if cv == v and cc == c and cheb_n(cn) >= 0:
                        cp[f, cheb_n(cn)] = i
            col_p.append(arr(cp, np.int32))
            rm = -np.ones((b.n, 2), np.int32)
            for i, (e, c, n, lam) in enumerate(b.row):
                o = out_index.get((int(e), int(c)))
                if o is not None and cheb_n(n) >= 0:
                    rm[i] = (o, cheb_n(n))
                else:
                    rm[i] = (-1, 0)
            row_p.append(arr(rm, np.int32))
        desc.buckets = arr(bd, np.int32)
        desc.bucket_offset = arr(offsets, np.int64)
        ptrs = [(ctypes.c_void_p * nb)(*modes_p), (ctypes.c_void_p * nb)(*col_p), (ctypes.c_void_p * nb)(*row_p)]
        keep.extend(ptrs)
        desc.modes, desc.colpos, desc.rowmap = (ctypes.cast(p, ctypes.c_void_p).value for p in ptrs)
        ncase = int(getattr(P, "ncase", 1))
        desc.ncase = ncase
        if ncase > 1:                      # stacked cases: the case of every system
            cp_ = (ctypes.c_void_p * nb)(*[arr(P.case_of[bi], np.int32) for bi in range(nb)])
            keep.append(cp_)
            desc.case_of = ctypes.cast(cp_, ctypes.c_void_p).value
        # conversions T -> C^(lambda) for lambda = 1..max (levels no row uses: identity, unused)
        nlam = max(tpl.conv) if tpl.conv else 0
        desc.nlam = nlam
        desc.conv = arr(np.stack([tpl.conv.get(l, np.eye(ny)) for l in range(1, nlam + 1)])
                        if nlam else np.zeros(1), np.float64)
        b0 = P.b0_dense()
        idx, val = [], []
        for bi, B0 in enumerate(b0):
            m, i = np.nonzero(B0)
            for mm, ii in zip(m, i):
                idx.append(offsets[bi] + mm * tpl.buckets[bi].n + ii)
                val.append([B0[mm, ii].real, B0[mm, ii].imag])
        desc.nb0 = len(idx)
        self._has_b0.append(len(idx) > 0)
        desc.b0_index = arr(idx if idx else [0], np.int64)
        desc.b0_value = arr(val if val else [[0.0, 0.0]], np.float64)
        h = ctypes.c_void_p()
        call("cng_rhs_create", ctypes.byref(desc), ctypes.byref(h))
        return h

    def F(self, X, out, stream=None) -> None:
        """out = F(X) (mode layout, complex128 device tensors); a GroupedProblem's groups in one
        launch per stage."""
        if len(self._rhs_all) == 1:
            call("cng_rhs_evaluate", self._rhs, X.data_ptr(), out.data_ptr(), _stream_handle(stream))
        else:
            call("cng_rhs_evaluate_group", len(self._rhs_all), self._rhs_arr, X.data_ptr(), out.data_ptr(),
                 _stream_handle(stream))

    # kernel launches of the step's pieces (the count a step reports; a grouped launch takes at
    # most 8 argument sets)
    _GRP = 8

    def f_launches(self) -> int:
        """Launches of one F evaluation."""
        g8 = lambda k: -(-k // self._GRP)
        nbk = sum(1 for ns in self.nsys if ns > 0)
        stages = 2 + 2 + (2 if self.d >= 2 else 0) + 1        # Chebyshev, x (or real parts), z, products
        if len(self._rhs_all) == 1:                  # unpack and pack: every bucket in one launch
            return 2 * g8(nbk) + stages + (1 if self.has_b0 else 0)
        ng = len(self._rhs_all)
        return 2 * g8(nbk) + stages * g8(ng) + g8(sum(self._has_b0))

    def mx_launches(self) -> int:
        """Launches of one M X."""
        real = [len(self._M[bi]) == 4 for bi in range(len(self.nsys))]
        return -(-sum(1 for r, ns in zip(real, self.nsys) if r and ns > 0) // self._GRP) + \
            sum(1 for r, ns in zip(real, self.nsys) if not r and ns > 0)

    def residual_launches(self, parts=None) -> int:
        """Launches of one residual() over ``parts`` (default: every bucket): one grouped launch for
        the split-form parts (per 8 of them), one per system for the others."""
        if parts is None:
            parts = [(bi, 0, ns) for bi, ns in enumerate(self.nsys)]
        nsplit, nvals = 0, 0
        for g in parts:
            bi, s0, s1 = (g, 0, self.nsys[g]) if isinstance(g, (int, np.integer)) else tuple(g)
            r = self._resid[bi]
            if r is not None and r[0] == "values":
                nvals += s1 - s0
            elif s1 > s0:
                nsplit += 1
        return -(-nsplit // self._GRP) + nvals

    def workspace_bytes(self) -> int:
        tot = 0
        for h in self._rhs_all:
            v = ctypes.c_uint64()
            call("cng_rhs_workspace_bytes", h, ctypes.byref(v))
            tot += int(v.value)
        return tot

    # ------------------------------------------------------------------ linear algebra
    def bucket(self, X, bi):
        b = self.tpl.buckets[bi]
        o = self.offsets[bi]
        return X[o:o + self.nsys[bi] * b.n]

    def MX(self, X, out, stream=None) -> None:
        """out = M X per bucket: the buckets with one real M (shared by their systems) in one
        grouped launch, the others one launch each."""
        s = _stream_handle(stream)
        real = [bi for bi in range(len(self.nsys)) if len(self._M[bi]) == 4 and self.nsys[bi] > 0]
        if real:
            parts = (_lib.MatvecPart * len(real))()
            for k, bi in enumerate(real):
                _, mv, ipM, ixM = self._M[bi]
                parts[k] = _lib.MatvecPart(self.nsys[bi], self.tpl.buckets[bi].n, ipM.data_ptr(), ixM.data_ptr(),
                                           mv.data_ptr(), self.bucket(X, bi).data_ptr(), self.bucket(out, bi).data_ptr())
            call("cng_csr_matvec_real_group", len(real), parts, s)
        for bi, b in enumerate(self.tpl.buckets):
            ip, ix = self._pat[bi]
            if len(self._M[bi]) == 4:                    # shared real values on M's own pattern: above
                continue
            vals, per = self._M[bi]
            call("cng_csr_matvec", self.nsys[bi], b.n, ip.data_ptr(), ix.data_ptr(), vals.data_ptr(), per,
                 self.bucket(X, bi).data_ptr(), self.bucket(out, bi).data_ptr(), s)

    def _Lvals(self, bi):
        torch = _torch()
        if self._L[bi] is None:
            self._L[bi] = torch.as_tensor(self.P.values(bi, "L"), device=self.device).contiguous()
        return self._L[bi]

    def factor(self, a: float, b_: float, stream=None):
        """Factorizations of a M + b L for every bucket (cached per (a, b), as the reference's
        FactorCache, system.py:58-82)."""
        key = (float(a), float(b_))
        f = self._factors.get(key)
        if f is None:
            torch = _torch()
            if self.factor_sets is not None:
                while len(self._factors) >= max(1, self.factor_sets):
                    self._factors.pop(next(iter(self._factors)))     # oldest set (its handles free on drop)
            vals_all = []
            for bi, b in enumerate(self.tpl.buckets):
                Mv, per = self._M[bi][:2]
                per = per if isinstance(per, int) else 0
                vals_all.append((a * (Mv if per else Mv.unsqueeze(0)) + b_ * self._Lvals(bi)).contiguous())
            shared = self._check_pairs(vals_all)
            torch.cuda.current_stream(self.device).synchronize()    # the values come from torch's stream
            f = []
            for bi, b in enumerate(self.tpl.buckets):
                if bi in shared:                 # solved with its primary's factors
                    f.append(_Partner(shared[bi], f[shared[bi]]))
                    continue
                vals = vals_all[bi]
                h = _Handle.shared(np.complex128, self.nsys[bi], b.n, b.indptr, b.indices, vals,
                                   list(range(b.r)), pivot=True, stream=_stream_handle(stream))
                if self.precision == "fp32":
                    call("cng_banded_make_fp32", h.h, _stream_handle(stream))
                rel = next(((dr, dc) for j, (i, dr, dc) in self._pairs.items() if i == bi and j in shared), None)
                if rel is not None:
                    call("cng_banded_share", h.h, np.ascontiguousarray(rel[0], np.int8).ctypes.data,
                         np.ascontiguousarray(rel[1], np.int8).ctypes.data, _stream_handle(stream))
                if self.compact:
                    call("cng_banded_compact", h.h, _stream_handle(stream))
                f.append(h)
            del vals_all
            self.shared = dict(shared)
            self._groups = None
            self._factors[key] = f
            if self.compact and self.autotune:
                from .autotune import tune_solve
                self.tuning = tune_solve(self, key, f, stream)
        return f

    def reset_operators(self) -> None:
        """The problem's operator values changed (a stacked problem's case parameters): drop the L
        values, the factor sets and the residual data made from them; they are rebuilt on next use
        (outside any capture). Solvers on this problem drop their captured graphs
        (``IVPSolver.operators_changed``)."""
        self._L = [None] * len(self.tpl.buckets)
        self._factors = {}
        self._resid = [None] * len(self.tpl.buckets)
        self._groups = None
        self.shared = {}

    def _check_pairs(self, vals_all) -> dict:
        """{partner: primary} of the structural pairs whose values satisfy the relation exactly at
        this (a, b): no zero entry in the primary (a zero carries no sign), and every entry of the
        partner equal to dr_i dc_j times the primary's (the reference's rule,
        python/conatus/timestep/shared_factors.py:104-138)."""
        torch = _torch()
        out = {}
        for j, (i, dr, dc) in self._pairs.items():
            A, B = vals_all[i], vals_all[j]
            if A.shape != B.shape:
                continue
            b = self.tpl.buckets[i]
            flip = torch.as_tensor((dr[b.coo_rows()] * dc[b.indices]) < 0, device=self.device)
            if bool((A == 0).any()):
                continue
            if bool(torch.equal(B, torch.where(flip.unsqueeze(0), -A, A))):
                out[j] = i
        return out

    def _residual_data(self, bi):
        """Device data of the FP64 refinement residual of bucket bi: M and every wavenumber monomial
        of L as one real-coefficient entry list per row (each coefficient is purely real or purely
        imaginary), with the per-system monomial values; or, for buckets carrying the reference's
        own values, per-system A values per (a, b)."""
        if self._resid[bi] is None:
            torch = _torch()
            b = self.tpl.buckets[bi]
            split = None
            if b.exact is None and b.m_is_constant():
                terms = self.P.split_terms(bi) if hasattr(self.P, "split_terms") else \
                    [(b.Lc[t], self.P.mono_values(bi)[:, t]) for t in range(b.monos.shape[0])
                     if np.any(b.Lc[t] != 0)]
                split = self._split_operator(b, [c for c, _ in terms])
            if split is None:
                self._resid[bi] = ("values", {})
            else:
                ptr, col, val, code, act, rowsets = split
                mv = np.stack([terms[k][1] for k in act], axis=1) if act else np.zeros((self.nsys[bi], 1))
                dv = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a, dtype=dt), device=self.device)
                self._resid[bi] = ("split", (dv(ptr, np.int32), dv(col, np.int32), dv(val, np.float64),
                                             dv(code, np.int8), dv(mv, np.float64), len(act), rowsets,
                                             np.asarray(mv, np.float64), {}))
        return self._resid[bi]

    def _rowscale(self, bi, a, c):
        """Per-(row, system) scales of the merged entry lists of bucket bi's split residual for
        (a, c): sum over the row's merged terms of rho_k (a for M, c mono_k(system) for L_k); None
        when the bucket has no merged rows. Made once per (a, c), outside any capture."""
        kind, data = self._residual_data(bi)
        if kind != "split" or not data[6]:
            return None
        rowsets, mvh, cache = data[6], data[7], data[8]
        key = (float(a), float(c))
        if key not in cache:
            torch = _torch()
            tab = self._rowscale_table(rowsets, mvh, self.tpl.buckets[bi].n, a, c)
            cache[key] = torch.as_tensor(tab, device=self.device)
            torch.cuda.current_stream(self.device).synchronize()
        return cache[key]

    @staticmethod
    def _rowscale_table(rowsets, mvh, n, a, c):
        """(n, systems) scales of the merged lists: row i, system m: sum over (k, rho) of the row's
        set of rho (a for k = -1, c mvh[m, k] otherwise); zero for rows without a merged list."""
        tab = np.zeros((n, mvh.shape[0]))
        for i, st in rowsets.items():
            acc = np.zeros(mvh.shape[0])
            for k, rho in st:
                acc += rho * (a if k < 0 else c * mvh[:, k])
            tab[i] = acc
        return tab

    @staticmethod
    def _split_operator(b, lrows):
        """Row lists (ptr, col, val, code, active terms) of M and the terms of L (coefficient rows
        ``lrows``, each scaled per system), or None when some coefficient is neither purely real nor
        purely imaginary."""
        t0 = int(np.nonzero(np.all(b.monos == 0, axis=1))[0][0])
        act = [t for t in range(len(lrows)) if np.any(lrows[t] != 0)]
        rows = b.coo_rows()
        ent = [[] for _ in range(b.n)]
        terms = [(-1, b.Mc[t0])] + [(k, lrows[t]) for k, t in enumerate(act)]
        for k, C in terms:
            nz = np.nonzero(C)[0]
            for p in nz:
                v = complex(C[p])
                if v.imag == 0:
                    ent[rows[p]].append((int(b.indices[p]), v.real, 2 * k))
                elif v.real == 0:
                    ent[rows[p]].append((int(b.indices[p]), v.imag, 2 * k + 1))
                else:
                    return None
        # terms of a row with the same columns and proportional values (on the channel: M and the
        # kx^2 and kz^2 parts of L share the conversion operator) become one entry list with a
        # per-(row, system) scale sum_k rho_k s_k (code 2 MERGED + imag), computed once per (a, b)
        ptr = np.zeros(b.n + 1, np.int64)
        col, val, code = [], [], []
        rowsets = {}
        for i in range(b.n):
            groups = {}
            for c_, v_, cd in ent[i]:
                groups.setdefault(cd >> 1, []).append((c_, v_, cd & 1))
            order = list(groups)
            merged = None
            for gi, k0 in enumerate(order):
                base = groups[k0]
                bc = [e[0] for e in base]
                bv = np.array([e[1] for e in base])
                st = [(k0, 1.0)]
                for k in order[gi + 1:]:
                    g = groups[k]
                    if [e[0] for e in g] != bc or any(e[2] != base[0][2] for e in g + base):
                        continue
                    gv = np.array([e[1] for e in g])
                    rho = gv[0] / bv[0]
                    if np.all(np.abs(gv - rho * bv) <= 1e-15 * np.abs(gv)):
                        st.append((k, float(rho)))
                if len(st) > 1:
                    merged = (k0, st)
                    break
            if merged is not None:
                k0, st = merged
                rowsets[i] = st
                for c_, v_, im in groups[k0]:
                    col.append(c_)
                    val.append(v_)
                    code.append(2 * SPLIT_MERGED + im)
            done = {k for k, _ in merged[1]} if merged is not None else set()
            for c_, v_, cd in ent[i]:
                if (cd >> 1) not in done:
                    col.append(c_)
                    val.append(v_)
                    code.append(cd)
            ptr[i + 1] = len(col)
        return ptr, np.array(col), np.array(val), np.array(code), act, rowsets

    def ensure_residual(self, a, b_) -> None:
        """Build the device data of residual(a, b, ...) now (the first call would, outside a graph
        capture; a capture cannot allocate)."""
        for bi, b in enumerate(self.tpl.buckets):
            kind, data = self._residual_data(bi)
            key = (float(a), float(b_))
            self._rowscale(bi, a, b_)
            if kind == "values" and key not in data:
                Mv, per = self._M[bi][:2]
                per = per if isinstance(per, int) else 0
                data[key] = (a * (Mv if per else Mv.unsqueeze(0).expand(self.nsys[bi], -1)) +
                             b_ * self._Lvals(bi)).contiguous()
        _torch().cuda.current_stream(self.device).synchronize()
        if self.precision == "fp32" and self._R2 is None:
            self._R2 = self.zeros()

    def residual(self, a, b_, x, rhs, out, stream=None, buckets=None, xT=None) -> None:
        """out = rhs - (a M + b L) x per bucket (all, or ``buckets``: bucket indices or (bucket,
        first system, end system) parts), FP64; ``xT``: x also row-major over the systems of each
        bucket (read by the split kernel instead)."""
        s = _stream_handle(stream)
        if buckets is None:
            parts = [(bi, 0, ns) for bi, ns in enumerate(self.nsys)]
        else:
            parts = [(g, 0, self.nsys[g]) if isinstance(g, (int, np.integer)) else tuple(g) for g in buckets]
        split = []                     # the split-form parts: one grouped launch
        for bi, s0, s1 in parts:
            b = self.tpl.buckets[bi]
            kind, data = self._residual_data(bi)
            xb, rb, ob = self.bucket(x, bi), self.bucket(rhs, bi), self.bucket(out, bi)
            if kind == "split":
                if s1 <= s0:
                    continue
                ptr, col, val, code, mv, nm = data[:6]
                rs = self._rowscale(bi, a, b_)
                split.append(_lib.ResidualPart(
                    self.nsys[bi], int(s0), int(s1), b.n, ptr.data_ptr(), col.data_ptr(), val.data_ptr(),
                    code.data_ptr(), mv.data_ptr(), nm, rs.data_ptr() if rs is not None else None, xb.data_ptr(),
                    self.bucket(xT, bi).data_ptr() if xT is not None else None, rb.data_ptr(), ob.data_ptr()))
                continue
            key = (float(a), float(b_))
            if key not in data:
                Mv, per = self._M[bi][:2]
                per = per if isinstance(per, int) else 0
                data[key] = (a * (Mv if per else Mv.unsqueeze(0).expand(self.nsys[bi], -1)) +
                             b_ * self._Lvals(bi)).contiguous()
                _torch().cuda.current_stream(self.device).synchronize()   # made on torch's stream
            ip, ix = self._pat[bi]
            A = data[key]
            for m in range(s0, s1):
                sl = slice(m * b.n, (m + 1) * b.n)
                call("cng_poly_residual", 1, b.n, ip.data_ptr(), ix.data_ptr(), A[m].data_ptr(), None, None, 0,
                     1.0, 0.0, xb[sl].data_ptr(), rb[sl].data_ptr(), ob[sl].data_ptr(), s)
        if split:
            arr = (_lib.ResidualPart * len(split))(*split)
            call("cng_split_residual_group", len(split), arr, float(a), float(b_), s)

    def solve(self, a: float, b_: float, rhs, out, stream=None) -> None:
        """out = (a M + b L)^{-1} rhs per bucket (rhs and out must not alias), every bucket in one
        launch. FP32 form: FP32 solve, then ``refine`` passes (default one) of FP64 residual and
        FP32 correction added in FP64."""
        fs = self.factor(a, b_, stream)
        self._solve_with(fs, a, b_, rhs, out, stream)

    def _solve_with(self, fs, a, b_, rhs, out, stream=None) -> None:
        s = _stream_handle(stream)
        if not self.compact:
            for bi, h in enumerate(fs):
                if self.precision == "fp64":
                    call("cng_banded_solve_mapped", h.h, self.bucket(rhs, bi).data_ptr(), None,
                         self.bucket(out, bi).data_ptr(), None, s)
                else:
                    raise ValueError("the FP32 form needs the compact solve")
            return
        nb = len(fs)
        if self.precision == "fp64":
            self._batch_call(fs, list(range(nb)), rhs, out, None, 0, 0, s)
            return
        if self._R2 is None:
            self._R2 = self.zeros()
        dense = all(getattr(h, "schedule", 0) < 0 for h in fs)
        groups = self._refine_groups() if (self.overlap_refine and not dense) else [list(range(nb))]
        if len(groups) == 1:
            self._refine_chain(fs, groups[0], a, b_, rhs, out, s)
            return
        # two chains (solve, residual, correction) on two streams: the FP64 residual of one group of
        # buckets runs beside the FP32 sweeps of the other (different pipes of the same SMs).
        # Measured against one chain: the channel's solve and refinement 3.73 -> 3.50 ms, RB
        # 256x64's step 0.38 -> 0.34 ms; staggering the chains (B's solve after A's) gained nothing
        # on the channel and lost on RB
        torch = _torch()
        if self._aux is None:
            self._aux = (torch.cuda.Stream(self.device), torch.cuda.Event(), torch.cuda.Event())
        aux, fork, join = self._aux
        main = torch.cuda.ExternalStream(s, device=self.device)
        fork.record(main)
        aux.wait_event(fork)
        self._refine_chain(fs, groups[1], a, b_, rhs, out, aux.cuda_stream)
        self._refine_chain(fs, groups[0], a, b_, rhs, out, s)
        join.record(aux)
        main.wait_event(join)

    def _refine_groups(self):
        """Two groups of about equal work (systems x length) for the FP32 refinement on two streams,
        as (bucket, first system, end system) parts; a shared pair's partner goes with its primary
        (one sweep solves both). Whole buckets are placed largest first; when one bucket outweighs
        all the others, it is split at a system boundary between the two groups."""
        if self._groups is None:
            partner_of = {i: j for j, i in self.shared.items()}
            units = [bi for bi in range(len(self.nsys)) if bi not in self.shared]
            per = {bi: self.tpl.buckets[bi].n * (2 if bi in partner_of else 1) for bi in units}
            work = {bi: self.nsys[bi] * per[bi] for bi in units}
            total = sum(work.values())
            big = max(units, key=lambda bi: work[bi])
            if len(units) > 0 and work[big] > total / 2 and self.nsys[big] >= 4:
                align = 1 if big in partner_of else 2          # warp groups of the compact streams
                rest = total - work[big]
                h = int(round((work[big] - rest) / (2 * per[big])))
                h = max(align, min(self.nsys[big] - align, h - h % align))
                g0 = [(bi, 0, self.nsys[bi]) for bi in sorted(units) if bi != big] + [(big, 0, h)]
                self._groups = [g0, [(big, h, self.nsys[big])]]
            else:
                g, w = [[], []], [0, 0]
                for bi in sorted(units, key=lambda u: -work[u]):
                    k = 0 if w[0] <= w[1] else 1
                    g[k].append((bi, 0, self.nsys[bi]))
                    w[k] += work[bi]
                self._groups = [sorted(x) for x in g if x]
        return self._groups

    def _with_partners(self, parts):
        """Parts plus the same system range of each part's shared partner (the residual's list)."""
        partner_of = {i: j for j, i in self.shared.items()}
        out = []
        for g in parts:
            bi, s0, s1 = (g, 0, self.nsys[g]) if isinstance(g, (int, np.integer)) else tuple(g)
            for e in ((bi, s0, s1), (partner_of[bi], s0, s1) if bi in partner_of else None):
                if e is not None and e not in out:
                    out.append(e)
        return out

    def _batch_call(self, fs, group, rhs, out, xt, fp32, accumulate, s) -> None:
        """One batched solve launch over ``group`` (bucket indices, or (bucket, first system, end
        system) parts): a shared pair's partner is solved in the same sweep as its primary
        (cng_banded_solve_batch2), over the same systems."""
        parts = [(g, 0, self.nsys[g]) if isinstance(g, (int, np.integer)) else tuple(g) for g in group]
        partner_of = {fs[bj].primary: bj for bj in range(len(fs)) if isinstance(fs[bj], _Partner)}
        prim = [p for p in parts if not isinstance(fs[p[0]], _Partner)]
        for p in parts:
            if isinstance(fs[p[0]], _Partner) and not any(q[0] == fs[p[0]].primary for q in prim):
                raise ValueError("a shared pair's partner is solved with its primary, in one launch")
        nb = len(prim)
        V = ctypes.c_void_p * nb
        ptr = lambda X, bi: self.bucket(X, bi).data_ptr() if bi is not None else None
        hs = V(*[fs[bi].h.value for bi, _, _ in prim])
        bp, xp = V(*[ptr(rhs, bi) for bi, _, _ in prim]), V(*[ptr(out, bi) for bi, _, _ in prim])
        b2 = x2 = xt1 = xt2 = rng = None
        if partner_of:
            b2 = V(*[ptr(rhs, partner_of.get(bi)) for bi, _, _ in prim])
            x2 = V(*[ptr(out, partner_of.get(bi)) for bi, _, _ in prim])
        if xt is not None:
            xt1 = V(*[ptr(xt, bi) for bi, _, _ in prim])
            if partner_of:
                xt2 = V(*[ptr(xt, partner_of.get(bi)) for bi, _, _ in prim])
        if any(s0 != 0 or s1 != self.nsys[bi] for bi, s0, s1 in prim):
            rng = (ctypes.c_int32 * (2 * nb))(*[int(v) for _, s0, s1 in prim for v in (s0, s1)])
        call("cng_banded_solve_batch2", nb, hs, bp, xp, b2, x2, xt1, xt2, rng, fp32, accumulate, s)

    def _refine_chain(self, fs, group, a, b_, rhs, out, s) -> None:
        """FP32 solve of the buckets in ``group``, then ``refine`` passes of FP64 residual and FP32
        correction added in FP64, all on stream ``s``."""
        # x also row-major over the systems (coalesced reads of the residual kernel), with the
        # compact schedules
        xt = None
        if all(getattr(fs[g if isinstance(g, (int, np.integer)) else g[0]], "schedule", 0) >= 0 for g in group):
            if self._XT is None:
                self._XT = self.zeros()
            xt = self._XT
        self._batch_call(fs, group, rhs, out, xt, 1, 0, s)
        for p in range(self.refine):
            self.residual(a, b_, out, rhs, self._R2, s, buckets=self._with_partners(group), xT=xt)
            self._batch_call(fs, group, self._R2, out, xt if p + 1 < self.refine else None, 1, 1, s)

    def solve_launch(self, fs, rhs, out, stream=None) -> None:
        """One batched solve launch with the factor set ``fs`` (FP32 factors in the FP32 form), no
        refinement: the unit the solve's roofline is measured on."""
        self._batch_call(fs, list(range(len(fs))), rhs, out, None, 1 if self.precision == "fp32" else 0, 0,
                         _stream_handle(stream))

    def zeros(self):
        torch = _torch()
        return torch.zeros(self.n_total, dtype=torch.complex128, device=self.device)

    # ------------------------------------------------------------------ layout helpers
    def to_device(self, C_list):
        torch = _torch()
        flat = np.concatenate([np.asarray(c, np.complex128).ravel() for c in C_list])
        return torch.as_tensor(flat, device=self.device)

    def to_host(self, X):
        x = X.detach().cpu().numpy()
        return [x[o:o + ns * b.n].reshape(ns, b.n) for o, ns, b in zip(self.offsets, self.nsys, self.tpl.buckets)]

    def __del__(self):
        for h in getattr(self, "_rhs_all", []):
            if h is not None and h.value:
                try:
                    _lib.lib().cng_rhs_destroy(h)
                except Exception:
                    pass


class _Partner:
    """Factor-list entry of a bucket solved with the factors of bucket ``primary`` (a shared pair:
    the partner's matrix is diag(dr) A diag(dc), python/conatus/timestep/shared_factors.py:40-60).
    Holds no device memory; shapes and schedule are the primary's."""

    def __init__(self, primary: int, handle):
        self.primary, self._p = primary, handle
        self.h = None
        for k in ("batch", "n", "rank", "kl", "ku", "ldab", "pivot"):
            setattr(self, k, getattr(handle, k))

    @property
    def schedule(self):
        return getattr(self._p, "schedule", 0)


class _Graph:
    def __init__(self, h):
        self.h = h

    def launch(self, stream):
        call("cng_graph_launch", self.h, stream)

    def __del__(self):
        if self.h is not None and self.h.value:
            try:
                _lib.lib().cng_graph_destroy(self.h)
            except Exception:
                pass


SBDF_SCHEMES = ("SBDF1", "SBDF2", "SBDF3", "SBDF4")
CN_SCHEMES = ("CNAB1", "CNAB2", "MCNAB2", "CNLF2")
RK_SCHEMES = ("RK111", "RK222", "RK443", "RKSMR", "RKGFY")


def cn_coefficients(name: str):
    """(a, b, c) of a constant-step CN-family multistep scheme (Wang & Ruuth 2008), a in units of
    1/dt: sum_j (a_j/dt) M X^{n+1-j} + b_j L X^{n+1-j} = sum_{j>=1} c_j F^{n+1-j}
    (python/conatus/timestep/schemes.py:91-103; the published coefficients)."""
    return {"CNAB1": ([1.0, -1.0], [0.5, 0.5], [0.0, 1.0]),
            "CNAB2": ([1.0, -1.0, 0.0], [0.5, 0.5, 0.0], [0.0, 1.5, -0.5]),
            "MCNAB2": ([1.0, -1.0, 0.0], [9 / 16, 6 / 16, 1 / 16], [0.0, 1.5, -0.5]),
            "CNLF2": ([0.5, 0.0, -0.5], [0.5, 0.0, 0.5], [0.0, 1.0, 0.0])}[name]


def rk_tableau(name: str):
    """(A, H, c) of an IMEX Runge-Kutta scheme in cumulative form M X_i = M X_0 + dt sum_j A_ij F_j
    - dt sum_j H_ij L X_j (python/conatus/timestep/schemes.py:106-143; the published tableaux:
    RK222 and RK443 of Ascher, Ruuth & Spiteri 1997, RKSMR of Spalart, Moser & Rogers 1991,
    RKGFY Heun / Crank-Nicolson)."""
    if name == "RK111":
        return [[0, 0], [1, 0]], [[0, 0], [0, 1]], [0, 1]
    if name == "RK222":
        g = (2 - math.sqrt(2)) / 2
        d = 1 - 1 / g / 2
        return ([[0, 0, 0], [g, 0, 0], [d, 1 - d, 0]], [[0, 0, 0], [0, g, 0], [0, 1 - g, g]], [0, g, 1])
    if name == "RK443":
        return ([[0, 0, 0, 0, 0], [1 / 2, 0, 0, 0, 0], [11 / 18, 1 / 18, 0, 0, 0],
                 [5 / 6, -5 / 6, 1 / 2, 0, 0], [1 / 4, 7 / 4, 3 / 4, -7 / 4, 0]],
                [[0, 0, 0, 0, 0], [0, 1 / 2, 0, 0, 0], [0, 1 / 6, 1 / 2, 0, 0],
                 [0, -1 / 2, 1 / 2, 1 / 2, 0], [0, 3 / 2, -3 / 2, 1 / 2, 1 / 2]],
                [0, 1 / 2, 2 / 3, 1 / 2, 1])
    if name == "RKSMR":
        al, be = (29 / 96, -3 / 40, 1 / 6), (37 / 160, 5 / 24, 1 / 6)
        ga, ze = (8 / 15, 5 / 12, 3 / 4), (-17 / 60, -5 / 12)
        A = [[0, 0, 0, 0], [ga[0], 0, 0, 0], [ga[0] + ze[0], ga[1], 0, 0],
             [ga[0] + ze[0], ga[1] + ze[1], ga[2], 0]]
        H = [[0, 0, 0, 0], [al[0], be[0], 0, 0], [al[0], be[0] + al[1], be[1], 0],
             [al[0], be[0] + al[1], be[1] + al[2], be[2]]]
        return A, H, [0, 8 / 15, 2 / 3, 1]
    if name == "RKGFY":
        return ([[0, 0, 0], [1, 0, 0], [1 / 2, 1 / 2, 0]], [[0, 0, 0], [1 / 2, 1 / 2, 0], [1 / 2, 0, 1 / 2]],
                [0, 1, 1])
    raise ValueError(f"unknown Runge-Kutta scheme {name!r}")


class IVPSolver:
    """IMEX time stepper on the device (see module docstring): SBDF1-4, the CN family (CNAB1,
    CNAB2, MCNAB2, CNLF2) and IMEX Runge-Kutta (RK111, RK222, RK443, RKSMR, RKGFY), start-up
    ``lower_order`` as the reference's default."""

    def __init__(self, problem, scheme: str = "SBDF2", dt: float = 1e-3, precision: str = "fp64",
                 device_problem: DeviceProblem | None = None, factor_sets: int | None = None,
                 refine: int | None = None, check_finite=True):
        if scheme in SBDF_SCHEMES:
            self.family, self.order = "sbdf", int(scheme[-1])
            self.ring = self.order
        elif scheme in CN_SCHEMES:
            self.family, self.order = "cn", 0
            self._cn = cn_coefficients(scheme)
            self.ring = len(self._cn[0]) - 1
        elif scheme in RK_SCHEMES:
            self.family, self.order = "rk", 0
            self._rk = rk_tableau(scheme)
            self.ring = 1
        else:
            raise ValueError(f"scheme {scheme!r}: one of {SBDF_SCHEMES + CN_SCHEMES + RK_SCHEMES}")
        self.scheme, self.dt = scheme, float(dt)
        self._finite_every = finite_cadence(check_finite)
        self._flag = None                    # device int64: first iteration found non-finite
        self._finite_ok = None               # (iteration, t) of the last check found finite
        self._probed = None                  # (iteration, t) of the last check launched
        self.dev = device_problem or DeviceProblem(problem, precision, factor_sets=factor_sets)
        # FP32 form: refinement passes per solve. The CN family carries -b_1 L X_n of the previous
        # step with a weight comparable to the implicit one, and with it the previous pressure (the
        # odd-even pressure mode of CNAB2 starts from any state that is not in balance); one pass
        # leaves its solve error in the pressure (3e-6 relative after 20 CNAB2 steps of RB 64x64),
        # two passes bring it to the FP32 F's own level (3e-8)
        if refine is not None:
            self.dev.refine = max(1, int(refine))
        elif self.family == "cn":
            self.dev.refine = 2
        z = self.dev.zeros
        self.X, self.R = z(), z()
        nh = self.ring if self.family != "rk" else 0
        self.MXh = [z() for _ in range(nh)]
        self.Fh = [z() for _ in range(nh)]
        self.LXh = [z() for _ in range(nh)] if self.family == "cn" else []     # -L X (negated)
        if self.family == "rk":
            S = len(self._rk[2]) - 1
            self._MX0 = z()
            self._Xs = [self.X] + [z() for _ in range(S - 1)]     # the last stage is written to X
            self._Fs = [z() if any(self._rk[0][m][j] != 0 for m in range(j + 1, S + 1)) else None
                        for j in range(S)]
            self._LXs = [z() if any(self._rk[1][m][j] != 0 for m in range(j + 1, S + 1)) else None
                         for j in range(S)]
            self._Xnew = z()
        self._zero = None
        self._warm = False
        self._side = None          # side stream of M X (and -L X), beside F
        # fork: M X on a side stream beside F (and, in the FP32 form, the refinement in two bucket
        # groups on two streams). A caller that keeps many solvers in flight (the serving loop)
        # turns it off: the device is busy with the other runs, and the extra streams and events
        # only add dependencies
        self.fork = True
        self.filled, self.head = 0, self.ring - 1
        self.t, self.iteration = 0.0, 0
        self._graphs = {}
        torch = _torch()
        self.stream = torch.cuda.Stream()
        # join: every call orders the solver's stream after torch's current stream and back (safe
        # default). A caller that keeps many solvers in flight on their own streams (the serving
        # loop) turns it off after one explicit wait, so that independent runs do not serialize.
        self.join = True
        self._shadow = None                  # FP32 form: the FP64 shadow of monitor_fp64
        self.mixed_error, self.mixed_error_last = {}, None

    def set_state(self, X, t: float = 0.0) -> None:
        """Initial state (mode layout tensor or list of per-bucket arrays); resets the history."""
        if isinstance(X, (list, tuple)):
            X = self.dev.to_device(X)
        self.X.copy_(X)
        self.t, self.iteration = float(t), 0
        self.filled, self.head = 0, self.ring - 1
        self._reset_finite()
        if self._shadow is not None:
            self._shadow.set_state(self.X, t)
            self.mixed_error, self.mixed_error_last = {}, None

    # ------------------------------------------------------------------ FP32 form: error monitor
    def monitor_fp64(self, every: int = 100, bound: float = 1e-6) -> None:
        """FP32 form: advance a plain FP64 shadow of this solver in lockstep (its own device problem)
        and record the relative L2 error per field (tau variables left out) of this run against it
        every ``every`` steps and at the end of every ``step`` / ``run`` / ``run_graph`` call, in
        ``self.mixed_error`` ({iteration: {field: error}}; the latest in ``mixed_error_last``). An
        error above ``bound`` warns (RuntimeWarning). The FP64 drop-in matches the reference step
        by step, so this is the mixed form's error against the FP64 path, at the cost of running it
        beside. Call after ``set_state`` and before the first step (the shadow starts from the same
        state and an empty history)."""
        if self.dev.precision != "fp32":
            raise ValueError("monitor_fp64: the solver is not the FP32 form")
        if self.iteration != 0 or self.filled != 0:
            raise ValueError("monitor_fp64: call it after set_state, before the first step")
        torch = _torch()
        self._shadow = IVPSolver(self.dev.P, scheme=self.scheme, dt=self.dt, precision="fp64",
                                 check_finite=self._finite_every or False)
        self._shadow.set_state(self.X, self.t)
        self._mon_every, self._mon_bound = max(1, int(every)), float(bound)
        tpl = self.dev.tpl
        self._mon_masks = {}
        for v, var in enumerate(tpl.variables):
            if var["name"].startswith("tau"):
                continue
            self._mon_masks[var["name"]] = [torch.as_tensor(b.col[:, 0] == v, device=self.X.device)
                                            for b in tpl.buckets]
        self.mixed_error, self.mixed_error_last = {}, None

    def _record_error(self) -> None:
        torch = _torch()
        self.stream.synchronize()
        self._shadow.stream.synchronize()
        dev = self.dev
        errs = {}
        for name, masks in self._mon_masks.items():
            num = den = 0.0
            for bi, (b, mask) in enumerate(zip(dev.tpl.buckets, masks)):
                ns = dev.nsys[bi]
                if ns == 0:
                    continue
                a = dev.bucket(self.X, bi).view(ns, b.n)[:, mask]
                r = dev.bucket(self._shadow.X, bi).view(ns, b.n)[:, mask]
                num += float(torch.sum(torch.abs(a - r) ** 2))
                den += float(torch.sum(torch.abs(r) ** 2))
            errs[name] = (num / den) ** 0.5 if den > 0 else 0.0
        self.mixed_error[int(self.iteration)] = errs
        self.mixed_error_last = errs
        worst = max(errs.values()) if errs else 0.0
        if worst > self._mon_bound:
            import warnings
            warnings.warn(f"FP32 form: relative L2 error {worst:.3g} against the FP64 shadow at iteration "
                          f"{self.iteration} (bound {self._mon_bound:g}; per field {errs})", RuntimeWarning,
                          stacklevel=3)

    def _monitored(self, fn, shadow_fn, steps: int) -> None:
        """Run ``steps`` steps through fn and the shadow through shadow_fn in chunks that end on the
        monitor's iterations; record the error there and at the end of the call."""
        left = int(steps)
        while left > 0:
            n = min(left, self._mon_every - self.iteration % self._mon_every)
            fn(n)
            shadow_fn(n)
            left -= n
            if self.iteration % self._mon_every == 0 or left == 0:
                self._record_error()

    def _reset_finite(self) -> None:
        """A new state: forget the finite-state checks of the previous one."""
        if self._flag is not None:
            self._flag.fill_(_FLAG_CLEAR)
        self._finite_ok = self._probed = None

    def operators_changed(self) -> None:
        """After ``DeviceProblem.reset_operators``: the captured graphs hold the old factor sets;
        they are captured again on next use."""
        self._graphs = {}

    def set_history(self, MX_list, F_list, LX_list=None) -> None:
        """History (newest first) of M X and F, and of L X for the CN family, e.g. to continue from
        another solver's state."""
        if self.family == "rk":
            raise ValueError("a Runge-Kutta scheme keeps no history")
        self.filled = len(MX_list)
        for j, (mx, f) in enumerate(zip(MX_list, F_list)):
            slot = (self.head - j) % self.ring
            self.MXh[slot].copy_(mx)
            self.Fh[slot].copy_(f)
            if self.family == "cn":
                self.LXh[slot].copy_(-LX_list[j])

    # ------------------------------------------------------------------ pieces of a step
    def _neg_LX(self, x, out, s):
        """out = -L x (the FP64 operator apply of the residual kernel with a = 0, b = 1)."""
        if self._zero is None:
            self._zero = self.dev.zeros()
        self.dev.residual(0.0, 1.0, x, self._zero, out, s)

    def _push(self, s):
        """History of the new state: M X (and -L X) on a side stream forked from the step's stream,
        F on the step's stream, joined before the combination (in a captured step the two become
        parallel branches of the graph)."""
        self.head = (self.head + 1) % self.ring
        self.dev.overlap_refine = self.fork
        if not self.fork:
            self.dev.MX(self.X, self.MXh[self.head], s)
            if self.family == "cn":
                self._neg_LX(self.X, self.LXh[self.head], s)
            self.dev.F(self.X, self.Fh[self.head], s)
            self.filled = min(self.filled + 1, self.ring)
            return
        torch = _torch()
        if self._side is None:
            self._side = (torch.cuda.Stream(), torch.cuda.Event(), torch.cuda.Event())
        side, fork, join = self._side
        fork.record(self.stream)
        side.wait_event(fork)
        hs = side.cuda_stream
        self.dev.MX(self.X, self.MXh[self.head], hs)
        if self.family == "cn":
            self._neg_LX(self.X, self.LXh[self.head], hs)
        self.dev.F(self.X, self.Fh[self.head], s)
        join.record(side)
        self.stream.wait_event(join)
        self.filled = min(self.filled + 1, self.ring)

    def _lincomb(self, base, terms, out, s):
        """out = base + sum of (negate, coef, vector) terms in order (cng_lincomb)."""
        k = len(terms)
        cs = (ctypes.c_double * max(k, 1))(*[t[1] for t in terms])
        ng = (ctypes.c_int32 * max(k, 1))(*[1 if t[0] else 0 for t in terms])
        vp = (ctypes.c_void_p * max(k, 1))(*[t[2].data_ptr() for t in terms])
        call("cng_lincomb", self.dev.n_total, None if base is None else base.data_ptr(), k, cs, ng, vp,
             out.data_ptr(), s)

    def _cn_now(self):
        """The scheme's coefficients once the history is full, CNAB1 before (lower-order start-up,
        integrator.py:577-579)."""
        return self._cn if self.filled >= self.ring else cn_coefficients("CNAB1")

    def _step_keys(self):
        """(a, b) of the solves of the next step."""
        if self.family == "sbdf":
            a, _ = SBDF[min(self.order, self.filled + 1)]
            return [(a[0] / self.dt, 1.0)]
        if self.family == "cn":
            filled = self.filled
            self.filled = min(self.filled + 1, self.ring)
            a, b, _ = self._cn_now()
            self.filled = filled
            return [(a[0] / self.dt, b[0])]
        A, H, c = self._rk
        return sorted({(1.0, self.dt * H[i][i]) for i in range(1, len(c))})

    def _step_factors(self, s):
        """Factor sets (and the other device data made on first use) of the next step, made
        outside any capture."""
        for a, b in self._step_keys():
            self.dev.factor(a, b, s)
            if self.dev.precision == "fp32":
                self.dev.ensure_residual(a, b)
        if self.family != "sbdf":
            self.dev.ensure_residual(0.0, 1.0)
            if self._zero is None:
                self._zero = self.dev.zeros()

    def _combine_solve(self, s):
        if self.family == "sbdf":
            q = min(self.order, self.filled)
            a, c = SBDF[q]
            slots = [(self.head - j) % self.order for j in range(q)]
            cs = (ctypes.c_double * q)(*[c[j + 1] for j in range(q)])
            ds = (ctypes.c_double * q)(*[a[j + 1] / self.dt for j in range(q)])
            Fp = (ctypes.c_void_p * q)(*[self.Fh[k].data_ptr() for k in slots])
            Mp = (ctypes.c_void_p * q)(*[self.MXh[k].data_ptr() for k in slots])
            call("cng_sbdf_rhs_fused", q, cs, ds, Fp, Mp, self.R.data_ptr(), self.dev.n_total,
                 1 if self.dev.precision == "fp32" else 0, s)
            self.dev.solve(a[0] / self.dt, 1.0, self.R, self.X, s)
            return
        # CN family (integrator.py:581-603): rhs = sum_{j>=1} c_j F_j - (a_j/dt) M X_j - b_j L X_j
        a, b, c = self._cn_now()
        terms = []
        for j in range(1, len(a)):
            if j > self.filled:
                break
            slot = (self.head - (j - 1)) % self.ring
            if c[j] != 0:
                terms.append((False, c[j], self.Fh[slot]))
            if a[j] != 0:
                terms.append((True, a[j] / self.dt, self.MXh[slot]))
            if b[j] != 0:
                terms.append((False, b[j], self.LXh[slot]))       # - b_j L X_j = + b_j (-L X_j)
        self._lincomb(None, terms, self.R, s)
        self.dev.solve(a[0] / self.dt, b[0], self.R, self.X, s)

    def _rk_stages(self, s):
        """One IMEX Runge-Kutta step (integrator.py:605-646): M X_i = M X_0 + dt sum_k A_ik F_k -
        dt sum_k H_ik L X_k, (M + dt H_ii L) X_i = rhs; X_s is the new state."""
        A, H, c = self._rk
        S = len(c) - 1
        dt = self.dt
        self.dev.MX(self.X, self._MX0, s)
        for i in range(1, S + 1):
            j = i - 1
            xj = self._Xs[j]
            if self._Fs[j] is not None:
                self.dev.F(xj, self._Fs[j], s)
            if self._LXs[j] is not None:
                self._neg_LX(xj, self._LXs[j], s)
            terms = []
            for k in range(i):
                if A[i][k] != 0:
                    terms.append((False, dt * A[i][k], self._Fs[k]))
                if H[i][k] != 0:
                    terms.append((False, dt * H[i][k], self._LXs[k]))   # - dt H L X = + dt H (-L X)
            self._lincomb(self._MX0, terms, self.R, s)
            out = self._Xs[i] if i < S else self._Xnew
            self.dev.solve(1.0, dt * H[i][i], self.R, out, s)
        # X_s -> X (the stage buffers keep X_0 = X)
        call("cng_lincomb", self.dev.n_total, self._Xnew.data_ptr(), 0, None, None, None, self.X.data_ptr(), s)

    def _advance(self, s):
        """The device work of one step (no factorization: see _step_factors)."""
        if self.family == "rk":
            self._rk_stages(s)
        else:
            self._push(s)
            self._combine_solve(s)

    def _enter(self):
        if self.join:
            self.stream.wait_stream(_torch().cuda.current_stream())

    def _leave(self):
        if self.join:
            _torch().cuda.current_stream().wait_stream(self.stream)

    def step(self) -> None:
        if self._shadow is not None:
            return self._monitored(lambda n: self._plain_step(), lambda n: self._shadow.step(), 1)
        self._plain_step()

    def _plain_step(self) -> None:
        self._enter()
        self._step()
        self._leave()

    def _step(self) -> None:
        s = _stream_handle(self.stream)
        self._step_factors(s)                       # outside the timed/captured work
        self._advance(s)
        self._warm = True
        self.t += self.dt
        self.iteration += 1

    def run(self, steps: int) -> None:
        """``steps`` plain steps; with the finite-state check on, the state is checked every
        ``check_finite`` steps and at the end of the call, and a blown-up run stops with
        NumericalError (integrator.py:745-767)."""
        if self._shadow is not None:
            return self._monitored(self._run, self._shadow.run, steps)
        self._run(steps)

    def _run(self, steps: int) -> None:
        self._enter()
        fe = self._finite_every
        s = _stream_handle(self.stream)
        for _ in range(int(steps)):
            self._step()
            if fe and self.iteration % fe == 0:
                self._probe(s)
                self._finite_raise("IVPSolver.run")
        if fe and int(steps) > 0:
            self._probe(s)
            self._finite_raise("IVPSolver.run (end of the call)")
        self._leave()

    # ------------------------------------------------------------------ finite-state check
    def _probe(self, s) -> None:
        """Launch the finite-state check of the current state on stream s (asynchronous)."""
        if self._flag is None:
            torch = _torch()
            self._flag = torch.full((1,), _FLAG_CLEAR, dtype=torch.int64, device=self.X.device)
            torch.cuda.current_stream(self.X.device).synchronize()
        call("cng_check_finite", self.X.data_ptr(), self.dev.n_total, int(self.iteration), self._flag.data_ptr(), s)
        self._probed = (int(self.iteration), float(self.t))

    def finite_status(self):
        """None while every check launched so far found the state finite, else the first iteration
        found non-finite. Reads a device flag: the checks must have completed (call after a
        synchronization of the solver's stream)."""
        if self._flag is None:
            return None
        v = int(self._flag.item())
        return None if v == _FLAG_CLEAR else v

    def _finite_raise(self, where: str) -> None:
        """Wait for the checks launched so far; raise NumericalError if one found the state
        non-finite, naming the iteration, the first non-finite variable and the last iteration
        checked finite (run_checks.check_state_finite, python/conatus/timestep/run_checks.py:67-99)."""
        self.stream.synchronize()
        bad = self.finite_status()
        if bad is None:
            self._finite_ok = self._probed
            return
        name, count = "?", 0
        C = self.dev.to_host(self.X)
        for v, var in enumerate(self.dev.tpl.variables):
            cnt = sum(int(np.count_nonzero(~np.isfinite(Cb[:, b.col[:, 0] == v])))
                      for Cb, b in zip(C, self.dev.tpl.buckets))
            if cnt:
                name, count = var["name"], cnt
                break
        last = self._finite_ok
        since = f"; last checked finite at iteration {last[0]} (t = {last[1]:.10g})" if last else ""
        raise NumericalError(
            f"{where}: non-finite state (NaN or inf) at iteration {bad}: unknown {name!r} ({count} "
            f"non-finite coefficient(s) now, at iteration {self.iteration}){since}; reduce dt (now "
            f"{self.dt:g}), raise the resolution or check the initial state; check_finite=False "
            "turns the check off")

    def run_graph(self, steps: int, unroll: int = 1, wait: bool = True) -> None:
        """``steps`` steps; once the history is full (at once for Runge-Kutta), the steps run as CUDA
        graph launches, each graph holding ``unroll`` steps (one graph per position of the history
        ring and length, captured on first use; a remainder shorter than ``unroll`` runs as
        one-step graphs). The finite-state check runs between graphs every ``check_finite`` steps
        and at the end of the call (graphs end on those iterations); ``wait``: wait for it at the
        end and raise NumericalError on a blown-up state, else leave the result to
        :meth:`finite_status` (a caller that keeps many runs in flight)."""
        if self._shadow is not None:
            return self._monitored(lambda n: self._run_graph(n, unroll, wait),
                                   lambda n: self._shadow.run_graph(n, unroll), steps)
        self._run_graph(steps, unroll, wait)

    def _run_graph(self, steps: int, unroll: int = 1, wait: bool = True) -> None:
        s = _stream_handle(self.stream)
        steps = int(steps)
        unroll = max(1, int(unroll))
        fe = self._finite_every
        ran = steps > 0
        self._enter()
        # plain steps until the history is full, and at least one (its first launches make the
        # lazily built device data -- tables, kernel attributes -- which a capture cannot make)
        while steps > 0 and (not self._warm or (self.family != "rk" and self.filled < self.ring)):
            self._step()
            steps -= 1
            if fe and self.iteration % fe == 0:
                self._probe(s)
        if steps <= 0:
            self._end_run_graph(s, ran, wait)
            self._leave()
            return
        self._step_factors(s)
        while steps > 0:
            u = unroll if steps >= unroll else 1
            if fe:                             # graphs end on the check's iterations
                u = min(u, fe - self.iteration % fe)
            key = ((self.head + 1) % self.ring, u)
            g = self._graphs.get(key)
            if g is None:
                self.stream.synchronize()
                call("cng_graph_begin", s)
                head0, filled0 = self.head, self.filled
                try:
                    for _ in range(u):
                        self._advance(s)
                finally:
                    h = ctypes.c_void_p()
                    call("cng_graph_end", s, ctypes.byref(h))
                g = self._graphs[key] = _Graph(h)
                self.head, self.filled = head0, filled0     # captured, not run
            g.launch(s)
            self.head = (self.head + u) % self.ring
            self.t += u * self.dt
            self.iteration += u
            steps -= u
            if fe and self.iteration % fe == 0:
                self._probe(s)
        self._end_run_graph(s, ran, wait)
        self._leave()

    def _end_run_graph(self, s, ran, wait) -> None:
        """The finite-state check at the end of a run_graph call: launched, and (``wait``) waited
        for, raising NumericalError on a blown-up state."""
        if self._finite_every and ran:
            if self._probed is None or self._probed[0] != self.iteration:
                self._probe(s)
            if wait:
                self._finite_raise("IVPSolver.run_graph (end of the call)")

    def step_host(self, host_in, host_out) -> None:
        """One step through host buffers: the state is copied in from ``host_in`` (pinned, mode
        layout), stepped (history kept), and copied out to ``host_out``."""
        self._enter()
        with _torch().cuda.stream(self.stream):
            self.X.copy_(host_in, non_blocking=True)
        if self.family == "rk" or self.filled >= self.ring:
            self.run_graph(1)
        else:
            self._step()
        with _torch().cuda.stream(self.stream):
            host_out.copy_(self.X, non_blocking=True)
        self.stream.synchronize()
        self._leave()

    # ------------------------------------------------------------------ checkpoints
    def checkpoint_payload(self):
        """(meta, host arrays) of a restart: the state, the multistep history (newest first: M X,
        F and, CN family, L X) and the clock, as the reference's ``_checkpoint_payload``
        (python/conatus/timestep/integrator.py:974-1007), on the mode layout."""
        self.stream.synchronize()
        meta = dict(scheme=self.scheme, dt=self.dt, startup="lower_order", n=int(self.dev.n_total),
                    iteration=int(self.iteration), t=float(self.t), nhist=int(self.filled),
                    nhist_LX=int(self.filled) if self.family == "cn" else 0,
                    problem=self.dev.tpl.name, precision=self.dev.precision,
                    layout="mode", fourier_sizes=list(self.dev.P.fourier_sizes))
        h = lambda a: a.detach().cpu().numpy()
        arrays = {"X": h(self.X)}
        for j in range(self.filled if self.family != "rk" else 0):
            slot = (self.head - j) % self.ring
            arrays[f"MX{j}"] = h(self.MXh[slot])
            arrays[f"F{j}"] = h(self.Fh[slot])
            if self.family == "cn":
                arrays[f"LX{j}"] = -h(self.LXh[slot])          # stored negated on the device
        return meta, arrays

    def save_checkpoint(self, path) -> str:
        """State + multistep history + clock as ``.npz`` (written to a temporary file, then
        renamed): a restart continues bit for bit. The reference's npz layout (integrator.py:
        1009-1036: ``meta`` JSON, ``X``, ``MX<i>``, ``F<i>``, ``LX<i>``), on the mode layout."""
        import json
        import os
        path = str(path)
        if not path.endswith(".npz"):
            path += ".npz"
        meta, arrays = self.checkpoint_payload()
        for k, a in arrays.items():
            if not np.all(np.isfinite(a)):
                raise ValueError(f"save_checkpoint: {k} holds NaN or infinity")
        part = path[:-4] + ".part.npz"
        np.savez(part, meta=json.dumps(meta), **arrays)
        os.replace(part, path)
        return path

    def load_checkpoint(self, path) -> None:
        """Restart from :meth:`save_checkpoint`: the numerical options must match the solver's
        (integrator.py:1038-1097: a restart never changes the numerics silently)."""
        import json
        path = str(path)
        with np.load(path, allow_pickle=False) as z:
            arrays = {k: z[k] for k in z.files}
        meta = json.loads(str(arrays.pop("meta")))
        mine = dict(scheme=self.scheme, dt=self.dt, n=int(self.dev.n_total), problem=self.dev.tpl.name,
                    layout="mode", fourier_sizes=list(self.dev.P.fourier_sizes))
        for k, v in mine.items():
            if meta.get(k) != v:
                raise ValueError(f"checkpoint mismatch on {k}: {meta.get(k)!r} vs {v!r} (a restart "
                                 "never changes the numerics silently)")
        nh = int(meta["nhist"])
        if self.family == "rk":
            nh = 0
        if nh > self.ring or arrays["X"].shape != (self.dev.n_total,):
            raise ValueError("checkpoint: state or history does not match the solver")
        torch = _torch()
        dev = self.X.device
        self.stream.synchronize()
        self.X.copy_(torch.as_tensor(arrays["X"], device=dev))
        self.head, self.filled = self.ring - 1, nh
        for j in range(nh):
            slot = (self.head - j) % self.ring
            self.MXh[slot].copy_(torch.as_tensor(arrays[f"MX{j}"], device=dev))
            self.Fh[slot].copy_(torch.as_tensor(arrays[f"F{j}"], device=dev))
            if self.family == "cn":
                self.LXh[slot].copy_(-torch.as_tensor(arrays[f"LX{j}"], device=dev))
        self.t, self.iteration = float(meta["t"]), int(meta["iteration"])
        self._reset_finite()
        torch.cuda.current_stream().synchronize()

    def state_to_host(self):
        self.stream.synchronize()
        return self.dev.to_host(self.X)

    def launches_per_step(self) -> int:
        """Kernels of this library launched by one steady step: M X (one grouped launch for the
        buckets with a shared real M), F (``DeviceProblem.f_launches``: unpack and pack of every
        bucket in one launch each, 2 Chebyshev transforms, 2 or 4 Fourier transforms, products,
        constant part), -L X (the residual with a = 0, CN and Runge-Kutta), the right-hand side
        combination and the solves (one batched launch, or one per bucket with the band kernel; the
        FP32 form adds the residual and a second solve per refinement group). Grouped launches take
        at most 8 argument sets each."""
        dev = self.dev
        nb = len(dev.tpl.buckets)
        f = dev.f_launches()
        mx = dev.mx_launches()
        lx = dev.residual_launches()                  # -L X: the residual with a = 0
        dense = bool(dev._factors) and all(getattr(h, "schedule", 0) < 0 for fs in dev._factors.values() for h in fs)
        one = (nb if dense else 1) if dev.compact else nb
        res = dev.residual_launches()                 # residual launches per refinement pass
        if dev.precision == "fp32" and dev.compact and not dense and dev.overlap_refine:
            groups = dev._refine_groups()
            one = len(groups)                         # one batched launch per group
            res = sum(dev.residual_launches(dev._with_partners(g)) for g in groups)
        solve = one if dev.precision == "fp64" else one + dev.refine * (one + res)
        if self.family == "sbdf":
            return mx + f + 1 + solve
        if self.family == "cn":
            return mx + lx + f + 1 + solve
        A, H, c = self._rk
        S = len(c) - 1
        return mx + sum(f for x in self._Fs if x is not None) + sum(lx for x in self._LXs if x is not None) \
            + S * (1 + solve) + 1

    def synchronize(self) -> None:
        self.stream.synchronize()
