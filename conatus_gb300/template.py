"""Problem templates: the set-up data of a Fourier^d x Chebyshev IVP, independent of the Fourier
resolution, in the layout the GB300 kernels use.

The reference discretizes a model once (python/conatus/discretize/plan.py:851, ``GlobalSystem``
in python/conatus/timestep/system.py:244-334): one system per Fourier group, its rows and columns
permuted into solver order (border rows first, interleaved Chebyshev order), groups with one
sparsity pattern batched into a "bucket", and RealFourier (cos, -sin) pairs solved as complex
systems (``complexify=True``, system.py:600-726, exact). A template keeps, per bucket:

* the sparsity pattern of ``a M + b L`` in solver order and the values of M and L as polynomials
  in the signed wavenumbers (kx, kz) of the group -- the reference's group matrices are built
  from derivative blocks ``(i k)^order`` (discretize/layout.py:48-56), so each entry is a
  polynomial in k; the coefficients are recovered exactly from the reference's own assembly
  evaluated at small integer wavenumbers (see ``conatus_gb300.reference_adapter``);
* which (variable, component, Chebyshev index) each solver column holds, and which (equation,
  component, Chebyshev index, ultraspherical level lambda) each row holds;
* the rule that lists its systems at any Fourier resolution (which Fourier directions are nonzero,
  and the sign s of the second direction for the complex modes exp(i(kx x + s kz z))).

Plus the explicit right-hand side in polynomial form (``FusedRHS.factor_list/outputs`` of
python/conatus/timestep/fused.py:524-537), the conversions T -> C^(lambda) of the equations
(discretize/ultraspherical.py:43-66) and the constant part of F (boundary data, forcing).

Device layout ("mode layout"): every system is one complex vector of length n in solver order; the
state X, M X and F of a bucket are (nsys, n) complex arrays. A system of mode (jx, jz, s) holds the
complex amplitudes C with f = w Re(C exp(i(kx x + s kz z))), w = 2^(1 - d_act) for d_act >= 1
nonzero Fourier indices (1 for the mean mode), the reference's complex view of the real group.
"""
from __future__ import annotations

import itertools
import json
from dataclasses import dataclass, field

import numpy as np

__all__ = ["Bucket", "ProblemTemplate", "Problem"]


@dataclass
class Bucket:
    kind: str                     # "real" (all Fourier indices zero) or "complex"
    n: int
    r: int                        # border rows (first r rows in solver order)
    active: tuple                 # per Fourier direction: nonzero index in this bucket
    sign: int                     # s of the second Fourier direction (+1 / -1)
    indptr: np.ndarray            # pattern of a M + b L in solver order
    indices: np.ndarray
    monos: np.ndarray             # (nmono, d) powers of the signed wavenumbers
    Mc: np.ndarray                # (nmono, nnz) complex coefficients of M
    Lc: np.ndarray                # (nmono, nnz) complex coefficients of L
    col: np.ndarray               # (n, 3) int: variable, flat component, Chebyshev index (-1: none)
    row: np.ndarray               # (n, 4) int: equation, flat component, Chebyshev index, lambda
    fit_error: float = 0.0        # max relative error of the polynomial form on the source build
    exact: tuple | None = None    # optional (M values, L values), each (nsys, nnz), of the systems
                                  # of one resolution, taken bit for bit from the reference
    dL: dict = field(default_factory=dict)   # parameter name -> (nmono, nnz): L = Lc + sum_p theta_p dL[p]

    @property
    def nnz(self) -> int:
        return int(self.indices.shape[0])

    def coo_rows(self) -> np.ndarray:
        return np.repeat(np.arange(self.n), np.diff(self.indptr))

    def m_is_constant(self) -> bool:
        """M does not depend on the wavenumbers (only the constant monomial is nonzero)."""
        k0 = np.nonzero(np.all(self.monos == 0, axis=1))[0]
        others = [t for t in range(self.monos.shape[0]) if t not in set(k0.tolist())]
        return bool(not others or np.all(self.Mc[others] == 0))


def sign_similarity(a: Bucket, b: Bucket):
    """(dr, dc), int8 vectors of +1/-1, with b's matrix = diag(dr) (a's matrix) diag(dc) at every
    mode and for every (a, b) combination of M and L, or None. Structural: a and b are the two
    sign views (kx, +kz) and (kx, -kz) of the same groups (same pattern and the same polynomials
    in the signed wavenumbers), so b's entry e is a's with kz -> -kz; it is + or - a's entry at
    every mode iff every term of e (in M and in L) has the same parity in kz, and the entry signs
    must factor as dr_i dc_j (a spanning forest of the pattern's bipartite graph gives the
    candidate, every entry checks it). A border row k (rows 0 .. r-1) must keep the sign of its
    diagonal: dr_k dc_k = +1. The reference's sign_similarity (python/conatus/timestep/
    shared_factors.py:104-138) checks the same relation on the assembled values; conatus_gb300.ivp
    checks the values too before sharing."""
    if (a.kind != "complex" or b.kind != "complex" or a.n != b.n or a.r != b.r or a.active != b.active
            or a.sign == b.sign or len(a.active) < 2 or not all(a.active)):
        return None
    if not (np.array_equal(a.indptr, b.indptr) and np.array_equal(a.indices, b.indices)
            and np.array_equal(a.monos, b.monos) and np.array_equal(a.Mc, b.Mc) and np.array_equal(a.Lc, b.Lc)):
        return None
    odd = (a.monos[:, 1] % 2 == 1)[:, None]             # terms odd in kz flip with the sign view
    used = (a.Mc != 0) | (a.Lc != 0)                    # (nmono, nnz)
    has_odd = np.any(used & odd, axis=0)
    has_even = np.any(used & ~odd, axis=0)
    if np.any(has_odd & has_even) or not np.all(has_odd | has_even):
        return None                                     # mixed parity (or an empty entry): no relation
    sgn = np.where(has_odd, -1, 1).astype(np.int8)      # entry sign of b relative to a
    n = a.n
    rows = np.repeat(np.arange(n), np.diff(a.indptr))
    cols = a.indices.astype(np.int64)
    # spanning forest of the bipartite graph (rows 0..n-1, columns n..2n-1), breadth first
    adj = [[] for _ in range(2 * n)]
    for e, (i, j) in enumerate(zip(rows, cols)):
        adj[i].append((n + j, e))
        adj[n + j].append((i, e))
    d = np.zeros(2 * n, np.int8)
    for root in range(2 * n):
        if d[root]:
            continue
        d[root] = 1
        queue = [root]
        while queue:
            v = queue.pop()
            for w, e in adj[v]:
                if not d[w]:
                    d[w] = d[v] * sgn[e]
                    queue.append(w)
    dr, dc = d[:n].copy(), d[n:].copy()
    if not np.array_equal(dr[rows] * dc[cols], sgn):
        return None                                     # entry signs do not factor as dr_i dc_j
    if a.r and not np.all(dr[:a.r] * dc[:a.r] == 1):
        return None                                     # a border row's s e_k would change sign
    return dr, dc


@dataclass
class ProblemTemplate:
    name: str
    axes: list                    # per coordinate: {coord, kind, N, L, a, M}
    cheb_axis: int                # index of the Chebyshev axis (-1: none)
    fourier_axes: list            # indices of the RealFourier axes, in order
    variables: list               # {name, ncomp, shape}
    equations: list               # {ncomp, shape}
    factors: list                 # (var, comp, orders per axis)
    outputs: list                 # (eq, comp, [(coef, (factor ids))]) -- constant terms excluded
    conv: dict                    # lambda -> (N, N) dense conversion T -> C^(lambda)
    buckets: list
    b0: list = field(default_factory=list)   # (bucket, mode tuple, position, value) of F(0)
    params: dict = field(default_factory=dict)
    source: dict = field(default_factory=dict)
    linear_params: list = field(default_factory=list)   # parameters L depends on linearly

    # ---------------------------------------------------------------- persistence
    def save(self, path: str) -> None:
        meta = dict(name=self.name, axes=self.axes, cheb_axis=self.cheb_axis,
                    fourier_axes=self.fourier_axes, variables=self.variables,
                    equations=self.equations,
                    factors=[[int(v), int(c), [int(o) for o in a]] for v, c, a in self.factors],
                    outputs=[[int(e), int(c), [[_cplx_json(co), [int(f) for f in fs]] for co, fs in m]]
                             for e, c, m in self.outputs],
                    lams=sorted(int(k) for k in self.conv),
                    buckets=[dict(kind=b.kind, n=b.n, r=b.r, active=list(map(bool, b.active)),
                                  sign=int(b.sign), fit_error=float(b.fit_error))
                             for b in self.buckets],
                    b0=[[int(bi), [int(j) for j in mode], int(pos), _cplx_json(v)]
                        for bi, mode, pos, v in self.b0],
                    params=self.params, source=self.source, linear_params=self.linear_params)
        arrays = {"meta": np.array(json.dumps(meta))}
        for lam, C in self.conv.items():
            arrays[f"conv_{lam}"] = C
        for i, b in enumerate(self.buckets):
            p = f"b{i}_"
            arrays[p + "indptr"] = b.indptr.astype(np.int32)
            arrays[p + "indices"] = b.indices.astype(np.int32)
            arrays[p + "monos"] = b.monos.astype(np.int32)
            arrays[p + "Mc"] = b.Mc
            arrays[p + "Lc"] = b.Lc
            arrays[p + "col"] = b.col.astype(np.int32)
            arrays[p + "row"] = b.row.astype(np.int32)
            for name, D in b.dL.items():
                arrays[p + "dL_" + name] = D
        np.savez_compressed(path, **arrays)

    @classmethod
    def load(cls, path: str) -> "ProblemTemplate":
        z = np.load(path, allow_pickle=False)
        meta = json.loads(str(z["meta"]))
        buckets = []
        for i, bm in enumerate(meta["buckets"]):
            p = f"b{i}_"
            bk = Bucket(bm["kind"], int(bm["n"]), int(bm["r"]), tuple(bm["active"]),
                        int(bm["sign"]), z[p + "indptr"], z[p + "indices"], z[p + "monos"],
                        z[p + "Mc"], z[p + "Lc"], z[p + "col"], z[p + "row"],
                        float(bm.get("fit_error", 0.0)))
            for name in meta.get("linear_params", []):
                bk.dL[name] = z[p + "dL_" + name]
            buckets.append(bk)
        return cls(name=meta["name"], axes=meta["axes"], cheb_axis=int(meta["cheb_axis"]),
                   fourier_axes=list(meta["fourier_axes"]), variables=meta["variables"],
                   equations=meta["equations"],
                   factors=[(v, c, tuple(a)) for v, c, a in meta["factors"]],
                   outputs=[(e, c, [(_cplx_from(co), tuple(fs)) for co, fs in m])
                            for e, c, m in meta["outputs"]],
                   conv={int(l): z[f"conv_{l}"] for l in meta["lams"]},
                   buckets=buckets,
                   b0=[(bi, tuple(mode), pos, _cplx_from(v)) for bi, mode, pos, v in meta["b0"]],
                   params=meta.get("params", {}), source=meta.get("source", {}),
                   linear_params=list(meta.get("linear_params", [])))

    # ---------------------------------------------------------------- derived
    def sign_pairs(self) -> dict:
        """Buckets solved with another bucket's factors: {partner index: (primary index, dr, dc)}
        (``sign_similarity``), each primary used once."""
        out, used = {}, set()
        for j, b in enumerate(self.buckets):
            for i, a in enumerate(self.buckets[:j]):
                if i in used or i in out:
                    continue
                rel = sign_similarity(a, b)
                if rel is not None:
                    out[j] = (i, rel[0], rel[1])
                    used.add(i)
                    break
        return out

    @property
    def ncheb(self) -> int:
        return self.axes[self.cheb_axis]["N"] if self.cheb_axis >= 0 else 1

    def instantiate(self, fourier_sizes=None, lengths=None, params=None) -> "Problem":
        """The systems of this template at the given RealFourier sizes (default: the template's) and,
        optionally, other periods of the Fourier directions (the operators are polynomials in the
        wavenumbers 2 pi j / L, so the period is a free parameter) and other values of the
        parameters L depends on linearly (``linear_params``)."""
        return Problem(self, fourier_sizes, lengths, params)

    def with_params(self, **values) -> "ProblemTemplate":
        """A copy whose L is evaluated at the given values of its linear parameters."""
        import copy
        t = copy.copy(self)
        t.buckets = []
        for b in self.buckets:
            nb = copy.copy(b)
            nb.Lc = b.Lc.copy()
            for name, v in values.items():
                if name not in b.dL:
                    raise KeyError(f"{self.name}: no linear parameter {name!r}")
                nb.Lc = nb.Lc + float(v) * b.dL[name]
            nb.dL = {}
            t.buckets.append(nb)
        t.linear_params = []
        t.params = dict(self.params, **{k: float(v) for k, v in values.items()})
        return t


def _cplx_json(v):
    v = complex(v)
    return [v.real, v.imag]


def _cplx_from(v):
    if isinstance(v, (list, tuple)):
        return complex(v[0], v[1])
    return complex(v)


class Problem:
    """A template at a Fourier resolution: the systems (modes, wavenumbers) of every bucket."""

    def __init__(self, tpl: ProblemTemplate, fourier_sizes=None, lengths=None, params=None):
        if params:
            tpl = tpl.with_params(**params)
        elif tpl.linear_params:
            tpl = tpl.with_params(**{k: tpl.params[k] for k in tpl.linear_params})
        self.tpl = tpl
        d = len(tpl.fourier_axes)
        if fourier_sizes is None:
            fourier_sizes = [tpl.axes[a]["N"] for a in tpl.fourier_axes]
        fourier_sizes = [int(s) for s in fourier_sizes]
        if len(fourier_sizes) != d:
            raise ValueError(f"{tpl.name}: {d} Fourier sizes expected, got {fourier_sizes}")
        for s in fourier_sizes:
            if s % 2 or s < 2:
                raise ValueError("Fourier sizes must be even (Nyquist convention)")
        self.fourier_sizes = fourier_sizes
        self.K = [s // 2 for s in fourier_sizes]
        self.lengths = [float(x) for x in lengths] if lengths is not None else \
            [tpl.axes[a]["L"] for a in tpl.fourier_axes]
        if len(self.lengths) != d:
            raise ValueError(f"{tpl.name}: {d} periods expected")
        # grid sizes: the reference's dealiasing rule floor(N * 3/2) scaled from the template
        self.modes, self.wavenumbers, self.offsets = [], [], []
        off = 0
        for b in tpl.buckets:
            ranges = [range(1, K) if act else range(0, 1) for act, K in zip(b.active, self.K)]
            modes = np.array(list(itertools.product(*ranges)), dtype=np.int64).reshape(-1, d) if d else \
                np.zeros((1, 0), np.int64)
            kw = np.zeros(modes.shape, dtype=np.float64)
            for j in range(d):
                kw[:, j] = 2 * np.pi * modes[:, j] / self.lengths[j]
            if d >= 2:
                kw[:, 1] *= b.sign
            self.modes.append(modes)
            self.wavenumbers.append(kw)
            self.offsets.append(off)
            off += modes.shape[0] * b.n
        self.n_total = off           # complex unknowns of the mode layout

    def axis_length(self, ax: int) -> float:
        """Length of coordinate axis ``ax`` of this instance."""
        if ax in self.tpl.fourier_axes:
            return self.lengths[self.tpl.fourier_axes.index(ax)]
        return self.tpl.axes[ax]["L"]

    @property
    def nsys(self):
        return [m.shape[0] for m in self.modes]

    def mono_values(self, bi: int) -> np.ndarray:
        """(nsys, nmono) values of the wavenumber monomials of bucket bi."""
        b = self.tpl.buckets[bi]
        kw = self.wavenumbers[bi]
        out = np.ones((kw.shape[0], b.monos.shape[0]), dtype=np.float64)
        for t, powers in enumerate(b.monos):
            for j, p in enumerate(powers):
                if p:
                    out[:, t] *= kw[:, j] ** int(p)
        return out

    def values(self, bi: int, which: str) -> np.ndarray:
        """(nsys, nnz) values of M or L ('M' / 'L') of every system of bucket bi: the reference's
        own values when the bucket carries them for this resolution, else the wavenumber
        polynomial."""
        b = self.tpl.buckets[bi]
        if b.exact is not None and b.exact[0].shape[0] == self.nsys[bi]:
            return np.array(b.exact[0] if which == "M" else b.exact[1], dtype=np.complex128)
        C = b.Mc if which == "M" else b.Lc
        return self.mono_values(bi).astype(np.complex128) @ C

    def set_exact(self, values) -> None:
        """Attach the reference's own (M, L) values per bucket, [(Mv, Lv)] with (nsys, nnz)."""
        for b, (Mv, Lv), ns in zip(self.tpl.buckets, values, self.nsys):
            if Mv.shape != (ns, b.nnz) or Lv.shape != (ns, b.nnz):
                raise ValueError("exact values do not match the bucket (nsys, nnz)")
            b.exact = (np.asarray(Mv), np.asarray(Lv))

    def d_active(self, bi: int) -> int:
        return int(sum(self.tpl.buckets[bi].active))

    def real_unknowns(self) -> int:
        """Unknowns of the reference's real global vector (N_u): complex systems count twice,
        except the modes with 2 active directions, whose two sign views share 4 real entries."""
        tot = 0
        for bi, b in enumerate(self.tpl.buckets):
            ns = self.nsys[bi]
            tot += ns * b.n * (1 if b.kind == "real" else 2)
        return tot

    def b0_dense(self):
        """Constant part of F in the mode layout: list per bucket of (nsys, n) complex arrays
        (zero where the template has no entry; modes absent at this resolution are dropped)."""
        out = [np.zeros((ns, b.n), np.complex128) for ns, b in zip(self.nsys, self.tpl.buckets)]
        for bi, mode, pos, v in self.tpl.b0:
            hit = np.nonzero(np.all(self.modes[bi] == np.asarray(mode, dtype=np.int64), axis=1))[0]
            if hit.size:
                out[bi][hit[0], pos] += v
        return out


class StackedProblem:
    """Cases of one template at one Fourier resolution, advanced as one problem (an ensemble):
    every bucket holds the systems of all cases (case-major), the F pipeline runs over every case in
    one pass (a case index per system), the solves over every system in one launch. The cases
    differ in the values of the template's linear parameters (L = L0 + sum_p theta_p dL_p, e.g. Ra
    for Rayleigh-Benard): their M, sparsity patterns, F and wavenumbers are the same.

    The reference runs ensemble members as separate batched solves of one discretization
    (python/conatus/ensembles/batched.py:442-613)."""

    def __init__(self, tpl: ProblemTemplate, fourier_sizes, params_list, lengths=None):
        if not params_list:
            raise ValueError("at least one case")
        names = set(params_list[0])
        for pr in params_list:
            if set(pr) != names or not names <= set(tpl.linear_params):
                raise ValueError(f"every case sets the same linear parameters of {tpl.name} "
                                 f"({tpl.linear_params})")
        self.base_tpl = tpl
        self.params = [dict(pr) for pr in params_list]
        self.ncase = len(params_list)
        first = Problem(tpl, fourier_sizes, lengths, params_list[0])
        self.tpl = first.tpl
        self.fourier_sizes, self.K, self.lengths = first.fourier_sizes, first.K, first.lengths
        nb = len(tpl.buckets)
        self._nsys_case = first.nsys
        self.modes = [np.concatenate([first.modes[bi]] * self.ncase) for bi in range(nb)]
        self.wavenumbers = [np.concatenate([first.wavenumbers[bi]] * self.ncase) for bi in range(nb)]
        self.case_of = [np.repeat(np.arange(self.ncase, dtype=np.int32), first.nsys[bi]) for bi in range(nb)]
        self._first = first
        self.offsets, off = [], 0
        for bi, b in enumerate(tpl.buckets):
            self.offsets.append(off)
            off += self.modes[bi].shape[0] * b.n
        self.n_total = off

    def axis_length(self, ax: int) -> float:
        return self._first.axis_length(ax)

    @property
    def nsys(self):
        return [m.shape[0] for m in self.modes]

    def mono_values(self, bi: int) -> np.ndarray:
        return np.concatenate([self._first.mono_values(bi)] * self.ncase)

    def _theta(self, name):
        return np.array([pr[name] for pr in self.params], dtype=np.float64)

    def values(self, bi: int, which: str) -> np.ndarray:
        b0 = self.base_tpl.buckets[bi]
        mv = self._first.mono_values(bi).astype(np.complex128)
        if which == "M":
            return np.concatenate([mv @ b0.Mc] * self.ncase)
        base = mv @ b0.Lc
        out = np.empty((self.ncase * base.shape[0], base.shape[1]), np.complex128)
        ns = base.shape[0]
        for c, pr in enumerate(self.params):
            v = base.copy()
            for name, th in pr.items():
                v = v + float(th) * (mv @ b0.dL[name])
            out[c * ns:(c + 1) * ns] = v
        return out

    def split_terms(self, bi: int):
        """Terms of L for the refinement residual: (coefficient row, per-system scale) -- the base
        rows L0_t with the monomial values, and the parameter rows dL_{p,t} with the monomial values
        times each system's theta_p."""
        b0 = self.base_tpl.buckets[bi]
        mv = self.mono_values(bi)
        out = []
        for t in range(b0.monos.shape[0]):
            if np.any(b0.Lc[t] != 0):
                out.append((b0.Lc[t], mv[:, t]))
        for name in self.params[0]:
            th = np.repeat(self._theta(name), self._nsys_case[bi])
            for t in range(b0.monos.shape[0]):
                if np.any(b0.dL[name][t] != 0):
                    out.append((b0.dL[name][t], mv[:, t] * th))
        return out

    def d_active(self, bi: int) -> int:
        return self._first.d_active(bi)

    def real_unknowns(self) -> int:
        return self._first.real_unknowns() * self.ncase

    def b0_dense(self):
        return [np.concatenate([x] * self.ncase) for x in self._first.b0_dense()]

    def case_state(self, C, c: int):
        """The mode-layout arrays of case ``c`` out of the stacked per-bucket arrays."""
        return [np.asarray(C[bi])[c * ns:(c + 1) * ns] for bi, ns in enumerate(self._nsys_case)]

    def stack_states(self, states):
        """Per-bucket stacked arrays from the cases' mode-layout states."""
        return [np.concatenate([st[bi] for st in states]) for bi in range(len(self._nsys_case))]


class _GroupedTemplate:
    """The bucket list of a GroupedProblem (its groups' buckets side by side) with the template
    attributes the device solver reads; F stays per group."""

    def __init__(self, tpls):
        t0 = tpls[0]
        for t in tpls[1:]:
            if (len(t.fourier_axes) != len(t0.fourier_axes) or (t.cheb_axis >= 0) != (t0.cheb_axis >= 0)
                    or [v["name"] for v in t.variables] != [v["name"] for v in t0.variables]):
                raise ValueError("grouped problems need the same variables and the same kinds of axes")
        self.parts = list(tpls)
        self.name = "+".join(t.name for t in tpls)
        self.variables = t0.variables
        self.fourier_axes = t0.fourier_axes
        self.cheb_axis = t0.cheb_axis
        self.axes = t0.axes
        self.buckets = [b for t in tpls for b in t.buckets]
        self.linear_params = list(t0.linear_params)

    def sign_pairs(self) -> dict:
        out, base = {}, 0
        for t in self.parts:
            for j, (i, dr, dc) in t.sign_pairs().items():
                out[base + j] = (base + i, dr, dc)
            base += len(t.buckets)
        return out


class GroupedProblem:
    """Problems of different sizes (or templates with the same variables) advanced as one: their
    buckets side by side in one mode layout, so that every kernel of a step is one launch for all
    of them — F by grouped launches (one per stage, each problem over its own block range), M X and
    the refinement residual by grouped launches, the solves by the batched multi-bucket launch, the
    right-hand side and the finite-state check over the joint vector. Each problem keeps its own
    arithmetic: a group member's trajectory is bit for bit the one it has alone. The groups are
    typically ``StackedProblem`` ensembles of one resolution each (Rayleigh-Benard cases of several
    Nz).

    The reference batches ensemble members of one discretization only
    (python/conatus/ensembles/batched.py:442-613)."""

    def __init__(self, problems):
        if not problems:
            raise ValueError("at least one problem")
        self.parts = list(problems)
        self.tpl = _GroupedTemplate([p.tpl for p in self.parts])
        self.bucket_of = [(g, bi) for g, p in enumerate(self.parts) for bi in range(len(p.tpl.buckets))]
        self.group_buckets = []
        k = 0
        for p in self.parts:
            nb = len(p.tpl.buckets)
            self.group_buckets.append(list(range(k, k + nb)))
            k += nb
        self.modes = [self.parts[g].modes[bi] for g, bi in self.bucket_of]
        self.offsets, off = [], 0
        for (g, bi), b in zip(self.bucket_of, self.tpl.buckets):
            self.offsets.append(off)
            off += self.parts[g].nsys[bi] * b.n
        self.n_total = off

    @property
    def nsys(self):
        return [self.parts[g].nsys[bi] for g, bi in self.bucket_of]

    @property
    def ncase(self) -> int:
        return sum(int(getattr(p, "ncase", 1)) for p in self.parts)

    @property
    def fourier_sizes(self):
        return tuple(tuple(p.fourier_sizes) for p in self.parts)

    def _part(self, bi):
        g, lb = self.bucket_of[bi]
        return self.parts[g], lb

    def mono_values(self, bi: int) -> np.ndarray:
        p, lb = self._part(bi)
        return p.mono_values(lb)

    def values(self, bi: int, which: str) -> np.ndarray:
        p, lb = self._part(bi)
        return p.values(lb, which)

    def split_terms(self, bi: int):
        p, lb = self._part(bi)
        if hasattr(p, "split_terms"):
            return p.split_terms(lb)
        b = p.tpl.buckets[lb]
        return [(b.Lc[t], p.mono_values(lb)[:, t]) for t in range(b.monos.shape[0]) if np.any(b.Lc[t] != 0)]

    def d_active(self, bi: int) -> int:
        p, lb = self._part(bi)
        return p.d_active(lb)

    def real_unknowns(self) -> int:
        return sum(p.real_unknowns() for p in self.parts)

    def b0_dense(self):
        return [x for p in self.parts for x in p.b0_dense()]

    def stack_states(self, states):
        """The joint per-bucket list from one mode-layout state per group."""
        if len(states) != len(self.parts):
            raise ValueError("one state per group")
        return [np.asarray(c) for st in states for c in st]

    def group_state(self, C, g: int):
        """Group g's per-bucket arrays out of the joint list."""
        return [C[bi] for bi in self.group_buckets[g]]
