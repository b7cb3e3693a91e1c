"""Adapter from a live reference ``IVPSolver`` to a :class:`ProblemTemplate` (the drop-in set-up).

Runs where the reference package is importable: it reads the reference's own discretization
(``GlobalSystem`` buckets and complex views, python/conatus/timestep/system.py:244-726; the
compiled RHS ``FusedRHS``, python/conatus/timestep/fused.py:280-537) and converts it into the
GB300 layout. Nothing numerical is re-derived: every matrix entry comes from the reference's
assembly.

Wavenumber polynomials. The reference builds a group's matrices from derivative blocks
``GroupItem.deriv(order)`` = powers of [[0, -k], [k, 0]] on (cos, -sin) pairs
(python/conatus/discretize/layout.py:48-56), so each entry of a bucket's complex view is a
polynomial in the group's signed wavenumbers. The adapter re-runs the reference's group assembly
(``GlobalSystem._build_group``) on copies of the group with integer wavenumbers on a tensor grid of
nodes, solves the small Vandermonde systems for the coefficients, and checks the result against
every real system of the bucket (``Bucket.fit_error``).
"""
from __future__ import annotations

import dataclasses
import itertools

import numpy as np
import scipy.sparse as sp

from .template import Bucket, ProblemTemplate

#: wavenumber nodes of the polynomial extraction (integers: exact powers; k = 0 is a different
#: group structure, so it is not a node)
NODES = (-2.0, -1.0, 1.0, 2.0, 3.0)
DEGREE = 4


def _flat_comp(comp, rank, dim):
    if rank == 0:
        return 0
    return int(np.ravel_multi_index(tuple(comp), (dim,) * rank))


def _unravel(flat, shape, rank):
    """(flat component, per-axis indices) of a flat index into an object's coefficient array."""
    idx = np.unravel_index(int(flat), shape)
    comp = idx[:rank]
    cshape = shape[:rank]
    cf = int(np.ravel_multi_index(comp, cshape)) if rank else 0
    return cf, idx[rank:]


class _Views:
    """Views of one bucket of the reference system: per system, (slot index, view key)."""

    def __init__(self, S, kind, entries, label, sign):
        self.S, self.kind, self.entries, self.label, self.sign = S, kind, entries, label, sign

    def view(self, slot, key, group=None):
        """(M, L, rperm, cperm, n_border, col_local, row_local, slot_obj, cm, rpart) of a system
        (cm/rpart only when assembled); with ``group``, the reference's assembly of that
        (fabricated) group, else the stored slot."""
        S = self.S
        cm = rpart = None
        if group is None:
            sl = S.slots[slot]
        else:
            parts = S._build_group(group, S.reduced)
            if len(parts) != 1:
                raise NotImplementedError("decouple=True (several blocks per group) is not supported")
            sl, cm, rpart = parts[0]
        if self.kind == "real":
            return (sl.M, sl.L, sl.rperm, sl.cperm, sl.n_border, np.arange(sl.size),
                    np.arange(sl.size), sl, cm, rpart)
        if self.kind == "cz":
            cz = sl.cz
            return cz.M, cz.L, cz.rperm, cz.cperm, cz.n_border, cz.cc, cz.rc, sl, cm, rpart
        v = sl.zs[key]
        return v.M, v.L, v.rperm, v.cperm, v.n_border, v.cols[0], v.rows[0], sl, cm, rpart


def _bucket_views(S):
    out = []
    for idx, _, _ in S._buckets:
        out.append(_Views(S, "real", [(i, None) for i in idx], S.slots[idx[0]].label, 1))
    for idx, *_ in S._cbuckets:
        out.append(_Views(S, "cz", [(i, None) for i in idx], S.slots[idx[0]].label, 1))
    for keys, *_ in S._zbuckets:
        v0 = S.slots[keys[0][0]].zs[keys[0][1]]
        sgn = int(v0.s[1]) if len(v0.s) > 1 else 1
        out.append(_Views(S, "zs", list(keys), S.slots[keys[0][0]].label, sgn))
    return out


def _permuted(A, rperm, cperm):
    return sp.csr_matrix(sp.csr_matrix(A)[rperm][:, cperm], dtype=np.complex128)


def _pattern_values(A, pat):
    """Values of sparse A on the CSR pattern ``pat`` (zeros where A has no entry); refuses entries
    of A outside the pattern."""
    A = sp.csr_matrix(A, dtype=np.complex128)
    outside = sp.csr_matrix(abs(A) > 0, dtype=np.int8) - sp.csr_matrix(abs(A) > 0, dtype=np.int8).multiply(pat)
    if outside.nnz and np.any(outside.data != 0):
        raise ValueError("matrix has entries outside the bucket pattern")
    rows = np.repeat(np.arange(pat.shape[0]), np.diff(pat.indptr))
    return np.asarray(A[rows, pat.indices]).ravel()


def template_from_solver(solver, name: str, params: dict | None = None,
                         exact_values: bool = False) -> ProblemTemplate:
    """Template of a reference ``IVPSolver`` built with ``complexify=True`` and
    ``f_backend="fused"`` (the polynomial form of F). ``exact_values``: also attach the reference's
    own M and L values of every system of this build (``Bucket.exact``), which the runtime then
    uses instead of the wavenumber polynomial -- the drop-in case, where the reference hands over
    its assembled matrices bit for bit."""
    S = solver.system
    plan = solver.plan
    dom = plan.domain
    coords = list(dom.coordsys.coords)
    from conatus.ir.bases import Chebyshev, RealFourier
    axes, cheb_axis, fourier_axes = [], -1, []
    for i, c in enumerate(coords):
        b = dom.basis(c)
        kind = "Chebyshev" if isinstance(b, Chebyshev) else "RealFourier" if isinstance(b, RealFourier) else None
        if kind is None:
            raise NotImplementedError(f"basis {type(b).__name__} (only RealFourier x Chebyshev)")
        if getattr(b, "map", None) is not None:
            raise NotImplementedError("mapped Chebyshev axes are not supported")
        axes.append(dict(coord=str(getattr(c, "name", c)), kind=kind, N=int(b.size), L=float(b.length),
                         a=float(b.bounds[0]), M=int(b.grid_size), dealias=float(b.dealias)))
        if kind == "Chebyshev":
            if cheb_axis >= 0:
                raise NotImplementedError("one Chebyshev axis at most")
            cheb_axis = i
        else:
            fourier_axes.append(i)
    if fourier_axes and not S.complexify:
        raise ValueError("the GB300 layout needs complexify=True (RealFourier pairs as complex systems)")
    d = len(fourier_axes)
    var_names = [v.name for v in S.variables]
    variables = [dict(name=v.name, rank=int(v.rank if hasattr(v, "rank") else len(v.tensorsig)),
                      shape=list(map(int, sh))) for v, sh in zip(S.variables, S.var_shapes)]
    equations = [dict(rank=int(eq.lhs.rank), shape=list(map(int, sh)))
                 for eq, sh in zip(plan.problem.equations, S.eq_shapes)]
    for v in variables:
        v["ncomp"] = int(np.prod(v["shape"][:v["rank"]])) if v["rank"] else 1
    for e in equations:
        e["ncomp"] = int(np.prod(e["shape"][:e["rank"]])) if e["rank"] else 1
    ndim = len(coords)

    # ---- F (polynomial form)
    fz = solver._fused
    if fz is None or fz.mode != "polynomial":
        raise ValueError("the solver needs f_backend='fused' with a polynomial right-hand side")
    factors = []
    for f, comp, a in fz.factor_list:
        vi = var_names.index(f.name)
        factors.append((vi, _flat_comp(comp, len(comp), ndim), tuple(int(x) for x in a)))
    outputs = []
    for k, comp, monos in fz.outputs:
        ms = [(complex(c), tuple(int(j) for j in fs)) for c, fs in monos if len(fs) > 0 and c != 0]
        outputs.append((int(k), _flat_comp(comp, len(comp), ndim), ms))

    # ---- conversions
    lams = sorted({int(l) for l in np.unique(S.rows_lam) if l > 0})
    conv = {}
    if cheb_axis >= 0:
        for lam in lams:
            conv[lam] = np.asarray(plan.layout.zconv(lam).toarray(), dtype=np.float64)

    def descr_cols(cm, local):
        out = np.zeros((len(local), 3), np.int64)
        for i, j in enumerate(local):
            k, fl, n = cm[j]
            rank = variables[k]["rank"]
            cf, _ = _unravel(fl, tuple(variables[k]["shape"]), rank)
            out[i] = (k, cf, -1 if n is None else int(n))
        return out

    def descr_rows(rpart, local):
        out = np.zeros((len(local), 4), np.int64)
        for i, j in enumerate(local):
            k, fl, n, lam = rpart[j]
            rank = equations[k]["rank"]
            cf, _ = _unravel(fl, tuple(equations[k]["shape"]), rank)
            out[i] = (k, cf, int(n), int(lam))
        return out

    if d == 0:
        monos = np.zeros((1, 0), np.int64)
    else:
        monos = np.array([p for p in itertools.product(range(DEGREE + 1), repeat=d) if sum(p) <= DEGREE],
                         dtype=np.int64)
    buckets = []
    for bv in _bucket_views(S):
        slot0, key0 = bv.entries[0]
        g0 = S.slots[slot0].group
        M0, L0, rp, cpm, nb, cl, rl, sl0, cm, rpart = bv.view(slot0, key0, g0)
        active = tuple(bool(g0[j].index != 0) for j in range(d)) if d else ()
        # union pattern over the real systems
        mats = []
        for slot, key in bv.entries:
            M, L, rpi, cpi, _, _, _, _, _, _ = bv.view(slot, key)
            if not (np.array_equal(rpi, rp) and np.array_equal(cpi, cpm)):
                raise ValueError(f"[{bv.label}] systems of one bucket with different orderings")
            mats.append((_permuted(M, rp, cpm), _permuted(L, rp, cpm), S.slots[slot].group))
        pat = sp.csr_matrix(sum(abs(M) + abs(L) for M, L, _ in mats) > 0, dtype=np.float64)
        pat.sort_indices()
        n = pat.shape[0]
        act_dirs = [j for j in range(d) if active[j]]
        if act_dirs:
            # evaluate the reference assembly on the node grid of the active directions
            node_sets = list(itertools.product(NODES, repeat=len(act_dirs)))
            use = [t for t, p in enumerate(monos) if all(p[j] == 0 for j in range(d) if j not in act_dirs)]
            V = np.array([[np.prod([kn[act_dirs.index(j)] ** monos[t][j] for j in act_dirs])
                           for t in use] for kn in node_sets])
            Ym, Yl = [], []
            for kn in node_sets:
                g = list(g0)
                for jj, j in enumerate(act_dirs):
                    kval = kn[jj] * (bv.sign if (j == 1 and d >= 2) else 1)
                    g[j] = dataclasses.replace(g0[j], k=float(kval))
                Mf, Lf, rpf, cpf, _, _, _, _, _, _ = bv.view(slot0, key0, tuple(g))
                if not (np.array_equal(rpf, rp) and np.array_equal(cpf, cpm)):
                    raise ValueError(f"[{bv.label}] fabricated group has another ordering")
                Ym.append(_pattern_values(_permuted(Mf, rp, cpm), pat))
                Yl.append(_pattern_values(_permuted(Lf, rp, cpm), pat))
            sol_m = np.linalg.lstsq(V.astype(np.complex128), np.array(Ym), rcond=None)[0]
            sol_l = np.linalg.lstsq(V.astype(np.complex128), np.array(Yl), rcond=None)[0]
            Mc = np.zeros((monos.shape[0], pat.nnz), np.complex128)
            Lc = np.zeros((monos.shape[0], pat.nnz), np.complex128)
            Mc[use] = sol_m
            Lc[use] = sol_l
            # the node grid is symmetric in sign and the powers are small integers: snap the
            # coefficients that are zero to rounding (pure k^p structure) to exact zero
            for C in (Mc, Lc):
                scale = np.abs(C).max(axis=0, keepdims=True) + 1e-300
                C[np.abs(C) < 1e-13 * scale] = 0
        else:
            Mc = np.zeros((monos.shape[0], pat.nnz), np.complex128)
            Lc = np.zeros((monos.shape[0], pat.nnz), np.complex128)
            t0 = int(np.nonzero(np.all(monos == 0, axis=1))[0][0])
            Mc[t0] = _pattern_values(mats[0][0], pat)
            Lc[t0] = _pattern_values(mats[0][1], pat)
        # check the polynomial form against every system of the bucket
        err = 0.0
        for M, L, grp in mats:
            kv = [float(grp[j].k) * (bv.sign if (j == 1 and d >= 2) else 1) for j in range(d)]
            mv = np.array([np.prod([kv[j] ** p[j] for j in range(d)]) for p in monos])
            for X, C in ((M, Mc), (L, Lc)):
                ref = _pattern_values(X, pat)
                got = mv @ C
                scale = max(np.abs(ref).max(), 1e-300)
                err = max(err, float(np.abs(got - ref).max() / scale))
        if err > 1e-12:
            raise ValueError(f"[{bv.label}] wavenumber polynomial does not reproduce the reference "
                             f"matrices (max relative error {err:.2e})")
        kind = "real" if bv.kind == "real" else "complex"
        bk = Bucket(kind, n, int(nb), active, int(bv.sign), pat.indptr.astype(np.int64),
                    pat.indices.astype(np.int64), monos, Mc, Lc,
                    descr_cols(cm, np.asarray(cl)[cpm]), descr_rows(rpart, np.asarray(rl)[rp]), err)
        if exact_values:
            bk.exact = (np.stack([_pattern_values(M, pat) for M, _, _ in mats]),
                        np.stack([_pattern_values(L, pat) for _, L, _ in mats]))
        buckets.append(bk)

    tpl = ProblemTemplate(name=name, axes=axes, cheb_axis=cheb_axis, fourier_axes=fourier_axes,
                          variables=variables, equations=equations, factors=factors,
                          outputs=outputs, conv=conv, buckets=buckets, params=dict(params or {}))
    # ---- constant part of F: the reference's F at X = 0, in the mode layout
    F0 = np.asarray(solver.F(np.zeros(S.n, dtype=S.dtype), solver.t))
    maps = reference_maps(solver)
    b0 = []
    for bi, mp in enumerate(maps):
        R = gather_rows(F0, mp)
        for m, i in zip(*np.nonzero(np.abs(R) > 0)):
            b0.append((bi, tuple(int(j) for j in mp["modes"][m]), int(i), complex(R[m, i])))
    tpl.b0 = b0
    # the template's own Fourier sizes must list the reference's systems in the same order
    prob = tpl.instantiate()
    for bi, mp in enumerate(maps):
        if not np.array_equal(prob.modes[bi], mp["modes"]):
            raise ValueError(f"bucket {bi}: mode order differs from the reference's")
    return tpl


def reference_maps(solver) -> list:
    """Per bucket: gather maps between the reference's real global vector and the mode layout.

    ``cols``/``rows`` (P, nsys, n) global indices and ``wc``/``wr`` (P,) complex weights with
    C[m, i] = sum_p wc[p] X[cols[p, m, i]] (state) and R[m, i] = sum_p wr[p] r[rows[p, m, i]]
    (right-hand sides), and ``modes`` (nsys, d) the Fourier indices of each system
    (system.py:544-597 for the bucket maps)."""
    S = solver.system
    d = len([1 for c in solver.plan.domain.coordsys.coords
             if type(solver.plan.domain.basis(c)).__name__ == "RealFourier"])
    out = []
    for idx, rows, cols in S._buckets:
        modes = np.array([[g.index for g in S.slots[i].group][:d] for i in idx], np.int64).reshape(len(idx), d)
        out.append(dict(cols=cols[None], rows=rows[None], wc=np.ones(1, complex), wr=np.ones(1, complex),
                        modes=modes, dact=0))
    for idx, rc, rs, cc, cs in S._cbuckets:
        modes = np.array([[g.index for g in S.slots[i].group][:d] for i in idx], np.int64).reshape(len(idx), d)
        out.append(dict(cols=np.stack([cc, cs]), rows=np.stack([rc, rs]),
                        wc=np.array([1, 1j]), wr=np.array([1, 1j]), modes=modes, dact=1))
    for keys, rows, cols, wr, wc in S._zbuckets:
        modes = np.array([[g.index for g in S.slots[i].group][:d] for i, _ in keys], np.int64)
        out.append(dict(cols=cols, rows=rows, wc=np.asarray(wr), wr=np.asarray(wr), modes=modes,
                        dact=int(np.log2(len(wr)))))
    return out


def gather_rows(vec, mp):
    return sum(w * vec[r] for w, r in zip(mp["wr"], mp["rows"]))


def gather_state(vec, mp):
    return sum(w * vec[c] for w, c in zip(mp["wc"], mp["cols"]))


def scatter_state(C_list, maps, n_real):
    """Mode layout -> the reference's real global vector (sum over the sign views)."""
    X = np.zeros(n_real)
    for C, mp in zip(C_list, maps):
        scale = 2.0 ** max(mp["dact"] - 1, 0)
        for w, c in zip(mp["wc"], mp["cols"]):
            np.add.at(X, c.ravel(), (np.conj(w) / scale * C).real.ravel())
    return X
