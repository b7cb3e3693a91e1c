"""Generate the golden fixtures of tests/golden/ from the reference (run where it is importable).

    python tests/golden/make_golden.py --ref REFERENCE_TREE

The reference tree is given by ``--ref`` or the environment variable ``CONATUS_REFERENCE``;
there is no default.

Banded fixtures (``banded_<case>.npz``): the bucket matrices a M + b L that the reference's
``GlobalSystem.factor`` builds for the problems of the benchmark configurations (at small
resolutions), seeded right-hand sides, and the solutions computed by the reference's own C++
``BorderedBanded`` (core/include/conatus/banded.hpp, compiled unmodified by oracle/Makefile),
forward and transposed.

The reference package is imported read-only with the oracle restatement of the banded solver
installed as ``conatus._core`` (the loader accepts a preloaded module,
python/conatus/runtime/__init__.py:55-59); the solutions themselves come from the compiled
reference core.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def import_reference(ref: str):
    sys.path.insert(0, os.path.join(ref, "python"))
    sys.path.insert(0, ROOT)
    from oracle.banded import install_as_reference_core
    install_as_reference_core()
    import conatus as cn
    return cn


# ------------------------------------------------------------------------------------------------
# problems of the benchmark configurations (small resolutions for the fixtures)

def burgers(cn, N=128, nu=0.01 / np.pi):
    m = cn.Model(cn.Box(x=cn.walls(-1, 1)), name="Burgers", nu=nu)
    m.scalar("u")
    m.equations("dt(u) - nu*lap(u) = -u*dx(u)")
    m.at("walls", u=0)
    return m


def rayleigh_benard(cn, Ra=1e6, Pr=1.0):
    m = cn.Model(cn.Box(x=cn.periodic(2 * np.pi / 3.117), z=cn.walls(0, 1)), name="RB",
                 Ra=Ra, Pr=Pr)
    m.velocity("u")
    m.pressure("p")
    m.scalar("T")
    m.equations("dt(u) + grad(p) - Pr*lap(u) = Pr*Ra*T*ez - u@grad(u)", "div(u) = 0",
                "dt(T) - lap(T) = -u@grad(T)")
    m.at("bottom", u=0, T=1)
    m.at("top", u=0, T=0)
    return m


def channel(cn, Re=4000.0):
    from conatus.problems import native
    return native.channel(Lx=4 * np.pi, Lz=2 * np.pi, Re=Re, pressure_gradient=2 / Re)


def kuramoto_sivashinsky(cn, L=22.0):
    from conatus.problems import native
    return native.kuramoto_sivashinsky(L=L)


# ------------------------------------------------------------------------------------------------

def _bucket_mats(system, a, b):
    """[(label, dtype, border count, [csr matrices])] of every solver bucket (real, complexified,
    complex-mode), exactly as GlobalSystem.factor assembles them (system.py:729-783)."""
    out = []
    for idx, _, _ in system._buckets:
        mats = []
        for i in idx:
            s = system.slots[i]
            A = (a * s.M + b * s.L).tocsr()[s.rperm][:, s.cperm].astype(system.dtype)
            mats.append(A)
        out.append((system.slots[idx[0]].label, np.dtype(system.dtype), system.slots[idx[0]].n_border, mats))
    for idx, *_ in system._cbuckets:
        czs = [system.slots[i].cz for i in idx]
        mats = [(a * cz.M + b * cz.L).tocsr()[cz.rperm][:, cz.cperm].astype(np.complex128) for cz in czs]
        out.append((system.slots[idx[0]].label + " (complex)", np.dtype(np.complex128), czs[0].n_border, mats))
    for keys, *_ in system._zbuckets:
        vs = [system.slots[i].zs[vi] for i, vi in keys]
        mats = [(a * v.M + b * v.L).tocsr()[v.rperm][:, v.cperm].astype(np.complex128) for v in vs]
        for A in mats:
            A.sort_indices()
        sgn = "".join("+" if t > 0 else "-" for t in vs[0].s)
        out.append((system.slots[keys[0][0]].label + f" (complex, s={sgn})", np.dtype(np.complex128),
                    vs[0].n_border, mats))
    return out


def banded_fixtures(cn, out_dir, rng):
    from oracle import ref
    cases = [
        ("burgers128", burgers(cn), dict(N=128, scheme="SBDF2", dt=1e-4), 1.5 / 1e-4),
        ("rb32x16", rayleigh_benard(cn), dict(N=(32, 16), scheme="SBDF2", dt=1e-4, complexify=True), 1.5 / 1e-4),
        ("channel8x17x8", channel(cn), dict(N=(8, 17, 8), scheme="SBDF3", dt=5e-3, complexify=True),
         (11 / 6) / 5e-3),
    ]
    for name, model, kw, a in cases:
        sim = model.simulate(**kw)
        system = sim.solver.system
        arrays = {}
        labels = []
        for bi, (label, dtype, nb, mats) in enumerate(_bucket_mats(system, a, 1.0)):
            mats = mats[:6]
            csr = [(A.shape[0], A.indptr.astype(np.int32), A.indices.astype(np.int32),
                    A.data.astype(dtype)) for A in mats]
            border = list(range(nb))
            R = ref.RefBatch(csr, border, dtype)
            n = csr[0][0]
            b = rng.standard_normal((len(csr), n))
            if dtype.kind == "c":
                b = b + 1j * rng.standard_normal((len(csr), n))
            x = R.solve(b)
            xt = R.solve(b, transpose=True)
            info = R.info(0)
            p = f"b{bi}_"
            arrays[p + "indptr"] = np.stack([c[1] for c in csr])
            arrays[p + "indices"] = np.concatenate([c[2] for c in csr])
            arrays[p + "data"] = np.concatenate([c[3] for c in csr])
            arrays[p + "nnz"] = np.array([len(c[3]) for c in csr], np.int64)
            arrays[p + "border"] = np.array(border, np.int32)
            arrays[p + "rhs"] = b
            arrays[p + "x"] = x
            arrays[p + "xt"] = xt
            arrays[p + "band"] = np.array([info["kl"], info["ku"]], np.int32)
            arrays[p + "cond"] = np.array([np.linalg.cond(A.toarray()) for A in mats])
            labels.append(f"{label}|n={n}|r={nb}|kl={info['kl']}|ku={info['ku']}")
        arrays["labels"] = np.array(labels)
        np.savez_compressed(os.path.join(out_dir, f"banded_{name}.npz"), **arrays)
        print(name, labels)


def step_fixtures(cn, out_dir, rng):
    """Step fixtures (``step_<case>.npz``): the reference's IVPSolver (fused F, complexify=True)
    from a seeded smooth state, a few start-up steps to fill the SBDF history, then one recorded
    step: X_n, the M X and F history, F(X_n) and X_{n+1} (reference real layout), with the maps
    between that layout and the mode layout of the problem template, and the reference's own M, L
    values. ``Xn1_perturbed``: the reference's X_{n+1} from X_n perturbed by about one ulp (three
    seeds) -- the spread of the reference's own arithmetic, the floor below which two correct
    FP64 implementations cannot be told apart."""
    from conatus_gb300.problems import make_problems as mp
    from conatus_gb300.reference_adapter import reference_maps, scatter_state, template_from_solver
    cases = [("burgers128", "burgers_n128"), ("rb32x16", "rb_nz16_32"), ("channel8x17x8", "channel_ny17_8"),
             ("ks64", "ks")]
    builds = {
        "burgers128": ("burgers", dict(N=128, scheme="SBDF2", dt=1e-4), {}),
        "rb32x16": ("rayleigh_benard", dict(N=(32, 16), scheme="SBDF2", dt=1e-4), dict(Ra=1e6, Pr=1.0)),
        "channel8x17x8": ("channel", dict(N=(8, 17, 8), scheme="SBDF3", dt=5e-3), dict(Re=4000.0)),
        "ks64": ("kuramoto_sivashinsky", dict(N=64, scheme="SBDF2", dt=1e-2), dict(L=37.0)),
    }
    for name, _ in cases:
        fn, kw, params = builds[name]
        sim = globals()[fn](cn, **params).simulate(complexify=True, f_backend="fused", **kw)
        s = sim.solver
        tpl = template_from_solver(s, name, params=params, exact_values=True)
        maps = reference_maps(s)
        P = tpl.instantiate()
        # seeded smooth state in the mode layout: decay with the Chebyshev index
        C = []
        for bi, b in enumerate(tpl.buckets):
            n_idx = np.maximum(b.col[:, 2], 0)
            amp = 0.05 * np.exp(-0.35 * n_idx)
            z = rng.standard_normal((P.nsys[bi], b.n)) + (0 if b.kind == "real" else 1j) * rng.standard_normal((P.nsys[bi], b.n))
            C.append(z * amp)
        X0 = scatter_state(C, maps, s.system.n)
        s.X = X0.astype(s.system.dtype)
        s.t, s.iteration = 0.0, 0
        s._reset_history()
        for _ in range(3):
            s.step()
        Xn = np.array(s.X)
        MXh = [np.array(v) for v in s._MXh]
        Fh = [np.array(v) for v in s._Fh]
        Fn = np.array(s.F(s.X, s.t))
        state = (np.array(s.X), s.t, s.iteration, list(s._MXh), list(s._Fh))
        s.step()
        Xn1 = np.array(s.X)
        MXn = np.array(s._MXh[0])             # the step pushed M X_n on its history
        # the reference's own rounding floor: the same step from X_n perturbed by ~1 ulp
        floors = []
        for trial in range(3):
            s.X = state[0] * (1 + 2.0 ** -52 * rng.standard_normal(state[0].shape))
            s.t, s.iteration = state[1], state[2]
            s._MXh.clear(); s._MXh.extend(state[3])
            s._Fh.clear(); s._Fh.extend(state[4])
            s.step()
            floors.append(np.array(s.X))
        arrays = dict(Xn=Xn, Xn1=Xn1, Fn=Fn, MXn=MXn, MXh=np.stack(MXh), Fh=np.stack(Fh), dt=kw["dt"],
                      order=int(kw["scheme"][-1]), nb=len(maps), Xn1_perturbed=np.stack(floors))
        for bi, m in enumerate(maps):
            p = f"m{bi}_"
            arrays[p + "cols"] = m["cols"].astype(np.int32)
            arrays[p + "rows"] = m["rows"].astype(np.int32)
            arrays[p + "wc"] = m["wc"]
            arrays[p + "wr"] = m["wr"]
            arrays[p + "dact"] = m["dact"]
            arrays[p + "Mv"], arrays[p + "Lv"] = tpl.buckets[bi].exact
        np.savez_compressed(os.path.join(out_dir, f"step_{name}.npz"), **arrays)
        print(name, "N_u", s.system.n, "history", len(MXh))


SCHEME_CASES = {
    # case -> (model, build kwargs (without the scheme), parameters, schemes)
    "rb32x16": ("rayleigh_benard", dict(N=(32, 16), dt=1e-4), dict(Ra=1e6, Pr=1.0),
                ("RK443", "RK222", "CNAB2", "MCNAB2", "CNLF2")),
    "burgers128": ("burgers", dict(N=128, dt=1e-4), {}, ("RK111", "RKSMR", "RKGFY", "CNAB1")),
    "channel8x17x8": ("channel", dict(N=(8, 17, 8), dt=5e-3), dict(Re=4000.0), ("RK443", "CNAB2")),
}


def scheme_fixtures(cn, out_dir, rng, steps=3):
    """Scheme fixtures (``scheme_<case>_<scheme>.npz``): the reference's IVPSolver with an IMEX
    Runge-Kutta or CN-family scheme (start-up ``lower_order``) from a seeded smooth state: X_0 and
    the states after each of ``steps`` steps (reference real layout), the maps to the mode layout and
    the reference's M, L values; ``Xs_perturbed``: the same steps from X_0 perturbed by about one
    ulp (three seeds), the reference's own rounding floor."""
    from conatus_gb300.reference_adapter import reference_maps, scatter_state, template_from_solver
    for name, (fn, kw, params, schemes) in SCHEME_CASES.items():
        for scheme in schemes:
            sim = globals()[fn](cn, **params).simulate(complexify=True, f_backend="fused", scheme=scheme, **kw)
            s = sim.solver
            tpl = template_from_solver(s, name, params=params, exact_values=True)
            maps = reference_maps(s)
            P = tpl.instantiate()
            C = []
            for bi, b in enumerate(tpl.buckets):
                n_idx = np.maximum(b.col[:, 2], 0)
                amp = 0.05 * np.exp(-0.35 * n_idx)
                z = rng.standard_normal((P.nsys[bi], b.n)) + (0 if b.kind == "real" else 1j) * rng.standard_normal((P.nsys[bi], b.n))
                C.append(z * amp)
            X0 = scatter_state(C, maps, s.system.n).astype(s.system.dtype)

            def run(x0):
                s.X = x0.copy()
                s.t, s.iteration = 0.0, 0
                s._reset_history()
                out = []
                for _ in range(steps):
                    s.step()
                    out.append(np.array(s.X))
                return np.stack(out)

            Xs = run(X0)
            pert = np.stack([run(X0 * (1 + 2.0 ** -52 * rng.standard_normal(X0.shape))) for _ in range(3)])
            arrays = dict(X0=X0, Xs=Xs, Xs_perturbed=pert, dt=kw["dt"], scheme=scheme, nb=len(maps))
            for bi, m in enumerate(maps):
                p = f"m{bi}_"
                arrays[p + "cols"] = m["cols"].astype(np.int32)
                arrays[p + "rows"] = m["rows"].astype(np.int32)
                arrays[p + "wc"] = m["wc"]
                arrays[p + "wr"] = m["wr"]
                arrays[p + "dact"] = m["dact"]
                arrays[p + "Mv"], arrays[p + "Lv"] = tpl.buckets[bi].exact
            np.savez_compressed(os.path.join(out_dir, f"scheme_{name}_{scheme}.npz"), **arrays)
            print(name, scheme, "N_u", s.system.n)


TRAJECTORY_CASES = {
    # case -> (model, build kwargs, parameters, committed template, template parameters, Fourier
    #          sizes, workload, recorded steps)
    "burgers128": ("burgers", dict(N=128, scheme="SBDF2", dt=1e-4), {}, "burgers_n128", None, None,
                   "burgers", (1000, 2500, 5000)),
    # the Rayleigh-Benard configuration (Ra = 1e6, dt = 1e-4) blows up in the reference itself
    # between steps 150 and 200 (convection sets in near t = 0.015 with velocities of order
    # sqrt(Ra) = 1e3, far beyond the advective limit of dt = 1e-4 on this grid): recorded up to step
    # 150; the configured length is run at Ra = 1e4, stable over the 2000 steps
    "rb256x64_ra1e6": ("rayleigh_benard", dict(N=(256, 64), scheme="SBDF2", dt=1e-4), dict(Ra=1e6, Pr=1.0),
                       "rb_nz64", None, [256], "rayleigh_benard", (50, 100, 150)),
    "rb256x64_ra1e4": ("rayleigh_benard", dict(N=(256, 64), scheme="SBDF2", dt=1e-4), dict(Ra=1e4, Pr=1.0),
                       "rb_nz64_ra", {"Ra": 1e4}, [256], "rayleigh_benard", (1000, 2000)),
    "channel16x17x16": ("channel", dict(N=(16, 17, 16), scheme="SBDF3", dt=5e-3), dict(Re=4000.0),
                        "channel_ny17", None, [16, 16], "channel", (100, 500)),
}


TRAJ_FLOOR = 1e-8      # a field's norm counts as at least this fraction of the state's norm


def field_spread(arrs, ref, floor=TRAJ_FLOOR):
    """Relative L2 difference per variable of coefficient arrays ``arrs`` against ``ref``, each
    field's norm taken at least ``floor`` times the norm of the whole state (the tau variables,
    zero up to rounding, are judged against the state)."""
    tot = sum(float(np.sum(np.asarray(r) ** 2)) for r in ref) ** 0.5
    return np.array([float(np.linalg.norm(np.asarray(a) - np.asarray(r))) /
                     max(float(np.linalg.norm(r)), floor * tot, 1e-300) for a, r in zip(arrs, ref)])


def trajectory_fixtures(cn, out_dir, seeds=2):
    """Trajectory fixtures (``traj_<case>.npz``): the reference's IVPSolver (fused F,
    complexify=True, start-up ``lower_order``) run over the configuration's whole length from the
    benchmark's initial state (``conatus_gb300.workloads``, mapped into the reference's layout), the
    state recorded at a few steps as the coefficient arrays of every variable (the layout-free form
    ``oracle.ivp.OracleProblem.to_arrays`` gives), so that a GPU run of the same length compares
    field by field with no teacher forcing. ``spread_s<step>``: per variable, the largest
    difference (``field_spread``) of the reference's own runs from the initial state perturbed by
    about one ulp (``seeds`` seeds): how far two correct FP64 runs drift apart by rounding alone."""
    import time
    sys.path.insert(0, ROOT)
    from conatus_gb300 import workloads as W
    from conatus_gb300.reference_adapter import gather_state, reference_maps, scatter_state
    from oracle.ivp import OracleProblem
    rng = np.random.default_rng(13)
    for name, (fn, kw, params, tname, tparams, sizes, wl, rec) in TRAJECTORY_CASES.items():
        t0 = time.time()
        sim = globals()[fn](cn, **params).simulate(complexify=True, f_backend="fused", **kw)
        s = sim.solver
        maps = reference_maps(s)
        P = W.load_template(tname).instantiate(sizes, params=tparams)
        for bi, (b, m) in enumerate(zip(P.tpl.buckets, maps)):
            if m["cols"].shape[-2:] != (P.nsys[bi], b.n) or not np.array_equal(m["modes"], P.modes[bi]):
                raise RuntimeError(f"{name}: bucket {bi} of the template does not match the reference build")
        C0 = W.initial_state(wl, P, seed=0)
        X0 = scatter_state(C0, maps, s.system.n).astype(s.system.dtype)
        op = OracleProblem(P)

        def run(x0):
            s.X = x0.copy()
            s.t, s.iteration = 0.0, 0
            s._reset_history()
            out, done = {}, 0
            for r in rec:
                s.run(r - done)
                done = r
                out[r] = op.to_arrays([gather_state(np.asarray(s.X), m) for m in maps])
            return out

        main = run(X0)
        spread = {r: np.zeros(len(P.tpl.variables)) for r in rec}
        for _ in range(seeds):
            pert = run(X0 * (1 + 2.0 ** -52 * rng.standard_normal(X0.shape)))
            for r in rec:
                spread[r] = np.maximum(spread[r], field_spread(pert[r], main[r]))
        arrays = dict(steps=np.array(rec, np.int64), dt=kw["dt"], scheme=kw["scheme"],
                      variables=np.array([v["name"] for v in P.tpl.variables]))
        for r in rec:
            for v, a in enumerate(main[r]):
                arrays[f"s{r}_v{v}"] = a
            arrays[f"spread_s{r}"] = spread[r]
        np.savez_compressed(os.path.join(out_dir, f"traj_{name}.npz"), **arrays)
        print(name, "steps", rec, "N_u", s.system.n, "spread", {r: np.round(np.log10(spread[r] + 1e-300), 1)
                                                               for r in rec}, f"{time.time() - t0:.1f} s")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CONATUS_REFERENCE"),
                    help="the reference source tree (or set CONATUS_REFERENCE)")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    if not args.ref:
        ap.error("the reference source tree is needed: pass --ref or set CONATUS_REFERENCE")
    cn = import_reference(args.ref)
    rng = np.random.default_rng(20261203)
    if args.only in ("", "banded"):
        banded_fixtures(cn, HERE, rng)
    if args.only in ("", "step"):
        step_fixtures(cn, HERE, np.random.default_rng(7))
    if args.only in ("", "scheme"):
        scheme_fixtures(cn, HERE, np.random.default_rng(11))
    if args.only in ("", "trajectory"):
        trajectory_fixtures(cn, HERE)


if __name__ == "__main__":
    main()
