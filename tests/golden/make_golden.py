"""Generate the golden fixtures of tests/golden/ from the reference (run where it is importable).

    python tests/golden/make_golden.py [--ref /root/reference]

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
# problems of the benchmark configurations (BASELINE configs, small resolutions for fixtures)

def burgers(cn, N=128):
    m = cn.Model(cn.Box(x=cn.walls(-1, 1)), name="Burgers", nu=0.01 / np.pi)
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
            labels.append(f"{label}|n={n}|r={nb}|kl={info['kl']}|ku={info['ku']}")
        arrays["labels"] = np.array(labels)
        np.savez_compressed(os.path.join(out_dir, f"banded_{name}.npz"), **arrays)
        print(name, labels)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    cn = import_reference(args.ref)
    rng = np.random.default_rng(20261203)
    if args.only in ("", "banded"):
        banded_fixtures(cn, HERE, rng)


if __name__ == "__main__":
    main()
