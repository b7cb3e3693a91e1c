"""Generate the problem templates of this directory from the reference (run where it is importable).

    python -m conatus_gb300.problems.make_problems --ref REFERENCE_TREE [--only NAME]

The reference tree is given by ``--ref`` or the environment variable ``CONATUS_REFERENCE``;
there is no default.

Each template is the reference's own discretization of a benchmark model (``template_from_solver``
in conatus_gb300/reference_adapter.py), built with ``complexify=True`` and ``f_backend="fused"``.
A template is independent of the Fourier resolution, so a small Fourier build suffices; the
Chebyshev resolution and the parameters are those of the benchmark configuration:

* ``burgers_n128``: u_t + u u_x = nu u_xx, x in [-1, 1], u = 0 at the walls, nu = 0.01/pi, N = 128;
* ``rb_nz64`` (and ``rb_nz16`` for tests): 2D Rayleigh-Benard, x periodic of length 2 pi/3.117,
  z in [0, 1], no-slip isothermal walls (T = 1 bottom, 0 top), Ra = 1e6, Pr = 1;
* ``channel_ny129`` (and ``channel_ny17`` for tests): plane channel, Lx = 4 pi, Lz = 2 pi,
  y in [-1, 1], Re = 4000, driving pressure gradient 2/Re;
* ``ks``: Kuramoto-Sivashinsky u_t + u u_x + u_xx + u_xxxx = 0 (any period: the length is set
  when the template is instantiated).
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

SPECS = {
    "burgers_n128": ("burgers", dict(N=128, scheme="SBDF2", dt=1e-4), {}),
    "rb_nz16": ("rayleigh_benard", dict(N=(16, 16), scheme="SBDF2", dt=1e-4), dict(Ra=1e6, Pr=1.0)),
    "rb_nz64": ("rayleigh_benard", dict(N=(16, 64), scheme="SBDF2", dt=1e-4), dict(Ra=1e6, Pr=1.0)),
    "channel_ny17": ("channel", dict(N=(8, 17, 8), scheme="SBDF3", dt=5e-3), dict(Re=4000.0)),
    "channel_ny129": ("channel", dict(N=(8, 129, 8), scheme="SBDF3", dt=5e-3), dict(Re=4000.0)),
    "ks": ("kuramoto_sivashinsky", dict(N=16, scheme="SBDF2", dt=1e-2), dict(L=22.0)),
}
# serving mix: Burgers at N = 64, 96, .. 512 with L linear in nu; RB at Nz = 32 .. 96 with L linear in Ra
LINEAR = {}
for _n in range(64, 513, 32):
    LINEAR[f"burgers_n{_n}_nu"] = ("burgers", dict(N=_n, scheme="SBDF2", dt=1e-4), "nu", {})
for _nz in (32, 48, 64, 80, 96):
    LINEAR[f"rb_nz{_nz}_ra"] = ("rayleigh_benard", dict(N=(16, _nz), scheme="SBDF2", dt=1e-4), "Ra", dict(Pr=1.0))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CONATUS_REFERENCE"),
                    help="the reference source tree (or set CONATUS_REFERENCE)")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    if not args.ref:
        ap.error("the reference source tree is needed: pass --ref or set CONATUS_REFERENCE")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden as mg
    cn = mg.import_reference(args.ref)
    from conatus_gb300.reference_adapter import template_from_solver
    for name, (fn, kw, pname, fixed) in LINEAR.items():
        if args.only and name != args.only and args.only != "linear":
            continue
        t0 = time.time()
        # L(theta) = L(1) + (theta - 1) (L(2) - L(1)): the parameter's terms are linear in it, so
        # both differences are exact; the template stores L_0 = L(1) - dL and dL
        tps = []
        for val in (1.0, 2.0):
            model = getattr(mg, fn)(cn, **dict(fixed, **{pname: val}))
            sim = model.simulate(complexify=True, f_backend="fused", **kw)
            tps.append(template_from_solver(sim.solver, name, params=dict(fixed, **{pname: val})))
        t1, t2 = tps
        for b1, b2 in zip(t1.buckets, t2.buckets):
            if not (np.array_equal(b1.indices, b2.indices) and np.array_equal(b1.Mc, b2.Mc)):
                raise ValueError(f"{name}: M or the pattern depends on {pname}")
            b1.dL = {pname: b2.Lc - b1.Lc}
            b1.Lc = b1.Lc - b1.dL[pname]
        t1.linear_params = [pname]
        t1.params = dict(fixed, **{pname: 1.0})
        t1.source = dict(reference="conatus 0.5.0", model=fn, build=dict(kw, complexify=True),
                         linear=f"L({pname}) = L0 + {pname} dL")
        t1.save(os.path.join(HERE, f"{name}.npz"))
        print(f"{name}: {len(t1.buckets)} buckets, {time.time() - t0:.1f}s")
    if args.only == "linear":
        return
    for name, (fn, kw, params) in SPECS.items():
        if args.only and name != args.only:
            continue
        t0 = time.time()
        model = getattr(mg, fn)(cn, **params)
        sim = model.simulate(complexify=True, f_backend="fused", **kw)
        tpl = template_from_solver(sim.solver, name, params=params)
        tpl.source = dict(reference="conatus 0.5.0", model=fn, build=dict(kw, complexify=True))
        tpl.save(os.path.join(HERE, f"{name}.npz"))
        print(f"{name}: {len(tpl.buckets)} buckets, fit error "
              f"{max(b.fit_error for b in tpl.buckets):.1e}, {time.time() - t0:.1f}s")


if __name__ == "__main__":
    main()
