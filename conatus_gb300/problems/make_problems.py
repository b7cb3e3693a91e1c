"""Generate the problem templates of this directory from the reference (run where it is importable).

    python -m conatus_gb300.problems.make_problems [--ref /root/reference] [--only NAME]

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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden as mg
    cn = mg.import_reference(args.ref)
    from conatus_gb300.reference_adapter import template_from_solver
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
