"""Oracle (test infrastructure only): times the reference's own CPU IMEX path on a benchmark
configuration, with its own compiled bordered-banded solver.

    CONATUS_REFERENCE=<tree> python -m oracle.time_reference --config channel [--steps 4] [--threads 8]

The reference package (``<tree>/python``) is imported read-only; ``conatus._core`` is the
reference's ``core/include/conatus/banded.hpp`` compiled unmodified by ``oracle/Makefile``
(``oracle.ref.install_compiled_core``), so the batched solves are the reference's C++ solves,
threaded over systems as its bindings thread them (``CONATUS_SOLVE_THREADS``), and its transforms
run on ``CN_FFT_WORKERS`` scipy.fft threads. The solver is ``Model.simulate(...)`` with the
configuration's resolution, scheme and step (python/conatus/model/model.py:912-935,
model/run.py:116-144); ``f_backend`` is the reference's default evaluator and its fused
polynomial form, the faster one reported, as in the reference's own GPU table
(docs/site/guide/benchmarks.md:271-275). Steps are timed one by one (median reported) after
warm-up steps that make the factorizations: the lower-order start-up takes one per order, so an
SBDF-q run warms up q steps (examples/benchmarks/cases.py:27-43 warms up before timing). Prints one
JSON line.

This is the measurement behind the CPU baseline that the port (oracle/ivp.py) is compared with.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CONFIGS = {
    "channel": dict(N=(192, 129, 192), scheme="SBDF3", dt=5e-3),
    "rayleigh_benard": dict(N=(256, 64), scheme="SBDF2", dt=1e-4),
    "burgers": dict(N=128, scheme="SBDF2", dt=1e-4),
}


def model(cn, config):
    if config == "channel":
        from conatus.problems import native
        return native.channel(Lx=4 * np.pi, Lz=2 * np.pi, Re=4000.0, pressure_gradient=2 / 4000.0)
    if config == "rayleigh_benard":
        m = cn.Model(cn.Box(x=cn.periodic(2 * np.pi / 3.117), z=cn.walls(0, 1)), name="RB",
                     Ra=1e6, Pr=1.0)
        m.velocity("u")
        m.pressure("p")
        m.scalar("T")
        m.equations("dt(u) + grad(p) - Pr*lap(u) = Pr*Ra*T*ez - u@grad(u)", "div(u) = 0",
                    "dt(T) - lap(T) = -u@grad(T)")
        m.at("bottom", u=0, T=1)
        m.at("top", u=0, T=0)
        return m
    m = cn.Model(cn.Box(x=cn.walls(-1, 1)), name="Burgers", nu=0.01 / np.pi)
    m.scalar("u")
    m.equations("dt(u) - nu*lap(u) = -u*dx(u)")
    m.at("walls", u=0)
    return m


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CONATUS_REFERENCE"),
                    help="the reference source tree (or set CONATUS_REFERENCE)")
    ap.add_argument("--config", default="channel", choices=list(CONFIGS))
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--threads", type=int, default=len(os.sched_getaffinity(0)))
    ap.add_argument("--f-backend", default="both", choices=["both", "evaluator", "fused"])
    ap.add_argument("--fourier", type=int, nargs="*", default=None,
                    help="Fourier sizes instead of the configuration's (the channel's CPU run at 192 x 192 "
                         "needs more host memory than 64 GB)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("the reference source tree is needed: pass --ref or set CONATUS_REFERENCE")
    os.environ["CONATUS_SOLVE_THREADS"] = str(args.threads)
    os.environ["CN_FFT_WORKERS"] = str(args.threads)
    sys.path.insert(0, os.path.join(args.ref, "python"))
    sys.path.insert(0, ROOT)
    from oracle.ref import install_compiled_core
    install_compiled_core()
    import conatus as cn
    cfg = dict(CONFIGS[args.config])
    if args.fourier:
        N = list(cfg["N"]) if isinstance(cfg["N"], tuple) else [cfg["N"]]
        if args.config == "channel":
            N[0], N[2] = args.fourier[0], args.fourier[-1]
        elif args.config == "rayleigh_benard":
            N[0] = args.fourier[0]
        cfg["N"] = tuple(N) if len(N) > 1 else N[0]
    backends = ["evaluator", "fused"] if args.f_backend == "both" else [args.f_backend]
    res = {}
    for fb in backends:
        t0 = time.perf_counter()
        sim = model(cn, args.config).simulate(f_backend=fb, **cfg)
        t_setup = time.perf_counter() - t0
        X = sim.solver.X
        rng = np.random.default_rng(0)
        sim.solver.X = X + 1e-3 * rng.standard_normal(X.shape)       # a generic state
        # the lower-order start-up: one factorization per order (SBDF1, 2, .. q); the steady steps
        # after it reuse the last one
        order = int(cfg["scheme"][-1])
        t0 = time.perf_counter()
        sim.run(steps=order)
        t_first = time.perf_counter() - t0
        per = []
        for _ in range(args.steps):
            t1 = time.perf_counter()
            sim.run(steps=1)
            per.append(time.perf_counter() - t1)
        res[fb] = dict(setup_s=t_setup, first_step_s=t_first, s_per_step=float(np.median(per)),
                       per_step=per, finite=bool(np.all(np.isfinite(sim.solver.X))))
        del sim
    best = min(res, key=lambda k: res[k]["s_per_step"])
    out = dict(config=args.config, build=cfg, threads=args.threads, unknowns=None,
               steps_per_s=1.0 / res[best]["s_per_step"], f_backend=best, runs=res,
               host=os.uname().machine, cores=len(os.sched_getaffinity(0)))
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
