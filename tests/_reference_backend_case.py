"""Cases of the reference's own scripts run through ``conatus_gb300.install()`` (driven by
tests/test_reference_backend*.py in a fresh interpreter each: installing patches the reference
package). Usage: python _reference_backend_case.py REFERENCE_PYTHON CASE; prints one JSON line."""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def burgers(cn):
    m = cn.Model(cn.Box(x=cn.walls(-1, 1)), name="Burgers", nu=0.01 / np.pi)
    m.scalar("u")
    m.equations("dt(u) - nu*lap(u) = -u*dx(u)")
    m.at("walls", u=0)
    return m


def rayleigh_benard(cn, Ra=1e6):
    m = cn.Model(cn.Box(x=cn.periodic(2 * np.pi / 3.117), z=cn.walls(0, 1)), name="RB", Ra=Ra, Pr=1.0)
    m.velocity("u")
    m.pressure("p")
    m.scalar("T")
    m.equations("dt(u) + grad(p) - Pr*lap(u) = Pr*Ra*T*ez - u@grad(u)", "div(u) = 0",
                "dt(T) - lap(T) = -u@grad(T)")
    m.at("bottom", u=0, T=1)
    m.at("top", u=0, T=0)
    return m


def channel(cn):
    from conatus.problems import native
    return native.channel(Lx=4 * np.pi, Lz=2 * np.pi, Re=4000.0, pressure_gradient=2 / 4000.0)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def main():
    refpy, case = sys.argv[1], sys.argv[2]
    sys.path.insert(0, refpy)
    sys.path.insert(0, ROOT)
    out = {"case": case}
    if case == "cpu_routing":
        # no GPU: the oracle core serves the reference's CPU path; backend="cuda" reaches this
        # package (and stops at the missing device), backend="cpu" stays the reference's
        from oracle.banded import install_as_reference_core
        install_as_reference_core()
        import conatus_gb300
        cn = conatus_gb300.install()
        from conatus_gb300.errors import CudaError
        from conatus_gb300.reference_backend import GB300IVPSolver, _scatter
        from conatus_gb300.reference_adapter import gather_rows, gather_state, reference_maps
        sim = channel(cn).simulate(N=(8, 17, 8), scheme="SBDF3", dt=5e-3)
        out["cpu_solver"] = type(sim.solver).__name__
        sim.run(steps=2)
        out["cpu_steps"] = int(sim.solver.iteration)
        try:
            dev = channel(cn).simulate(N=(8, 17, 8), scheme="SBDF3", dt=5e-3, backend="cuda")
            out["cuda"] = "built " + type(dev.solver).__name__
        except CudaError as e:
            out["cuda"] = "CudaError: " + str(e)
        import torch
        out["cuda_device"] = bool(torch.cuda.is_available())
        # the layout maps of the route: state and right-hand side rows round trip exactly
        s = channel(cn).simulate(N=(8, 17, 8), scheme="SBDF3", dt=5e-3, complexify=True,
                                 f_backend="fused").solver
        maps = reference_maps(s)
        rng = np.random.default_rng(0)
        X = rng.standard_normal(s.system.n)
        C = [gather_state(X, m) for m in maps]
        out["state_roundtrip"] = rel(_scatter(C, maps, s.system.n, "cols"), X)
        R = [gather_rows(X, m) for m in maps]
        out["rows_roundtrip"] = rel(_scatter(R, maps, s.system.n, "rows"), X)
        out["is_gb300_class"] = GB300IVPSolver.__name__
    elif case in ("burgers", "burgers_fp32"):
        import conatus_gb300
        cn = conatus_gb300.install("fp32" if case.endswith("fp32") else "fp64")
        sim = burgers(cn).simulate(N=128, scheme="SBDF2", dt=1e-4, backend="cuda")
        out["solver"] = type(sim.solver).__name__
        sim.initial(u=lambda x: -np.sin(np.pi * x))
        u0 = sim.coeffs("u")
        if case.endswith("fp32"):                     # the run reports its error against FP64
            sim.solver.monitor_fp64(every=250)
        sim.run(steps=1000)
        out["t"], out["iteration"] = float(sim.t), int(sim.solver.iteration)
        out["u1000"] = sim.coeffs("u").tolist()
        if case.endswith("fp32"):
            out["mixed_error"] = {str(k): v for k, v in sim.solver.mixed_error.items()}
        # the reference's own CPU path on the same script, its banded solves on this package's
        # GPU core (conatus._core = conatus_gb300.core)
        cpu = burgers(cn).simulate(N=128, scheme="SBDF2", dt=1e-4)
        cpu.initial(u=lambda x: -np.sin(np.pi * x))
        out["u0_same"] = rel(cpu.coeffs("u"), u0)
        cpu.run(steps=1000)
        out["cpu_core"] = type(sys.modules["conatus._core"]).__name__ + ":" + sys.modules["conatus._core"].__name__
        out["dev_vs_cpu"] = rel(out["u1000"], cpu.coeffs("u"))
    elif case == "channel":
        import conatus_gb300
        cn = conatus_gb300.install()
        from conatus_gb300 import workloads as W
        sim = channel(cn).simulate(N=(8, 17, 8), scheme="SBDF3", dt=5e-3, backend="cuda")
        cpu = channel(cn).simulate(N=(8, 17, 8), scheme="SBDF3", dt=5e-3, complexify=True,
                                   f_backend="fused")
        P = sim.solver.template.instantiate()
        X0 = sim.solver._real(W.channel_state(P, seed=2))
        sim.solver.X = X0
        cpu.solver.X = X0.copy()
        sim.run(steps=20)
        cpu.run(steps=20)
        out["fields"] = {v: rel(sim.coeffs(v), cpu.coeffs(v)) for v in ("u", "p")}
        # checkpoints in the reference's format: GB300 -> reference and reference -> GB300
        path = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"ck_{os.getpid()}.npz")
        sim.solver.save_checkpoint(path)
        cpu2 = channel(cn).simulate(N=(8, 17, 8), scheme="SBDF3", dt=5e-3, complexify=True,
                                    f_backend="fused")
        cpu2.solver.load_checkpoint(path)
        sim.run(steps=10)
        cpu2.run(steps=10)
        out["after_restart"] = {v: rel(sim.coeffs(v), cpu2.coeffs(v)) for v in ("u", "p")}
        cpu.solver.save_checkpoint(path)
        dev2 = channel(cn).simulate(N=(8, 17, 8), scheme="SBDF3", dt=5e-3, backend="cuda")
        dev2.solver.load_checkpoint(path)
        cpu.run(steps=10)
        dev2.run(steps=10)
        out["restart_from_reference"] = {v: rel(dev2.coeffs(v), cpu.coeffs(v)) for v in ("u", "p")}
        out["clock"] = [float(dev2.t), int(dev2.solver.iteration), float(cpu.t), int(cpu.solver.iteration)]
        os.remove(path)
    elif case == "blowup":
        import conatus_gb300
        cn = conatus_gb300.install()
        from conatus.errors import NumericalError
        from conatus_gb300 import workloads as W
        sim = rayleigh_benard(cn).simulate(N=(256, 64), scheme="SBDF2", dt=1e-4, backend="cuda")
        P = sim.solver.template.instantiate()
        sim.solver.X = sim.solver._real(W.rayleigh_benard_state(P, seed=0))
        try:
            sim.run(steps=300)
            out["raised"] = None
        except NumericalError as e:
            out["raised"] = str(e)
        out["iteration"] = int(sim.solver.iteration)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
