"""The reference's own entry points on the GB300 step: ``install()`` makes ``backend="cuda"`` of
``Model.simulate`` / ``Simulation`` / ``IVPSolver`` run the whole IMEX step here.

The reference selects its GPU path by ``backend="cuda"`` (python/conatus/model/model.py:912-935,
model/run.py:116-144, timestep/integrator.py:161-218); that path needs CuPy, which neither the GPU
host nor this container has. ``install()`` (before or after ``import conatus``):

* inserts ``conatus_gb300.core`` as ``conatus._core`` when no core is loaded yet, so the reference
  imports, and its CPU path's bordered-banded solves run on the GPU (the nanobind surface of
  core/bindings/module.cpp);
* adds one dispatcher to ``IVPSolver.__new__``, the hook the reference itself uses to send polar
  and spherical plans to their solvers (timestep/polar.py:495-502, timestep/sphere.py:353-363):
  ``IVPSolver(plan, scheme, dt, backend="cuda", ...)`` on a RealFourier x Chebyshev plan returns a
  :class:`GB300IVPSolver`, with the public surface ``Simulation`` uses (``set_state``, ``run``,
  ``step``, ``run_graph``, ``t``, ``iteration``, ``X``, ``coeffs``, ``grid``,
  ``save_checkpoint``, ``load_checkpoint``, ``explain``).

A script written for the reference then runs unchanged after ``import conatus_gb300;
conatus_gb300.install()``: ``m.simulate(N=..., scheme=..., dt=..., backend="cuda")`` and
``sim.run(steps=n)``. The set-up is the reference's own: its CPU solver is built with
``complexify=True`` and ``f_backend="fused"`` (exact reformulations the reference offers, the same
numbers), its discretization becomes a template with the reference's own M and L values
(``reference_adapter.template_from_solver(..., exact_values=True)``), and every step runs on the
device (``conatus_gb300.ivp.IVPSolver``). State, history and clock move between the two layouts
only when the caller reads or writes them. What the device path does not cover is refused, never
run on the CPU instead: ``decouple=True``, a time-dependent right-hand side
(``time_parameter``), bases other than RealFourier x one Chebyshev axis, complex monomial
coefficients, monomials of more than four factors, ``run(record=..., cache=...)``.
"""
from __future__ import annotations

import sys
from collections import deque

import numpy as np

__all__ = ["install", "GB300IVPSolver"]

_STATE = {"precision": "fp64", "installed": False}


def install(precision: str = "fp64"):
    """Route the reference's ``backend="cuda"`` to the GB300 step (see module docstring).
    ``precision``: "fp64" (the plain drop-in) or "fp32" (FP32 transforms, products and solves with
    FP64 refinement, state and history). Returns the reference package."""
    if precision not in ("fp64", "fp32"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    _STATE["precision"] = precision
    if "conatus._core" not in sys.modules:
        from . import core
        core.install()
    import conatus
    from conatus.timestep.integrator import IVPSolver
    if not _STATE["installed"]:
        prev = IVPSolver.__new__

        def _dispatch_new(cls, plan=None, *args, **kwargs):
            if cls is IVPSolver and kwargs.get("backend") == "cuda" and _cartesian(plan):
                return GB300IVPSolver(IVPSolver, plan, *args, **kwargs)
            return prev(cls, plan, *args, **kwargs)

        IVPSolver.__new__ = _dispatch_new
        _STATE["installed"] = True
    return conatus


def _cartesian(plan) -> bool:
    """A RealFourier x Chebyshev plan (what the device path covers); polar and spherical plans keep
    the reference's own dispatch."""
    if plan is None or getattr(plan, "is_polar", False) or getattr(plan, "is_sphere", False):
        return False
    from conatus.ir.bases import Chebyshev, RealFourier
    dom = plan.domain
    return all(isinstance(dom.basis(c), (Chebyshev, RealFourier)) for c in dom.coordsys.coords)


def _scatter(C_list, maps, n_real, key):
    """Mode layout -> the reference's real global vector (state: key "cols"; right-hand side rows:
    key "rows"), the inverse of the gather maps."""
    X = np.zeros(n_real)
    for C, mp in zip(C_list, maps):
        scale = 2.0 ** max(mp["dact"] - 1, 0)
        w = mp["wc"] if key == "cols" else mp["wr"]
        for wp, idx in zip(w, mp[key]):
            np.add.at(X, idx.ravel(), (np.conj(wp) / scale * np.asarray(C)).real.ravel())
    return X


class GB300IVPSolver:
    """``IVPSolver(plan, scheme, dt, backend="cuda", ...)`` after ``install()``: the reference's
    discretization, every step on the device (see module docstring)."""

    backend = "cuda"

    def __init__(self, ref_cls, plan, scheme, dt, *, reduced=None, ordering="interleaved",
                 startup="lower_order", startup_substeps=2, time_parameter=None, backend="cuda",
                 f_backend="evaluator", complexify=False, decouple=False, bc_time="auto",
                 check_finite=True):
        from .ivp import IVPSolver
        from .reference_adapter import reference_maps, template_from_solver
        if decouple:
            raise NotImplementedError("GB300 backend: decouple=True (a block split the device "
                                      "layout does not hold); use the default decouple=False")
        if time_parameter:
            raise NotImplementedError("GB300 backend: a time-dependent right-hand side "
                                      "(time_parameter) is not compiled to the device")
        if startup != "lower_order":
            raise NotImplementedError("GB300 backend: startup='lower_order' only")
        # the reference's own set-up (discretization, conversions, the fused polynomial F), on the
        # CPU, in the complexified layout (complexify=True, f_backend="fused": the reference's exact
        # reformulations; complexify / f_backend as given are accepted and replaced)
        self._host = ref_cls(plan, scheme, dt, reduced=reduced, ordering=ordering, startup=startup,
                             startup_substeps=startup_substeps, backend="cpu", f_backend="fused",
                             complexify=True, decouple=False, bc_time=bc_time, check_finite=check_finite)
        self.plan, self.scheme, self.dt = plan, scheme, float(dt)
        self.requested = dict(f_backend=f_backend, complexify=complexify)
        name = getattr(getattr(plan, "problem", None), "name", None) or "reference"
        self.template = template_from_solver(self._host, str(name), params=dict(plan.params),
                                             exact_values=True)
        self._maps = reference_maps(self._host)
        self._n = int(self._host.system.n)
        self._dtype = self._host.system.dtype
        P = self.template.instantiate()
        self.precision = _STATE["precision"]
        self._gpu = IVPSolver(P, scheme=scheme, dt=dt, precision=self.precision, check_finite=check_finite)
        self._gpu.set_state(self._modes(np.asarray(self._host.X)))

    # ---- layouts
    def _modes(self, X):
        from .reference_adapter import gather_state
        X = np.asarray(X)
        return [gather_state(X, m).astype(np.complex128) for m in self._maps]

    def _rows(self, r):
        from .reference_adapter import gather_rows
        r = np.asarray(r)
        return [gather_rows(r, m).astype(np.complex128) for m in self._maps]

    def _real(self, C_list, key="cols"):
        return _scatter(C_list, self._maps, self._n, key).astype(self._dtype)

    # ---- state and clock
    @property
    def X(self):
        """The state in the reference's layout (a host copy of the device state)."""
        return self._real(self._gpu.state_to_host())

    @X.setter
    def X(self, value):
        """Overwrite the state (the multistep history is kept, as assigning the reference's X)."""
        dev = self._gpu.dev
        self._gpu.stream.synchronize()
        self._gpu.X.copy_(dev.to_device(self._modes(value)))
        self._gpu._reset_finite()
        if self._gpu._shadow is not None:             # the FP64 shadow of monitor_fp64 follows
            self._gpu._shadow.stream.synchronize()
            self._gpu._shadow.X.copy_(self._gpu.X)
            self._gpu._shadow._reset_finite()

    def monitor_fp64(self, every: int = 100, bound: float = 1e-6) -> None:
        """The FP32 form (``install(precision="fp32")``): record the run's per-field error against
        an FP64 shadow every ``every`` steps and at the end of every call, in ``mixed_error``
        (``conatus_gb300.ivp.IVPSolver.monitor_fp64``). Call after ``set_state``, before stepping."""
        self._gpu.monitor_fp64(every, bound)

    mixed_error = property(lambda self: self._gpu.mixed_error)

    t = property(lambda self: self._gpu.t, lambda self, v: setattr(self._gpu, "t", float(v)))
    iteration = property(lambda self: self._gpu.iteration,
                         lambda self, v: setattr(self._gpu, "iteration", int(v)))

    def set_state(self, data, t: float = 0.0) -> None:
        """Initial condition, as the reference's ``set_state`` (integrator.py:262-276): the
        reference builds the state from the data, the device takes it; the history restarts."""
        self._host.set_state(data, t)
        self._gpu.set_state(self._modes(self._host.X), t=float(t))

    def coeffs(self, name: str) -> np.ndarray:
        self._host.X = self.X
        return self._host.coeffs(name)

    def grid(self, name: str) -> np.ndarray:
        self._host.X = self.X
        return self._host.grid(name)

    # ---- stepping (always on the device)
    def _numerical(self, err):
        from conatus.errors import NumericalError
        return NumericalError(str(err), where="IVPSolver.run (GB300 backend)",
                              why="the run has blown up (a numerical instability, or a physical one "
                                  "the resolution cannot follow)",
                              fix="reduce dt, raise the resolution N, or check the initial state")

    def step(self) -> None:
        self._gpu.step()

    def run(self, steps: int, callback=None, every: int | None = None, *, record=None, cache: bool = False):
        """``steps`` steps on the device (graph replays), ``callback(self)`` every ``every`` steps,
        the finite-state check every 100 steps and at the end (integrator.py:745-767)."""
        from .errors import NumericalError
        if record is not None or cache:
            raise NotImplementedError("GB300 backend: run(record=..., cache=...) (the run registry "
                                      "records the reference's CPU solver)")
        steps = self._host._run_arguments(steps, callback, every)
        try:
            if callback is None:
                self._gpu.run_graph(steps)
            else:
                done = 0
                while done < steps:
                    k = min(steps - done, every - self.iteration % every)
                    self._gpu.run_graph(k)
                    done += k
                    if self.iteration % every == 0:
                        callback(self)
        except NumericalError as err:
            raise self._numerical(err) from None
        return None

    def run_graph(self, steps: int, *args, **kwargs):
        return self.run(steps)

    # ---- checkpoints in the reference's own format (integrator.py:974-1161)
    def _to_host(self):
        g = self._gpu
        meta, arrays = g.checkpoint_payload()
        h = self._host
        h.X = self._real(_split(arrays["X"], g))
        nh = int(meta["nhist"])
        h._MXh = deque(self._real(_split(arrays[f"MX{j}"], g), "rows") for j in range(nh))
        h._Fh = deque(self._real(_split(arrays[f"F{j}"], g), "rows") for j in range(nh))
        h._LXh = deque(self._real(_split(arrays[f"LX{j}"], g), "rows") for j in range(int(meta["nhist_LX"])))
        h.t, h.iteration = float(meta["t"]), int(meta["iteration"])

    def save_checkpoint(self, path, **kw):
        """The reference's checkpoint file (its ``save_checkpoint``): state, multistep history and
        clock mapped to its layout; a reference run restarts from it and the converse."""
        self._to_host()
        return self._host.save_checkpoint(path, **kw)

    def load_checkpoint(self, path, **kw) -> None:
        h = self._host
        h.load_checkpoint(path, **kw)
        g = self._gpu
        g.set_state(self._modes(h.X), t=float(h.t))
        if g.family != "rk" and len(h._MXh):
            dev = g.dev
            mx = [dev.to_device(self._rows(v)) for v in h._MXh]
            f = [dev.to_device(self._rows(v)) for v in h._Fh]
            lx = [dev.to_device(self._rows(v)) for v in h._LXh] if g.family == "cn" else None
            g.set_history(mx, f, lx)
        g.iteration = int(h.iteration)

    def explain(self) -> str:
        return (f"GB300 backend (conatus_gb300, {self.precision}): the reference's discretization "
                f"({len(self.template.buckets)} buckets, complexified, fused F), every step on the "
                f"device\n" + self._host.explain())

    def __getattr__(self, name):
        # the reference solver's other attributes (plan data, system layout, options), read with
        # the current state; the step itself never runs there
        if name.startswith("__") or name in ("_host", "_gpu"):
            raise AttributeError(name)
        if name in ("F", "flowmap", "_sbdf_step", "_cn_step", "rk_stages", "_capture_graph"):
            raise NotImplementedError(f"GB300 backend: IVPSolver.{name} is not available (the step "
                                      "runs on the device; read the state with X, coeffs or grid)")
        return getattr(self._host, name)


def _split(flat, g):
    """Per-bucket (nsys, n) arrays of a flat mode-layout vector of solver ``g``."""
    dev = g.dev
    return [flat[o:o + ns * b.n].reshape(ns, b.n) for o, ns, b in zip(dev.offsets, dev.nsys, dev.tpl.buckets)]
