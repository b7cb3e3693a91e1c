"""Ensembles: many independent trajectories advanced together on the device.

``FourierEnsemble`` advances members of a one-dimensional periodic template (Kuramoto-Sivashinsky
for the benchmark) whose sizes N and periods L differ member to member, all in one kernel launch per
step (``cng_fourier_ensemble_step``: one CTA per member, the dealiased right-hand side, the SBDF
combination and the diagonal implicit solve fused), with the history ring in device memory and the
steady state of the loop replayed as CUDA graphs. The reference stacks ensemble members of one
discretization into batched solves (python/conatus/ensembles/ensemble.py:39-200,
ensembles/batched.py:442-613); it cannot mix sizes in one batch.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import call
from .ivp import SBDF, _stream_handle, _torch, smooth_size
from .template import ProblemTemplate

__all__ = ["FourierEnsemble", "ks_members"]


def ks_members(count: int, seed: int = 0, lmin: float = 22.0, lmax: float = 100.0):
    """Periods L ~ U[lmin, lmax] and sizes N = next power of two >= 2 L (the KS ensemble config)."""
    rng = np.random.default_rng(seed)
    L = rng.uniform(lmin, lmax, count)
    N = np.array([1 << int(math.ceil(math.log2(2 * x))) for x in L])
    return N, L


class FourierEnsemble:
    """Members of a one-dimensional periodic template advanced in one launch per step."""

    def __init__(self, tpl: ProblemTemplate, sizes, lengths, scheme: str = "SBDF2", dt: float = 0.01,
                 precision: str = "fp32"):
        torch = _torch()
        _lib.lib()
        if tpl.cheb_axis >= 0 or len(tpl.fourier_axes) != 1:
            raise ValueError("FourierEnsemble needs a template with one RealFourier axis only")
        if scheme not in SBDF and scheme not in ("SBDF1", "SBDF2", "SBDF3", "SBDF4"):
            raise ValueError(scheme)
        self.tpl = tpl
        self.order = int(scheme[-1])
        self.dt = float(dt)
        self.precision = precision
        self.N = np.asarray(sizes, dtype=np.int64)
        self.L = np.asarray(lengths, dtype=np.float64)
        if self.N.shape != self.L.shape or np.any(self.N % 2):
            raise ValueError("one even size and one period per member")
        self.nmem = len(self.N)
        dealias = tpl.axes[tpl.fourier_axes[0]].get("dealias", 1.5)
        self.M = np.array([smooth_size(int(math.floor(n * dealias))) for n in self.N])
        K = self.N // 2
        self.offsets = np.concatenate([[0], np.cumsum(K)[:-1]]).astype(np.int64)
        self.n_total = int(K.sum())
        plan_sizes = sorted(set(int(m) for m in self.M))
        if len(plan_sizes) > 4:
            raise ValueError("at most 4 distinct grid sizes per ensemble")
        self.plan_sizes = plan_sizes
        dev = torch.device("cuda")
        t = lambda a, dt_: torch.as_tensor(np.ascontiguousarray(a, dtype=dt_), device=dev)
        self._arrs = dict(N=t(self.N, np.int32), M=t(self.M, np.int32), off=t(self.offsets, np.int64),
                          L=t(self.L, np.float64),
                          plan=t([plan_sizes.index(int(m)) for m in self.M], np.int32))
        self.desc = self._describe()
        z = lambda: torch.zeros(self.n_total, dtype=torch.complex128, device=dev)
        self.X = z()
        self.MXh = [z() for _ in range(self.order)]
        self.Fh = [z() for _ in range(self.order)]
        self.head, self.filled = self.order - 1, 0
        self.t, self.iteration = 0.0, 0
        self.stream = torch.cuda.Stream()
        self._graphs = {}
        self.join = True          # as IVPSolver.join: order the stream after torch's current stream

    def _describe(self):
        tpl = self.tpl
        D = _lib_desc()
        D.nmem = self.nmem
        D.precision = 1 if self.precision == "fp32" else 0
        if len(tpl.outputs) != 1:
            raise NotImplementedError("one output equation")
        facs = [a[0] for _, _, a in tpl.factors]
        D.nfactors = len(facs)
        monos = tpl.outputs[0][2]
        D.nmono = len(monos)
        if not (1 <= D.nfactors <= 4 and 1 <= D.nmono <= 4):
            raise NotImplementedError("up to 4 factors and 4 monomials")
        for f, o in enumerate(facs):
            D.factor_order[f] = int(o)
        for mi, (co, fs) in enumerate(monos):
            D.mono_coef[mi] = complex(co).real
            for q in range(4):
                D.mono_factors[4 * mi + q] = int(fs[q]) if q < len(fs) else -1
        mean = next(b for b in tpl.buckets if b.kind == "real")
        wave = next(b for b in tpl.buckets if b.kind != "real")
        if mean.n != 1 or wave.n != 1:
            raise NotImplementedError("diagonal (1 x 1) systems only")
        t0 = int(np.nonzero(np.all(mean.monos == 0, axis=1))[0][0])
        D.m_mean[0], D.m_mean[1] = mean.Mc[t0, 0].real, mean.Mc[t0, 0].imag
        D.l_mean[0], D.l_mean[1] = mean.Lc[t0, 0].real, mean.Lc[t0, 0].imag
        for tt, (pw,) in enumerate(wave.monos):
            if pw > 4:
                continue
            D.m_poly[2 * pw] += wave.Mc[tt, 0].real
            D.m_poly[2 * pw + 1] += wave.Mc[tt, 0].imag
            D.l_poly[2 * pw] += wave.Lc[tt, 0].real
            D.l_poly[2 * pw + 1] += wave.Lc[tt, 0].imag
        D.nplans = len(self.plan_sizes)
        for p, m in enumerate(self.plan_sizes):
            D.plan_sizes[p] = m
            t64, t32 = ctypes.c_void_p(), ctypes.c_void_p()
            call("cng_twiddle_table", m, 0, ctypes.byref(t64))
            call("cng_twiddle_table", m, 1, ctypes.byref(t32))
            D.twiddles64[p] = t64.value
            D.twiddles32[p] = t32.value
        a = self._arrs
        D.size_dev, D.grid_dev, D.offset_dev = a["N"].data_ptr(), a["M"].data_ptr(), a["off"].data_ptr()
        D.length_dev, D.plan_dev = a["L"].data_ptr(), a["plan"].data_ptr()
        return D

    # ------------------------------------------------------------------ state
    def set_state(self, C_list, t: float = 0.0) -> None:
        """Per member, its N/2 complex mode amplitudes (C_0 real)."""
        flat = np.concatenate([np.asarray(c, np.complex128).ravel() for c in C_list])
        if flat.size != self.n_total:
            raise ValueError("state size mismatch")
        self.X.copy_(_torch().as_tensor(flat, device=self.X.device))
        self.head, self.filled = self.order - 1, 0
        self.t, self.iteration = float(t), 0

    def state(self):
        x = self.X.detach().cpu().numpy()
        return [x[o:o + n // 2] for o, n in zip(self.offsets, self.N)]

    def random_state(self, seed: int = 0, amplitude: float = 0.1, kmax: int = 8):
        """Seeded Fourier amplitudes of size ``amplitude`` for mode indices 1..kmax (the KS config)."""
        rng = np.random.default_rng(seed)
        out = []
        for n in self.N:
            c = np.zeros(n // 2, np.complex128)
            k = min(kmax, n // 2 - 1)
            c[1:k + 1] = amplitude * (rng.standard_normal(k) + 1j * rng.standard_normal(k))
            out.append(c)
        return out

    # ------------------------------------------------------------------ stepping
    def _launch(self, s):
        q = min(self.order, self.filled + 1)
        a, c = SBDF[q]
        nxt = (self.head + 1) % self.order
        slots = [(nxt - j) % self.order for j in range(q)]
        cs = (ctypes.c_double * q)(*[c[j + 1] for j in range(q)])
        ds = (ctypes.c_double * q)(*[a[j + 1] / self.dt for j in range(q)])
        mx = (ctypes.c_void_p * q)(*[self.MXh[k].data_ptr() for k in slots])
        fp = (ctypes.c_void_p * q)(*[self.Fh[k].data_ptr() for k in slots])
        call("cng_fourier_ensemble_step", ctypes.byref(self.desc), self.X.data_ptr(), mx, fp, q, cs, ds,
             a[0] / self.dt, s)
        return nxt

    def step(self) -> None:
        torch = _torch()
        if self.join:
            self.stream.wait_stream(torch.cuda.current_stream())
        self.head = self._launch(_stream_handle(self.stream))
        self.filled = min(self.filled + 1, self.order)
        self.t += self.dt
        self.iteration += 1
        if self.join:
            torch.cuda.current_stream().wait_stream(self.stream)

    def run(self, steps: int) -> None:
        for _ in range(int(steps)):
            self.step()

    def run_graph(self, steps: int, unroll: int = 1) -> None:
        """``steps`` steps; after the start-up, graph launches of ``unroll`` steps each (one graph
        per ring phase and length; a remainder shorter than ``unroll`` runs as one-step graphs)."""
        torch = _torch()
        steps = int(steps)
        unroll = max(1, int(unroll))
        while steps > 0 and self.filled < self.order:
            self.step()
            steps -= 1
        if steps <= 0:
            return
        s = _stream_handle(self.stream)
        if self.join:
            self.stream.wait_stream(torch.cuda.current_stream())
        while steps > 0:
            u = unroll if steps >= unroll else 1
            key = ((self.head + 1) % self.order, u)
            g = self._graphs.get(key)
            if g is None:
                self.stream.synchronize()
                call("cng_graph_begin", s)
                h = ctypes.c_void_p()
                head0 = self.head
                try:
                    for _ in range(u):
                        self.head = self._launch(s)
                finally:
                    self.head = head0
                    call("cng_graph_end", s, ctypes.byref(h))
                from .ivp import _Graph
                g = self._graphs[key] = _Graph(h)
            g.launch(s)
            self.head = (self.head + u) % self.order
            self.t += u * self.dt
            self.iteration += u
            steps -= u
        if self.join:
            torch.cuda.current_stream().wait_stream(self.stream)

    def mode_updates(self) -> int:
        """Real unknowns per step (2 per complex amplitude, 1 for the mean modes)."""
        return int(sum(self.N) - self.nmem)


def _lib_desc():
    class Desc(ctypes.Structure):
        _fields_ = [("nmem", ctypes.c_int32), ("precision", ctypes.c_int32), ("nfactors", ctypes.c_int32),
                    ("nmono", ctypes.c_int32), ("nplans", ctypes.c_int32),
                    ("size_dev", ctypes.c_void_p), ("grid_dev", ctypes.c_void_p),
                    ("offset_dev", ctypes.c_void_p), ("length_dev", ctypes.c_void_p),
                    ("plan_dev", ctypes.c_void_p), ("plan_sizes", ctypes.c_int32 * 4),
                    ("twiddles64", ctypes.c_void_p * 4), ("twiddles32", ctypes.c_void_p * 4),
                    ("factor_order", ctypes.c_int32 * 4), ("mono_coef", ctypes.c_double * 4),
                    ("mono_factors", ctypes.c_int32 * 16), ("m_poly", ctypes.c_double * 10),
                    ("l_poly", ctypes.c_double * 10), ("m_mean", ctypes.c_double * 2),
                    ("l_mean", ctypes.c_double * 2)]
    return Desc()
