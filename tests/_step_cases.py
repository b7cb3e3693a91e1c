"""Readers of the step golden fixtures (tests/golden/step_*.npz) and the problem templates."""
from __future__ import annotations

import os

import numpy as np

from conftest import ROOT, golden

PROBLEMS = os.path.join(ROOT, "conatus_gb300", "problems")
# fixture -> (template, Fourier sizes of the fixture's build)
STEP_CASES = {
    "step_burgers128.npz": ("burgers_n128", []),
    "step_rb32x16.npz": ("rb_nz16", [32]),
    "step_channel8x17x8.npz": ("channel_ny17", [8, 8]),
    "step_ks64.npz": ("ks", [64]),
}
# periods of the fixtures whose period differs from the template's
STEP_LENGTHS = {"step_ks64.npz": [37.0]}


def template(name):
    from conatus_gb300.template import ProblemTemplate
    return ProblemTemplate.load(os.path.join(PROBLEMS, name + ".npz"))


def load_step(fixture, exact=True):
    """(problem, fixture arrays, maps) of a step fixture. ``exact``: the systems use the
    reference's own M and L values recorded in the fixture (the drop-in case); else the
    template's wavenumber polynomials."""
    tname, sizes = STEP_CASES[fixture]
    P = template(tname).instantiate(sizes or None, STEP_LENGTHS.get(fixture))
    g = golden(fixture)
    maps = []
    for bi in range(int(g["nb"])):
        p = f"m{bi}_"
        maps.append(dict(cols=g[p + "cols"], rows=g[p + "rows"], wc=g[p + "wc"], wr=g[p + "wr"],
                         dact=int(g[p + "dact"])))
    if exact:
        P.set_exact([(g[f"m{bi}_Mv"], g[f"m{bi}_Lv"]) for bi in range(int(g["nb"]))])
    return P, g, maps


def gather_rows(vec, mp):
    return sum(w * vec[r] for w, r in zip(mp["wr"], mp["rows"]))


def gather_state(vec, mp):
    return sum(w * vec[c] for w, c in zip(mp["wc"], mp["cols"]))


def scatter_state(C_list, maps, n_real):
    X = np.zeros(n_real)
    for C, mp in zip(C_list, maps):
        scale = 2.0 ** max(mp["dact"] - 1, 0)
        for w, c in zip(mp["wc"], mp["cols"]):
            np.add.at(X, c.ravel(), (np.conj(w) / scale * np.asarray(C)).real.ravel())
    return X


def field_errors(P, C, C_ref, floor=0.0):
    """Relative L2 error per variable (over every system), mode layout. ``floor``: the norm of a
    field is taken at least ``floor`` times the norm of the whole state (a field that is zero up
    to rounding, such as a gauge tau, is then judged against the state, not against itself)."""
    out = {}
    tot = sum(float(np.sum(np.abs(np.asarray(c)) ** 2)) for c in C_ref)
    for v, var in enumerate(P.tpl.variables):
        num = den = 0.0
        for bi, b in enumerate(P.tpl.buckets):
            sel = b.col[:, 0] == v
            num += float(np.sum(np.abs(np.asarray(C[bi])[:, sel] - np.asarray(C_ref[bi])[:, sel]) ** 2))
            den += float(np.sum(np.abs(np.asarray(C_ref[bi])[:, sel]) ** 2))
        den = max(den, floor ** 2 * tot)
        out[var["name"]] = (num / den) ** 0.5 if den > 0 else num ** 0.5
    return out


def field_tolerances(P, g, maps, base=1e-12, factor=10.0):
    """Per-field tolerance of a step parity check: ``base`` (1e-12 relative L2), raised to
    ``factor`` times the reference's own rounding floor of that field (the spread of its X_{n+1}
    when X_n is perturbed by one ulp, recorded in the fixture)."""
    ref = [gather_state(g["Xn1"], m) for m in maps]
    tol = {k: base for k in (v["name"] for v in P.tpl.variables)}
    for Xp in g["Xn1_perturbed"]:
        pert = [gather_state(Xp, m) for m in maps]
        for k, e in field_errors(P, pert, ref).items():
            tol[k] = max(tol[k], factor * e)
    return tol


# scheme trajectories: a field's norm counts as at least this fraction of the state's norm
SCHEME_FLOOR = 1e-8
# scheme fixtures: case -> (template, Fourier sizes)
SCHEME_CASES = {"rb32x16": ("rb_nz16", [32]), "burgers128": ("burgers_n128", []),
                "channel8x17x8": ("channel_ny17", [8, 8])}


def scheme_fixtures():
    import glob
    from conftest import GOLDEN
    return sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "scheme_*.npz")))


def load_scheme(fixture):
    """(problem with the reference's own M and L values, fixture arrays, maps, scheme name) of a
    scheme fixture (``scheme_<case>_<scheme>.npz``)."""
    case = fixture[len("scheme_"):-len(".npz")].rsplit("_", 1)[0]
    tname, sizes = SCHEME_CASES[case]
    P = template(tname).instantiate(sizes or None)
    g = golden(fixture)
    maps = []
    for bi in range(int(g["nb"])):
        p = f"m{bi}_"
        maps.append(dict(cols=g[p + "cols"], rows=g[p + "rows"], wc=g[p + "wc"], wr=g[p + "wr"],
                         dact=int(g[p + "dact"])))
    P.set_exact([(g[f"m{bi}_Mv"], g[f"m{bi}_Lv"]) for bi in range(int(g["nb"]))])
    return P, g, maps, str(g["scheme"])


def trajectory_tolerances(P, g, maps, step, base=1e-12, factor=10.0, tau_base=1e-10):
    """Per-field tolerance after ``step`` + 1 steps: ``base`` for the fields (``tau_base`` for the
    tau variables, auxiliary unknowns of the boundary rows), raised to ``factor`` times the spread of
    the reference's own trajectories from X_0 perturbed by one ulp."""
    ref = [gather_state(g["Xs"][step], m) for m in maps]
    tol = {k: (tau_base if k.startswith("tau") else base) for k in (v["name"] for v in P.tpl.variables)}
    for Xp in g["Xs_perturbed"]:
        pert = [gather_state(Xp[step], m) for m in maps]
        for k, e in field_errors(P, pert, ref, floor=SCHEME_FLOOR).items():
            tol[k] = max(tol[k], factor * e)
    return tol
