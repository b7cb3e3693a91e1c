"""CPU: the committed problem templates (the set-up the GPU machine runs from) load, carry valid
sparsity patterns and wavenumber polynomials within their recorded fit, and give the benchmark
configurations the reference's unknown counts (the channel 192x129x192: 19 043 083 real unknowns
in one real and four complex buckets)."""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from conftest import ROOT

TEMPLATES = sorted(glob.glob(os.path.join(ROOT, "conatus_gb300", "problems", "*.npz")))


def test_templates_present():
    names = {os.path.basename(f)[:-4] for f in TEMPLATES}
    assert {"channel_ny129", "channel_ny17", "rb_nz64", "rb_nz16", "burgers_n128", "ks"} <= names


@pytest.mark.parametrize("path", TEMPLATES, ids=lambda p: os.path.basename(p)[:-4])
def test_template_patterns_and_fit(path):
    from conatus_gb300.template import ProblemTemplate
    t = ProblemTemplate.load(path)
    assert t.buckets
    for b in t.buckets:
        ip, ix = b.indptr, b.indices
        assert ip.shape == (b.n + 1,) and ip[0] == 0 and ip[-1] == ix.shape[0]
        assert np.all(np.diff(ip) >= 0)
        assert ix.min() >= 0 and ix.max() < b.n
        rows = b.coo_rows()
        assert np.unique(rows.astype(np.int64) * b.n + ix).size == ix.size   # no duplicate entries
        assert 0 <= b.r <= b.n and b.r <= 64
        assert b.Mc.shape == b.Lc.shape == (b.monos.shape[0], ix.size)
        assert np.all(np.isfinite(b.Mc)) and np.all(np.isfinite(b.Lc))
        assert b.col.shape == (b.n, 3) and b.row.shape == (b.n, 4)
        # the polynomial form reproduced the source build's matrices (parameter-linear templates
        # fit the parameter too, hence their wider bound)
        assert b.fit_error <= (1e-13 if t.linear_params else 4e-15), (b.kind, b.fit_error)
        for name in t.linear_params:
            assert b.dL[name].shape == b.Lc.shape
    for lam, C in t.conv.items():
        assert C.shape[0] == C.shape[1] == t.ncheb and np.all(np.isfinite(C))


@pytest.mark.parametrize("config, unknowns, nsys, n", [
    ("channel", 19_043_083, [1, 95, 95, 9025, 9025], [523, 522, 522, 522, 522]),
    ("rayleigh_benard", 66_811, [1, 127], [263, 262]),
    ("burgers", 130, [1], [130]),
])
def test_benchmark_configurations(config, unknowns, nsys, n):
    from conatus_gb300 import workloads
    P = workloads.problem(config)
    assert P.real_unknowns() == unknowns
    assert list(P.nsys) == nsys
    assert [b.n for b in P.tpl.buckets] == n
