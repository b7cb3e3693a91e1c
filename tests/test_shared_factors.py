"""CPU: shared factors of sign-similar buckets (the reference's SharedFactor,
python/conatus/timestep/shared_factors.py): the template-level relation and the planner's bytes."""
from __future__ import annotations

import copy

import numpy as np
import pytest

from _step_cases import template


@pytest.mark.parametrize("name,sizes", [("channel_ny17", [16, 12]), ("channel_ny129", [8, 8])])
def test_channel_pairs_hold_on_the_values(name, sizes):
    """The (kx, -kz) bucket of the channel is diag(dr) A diag(dc) of the (kx, +kz) bucket, exactly,
    at every mode and for any combination a M + b L; the border rows keep their diagonal's sign."""
    tpl = template(name)
    pairs = tpl.sign_pairs()
    assert list(pairs) == [4] and pairs[4][0] == 3
    _, dr, dc = pairs[4]
    b = tpl.buckets[3]
    assert np.all(dr[:b.r] * dc[:b.r] == 1)
    assert 0 < np.count_nonzero(dr < 0) < b.n
    P = tpl.instantiate(sizes)
    S = (dr[b.coo_rows()] * dc[b.indices]).astype(float)
    for a, c in [(1.0, 1.0), (11 / 6 / 5e-3, 1.0), (1.0, 0.25)]:
        A = a * P.values(3, "M") + c * P.values(3, "L")
        B = a * P.values(4, "M") + c * P.values(4, "L")
        assert np.all(A != 0) and np.array_equal(B, S[None, :] * A)


@pytest.mark.parametrize("name", ["rb_nz16", "rb_nz64", "burgers_n128", "ks"])
def test_no_pairs_without_two_fourier_directions(name):
    assert template(name).sign_pairs() == {}


def test_relation_refused_on_mixed_parity_and_border_sign():
    from conatus_gb300.template import sign_similarity
    tpl = template("channel_ny17")
    a, b = tpl.buckets[3], tpl.buckets[4]
    assert sign_similarity(a, b) is not None
    # an entry whose terms mix even and odd powers of kz is + or - the other at no mode
    c = copy.copy(b)
    c.Lc = b.Lc.copy()
    e = int(np.nonzero(b.Lc[0])[0][0])                    # an entry with a constant term
    odd = int(np.nonzero(b.monos[:, 1] == 1)[0][0])
    c.Lc[odd, e] = 1.0
    a2 = copy.copy(a)
    a2.Lc = c.Lc
    assert sign_similarity(a2, c) is None
    # different polynomials: not the two sign views of one bucket
    d = copy.copy(b)
    d.Mc = b.Mc * 2
    assert sign_similarity(a, d) is None
    # same sign: not a pair
    assert sign_similarity(a, a) is None


def test_planner_counts_one_factor_set_per_pair():
    from conatus_gb300 import memory
    P = template("channel_ny129").instantiate([64, 64])
    shared = memory.plan_ivp(P, "SBDF3")
    alone = memory.plan_ivp(P, "SBDF3", share=False)
    assert shared["factors"] < 0.6 * alone["factors"]
    assert shared["total"] < alone["total"]
