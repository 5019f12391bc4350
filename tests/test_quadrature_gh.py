"""The Gauss-Hermite velocity grid and the higher-order moments (CPU).

* The half-range rule computed from its weight function matches the table of
  the reference's GaussHermite routine (tests/golden/gauss_hermite_half_range
  .json, extracted by tests/golden/make_golden.py) for 8 and 16 nodes.  The
  reference's 7-node table is not the exact Gauss rule (its nodes differ from
  it by up to 9e-5), so for 7 nodes both are checked on the moments they
  integrate.
* Known answers of the oracle's DETFP and HOT/HOQ on the initial Maxwellian,
  which a Gauss-Hermite grid integrates exactly.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def cm(pkg):
    from hyb_gb300 import cases
    return cases


@pytest.fixture(scope="module")
def table(golden_dir):
    with open(os.path.join(golden_dir, "gauss_hermite_half_range.json")) as fh:
        return json.load(fh)["tables"]


@pytest.mark.parametrize("n", [8, 16])
def test_half_range_rule_matches_reference_table(cm, table, n):
    a, h = cm.half_range_hermite(n)
    ra, rh = np.array(table[str(n)]["nodes"]), np.array(table[str(n)]["weights"])
    assert np.abs(a - ra).max() < 1e-12
    assert np.abs(h / rh - 1.0).max() < 5e-12


def test_seven_point_rules_integrate_the_low_moments(cm, table):
    a, h = cm.half_range_hermite(7)
    ra, rh = np.array(table["7"]["nodes"]), np.array(table["7"]["weights"])
    for p in range(6):
        exact = math.gamma((p + 1) / 2.0) / 2.0
        assert abs((h * a ** p).sum() / exact - 1.0) < 1e-12
        assert abs((rh * ra ** p).sum() / exact - 1.0) < 5e-9
    for p in range(6, 14):      # the Gauss rule is exact to degree 13
        exact = math.gamma((p + 1) / 2.0) / 2.0
        assert abs((h * a ** p).sum() / exact - 1.0) < 1e-12
    assert np.abs(a - ra).max() < 1e-4


@pytest.mark.parametrize("n2", [14, 16, 32])
def test_full_grid_integrates_gaussian_moments(cm, n2):
    v, w = cm.grid_gh(n2)
    assert np.allclose(v, -v[::-1]) and np.allclose(w, w[::-1])
    g = np.exp(-v * v)
    for p in range(0, 9, 2):
        exact = math.gamma((p + 1) / 2.0)
        assert abs((w * g * v ** p).sum() / exact - 1.0) < 1e-12


def test_oracle_maxwellian_moments_on_gh_grid(cm):
    c = cm.couette_small(ncy=16, nvx=16, nvy=16, quadrature="gh", uw=0.0, dt=0.01)
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    S = o.s_gkua().reshape(c.ny + 7, c.nx + 7, 11)[4:4 + c.ny - 1, 4:4 + c.nx - 1, :]
    assert np.abs(S[..., 0] - 1.0).max() < 1e-12         # density
    assert np.abs(S[..., 1:3]).max() < 1e-12             # velocity
    assert np.abs(S[..., 3] - 1.0).max() < 1e-12         # temperature
    hot, hoq = o.hoq()
    hot = hot.reshape(c.ny + 7, c.nx + 7, 6)[4:4 + c.ny - 1, 4:4 + c.nx - 1, :]
    hoq = hoq.reshape(c.ny + 7, c.nx + 7, 4)[4:4 + c.ny - 1, 4:4 + c.nx - 1, :]
    # at rest, T = 1: odd moments vanish; sum (G c^2 + H) vx^2 = <vx^2 c^2> +
    # <vx^2>/2 = 1 + 1/4 with <.> the mean over exp(-c^2)/pi
    assert np.abs(hot).max() < 1e-12
    assert np.abs(hoq[..., 0] - 1.25).max() < 1e-12 and np.abs(hoq[..., 2] - 1.25).max() < 1e-12
    assert np.abs(hoq[..., 1]).max() < 1e-12 and np.abs(hoq[..., 3]).max() == 0.0
