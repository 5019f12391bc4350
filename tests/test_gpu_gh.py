"""Gauss-Hermite velocity grids and the higher-order moments on the GPU.

The kinetic path with a 2 x 8-node Gauss-Hermite grid against the oracle
(FP64: the same tolerances as the Newton-Cotes parity tests), and
HOT_GKUA / HOQ_GKUA from hyb_download_hoq against the oracle's orc_hoq
(FP64 1e-11 of the field's magnitude; mixed precision 1e-5).
"""
import numpy as np
import pytest

from test_gpu_parity import _cmp_state, _pair

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cases_mod(pkg):
    from hyb_gb300 import cases
    return cases


def _interior(c, a, k):
    return a.reshape(c.ny + 7, c.nx + 7, k)[4:4 + c.ny - 1, 4:4 + c.nx - 1, :]


def _cmp_hoq(c, g, o, tol):
    hg, qg = g.hoq()
    ho, qo = o.hoq()
    for a, b, k in ((hg, ho, 6), (qg, qo, 4)):
        A, B = _interior(c, a, k), _interior(c, b, k)
        scale = max(np.abs(B).max(), 1e-300)
        assert np.abs(A - B).max() <= tol * scale, (k, np.abs(A - B).max() / scale)


def test_gh_grid_fp64_matches_oracle(cases_mod):
    c = cases_mod.couette_small(ncy=32, nvx=16, nvy=16, quadrature="gh", uw=0.3, t_top=1.2, dt=0.02)
    g, o = _pair(c, 0)
    _cmp_state(c, g, o, 1e-12)
    g.step(3)
    o.step(3)
    _cmp_state(c, g, o, 1e-11)
    _cmp_hoq(c, g, o, 1e-11)


def test_hoq_newton_cotes_and_mixed(cases_mod):
    c = cases_mod.couette_small(ncy=32, nvx=16, nvy=16, uw=0.3, dt=0.05)
    g, o = _pair(c, 0)
    g.step(2)
    o.step(2)
    _cmp_hoq(c, g, o, 1e-11)
    gm, om = _pair(c, 1)
    gm.step(2)
    om.step(2)
    _cmp_hoq(c, gm, om, 1e-5)
