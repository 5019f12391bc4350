"""The CPU oracle against the reference's own output (no GPU).

tests/golden/flow2d_gkua_step0.json holds the step-0 moment field that the
reference wrote for its shipped cylinder case (see make_golden.py).  The
oracle must reproduce it from the same inputs: the Gauss-Legendre grid with
the reference's REAL(4) node table, the initial Maxwellian, DETFP's moment
sums and primitive conversion, and CF from sub_init.f90's cfc.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def gold(golden_dir):
    with open(os.path.join(golden_dir, "flow2d_gkua_step0.json")) as fh:
        return json.load(fh)


def _gl_case(pkg, inp, single):
    from hyb_gb300 import cases
    c = cases.couette_small(ncx=4, ncy=8, nvx=4, nvy=4, kn=0.1)
    v, w = O.grid_gl(inp["dv"], inp["intervals"], inp["vdown"], inp["kgln"], 1 if single else 0)
    c.vgrid = lambda: (v, w, v, w)
    c.nvx = c.nvy = len(v)
    cfc, re = O.cfc_vhs(inp["mole_mass"], inp["gamma"], inp["alpha"], inp["omega"], inp["vis_ref"],
                        inp["tref"], inp["ma"], inp["nd_inf"], inp["t_inf"], inp["lref"])
    base = c.params

    def params():
        p = base()
        p.cfc = cfc
        p.x1s = 1.0 - inp["omega"]
        return p
    c.params = params
    return c


def _cell(o, k, i=2, j=3):
    S = o.s_gkua().reshape(-1, 11)
    P = o.nx + 7
    return S[(i + 3) + P * (j + 3)][k]


@pytest.mark.parametrize("single", [True])
def test_step0_moments_match_reference_output(pkg, gold, single):
    inp, val = gold["inputs"], gold["values"]
    c = _gl_case(pkg, inp, single)
    o = O.Oracle(c, threads=1)
    u0 = math.sqrt(inp["gamma"] / 2.0) * inp["ma"] * math.cos(inp["aoa"])   # sub_init.f90:426
    o.init_maxwellian(1.0, u0, 0.0, 1.0)
    d, u, v, T = (_cell(o, k) for k in range(4))
    pxx, pyy, pxy, qx, qy, pzz = (_cell(o, k) for k in (4, 5, 6, 7, 8, 9))
    tol = 0.6e-10   # half a unit of the 10th printed decimal
    assert abs(d - val["d"]) < tol
    assert abs(u - val["u"]) < tol
    assert abs(v - val["v"]) < tol
    assert abs(T - val["T"]) < tol
    assert abs(d * T - val["p"]) < tol
    assert abs((pxx - d * T) - val["txx"]) < tol
    assert abs((pyy - d * T) - val["tyy"]) < tol
    assert abs(pxy - val["txy"]) < tol
    assert abs(qx - val["qx"]) < tol
    assert abs(qy - val["qy"]) < tol
    assert abs((pzz - d * T) - val["tzz"]) < tol
    cf = o.cf().reshape(-1)[(2 + 3) + (c.nx + 7) * (3 + 3)]
    assert abs(cf - val["cf"]) < 2e-9


def test_double_precision_table_does_not_match(pkg, gold):
    """The REAL(4) rounding of the node table is visible in the output: a
    double-precision Gauss-Legendre rule misses the printed digits."""
    inp, val = gold["inputs"], gold["values"]
    c = _gl_case(pkg, inp, single=False)
    o = O.Oracle(c, threads=1)
    u0 = math.sqrt(inp["gamma"] / 2.0) * inp["ma"]
    o.init_maxwellian(1.0, u0, 0.0, 1.0)
    assert abs(_cell(o, 1) - val["u"]) > 1e-10 or abs(_cell(o, 3) - val["T"]) > 1e-10


def test_gl_grid_matches_python_builder(pkg):
    from hyb_gb300 import cases
    for single in (True, False):
        v1, w1 = O.grid_gl(1.2, 15, -9.0, 4, 1 if single else 0)
        v2, w2 = cases.grid_gl(1.2, 15, -9.0, 4, single)
        np.testing.assert_allclose(v1, v2, rtol=0, atol=1e-15)
        np.testing.assert_allclose(w1, w2, rtol=0, atol=1e-15)
