"""CPU checks of the oracle on the boundary combinations beyond the Couette
channel (walls or periodicity on either axis), which the GPU parity tests of
the specialised sweep compare against.

* The Maxwellian at rest in a fully periodic box is a fixed point of the
  kinetic step, in both sweep orders, to the error of the velocity
  quadrature: every flux difference vanishes and the Shakhov target equals
  f once the discrete moments are exact.  33 nodes per axis on [-5, 5] make
  them exact to ~1e-12; the reference's Newton-Cotes pattern is a Simpson
  rule only for an odd node count (GKUA_DETFP.f90:419-444), so even counts
  leave a drift of the moments that no iteration removes.
* From a seeded +-10% perturbation, on every combination, both iterations
  (the reference's at dt 0.05, the upwind-ordered one at dt 1e6 with the mass
  pin) keep every value finite and at or above the 1e-30 floor
  (GKUA_Residual.f90:104-105).
"""
import itertools

import numpy as np
import pytest

from oracle import oracle as O

FLOOR = 1.0e-30


def _case(cases, T, xper, yper, **kw):
    P, W = T.HYB_BC_PERIODIC, T.HYB_BC_WALL
    kx, ky = (P if xper else W), (P if yper else W)
    d = dict(ncx=8, ncy=16, nvx=17, nvy=17, bcs=(kx, ky, kx, ky))
    d.update(kw)
    return cases.couette_small(**d)


def _interior(case, frd):
    return frd.reshape(case.nv, case.ny + 7, case.nx + 7, 2)[:, 4:4 + case.ny - 1, 4:4 + case.nx - 1]


@pytest.mark.parametrize("order,dt", [(0, 0.05), (1, 1.0e6)])
def test_maxwellian_at_rest_is_a_fixed_point_of_the_periodic_box(pkg, order, dt):
    from hyb_gb300 import cases, hyb_types as T
    c = _case(cases, T, True, True, nvx=33, nvy=33, dt=dt, sweep_order=order, mass_pin=order)
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    b = _interior(c, o.frd())
    o.step(3)
    a = _interior(c, o.frd())
    assert np.abs(a - b).max() <= 1e-8 * np.abs(b).max()


@pytest.mark.parametrize("xper,yper", list(itertools.product([False, True], repeat=2)))
def test_every_boundary_combination_stays_finite_above_the_floor(pkg, xper, yper):
    from hyb_gb300 import cases, hyb_types as T
    runs = [(dict(dt=0.05), 8), (dict(dt=1.0e6, sweep_order=1, mass_pin=1), 8)]
    for kw, nstep in runs:
        c = _case(cases, T, xper, yper, **kw)
        o = O.Oracle(c, threads=0)
        o.init_maxwellian()
        f = o.frd()
        rng = np.random.default_rng(3)
        o.upload_f(f * (1.0 + 0.2 * (rng.random(f.shape) - 0.5)))
        for _ in range(nstep):
            r = o.step(5)
            assert np.isfinite(r["max_rms"]), kw
        fi = _interior(c, o.frd())
        assert np.isfinite(fi).all(), kw
        assert fi.min() >= FLOOR * (1 - 1e-12), kw
        s = o.s_gkua().reshape(c.ny + 7, c.nx + 7, 11)[4:4 + c.ny - 1, 4:4 + c.nx - 1]
        assert np.isfinite(s).all() and s[..., 0].min() > 0.0, kw
