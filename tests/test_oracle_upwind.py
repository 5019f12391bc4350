"""CPU checks of the oracle's upwind-ordered kinetic step and mass pin.

The velocity grids are 32^2 Newton-Cotes on [-5, 5]: coarser grids leave a
conservation defect of the discrete equilibrium that stalls the residual.
The oracle (oracle/hyb_oracle.c, orc_kinetic_step) restates the reference's
GKUA_Residual (Hybrid2D/src/GKUA_Residual.f90:28-112) and, as options with no
counterpart in the reference, the upwind-ordered sweep and the mass pin.
A converged state has RHS = 0 whatever operator the implicit step uses, so
with the total mass pinned the upwind-ordered iteration at dt = 1e6 and the
reference iteration at the reference's small dt must end on the same fields.
"""
import numpy as np

from oracle import oracle as O


def _run(case, tol, cap, chunk):
    o = O.Oracle(case, threads=0)
    o.init_maxwellian()
    it, r = 0, None
    while it < cap:
        r = o.step(chunk)
        it += chunk
        if r["max_rms"] < tol:
            break
    s = o.s_gkua().reshape(case.ny + 7, case.nx + 7, 11)[4:4 + case.ny - 1, 4:4 + case.nx - 1, :10]
    return it, r["max_rms"], s


def test_upwind_and_reference_orders_reach_one_fixed_point(pkg):
    from hyb_gb300 import cases
    kw = dict(ncy=32, nvx=32, nvy=32, kn=0.1, uw=0.2, t_top=1.1, mass_pin=1)
    it_u, r_u, s_u = _run(cases.couette_small(dt=1.0e6, sweep_order=1, **kw), 1e-9, 2000, 50)
    it_r, r_r, s_r = _run(cases.couette_small(dt=0.05, sweep_order=0, **kw), 1e-9, 20000, 250)
    assert r_u < 1e-9 and r_r < 1e-9
    assert it_u * 3 < it_r, (it_u, it_r)
    for k in range(10):
        scale = max(np.abs(s_r[..., k]).max(), 1e-3)
        assert np.abs(s_u[..., k] - s_r[..., k]).max() <= 1e-7 * scale, k
    # the pinned total mass is the initial one (uniform mesh: the mean density)
    assert abs(s_u[..., 0].mean() - 1.0) < 1e-9


def test_mass_drifts_without_pin(pkg):
    """Without the pin the fixed point depends on the path: the upwind
    iteration at dt = 1e6 ends on a different total mass than the pinned one."""
    from hyb_gb300 import cases
    kw = dict(ncy=32, nvx=32, nvy=32, kn=0.1, uw=0.2, t_top=1.1)
    _, r, s = _run(cases.couette_small(dt=1.0e6, sweep_order=1, **kw), 1e-9, 2000, 50)
    assert r < 1e-9
    assert abs(s[..., 0].mean() - 1.0) > 1e-6
