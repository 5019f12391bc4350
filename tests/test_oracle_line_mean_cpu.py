"""CPU checks of the line-averaged correction of the synthetic solve
(line_mean, oracle/hyb_oracle_ns.c ns_line_mean and ns_line_harmonics),
which the GPU kernels k_ns_lmean_rows / k_ns_lines_pcr<true> /
k_ns_lmean_seq / k_ns_lharm_rows / k_ns_lharm_seq / k_ns_lmean_fill are
tested against.

Line Gauss-Seidel across the periodic axis builds up the correction that is
constant along that axis over O((cells across / line length)^2) passes; the
coarse solve of the line system averaged over the lines gives it in one.  On
a Kn 0.01 channel with 32 cells across and 48 along the wall normal (33^2
velocities on [-6, 6], plates +-0.5, walls 1 / 1.2, upwind order at dt 1e6,
mass pin, band to the walls, line solver of 20 inner iterations at CFL 300),
40 outer iterations take the residual to 1.9e-6 with it and 5.3e-3 without.
"""
import os

import pytest

from oracle import oracle as O

# every host core: an earlier test may have left the oracle at one thread
THREADS = os.cpu_count() or 1


def _run(cases, line_mean, nit):
    c = cases.Case(name="kn0.01-32x48", ncx=32, ncy=48, nvx=33, nvy=33, vmax=6.0, kn=0.01, uw=0.5, t_top=1.2,
                   dt=1.0e6, sweep_order=1, mass_pin=1)
    o = O.Oracle(c, threads=THREADS)
    o.init_maxwellian()
    o.convert_ns()
    o.gsis(wall_band=1, correct_f=1, ns_solver=2, line_mean=line_mean, cfl=300.0, max_inner=20, inner_tol=0.0,
           inner_rtol=1e-4)
    r = o.step(nit)
    assert o.gsis_skipped() == 0
    return r["max_rms"]


def test_line_mean_accelerates_the_synthetic_solve(pkg):
    from hyb_gb300 import cases
    with_lm, without = _run(cases, 1, 40), _run(cases, 0, 40)
    assert with_lm < 1e-5, with_lm
    assert with_lm < 1e-2 * without, (with_lm, without)


@pytest.mark.parametrize("solver", [0, 1])
def test_line_mean_is_ignored_without_the_line_solver_in_the_oracle(pkg, solver):
    """The oracle takes line_mean only in the line solver (the library
    rejects it elsewhere): with LU-SGS or ADI the runs are bit-identical."""
    from hyb_gb300 import cases
    c = cases.couette_small(ncx=8, ncy=16, nvx=17, nvy=17, dt=0.02)
    out = []
    for lm in (0, 1):
        o = O.Oracle(c, threads=THREADS)
        o.init_maxwellian()
        o.convert_ns()
        o.gsis(ns_solver=solver, line_mean=lm, max_inner=8, inner_tol=0.0, inner_rtol=0.0, cfl=20.0)
        o.step(2)
        out.append(o.frd())
    assert (out[0] == out[1]).all()


def test_harmonics_accelerate_the_sine_case(pkg):
    """line_mean 3: the constant mode and the first two harmonics across the
    periodic axis (complex averaged systems).  On the sine-wall case at
    64 x 64 (48^2 on [-5, 5], Kn 0.005, T_w = 1 + 0.1 sin 2 pi x, plates
    +-0.3; upwind order at dt 1e6, mass pin, band to the walls, line solver
    of 16 inner iterations at CFL 600, correction relaxed to 0.7), 30 outer
    iterations take the residual to 3.0e-5 with them, 9.3e-4 with the
    constant mode alone and 1.0e-2 without either."""
    from hyb_gb300 import cases
    out = {}
    for lm in (1, 3):
        c = cases.couette_sine(ncx=64, ncy=64, dt=1.0e6, sweep_order=1, mass_pin=1, precision=0)
        o = O.Oracle(c, threads=THREADS)
        o.init_maxwellian()
        o.convert_ns()
        o.gsis(wall_band=1, correct_f=1, ns_solver=2, cfl=600.0, max_inner=16, inner_tol=0.0, inner_rtol=1e-8,
               relax_pct=70, line_mean=lm)
        out[lm] = o.step(30)["max_rms"]
        assert o.gsis_skipped() == 0
    assert out[3] < 1e-4 and out[3] < 0.1 * out[1], out


@pytest.mark.parametrize("ns_scheme,floor", [(1, 1e-5), (2, None)])
def test_the_limiter_sets_the_coarse_mesh_floor(pkg, ns_scheme, floor):
    """The 4 x 32 Kn 0.01 channel (48^2 on [-6, 6]): with the NND limiter in
    the synthetic equation's reconstruction (ns_scheme 1) the coupled
    iteration stalls at 4.3e-5; with the unlimited NND stencil (2) it
    reaches 2e-10 within 60 outer iterations."""
    from hyb_gb300 import cases
    c = cases.Case(name="kn0.01-4x32", ncx=4, ncy=32, nvx=48, nvy=48, vmax=6.0, kn=0.01, uw=0.5, t_top=1.2,
                   dt=1.0e6, sweep_order=1, mass_pin=1)
    o = O.Oracle(c, threads=THREADS)
    o.init_maxwellian()
    o.convert_ns()
    o.gsis(wall_band=1, correct_f=1, ns_solver=2, line_mean=1, cfl=300.0, max_inner=20, inner_tol=0.0,
           inner_rtol=1e-4, ns_scheme=ns_scheme)
    r = o.step(60)["max_rms"]
    if floor is None:
        assert r < 1e-9, r
    else:
        assert r > floor, r


def test_moments_only_correction_finishes_the_sine_case(pkg):
    """The sine-wall case at 64 x 64 (48^2 on [-5, 5], Kn 0.005): with the
    harmonics and the unlimited NND stencil the coupled iteration settles
    near 4e-8 with the distribution correction on; reconfigured to correct
    the moments only it falls below 1e-8 within 20 more outer iterations
    (4.9e-9 in the oracle)."""
    from hyb_gb300 import cases
    c = cases.couette_sine(ncx=64, ncy=64, dt=1.0e6, sweep_order=1, mass_pin=1, precision=0)
    gk = dict(wall_band=1, correct_f=1, ns_solver=2, cfl=600.0, max_inner=16, inner_tol=0.0, inner_rtol=1e-8,
              relax_pct=70, line_mean=3, ns_scheme=2)
    o = O.Oracle(c, threads=THREADS)
    o.init_maxwellian()
    o.convert_ns()
    o.gsis(**gk)
    r50 = o.step(50)["max_rms"]
    assert 1e-8 < r50 < 1e-6, r50
    o.gsis(**dict(gk, correct_f=0))
    r70 = o.step(20)["max_rms"]
    assert r70 < 1e-8, r70
    assert o.gsis_skipped() == 0
