"""GPU parity of the synthetic solve with the band reaching the walls and
with the block line-implicit inner solver.

wall_band extends the band of the GSIS coupling (Hybrid2D/src/Hybrid_Sub.f90:
45-153, band 3..n-3 in sub_NS_singlegrid.f90:23-30) to the wall cells, with
the reference's no-slip reflection of boundary_wall
(Hybrid2D/src/sub_boundary.f90:51-118) about the kinetic state at the wall
face.  ns_solver 2 solves the matrix of du_LU_SGS_2D
(Hybrid2D/src/sub_LU_SGS.f90:26-111) exactly along each wall-normal line.
The oracle (oracle/hyb_oracle_ns.c) restates both in FP64.  The GPU line
solver eliminates in FP32 (it preconditions an FP64 residual), so its
per-step states agree with the oracle to 1e-5 (measured 2.4e-7 to 1.2e-6
after three outer iterations) and its converged state to the same 1e-10 as
every FP64 path.
"""
import numpy as np
import pytest

from oracle import oracle as O

from test_gpu_parity import _cmp_state

pytestmark = pytest.mark.gpu

FIXED = dict(max_inner=12, inner_tol=0.0, inner_rtol=0.0)


@pytest.fixture(scope="module")
def cases_mod(pkg):
    from hyb_gb300 import cases
    return cases


def _pair(case, precision, **gk):
    from hyb_gb300 import abi
    g = abi.Solver(case, precision=precision)
    o = O.Oracle(case, threads=0)
    g.init_maxwellian()
    o.init_maxwellian()
    o.convert_ns()
    g.gsis(**gk)
    o.gsis(**gk)
    return g, o


def _shape(cases_mod, shape, **kw):
    if shape == "small":
        return cases_mod.couette_small(ncy=32, nvx=16, nvy=16, **kw)
    if shape == "transposed":
        return cases_mod.couette_small(ncx=40, ncy=8, nvx=12, nvy=12, **kw)
    return cases_mod.couette_small(ncx=16, ncy=96, nvx=12, nvy=12, t_pert=0.1, **kw)


@pytest.mark.parametrize("shape", ["small", "transposed", "sine"])
def test_wall_band_lusgs_matches_oracle(cases_mod, shape):
    c = _shape(cases_mod, shape, dt=0.02)
    g, o = _pair(c, 0, wall_band=1, correct_f=1, cfl=20.0, **FIXED)
    for _ in range(3):
        g.step(1)
        o.step(1)
    _cmp_state(c, g, o, 1e-10)


@pytest.mark.parametrize("shape,cfl", [("small", 100.0), ("transposed", 100.0), ("sine", 20.0)])
def test_line_solver_matches_oracle(cases_mod, shape, cfl):
    c = _shape(cases_mod, shape, dt=1.0e6, sweep_order=1, mass_pin=1)
    g, o = _pair(c, 0, wall_band=1, correct_f=1, ns_solver=2, cfl=cfl, **FIXED)
    for _ in range(3):
        g.step(1)
        o.step(1)
    assert g.gsis_skipped() == o.gsis_skipped() == 0
    _cmp_state(c, g, o, 1e-5)


def test_out_of_range_correction_is_skipped(cases_mod):
    """The 16 x 96 sine channel at Kn 0.1 from rest: with the line solver at
    CFL 100 the third synthetic solve drives the NS temperature below 0.1
    (the reference STOPs there); the outer iteration keeps its kinetic step,
    the GPU and the oracle skip the same correction, and their states still
    agree."""
    c = _shape(cases_mod, "sine", dt=1.0e6, sweep_order=1, mass_pin=1)
    g, o = _pair(c, 0, wall_band=1, correct_f=1, ns_solver=2, cfl=100.0, **FIXED)
    for _ in range(4):
        g.step(1)
        o.step(1)
    assert g.gsis_skipped() == o.gsis_skipped() >= 1
    _cmp_state(c, g, o, 1e-5)


def test_relaxed_correction_matches_oracle(cases_mod):
    c = _shape(cases_mod, "small", dt=0.02)
    g, o = _pair(c, 0, wall_band=1, correct_f=1, relax_pct=70, cfl=20.0, **FIXED)
    for _ in range(3):
        g.step(1)
        o.step(1)
    _cmp_state(c, g, o, 1e-10)


def test_line_solver_gsis_converges_to_the_oracle_fixed_point(cases_mod):
    """Kn 0.01 channel (4 x 128 cells, 48^2 velocities on [-6, 6], plates
    +-0.5, walls 1 / 1.2) with the upwind-ordered kinetic step at dt 1e6,
    the mass pin, the wall band and the line solver: residual 1e-8 within
    120 outer iterations; after 240 the converged moments equal the
    oracle's run of the same iteration to 1e-10."""
    c = cases_mod.Case(name="kn0.01-4x128", ncx=4, ncy=128, nvx=48, nvy=48, vmax=6.0, kn=0.01, uw=0.5,
                       t_top=1.2, dt=1.0e6, sweep_order=1, mass_pin=1)
    gk = dict(wall_band=1, correct_f=1, ns_solver=2, cfl=300.0, max_inner=20, inner_tol=0.0, inner_rtol=1e-4)
    g, o = _pair(c, 0, **gk)
    it, it8 = 0, None
    while it < 240:
        rg = g.step(10)
        ro = o.step(10)
        it += 10
        if it8 is None and rg["max_rms"] < 1e-8:
            it8 = it
    assert it8 is not None and it8 <= 120, (it8, rg)
    # the residual settles near 2e-10: the velocity grid's conservation
    # defect; the state itself keeps converging to the same fixed point
    assert rg["max_rms"] < 1e-9 and ro["max_rms"] < 1e-9, (rg, ro)
    sg, _ = g.moments()
    so = o.s_gkua()
    n = (c.ny + 7, c.nx + 7, 11)
    Sg = sg.reshape(n)[4:4 + c.ny - 1, 4:4 + c.nx - 1, :10]
    So = so.reshape(n)[4:4 + c.ny - 1, 4:4 + c.nx - 1, :10]
    for k in range(10):
        d = np.abs(Sg[..., k] - So[..., k]).max()
        assert d <= 1e-10 * max(np.abs(So[..., k]).max(), 1e-2), (k, d)


def _line_mean_case(cases_mod, kind, **kw):
    """Wall-normal lines with a periodic axis across them: lines along j
    (the channel), lines along i (walls on the x faces), and lines of 519
    cells, above the 512 cells a CTA reduces (the sequential paths)."""
    from hyb_gb300 import hyb_types as T
    P, W = T.HYB_BC_PERIODIC, T.HYB_BC_WALL
    if kind == "along_j":
        return cases_mod.couette_small(ncx=24, ncy=32, nvx=16, nvy=16, **kw)
    if kind == "along_i":
        return cases_mod.couette_small(ncx=32, ncy=24, nvx=16, nvy=16, bcs=(W, P, W, P), t_top=1.2, **kw)
    return cases_mod.couette_small(ncx=6, ncy=520, nvx=16, nvy=16, **kw)


@pytest.mark.parametrize("line_mean", [1, 3])
@pytest.mark.parametrize("kind", ["along_j", "along_i", "long", "sine"])
def test_line_mean_matches_oracle(cases_mod, kind, line_mean):
    """line_mean: before the colour passes of each inner iteration, the
    line system averaged over the lines is solved and copied to every line;
    line_mean 3 adds the first two harmonics across the periodic axis, each
    a complex averaged system.  GPU (FP32 elimination, FP64 residual and
    update) against the oracle's FP64 restatement after three outer
    iterations."""
    if kind == "sine":
        c = _shape(cases_mod, "sine", dt=1.0e6, sweep_order=1, mass_pin=1)
    else:
        c = _line_mean_case(cases_mod, kind, dt=1.0e6, sweep_order=1, mass_pin=1)
    cfl = 20.0 if kind == "sine" else 100.0      # at CFL 100 the sine case's NS state leaves the range
    g, o = _pair(c, 0, wall_band=1, correct_f=1, ns_solver=2, line_mean=line_mean, cfl=cfl, **FIXED)
    for _ in range(3):
        g.step(1)
        o.step(1)
    assert g.gsis_skipped() == o.gsis_skipped() == 0
    _cmp_state(c, g, o, 1e-5)


def test_line_mean_needs_the_line_solver(cases_mod):
    from hyb_gb300 import abi, hyb_types as T
    c = _line_mean_case(cases_mod, "along_j", dt=0.02)
    s = abi.Solver(c, precision=0)
    with pytest.raises(abi.HybError) as e:
        s.gsis(ns_solver=0, line_mean=1, **FIXED)
    assert e.value.rc == T.HYB_ERR_INVALID
    with pytest.raises(abi.HybError) as e:     # at most three harmonics
        s.gsis(ns_solver=2, line_mean=5, **FIXED)
    assert e.value.rc == T.HYB_ERR_INVALID
    s.close()


def test_line_mean_converges_to_the_oracle_fixed_point(cases_mod):
    """Kn 0.01 channel with 16 cells across the periodic axis (16 x 128,
    48^2 velocities on [-6, 6], plates +-0.5, walls 1 / 1.2), upwind order
    at dt 1e6, mass pin, band to the walls, line solver with line_mean:
    residual 1e-8 within 100 outer iterations (the oracle: 70), and after
    160 the converged moments equal the oracle's run of the same iteration
    to 1e-10.  (Meshes of 32 or 64 cells along the wall normal stall near
    4e-5 / 1.5e-7 with or without line_mean, in the oracle as on the GPU.)"""
    c = cases_mod.Case(name="kn0.01-16x128", ncx=16, ncy=128, nvx=48, nvy=48, vmax=6.0, kn=0.01, uw=0.5,
                       t_top=1.2, dt=1.0e6, sweep_order=1, mass_pin=1)
    gk = dict(wall_band=1, correct_f=1, ns_solver=2, line_mean=1, cfl=300.0, max_inner=20, inner_tol=0.0,
              inner_rtol=1e-4)
    g, o = _pair(c, 0, **gk)
    it, it8 = 0, None
    while it < 160:
        rg = g.step(10)
        ro = o.step(10)
        it += 10
        if it8 is None and rg["max_rms"] < 1e-8:
            it8 = it
    assert it8 is not None and it8 <= 100, (it8, rg)
    assert rg["max_rms"] < 1e-9 and ro["max_rms"] < 1e-9, (rg, ro)
    sg, _ = g.moments()
    so = o.s_gkua()
    n = (c.ny + 7, c.nx + 7, 11)
    Sg = sg.reshape(n)[4:4 + c.ny - 1, 4:4 + c.nx - 1, :10]
    So = so.reshape(n)[4:4 + c.ny - 1, 4:4 + c.nx - 1, :10]
    for k in range(10):
        d = np.abs(Sg[..., k] - So[..., k]).max()
        assert d <= 1e-10 * max(np.abs(So[..., k]).max(), 1e-2), (k, d)


def test_unlimited_nnd_stencil_matches_oracle(cases_mod):
    """ns_scheme 2 (the NND stencil of the synthetic equation without its
    limiter) with the line solver and two harmonics, then the moments-only
    correction: the sine case's finishing configuration, on the 4 x 32
    channel against the oracle after three outer iterations of each."""
    c = _shape(cases_mod, "small", dt=1.0e6, sweep_order=1, mass_pin=1)
    gk = dict(wall_band=1, correct_f=1, ns_solver=2, line_mean=3, ns_scheme=2, cfl=20.0, **FIXED)
    g, o = _pair(c, 0, **gk)
    for _ in range(3):
        g.step(1)
        o.step(1)
    _cmp_state(c, g, o, 1e-5)
    g.gsis(**dict(gk, correct_f=0))
    o.gsis(**dict(gk, correct_f=0))
    for _ in range(3):
        g.step(1)
        o.step(1)
    assert g.gsis_skipped() == o.gsis_skipped() == 0
    _cmp_state(c, g, o, 1e-5)
