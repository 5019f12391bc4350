"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

FP64 path: same algorithm, summation order may differ -> per-step fields
within 1e-11 relative (to the field's magnitude), converged fields within
1e-10.  Mixed path (FP32 f / FP64 moments): error against the FP64 oracle
stated and bounded (5e-5 relative after a few steps).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pair(case, precision):
    from hyb_gb300 import abi
    g = abi.Solver(case, precision=precision)
    o = O.Oracle(case, threads=0)
    g.init_maxwellian()
    o.init_maxwellian()
    o.convert_ns()          # the device init ends with Convert_NS as well
    return g, o


def _interior_f(case, frd):
    f = frd.reshape(case.nv, case.ny + 7, case.nx + 7, 2)
    return f[:, 4:4 + case.ny - 1, 4:4 + case.nx - 1, :]


def _rel(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


def _s_ring(case, s):
    """S_GKUA restricted to the cells the solver defines: 0..nx x 0..ny
    without the four corners (those are set by Convert_NS)."""
    S = s.reshape(case.ny + 7, case.nx + 7, 11)[3:3 + case.ny + 1, 3:3 + case.nx + 1, :10].copy()
    for (j, i) in [(0, 0), (0, -1), (-1, 0), (-1, -1)]:
        S[j, i, :] = 0.0
    return S


def _hot_faces(case, arrs):
    nx, ny = case.nx, case.ny
    ti, qi, tj, qj = arrs
    ti = ti.reshape(ny + 3, nx + 3, 4)[2:2 + ny - 1, 2:2 + nx, :]       # i=1..nx, j=1..ny-1
    qi = qi.reshape(ny + 3, nx + 3, 2)[2:2 + ny - 1, 2:2 + nx, :]
    tj = tj.reshape(ny + 3, nx + 3, 4)[2:2 + ny, 2:2 + nx - 1, :]       # i=1..nx-1, j=1..ny
    qj = qj.reshape(ny + 3, nx + 3, 2)[2:2 + ny, 2:2 + nx - 1, :]
    return ti, qi, tj, qj


@pytest.fixture(scope="module")
def cases_mod(pkg):
    from hyb_gb300 import cases
    return cases


def _cmp_state(case, g, o, tol):
    fg, fo = _interior_f(case, g.download_f()), _interior_f(case, o.frd())
    assert _rel(fg, fo) < tol, ("f", _rel(fg, fo))
    sg, cg = g.moments()
    so = o.s_gkua()
    Sg, So = _s_ring(case, sg), _s_ring(case, so)
    for k in range(10):
        assert _rel(Sg[..., k], So[..., k]) < tol or np.abs(Sg[..., k] - So[..., k]).max() < tol, ("S", k)
    hg, ho = _hot_faces(case, g.hot()), _hot_faces(case, o.hot())
    for a, b, name in zip(hg, ho, ("tao_i", "q_i", "tao_j", "q_j")):
        assert np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-3), name


@pytest.mark.parametrize("scheme", [0, 1, 3])
def test_fp64_one_step_matches_oracle(cases_mod, scheme):
    c = cases_mod.couette_small(ncy=32, nvx=16, nvy=16, scheme=scheme, dt=0.05)
    g, o = _pair(c, 0)
    _cmp_state(c, g, o, 1e-12)          # initial state (moments of the Maxwellian)
    rg = g.step(1)
    ro = o.step(1)
    _cmp_state(c, g, o, 1e-11)
    for k in range(4):
        assert abs(rg["res_rms"][k] - ro["res_rms"][k]) <= 1e-10 * max(ro["res_rms"][k], 1e-12)


def test_fp64_twenty_steps_couette_small(cases_mod):
    c = cases_mod.couette_small(dt=0.05)            # 4x64 cells, 32^2 velocities
    g, o = _pair(c, 0)
    for _ in range(4):
        rg = g.step(5)
        ro = o.step(5)
    _cmp_state(c, g, o, 1e-10)
    assert abs(rg["max_rms"] - ro["max_rms"]) <= 1e-9 * ro["max_rms"]


def test_fp64_transposed_orientation(cases_mod):
    """More cells along the periodic axis than across: the scan runs along
    the periodic direction and the march along the walls."""
    c = cases_mod.couette_small(ncx=40, ncy=8, nvx=12, nvy=12, dt=0.05)
    g, o = _pair(c, 0)
    g.step(3)
    o.step(3)
    _cmp_state(c, g, o, 1e-11)


def test_fp64_stretched_mesh(cases_mod):
    """Non-uniform spacing takes the per-face geometry path of the sweep."""
    c = cases_mod.couette_small(ncy=32, nvx=12, nvy=12, dt=0.02, stretch=1.5)
    g, o = _pair(c, 0)
    g.step(3)
    o.step(3)
    _cmp_state(c, g, o, 1e-11)


@pytest.mark.parametrize("precision", [0, 1])
def test_odd_velocity_counts(cases_mod, precision):
    """Velocity counts that are not multiples of the moment kernel's stage
    slot (4 FP32 / 2 FP64 velocities) or of its 8-velocity sum blocks."""
    c = cases_mod.couette_small(ncy=32, nvx=13, nvy=11, dt=0.05)
    g, o = _pair(c, precision)
    if precision == 0:
        _cmp_state(c, g, o, 1e-12)
        g.step(2)
        o.step(2)
        _cmp_state(c, g, o, 1e-11)
    else:
        g.step(2)
        o.step(2)
        Sg, So = _s_ring(c, g.moments()[0]), _s_ring(c, o.s_gkua())
        assert _rel(Sg[..., 0], So[..., 0]) < 5e-6 and _rel(Sg[..., 3], So[..., 3]) < 5e-6


def test_mixed_precision_error_is_bounded(cases_mod):
    c = cases_mod.couette_small(ncy=32, nvx=16, nvy=16, dt=0.05)
    g, o = _pair(c, 1)
    g.step(10)
    o.step(10)
    sg, _ = g.moments()
    Sg, So = _s_ring(c, sg), _s_ring(c, o.s_gkua())
    err_rho = _rel(Sg[..., 0], So[..., 0])
    err_u = np.abs(Sg[..., 1] - So[..., 1]).max() / np.abs(So[..., 1]).max()
    err_t = _rel(Sg[..., 3], So[..., 3])
    assert err_rho < 5e-6 and err_t < 5e-6 and err_u < 5e-5, (err_rho, err_u, err_t)


def test_upload_download_roundtrip(cases_mod):
    c = cases_mod.couette_small(ncy=16, nvx=8, nvy=8)
    from hyb_gb300 import abi
    g = abi.Solver(c, precision=0)
    g.init_maxwellian()
    f = g.download_f()
    rng = np.random.default_rng(1)
    fi = _interior_f(c, f)
    fi *= 1.0 + 0.01 * rng.standard_normal(fi.shape)
    f2 = np.zeros_like(f)
    _interior_f(c, f2)[...] = fi
    g.upload_f(f2)
    back = _interior_f(c, g.download_f())
    assert np.array_equal(back, fi)
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    f3 = o.frd()
    _interior_f(c, f3)[...] = fi
    o.upload_f(f3)
    sg, _ = g.moments()
    assert _rel(_s_ring(c, sg)[1:-1, 1:-1], _s_ring(c, o.s_gkua())[1:-1, 1:-1]) < 1e-12


def test_step_errors_are_status_codes(cases_mod):
    from hyb_gb300 import abi, hyb_types as T
    c = cases_mod.couette_small(ncy=16, nvx=8, nvy=8)
    g = abi.Solver(c, precision=0)
    g.init_maxwellian()
    with pytest.raises(abi.HybError) as e:
        g.residual()                 # no RHS stored before the first step
    assert e.value.rc == T.HYB_ERR_INVALID
    assert g.L.hyb_step(g.h, 0, None) == T.HYB_ERR_INVALID
