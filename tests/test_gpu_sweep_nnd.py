"""The specialised FP32 sweep (k_sweep_nnd: uniform mesh, reference order,
NND, four scan cells per thread) on every combination of periodic and wall
scan and march axes, in both axis roles.

It forms the same face values with the same operations as the generic sweep
kernel (the limiter's zero-slope sign aside), so on the same FP32 state the
two agree to rounding; both are checked against the oracle within the mixed
path's tolerance.  The generic kernel is selected by HYB_SWEEP_GENERIC=1 at
context creation.  The state is a seeded perturbation of the Maxwellian, so
that fully periodic meshes have something to transport.
"""
import itertools

import numpy as np
import pytest

from oracle import oracle as O

from test_gpu_parity import _interior_f, _rel, _s_ring

pytestmark = pytest.mark.gpu

MIXED_TOL = 5e-5          # FP32 distribution against the FP64 oracle
TWIN_TOL = 4e-7           # the two FP32 kernels on the same state, relative to max |f|


@pytest.fixture(scope="module")
def mods(pkg):
    from hyb_gb300 import abi, cases, hyb_types as T
    return abi, cases, T


def _case(cases, T, pera, perb, sj, na=128, **kw):
    """A scan axis of na cells (4 cells per thread) of the given boundary
    kinds; the scan axis is y when sj, else x."""
    P, W = T.HYB_BC_PERIODIC, T.HYB_BC_WALL
    ka, kb = (P if pera else W), (P if perb else W)
    if sj:
        d = dict(ncx=12, ncy=na, bcs=(kb, ka, kb, ka))
    else:
        d = dict(ncx=na, ncy=12, bcs=(ka, kb, ka, kb))
    d.update(nvx=8, nvy=8, dt=0.05, precision=T.HYB_PREC_MIXED)
    d.update(kw)
    return cases.couette_small(**d)


def _perturbed(f, seed):
    rng = np.random.default_rng(seed)
    return f * (1.0 + 0.2 * (rng.random(f.shape) - 0.5))


@pytest.mark.parametrize("order,na", [(0, 128), (0, 256), (1, 128)])
@pytest.mark.parametrize("pera,perb,sj", list(itertools.product([False, True], repeat=3)))
def test_nnd_matches_generic_kernel_and_oracle(mods, monkeypatch, pera, perb, sj, order, na):
    """order 1: the upwind order (mirrored frames per velocity) at dt 1e6 with
    the mass pin, as the fast-converging runs use it."""
    abi, cases, T = mods
    kw = dict(sweep_order=1, mass_pin=1, dt=1.0e6) if order else {}
    c = _case(cases, T, pera, perb, sj, na=na, **kw)
    g = abi.Solver(c, precision=T.HYB_PREC_MIXED)
    g.init_maxwellian()
    g.upload_f(_perturbed(g.download_f(), 11))
    f0 = g.download_f()                     # the FP32 values, exact in FP64
    monkeypatch.setenv("HYB_SWEEP_GENERIC", "1")
    h = abi.Solver(c, precision=T.HYB_PREC_MIXED)
    monkeypatch.delenv("HYB_SWEEP_GENERIC")
    h.upload_f(f0)
    o = O.Oracle(c, threads=0)
    o.upload_f(f0)
    for _ in range(3):
        rg = g.step(1)
        rh = h.step(1)
        o.step(1)
    fg, fh = g.download_f(), h.download_f()
    assert np.abs(fg - fh).max() <= TWIN_TOL * np.abs(fh).max()
    for k in range(4):
        assert abs(rg["res_rms"][k] - rh["res_rms"][k]) <= 1e-5 * max(rh["res_rms"][k], 1e-12)
    fi, fo = _interior_f(c, fg), _interior_f(c, o.frd())
    assert _rel(fi, fo) < MIXED_TOL, _rel(fi, fo)
    Sg, So = _s_ring(c, g.moments()[0]), _s_ring(c, o.s_gkua())
    for k in range(10):
        assert _rel(Sg[..., k], So[..., k]) < MIXED_TOL or np.abs(Sg[..., k] - So[..., k]).max() < MIXED_TOL, k


@pytest.mark.parametrize("pera,perb", [(False, True), (True, False)])
def test_nnd_widest_rows_match_generic_kernel_and_oracle(mods, monkeypatch, pera, perb):
    """A 1024-cell scan axis: 256 threads and 8 warps per velocity, so the
    cross-warp carry of the scan runs over up to 7 warp aggregates."""
    abi, cases, T = mods
    c = _case(cases, T, pera, perb, True, na=1024, nvx=4, nvy=4)
    c.ncx = 6
    g = abi.Solver(c, precision=T.HYB_PREC_MIXED)
    g.init_maxwellian()
    g.upload_f(_perturbed(g.download_f(), 5))
    f0 = g.download_f()
    monkeypatch.setenv("HYB_SWEEP_GENERIC", "1")
    h = abi.Solver(c, precision=T.HYB_PREC_MIXED)
    monkeypatch.delenv("HYB_SWEEP_GENERIC")
    h.upload_f(f0)
    o = O.Oracle(c, threads=0)
    o.upload_f(f0)
    for _ in range(2):
        g.step(1)
        h.step(1)
        o.step(1)
    fg, fh = g.download_f(), h.download_f()
    assert np.abs(fg - fh).max() <= TWIN_TOL * np.abs(fh).max()
    fi, fo = _interior_f(c, fg), _interior_f(c, o.frd())
    assert _rel(fi, fo) < MIXED_TOL, _rel(fi, fo)


def test_nnd_rhs_only_pass_matches_generic_kernel(mods, monkeypatch):
    """The RHS-only pass of the synthetic solve (f left unchanged) and the
    RHS store of the last iteration run through the same kernel."""
    abi, cases, T = mods
    c = _case(cases, T, False, True, True, dt=0.02)
    gk = dict(max_inner=12, inner_tol=0.0, inner_rtol=0.0, cfl=20.0)
    runs = []
    for generic in (0, 1):
        if generic:
            monkeypatch.setenv("HYB_SWEEP_GENERIC", "1")
        s = abi.Solver(c, precision=T.HYB_PREC_MIXED)
        monkeypatch.delenv("HYB_SWEEP_GENERIC", raising=False)
        s.init_maxwellian()
        s.gsis(**gk)
        r = s.step(3)
        runs.append((s.download_f(), r))
    (fa, ra), (fb, rb) = runs
    assert np.abs(fa - fb).max() <= TWIN_TOL * np.abs(fb).max()
    for k in range(4):
        assert abs(ra["res_rms"][k] - rb["res_rms"][k]) <= 1e-5 * max(rb["res_rms"][k], 1e-12)
