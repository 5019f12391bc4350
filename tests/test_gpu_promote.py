"""hyb_set_precision: a mixed-precision context finishes in FP64 on the device.

The FP32 distribution is widened on the GPU (every FP32 value is exact in
FP64), so the promoted context must step exactly like a fresh FP64 context
into which the same distribution is uploaded through the host.  A mixed
run whose FP32 residual has stalled then converges to 1e-8 without a host
round trip of f, to the fields of the FP64 run within the mixed path's
stated error.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods(pkg):
    from hyb_gb300 import abi, cases, hyb_types as T
    return abi, cases, T


def _interior_s(case, s):
    return s.reshape(case.ny + 7, case.nx + 7, 11)[4:4 + case.ny - 1, 4:4 + case.nx - 1, :10]


@pytest.mark.parametrize("gsis", [0, 1])
def test_promoted_context_steps_like_an_fp64_context(mods, gsis):
    abi, cases, T = mods
    # no mass pin here: hyb_upload_f takes the uploaded state's mass as m0,
    # the promoted context keeps the initial one
    c = cases.couette_small(ncy=32, nvx=16, nvy=16, dt=1.0e6, sweep_order=1)
    gk = dict(wall_band=1, correct_f=1, ns_solver=0, cfl=20.0, max_inner=12, inner_tol=0.0, inner_rtol=0.0)
    m = abi.Solver(c, precision=T.HYB_PREC_MIXED)
    m.init_maxwellian()
    if gsis:
        m.gsis(**gk)
    m.step(5)
    frd = m.download_f()
    m.set_precision(T.HYB_PREC_FP64)
    d = abi.Solver(c, precision=T.HYB_PREC_FP64)
    d.upload_f(frd)
    if gsis:
        d.gsis(**gk)
    rm = m.step(4)
    rd = d.step(4)
    fm, fd = m.download_f(), d.download_f()
    assert np.abs(fm - fd).max() <= 1e-13 * np.abs(fd).max()
    Sm, Sd = _interior_s(c, m.moments()[0]), _interior_s(c, d.moments()[0])
    assert np.abs(Sm - Sd).max() <= 1e-12
    assert abs(rm["max_rms"] - rd["max_rms"]) <= 1e-10 * rd["max_rms"]


def test_promotion_rules(mods):
    abi, cases, T = mods
    c = cases.couette_small(ncy=16, nvx=8, nvy=8)
    d = abi.Solver(c, precision=T.HYB_PREC_FP64)
    d.set_precision(T.HYB_PREC_FP64)                      # same precision: no-op
    with pytest.raises(abi.HybError) as e:
        d.set_precision(T.HYB_PREC_MIXED)                 # only MIXED -> FP64
    assert e.value.rc == T.HYB_ERR_UNSUPPORTED


def test_mixed_run_finishes_in_fp64_on_the_device(mods):
    """The 4x64 Kn 0.1 channel, upwind-ordered kinetic iteration at dt 1e6
    with the mass pin: the FP32 residual stops falling near 1e-6; promoted
    at that point, the run reaches 1e-8 and its fields agree with an FP64
    run of the same iteration to 1e-7."""
    abi, cases, T = mods
    c = cases.couette_small(dt=1.0e6, sweep_order=1, mass_pin=1)
    runs = {}
    for prec in (T.HYB_PREC_MIXED, T.HYB_PREC_FP64):
        s = abi.Solver(c, precision=prec)
        s.init_maxwellian()
        it, promoted, prev = 0, None, None
        while it < 600:
            r = s.step(10)
            it += 10
            res = r["max_rms"]
            if prec == T.HYB_PREC_MIXED and promoted is None and prev is not None and res > 0.5 * prev:
                s.set_precision(T.HYB_PREC_FP64)          # the FP32 residual stopped falling
                promoted = it
            prev = res
            if res < 1e-8:
                break
        runs[prec] = (it, res, promoted, _interior_s(c, s.moments()[0]))
    it_m, res_m, promoted, Sm = runs[T.HYB_PREC_MIXED]
    it_d, res_d, _, Sd = runs[T.HYB_PREC_FP64]
    assert res_m < 1e-8 and res_d < 1e-8, (runs[T.HYB_PREC_MIXED][:3], runs[T.HYB_PREC_FP64][:3])
    assert promoted is not None and promoted < it_m
    for k in range(4):
        scale = max(np.abs(Sd[..., k]).max(), 1e-2)
        assert np.abs(Sm[..., k] - Sd[..., k]).max() <= 1e-7 * scale, k
