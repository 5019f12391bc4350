"""Converged-field parity with the reference's own iteration.

The 4x64 Couette channel at Kn 0.1 (32^2 Newton-Cotes velocities on [-5, 5],
plates at +-0.2), run with the reference's kinetic step exactly as
GKUA_Residual writes it (Hybrid2D/src/GKUA_Residual.f90:28-112: forward sweep
in increasing (i, j), backward step on the forward values, dt_global 0.01,
NND) until the residual of DETFP_res (Hybrid2D/src/GKUA_DETFP_RES.f90:45-54)
is below 1e-8, on the GPU in FP64 and in the CPU oracle: the converged
moments agree to 1e-10 relative.  The mixed-precision GPU path, stopped on
its FP32 floor and finished in FP64 on the device (hyb_set_precision),
reaches the reference's fields within 1e-5 relative: this iteration does not
conserve mass, so its FP32 part ends on a neighbouring member of the
mass-indexed family of steady states (measured: a uniform density shift of
8.2e-6).  With the mass pin the two precisions end on the same member to
1e-7 (tests/test_gpu_promote.py).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _interior(case, s):
    return s.reshape(case.ny + 7, case.nx + 7, 11)[4:4 + case.ny - 1, 4:4 + case.nx - 1, :10]


def _run_gpu(abi, c, prec, promote=False):
    from hyb_gb300 import hyb_types as T
    s = abi.Solver(c, precision=prec)
    s.init_maxwellian()
    it, prev = 0, None
    while it < 6000:
        r = s.step(50)
        it += 50
        if promote and prec == T.HYB_PREC_MIXED and prev is not None and r["max_rms"] > 0.95 * prev:
            s.set_precision(T.HYB_PREC_FP64)
            prec = T.HYB_PREC_FP64
        prev = r["max_rms"]
        if r["max_rms"] < 1e-8:
            break
    return it, r["max_rms"], _interior(c, s.moments()[0])


def test_reference_iteration_converges_to_the_oracle_fields(pkg):
    from hyb_gb300 import abi, cases
    c = cases.couette_small(dt=0.01)
    it_g, res_g, Sg = _run_gpu(abi, c, 0)
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    it_o = 0
    while it_o < 6000:
        ro = o.step(50)
        it_o += 50
        if ro["max_rms"] < 1e-8:
            break
    So = _interior(c, o.s_gkua())
    assert res_g < 1e-8 and ro["max_rms"] < 1e-8 and it_g == it_o, (it_g, res_g, it_o, ro["max_rms"])
    for k in range(10):
        scale = max(np.abs(So[..., k]).max(), 1e-3)
        assert np.abs(Sg[..., k] - So[..., k]).max() <= 1e-10 * scale, k
    # the mixed path, finished in FP64 on the device, ends on the same fields
    it_m, res_m, Sm = _run_gpu(abi, c, 1, promote=True)
    assert res_m < 1e-8, (it_m, res_m)
    for k in range(4):
        scale = max(np.abs(So[..., k]).max(), 1e-3)
        assert np.abs(Sm[..., k] - So[..., k]).max() <= 1e-5 * scale, k
