"""Bounded device waits that run out, on the GPU, without a fault.

Every mbarrier wait of the kinetic sweep and of the moment pass, and the
grid barrier of the synthetic solve's cooperative inner loop, give up after
a limit of SM clocks, set an error word and return; the host reports
HYB_ERR_TIMEOUT.  hyb_test_stall plants, for one step, a wait that nothing
completes (a row copy the sweep never issues; a block that never arrives at
the grid barrier) and shortens the limit to a few hundred microseconds.  The
tests check the status and that the same context then steps on exactly as
the oracle does.
"""
import numpy as np
import pytest

from oracle import oracle as O

from test_gpu_parity import _cmp_state

pytestmark = pytest.mark.gpu

SPIN = 400_000          # SM clocks, about 0.2 ms at 2 GHz


@pytest.fixture(scope="module")
def mods(pkg):
    from hyb_gb300 import abi, cases, hyb_types as T
    return abi, cases, T


def _pair(abi, case, precision):
    g = abi.Solver(case, precision=precision)
    o = O.Oracle(case, threads=0)
    g.init_maxwellian()
    o.init_maxwellian()
    o.convert_ns()
    return g, o


@pytest.mark.parametrize("precision,order,ncy", [(0, 0, 32), (1, 0, 32), (0, 1, 32), (1, 0, 128)])
def test_sweep_row_wait_runs_out_and_context_recovers(mods, precision, order, ncy):
    """ncy = 128 runs the specialised FP32 NND sweep (4 cells per thread)."""
    abi, cases, T = mods
    c = cases.couette_small(ncy=ncy, nvx=16, nvy=16, dt=0.05 if order == 0 else 1.0e6, sweep_order=order)
    g, o = _pair(abi, c, precision)
    g.step(2)
    o.step(2)
    f_before = g.download_f()
    g.test_stall(T.HYB_STALL_SWEEP_ROW, SPIN)
    with pytest.raises(abi.HybError) as e:
        g.step(1)
    assert e.value.rc == T.HYB_ERR_TIMEOUT
    # the CTAs returned before writing f: the state is the one before the step
    assert np.array_equal(g.download_f(), f_before)
    g.step(2)
    o.step(2)
    _cmp_state(c, g, o, 1e-11 if precision == 0 else 5e-5)


def test_grid_barrier_wait_runs_out_and_context_recovers(mods):
    """The cooperative LU-SGS inner loop (band 3..n-3, small mesh): with one
    block that never arrives, every block gives up at the first barrier.  The
    outer iteration's kinetic part has run; the oracle replays that step
    without the synthetic solve, and both then continue with it."""
    abi, cases, T = mods
    c = cases.couette_small(ncy=32, nvx=16, nvy=16, dt=0.02)
    g, o = _pair(abi, c, 0)
    gk = dict(max_inner=12, inner_tol=0.0, inner_rtol=0.0, cfl=20.0)
    g.gsis(**gk)
    o.gsis(**gk)
    g.step(1)
    o.step(1)
    g.test_stall(T.HYB_STALL_NS_BARRIER, SPIN)
    with pytest.raises(abi.HybError) as e:
        g.step(1)
    assert e.value.rc == T.HYB_ERR_TIMEOUT
    o.gsis(enable=0)
    o.step(1)
    o.gsis(**gk)
    for _ in range(2):
        g.step(1)
        o.step(1)
        assert g.gsis_last_inner() == o.gsis_last_inner() == gk["max_inner"]
    _cmp_state(c, g, o, 1e-10)


def test_stall_arguments_are_checked(mods):
    abi, cases, T = mods
    g = abi.Solver(cases.couette_small(ncy=16, nvx=8, nvy=8), precision=0)
    with pytest.raises(abi.HybError):
        g.test_stall(7, SPIN)
    with pytest.raises(abi.HybError):
        g.test_stall(T.HYB_STALL_SWEEP_ROW, 0)
    g.test_stall(T.HYB_STALL_NONE, SPIN)
    g.init_maxwellian()
    g.step(1)
