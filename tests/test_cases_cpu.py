"""The benchmark workloads' set-up (host side, no GPU).

The named configurations carry the sizes and physical parameters of the
workloads they stand for. The batch manifest is seeded, stays within its
stated ranges and has every mesh and velocity-grid size. The bench's dt
rule keeps dt / dy, and with it the kinetic CFL, equal over the instances.
The wall tables of the sine case follow T_w(x) = 1 + 0.1 sin(2 pi x) at the
face centres.
"""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def cm(pkg):
    from hyb_gb300 import cases
    return cases


def test_named_configurations(cm):
    from hyb_gb300 import hyb_types as T
    s = cm.couette_small()
    assert (s.ncx, s.ncy, s.nvx, s.nvy, s.vmax, s.kn, s.uw) == (4, 64, 32, 32, 5.0, 0.1, 0.2)
    assert s.t_bottom == s.t_top == 1.0 and s.precision == T.HYB_PREC_FP64
    g = cm.couette_large()
    assert (g.ncx, g.ncy, g.nvx, g.nvy, g.vmax, g.kn, g.uw) == (128, 512, 64, 64, 6.0, 0.01, 0.5)
    assert (g.t_bottom, g.t_top) == (1.0, 1.2) and g.precision == T.HYB_PREC_MIXED
    assert g.cells * g.nv == 268_435_456
    w = cm.couette_sine()
    assert (w.ncx, w.ncy, w.nvx, w.nvy, w.vmax, w.kn, w.uw, w.t_pert) == (512, 512, 48, 48, 5.0, 0.005, 0.3, 0.1)
    assert w.cells * w.nv == 603_979_776      # "about 600 M" cell-velocities, 1.2 G values with G and H


def test_gas_and_collision_parameters(cm):
    p = cm.couette_small().params()
    assert p.cpr == pytest.approx((1.0 - 2.0 / 3.0) / 2.5)     # Shakhov 1 - Pr over 5/2
    assert p.x1s == pytest.approx(0.5)                          # hard sphere, omega 0.5
    assert p.cfc == pytest.approx(math.sqrt(math.pi) / (2.0 * 0.1))


def test_sine_wall_temperature(cm):
    c = cm.couette_sine(ncx=16, ncy=8, nvx=8, nvy=8)
    _, _, t = c.walls()
    xc = (np.arange(16) + 0.5) / 16
    ref = 1.0 + 0.1 * np.sin(2.0 * np.pi * xc)
    assert np.allclose(t[1], ref) and np.allclose(t[3], ref)


def test_batch_manifest_is_seeded_and_in_range(cm):
    a, b = cm.batch_manifest(), cm.batch_manifest()
    assert a == b and len(a) == 256
    assert a != cm.batch_manifest(seed=1)
    sizes = set()
    for d in a:
        assert d["ncx"] == 4 and d["ncy"] in (32, 64, 128, 256)
        assert d["nvx"] == d["nvy"] and d["nvx"] in (24, 32, 48, 64)
        assert d["vmax"] == (5.0 if d["nvx"] < 48 else 6.0)
        assert 1e-3 <= d["kn"] <= 10.0
        assert 0.05 <= d["uw"] <= 0.8
        assert d["t_bottom"] == 1.0 and 0.8 <= d["t_top"] <= 1.5
        sizes.add((d["ncy"], d["nvx"]))
    assert len(sizes) == 16                    # every mesh x velocity-grid size occurs
    kn = np.log10([d["kn"] for d in a])
    assert kn.min() < -2.5 and kn.max() > 0.5  # log-uniform over four decades


def test_bench_batch_cases_keep_the_kinetic_cfl(cm):
    # bench.py scales dt with the cell size, so that dt / dy (and with it the
    # kinetic CFL of a velocity range) is the same for every instance
    import bench
    cl = bench.batch_cases()
    assert len(cl) == 256 and all(c.precision == 1 for c in cl)
    ratios = {round(c.dt * c.ncy / c.ly, 12) for c in cl}
    assert ratios == {0.64}


def test_bench_time_to_residual_report_shape(cm, monkeypatch):
    """time_to_residual's bookkeeping (field errors against the FP64 runs,
    the wall-time ratios of the large case) on stand-in runs: no GPU, no
    solver; every run the bench makes returns a fixed record."""
    import numpy as np
    import bench
    calls = []

    def fake(name, case, prec, gsis=None, promote=False, learned=False, tol=1e-8, max_iters=8000, chunk=50,
             wall_s=None):
        calls.append((name, case.name, prec, promote, learned, max_iters))
        S = np.full((case.ncy - 1, case.ncx - 1, 4), 1.0 + 1e-9 * len(calls))
        return {"seconds": 10.0 if "fp64" in name and "to_fp64" not in name else 4.0, "iterations": 100,
                "residual": 5e-9, "reached": True}, S

    monkeypatch.setattr(bench, "_ttr_run", fake)
    out = bench.time_to_residual(large=True)
    lg = out["large"]["runs"]
    assert set(lg) == {"gsis_fp64_line_mean", "gsis_mixed_line_mean_to_fp64",
                       "gsis_mixed_learned_line_mean_to_fp64", "gsis_mixed_without_line_mean", "plain_mixed"}
    for name in ("gsis_mixed_line_mean_to_fp64", "gsis_mixed_learned_line_mean_to_fp64"):
        assert lg[name]["wall_time_ratio_fp64_over_this"] == 2.5
        assert set(lg[name]["field_rel_err_vs_fp64"]) == {"rho", "u", "v", "T"}
    assert all(r["field_rel_err_vs_fp64"] is not None for r in out["runs"].values())
    # the large case's runs are the 128x512 workload; the learned one loads the closure
    large = [c for c in calls if c[1].startswith("couette-128x512")]
    assert len(large) == 5 and sum(c[4] for c in large) == 1


def test_bench_time_to_residual_sine_report_shape(cm, monkeypatch):
    import numpy as np
    import bench
    calls = []

    def fake(name, case, prec, gsis=None, promote=False, learned=False, tol=1e-8, max_iters=8000, chunk=50,
             wall_s=None, finish_below=None, finish_gsis=None):
        calls.append((name, case.name, (gsis or {}).get("line_mean", 0), learned, max_iters))
        return {"seconds": 1.0, "iterations": max_iters, "residual": 1e-3, "reached": False}, np.zeros(1)

    monkeypatch.setattr(bench, "_ttr_run", fake)
    out = bench.time_to_residual_sine()
    assert set(out["runs"]) == {"plain_mixed", "gsis_mixed_harmonics", "gsis_mixed_learned_harmonics",
                                "gsis_mixed_line_mean", "gsis_mixed_without_line_mean",
                                "gsis_mixed_harmonics_to_fp64_then_moments_only"}
    assert all(c[1].startswith("couette-512x512") for c in calls)
    assert [c[2] for c in calls] == [0, 3, 3, 1, 0, 3]
    assert [c[3] for c in calls] == [False, False, True, False, False, False]


class _FakeSolver:
    """Stands in for abi.Solver in the time-to-residual runner: the residual
    falls by 0.7 per outer iteration to a floor of 5e-8 while the synthetic
    solve corrects the distribution, and by 0.95 per iteration below it
    once it corrects the moments only or is off."""

    def __init__(self, case, precision=0):
        self.case, self.res, self.floored, self.calls = case, 1.0, False, []

    def init_maxwellian(self):
        pass

    def attach_mlp(self, m):
        pass

    def gsis(self, **kw):
        self.floored = kw.get("enable", 1) == 1 and kw.get("correct_f", 0) == 1
        self.calls.append(("gsis", kw.get("enable", 1), kw.get("correct_f", 0)))

    def set_precision(self, p):
        self.calls.append(("precision", p))

    def step(self, n):
        for _ in range(n):
            self.res = max(5e-8, 0.7 * self.res) if self.floored else 0.95 * self.res
        return {"max_rms": self.res}

    def moments(self):
        import numpy as np
        c = self.case
        return np.zeros((c.ny + 7) * (c.nx + 7) * 11), None

    def gsis_skipped(self):
        return 0

    def close(self):
        pass


def test_bench_finishes_with_the_moments_only_correction_at_the_synthetic_floor(cm, monkeypatch):
    import bench
    from hyb_gb300 import hyb_types as T
    made = []

    def make(case, precision=0):
        made.append(_FakeSolver(case, precision))
        return made[-1]

    monkeypatch.setattr(bench.abi, "Solver", make)
    c = cm.couette_small(dt=1.0e6, sweep_order=1, mass_pin=1)
    g = dict(ns_solver=2, line_mean=3, ns_scheme=2, correct_f=1)
    out, _ = bench._ttr_run("x", c, T.HYB_PREC_FP64, g, False, False, tol=1e-8, max_iters=2000, chunk=10,
                            finish_below=1e-6, finish_gsis=dict(g, correct_f=0))
    assert out["reached"] and out["finish_from_iteration"] is not None
    assert made[-1].calls == [("gsis", 1, 1), ("gsis", 1, 0)]
    # without the finishing switch the run stays on the floor
    out2, _ = bench._ttr_run("x", c, T.HYB_PREC_FP64, g, False, False, tol=1e-8, max_iters=300, chunk=10)
    assert not out2["reached"] and "finish_from_iteration" not in out2
