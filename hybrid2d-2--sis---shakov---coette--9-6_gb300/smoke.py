"""One tiny kinetic iteration on cuda:0 checked against the CPU oracle."""
import sys
import time

import numpy as np

from . import abi, cases


def run():
    from oracle import oracle as O   # the checker only
    c = cases.couette_small(ncy=32, nvx=16, nvy=16, dt=0.05)
    t0 = time.time()
    g = abi.Solver(c, precision=0)
    g.init_maxwellian()
    rg = g.step(2)
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    ro = o.step(2)
    P = (c.nx + 7) * (c.ny + 7)
    fg = g.download_f().reshape(c.nv, c.ny + 7, c.nx + 7, 2)[:, 4:4 + c.ny - 1, 4:4 + c.nx - 1]
    fo = o.frd().reshape(c.nv, c.ny + 7, c.nx + 7, 2)[:, 4:4 + c.ny - 1, 4:4 + c.nx - 1]
    err = float(np.abs(fg - fo).max() / np.abs(fo).max())
    rerr = abs(rg["max_rms"] - ro["max_rms"]) / ro["max_rms"]
    launches = g.launches()
    g.close()
    print(f"smoke: {c.name} fp64 2 steps on cuda:0: max rel f err {err:.2e}, residual rel err {rerr:.2e}, "
          f"{launches} kernel launches, {time.time() - t0:.1f}s")
    if not (err < 1e-11 and rerr < 1e-9):
        raise AssertionError(f"GPU result differs from the oracle: f {err:.3e} residual {rerr:.3e}")
    # mixed precision path as well
    g = abi.Solver(c, precision=1)
    g.init_maxwellian()
    rm = g.step(2)
    g.close()
    if not (abs(rm["max_rms"] - ro["max_rms"]) < 1e-3 * ro["max_rms"]):
        raise AssertionError("mixed-precision residual far from the FP64 oracle")
    # a 128-cell scan axis: the specialised FP32 sweep (k_sweep_nnd4) and the
    # packed FP32 moment pass (k_moments_f2), as on the large workloads
    c = cases.couette_small(name="couette-4x128-nv8-kn0.1", ncy=128, nvx=8, nvy=8, dt=0.05)
    g = abi.Solver(c, precision=1)
    g.init_maxwellian()
    rm = g.step(2)
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    ro = o.step(2)
    fg = g.download_f().reshape(c.nv, c.ny + 7, c.nx + 7, 2)[:, 4:4 + c.ny - 1, 4:4 + c.nx - 1]
    fo = o.frd().reshape(c.nv, c.ny + 7, c.nx + 7, 2)[:, 4:4 + c.ny - 1, 4:4 + c.nx - 1]
    g.close()
    err = float(np.abs(fg - fo).max() / np.abs(fo).max())
    print(f"smoke: {c.name} mixed 2 steps on cuda:0: max rel f err {err:.2e} (FP32 distribution)")
    if not (err < 5e-5 and abs(rm["max_rms"] - ro["max_rms"]) < 1e-3 * ro["max_rms"]):
        raise AssertionError(f"mixed-precision GPU result far from the FP64 oracle: f {err:.3e}")
    # the synthetic solve: band to the walls, line solver with the
    # line-averaged correction and two harmonics across the periodic axis,
    # on a sine-wall channel (16 x 96, 12^2 velocities), three outer
    # iterations; the line elimination is FP32, so 1e-5
    c = cases.couette_small(name="couette-16x96-nv12-kn0.1-sine", ncx=16, ncy=96, nvx=12, nvy=12, t_pert=0.1,
                            dt=1.0e6, sweep_order=1, mass_pin=1)
    gk = dict(wall_band=1, correct_f=1, ns_solver=2, line_mean=3, cfl=20.0, max_inner=12, inner_tol=0.0,
              inner_rtol=0.0)
    g = abi.Solver(c, precision=0)
    g.init_maxwellian()
    g.gsis(**gk)
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    o.convert_ns()
    o.gsis(**gk)
    for _ in range(3):
        g.step(1)
        o.step(1)
    fg = g.download_f().reshape(c.nv, c.ny + 7, c.nx + 7, 2)[:, 4:4 + c.ny - 1, 4:4 + c.nx - 1]
    fo = o.frd().reshape(c.nv, c.ny + 7, c.nx + 7, 2)[:, 4:4 + c.ny - 1, 4:4 + c.nx - 1]
    skipped = (g.gsis_skipped(), o.gsis_skipped())
    g.close()
    err = float(np.abs(fg - fo).max() / np.abs(fo).max())
    print(f"smoke: {c.name} GSIS (line solver, line_mean 3) 3 outer iterations on cuda:0: max rel f err {err:.2e}")
    if not (err < 1e-5 and skipped == (0, 0)):
        raise AssertionError(f"synthetic solve far from the oracle: f {err:.3e}, skipped {skipped}")


if __name__ == "__main__":
    sys.exit(run())
