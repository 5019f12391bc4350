"""Parity at the benchmark workloads' full sizes.

* The single large Couette (128 x 512 cells, 64^2 velocities, Kn 0.01):
  two outer iterations on the GPU against the FP64 oracle run on all host
  cores. The FP64 path must agree to 1e-11 of each field's magnitude in f
  and S_GKUA. The mixed path (FP32 f, FP64 moments) must agree to 5e-5 in f
  and 1e-5 in S_GKUA.
* The 512 x 512 Couette with the sinusoidal wall temperature (48^2
  velocities, Kn 0.005): one outer iteration, same tolerances.
* The seeded 256-instance batch, run whole: after two iterations, instances
  of every mesh size and velocity grid agree with the FP64 oracle to the
  mixed-precision tolerances.

f is compared one block of velocities at a time, so that the host needs
only one f-sized FP64 array beside the oracle's own.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _mem_available_gb():
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 1024 ** 2
    except OSError:
        pass
    return 0.0


@pytest.fixture(scope="module")
def cases_mod(pkg):
    from hyb_gb300 import cases
    return cases


def _f_rel(case, fg_flat, fo_flat, block=256):
    """max |f_gpu - f_oracle| over the interior / max |f_oracle|, by velocity blocks."""
    fg = fg_flat.reshape(case.nv, case.ny + 7, case.nx + 7, 2)
    fo = fo_flat.reshape(case.nv, case.ny + 7, case.nx + 7, 2)
    num = den = 0.0
    for v0 in range(0, case.nv, block):
        a = fg[v0:v0 + block, 4:4 + case.ny - 1, 4:4 + case.nx - 1, :]
        b = fo[v0:v0 + block, 4:4 + case.ny - 1, 4:4 + case.nx - 1, :]
        num = max(num, float(np.abs(a - b).max()))
        den = max(den, float(np.abs(b).max()))
    return num / max(den, 1e-300)


# components of S_GKUA(1:10) measured against one magnitude: density,
# velocity (u, v), temperature, stress (Pxx, Pyy, Pxy, tau_zz), heat flux
_S_GROUPS = ((0,), (1, 2), (3,), (4, 5, 6, 9), (7, 8))


def _s_rel(case, sg, so):
    """per-component max difference of S_GKUA(1:10) on the interior cells,
    relative to the magnitude of the component's field (velocity, stress and
    heat flux taken as a whole: their small components are near zero)"""
    A = sg.reshape(case.ny + 7, case.nx + 7, 11)[4:4 + case.ny - 1, 4:4 + case.nx - 1, :10]
    B = so.reshape(case.ny + 7, case.nx + 7, 11)[4:4 + case.ny - 1, 4:4 + case.nx - 1, :10]
    out = [0.0] * 10
    for grp in _S_GROUPS:
        scale = max(max(float(np.abs(B[..., k]).max()) for k in grp), 1e-12)
        for k in grp:
            out[k] = float(np.abs(A[..., k] - B[..., k]).max()) / scale
    return out


@pytest.fixture(scope="module")
def large_oracle(cases_mod):
    if _mem_available_gb() < 48.0:
        pytest.skip("needs about 30 GB of host memory for the full-size FP64 oracle")
    c = cases_mod.couette_large()
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    o.convert_ns()
    o.step(2)
    return c, o.frd(), o.s_gkua()


@pytest.mark.parametrize("precision,ftol,stol", [(0, 1e-11, 1e-11), (1, 5e-5, 1e-5)])
def test_large_couette_full_size(large_oracle, precision, ftol, stol):
    from hyb_gb300 import abi
    c, fo, so = large_oracle
    g = abi.Solver(c, precision=precision)
    g.init_maxwellian()
    g.step(2)
    assert _f_rel(c, g.download_f(), fo) < ftol
    s = _s_rel(c, g.moments()[0], so)
    assert max(s) < stol, s
    g.close()


@pytest.fixture(scope="module")
def sine_oracle(cases_mod):
    if _mem_available_gb() < 96.0:
        pytest.skip("needs about 60 GB of host memory for the full-size FP64 oracle")
    c = cases_mod.couette_sine()
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    o.convert_ns()
    o.step(1)
    return c, o.frd(), o.s_gkua()


@pytest.mark.parametrize("precision,ftol,stol", [(0, 1e-11, 1e-11), (1, 5e-5, 1e-5)])
def test_sine_couette_full_size(sine_oracle, precision, ftol, stol):
    from hyb_gb300 import abi
    c, fo, so = sine_oracle
    g = abi.Solver(c, precision=precision)
    g.init_maxwellian()
    g.step(1)
    assert _f_rel(c, g.download_f(), fo) < ftol
    s = _s_rel(c, g.moments()[0], so)
    assert max(s) < stol, s
    g.close()


def test_batch_manifest_full_size(cases_mod):
    from hyb_gb300 import abi
    cl = [cases_mod.Case(precision=1, dt=0.01 * 64.0 / d["ncy"], **d) for d in cases_mod.batch_manifest()]
    b = abi.Batch(cl, precision=1)
    b.init_maxwellian()
    res = b.step(2)
    assert all(np.isfinite(r["max_rms"]) for r in res)
    # one instance of every (mesh, velocity grid) size present
    picked = {}
    for k, c in enumerate(cl):
        picked.setdefault((c.ncy, c.nvx), k)
    for (ncy, nvx), k in sorted(picked.items()):
        c = cl[k]
        o = O.Oracle(c, threads=0)
        o.init_maxwellian()
        o.convert_ns()
        o.step(2)
        inst = b.instance(k)
        assert _f_rel(c, inst.download_f(), o.frd()) < 5e-5, (k, ncy, nvx)
        s = _s_rel(c, inst.moments()[0], o.s_gkua())
        assert max(s) < 1e-5, (k, ncy, nvx, s)
    b.close()
