"""A native host of the C ABI (tests/c_host/hyb_host_couette.c), compiled
with the system C compiler against include/hyb_dvm.h and the built library.
It makes the call sequence of the patched Fortran host (create, Maxwellian,
one hyb_step per outer iteration, moments and FRD downloads) on arrays in
the reference's own layouts.

CPU: the host compiles and links against the ABI.  GPU: its downloads equal
those of the Python binding on the same case bit for bit (one library, the
same inputs, deterministic kernels), and match the oracle within the FP64
parity tolerance.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "c_host", "hyb_host_couette.c")
MAGIC = 0x48594231


def _lib_dir():
    from hyb_gb300 import abi
    return os.path.dirname(abi.LIB_PATH)


def _compile(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = _lib_dir()
    if not os.path.exists(os.path.join(lib, "libhyb_gb300.so")):
        pytest.skip("library not built")
    exe = str(tmp_path / "hyb_host_couette")
    cuda_lib = "/usr/local/cuda/lib64"
    cmd = [cc, "-O2", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", lib, "-lhyb_gb300", "-Wl,-rpath," + lib, "-Wl,-rpath-link," + cuda_lib, "-Wl,-rpath," + cuda_lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_native_host_compiles_against_the_abi(pkg, tmp_path):
    exe = _compile(tmp_path)
    assert os.path.exists(exe)


def _write_input(path, case, nsteps):
    from hyb_gb300 import hyb_types as T
    X, Y = case.nodes()
    vi, wi, vj, wj = case.vgrid()
    u, v, t = case.walls()
    hdr = np.array([MAGIC, C.sizeof(T.HybParams), case.nx, case.ny, case.nvx, case.nvy, nsteps] + list(case.bcs),
                   dtype=np.int32)
    with open(path, "wb") as fh:
        fh.write(hdr.tobytes())
        fh.write(bytes(case.params()))
        for a in (X.ravel(order="F"), Y.ravel(order="F"), vi, wi, vj, wj):
            fh.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        for f in range(4):
            if case.bcs[f] == T.HYB_BC_WALL:
                for a in (u[f], v[f], t[f]):
                    fh.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())


@pytest.mark.gpu
def test_native_host_matches_python_binding_and_oracle(pkg, tmp_path):
    from hyb_gb300 import abi, cases
    exe = _compile(tmp_path)
    c = cases.couette_small(ncy=32, nvx=16, nvy=16, dt=0.05)
    nsteps = 4
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(fin, c, nsteps)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(fout, dtype=np.float64)
    P = (c.nx + 7) * (c.ny + 7)
    n_res, n_s, n_cf, n_f = 9 * nsteps, 11 * P, (c.nx + 3) * (c.ny + 3), 2 * P * c.nv
    assert raw.size == n_res + n_s + n_cf + n_f
    res = raw[:n_res].reshape(nsteps, 9)
    S = raw[n_res:n_res + n_s]
    cf = raw[n_res + n_s:n_res + n_s + n_cf]
    frd = raw[n_res + n_s + n_cf:]
    # the Python binding, same case
    g = abi.Solver(c, precision=0)
    g.init_maxwellian()
    rg = [g.step(1) for _ in range(nsteps)]
    Sg, cfg = g.moments()
    fg = g.download_f()
    g.close()
    for k in range(nsteps):
        assert np.array_equal(res[k, 4:8], np.asarray(rg[k]["res_rms"])), k
        assert np.array_equal(res[k, 0:4], np.asarray(rg[k]["res_max"])), k
    assert np.array_equal(S, Sg) and np.array_equal(cf, cfg) and np.array_equal(frd, fg)
    # the oracle
    o = O.Oracle(c, threads=0)
    o.init_maxwellian()
    ro = o.step(nsteps)
    fo = o.frd()
    nv, ny, nx = c.nv, c.ny + 7, c.nx + 7
    a = frd.reshape(nv, ny, nx, 2)[:, 4:4 + c.ny - 1, 4:4 + c.nx - 1]
    b = fo.reshape(nv, ny, nx, 2)[:, 4:4 + c.ny - 1, 4:4 + c.nx - 1]
    assert np.abs(a - b).max() <= 1e-11 * np.abs(b).max()
    assert abs(res[-1, 8] - ro["max_rms"]) <= 1e-9 * ro["max_rms"]
