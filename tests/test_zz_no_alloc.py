"""hyb_detfp_noalloc: DETFP on caller-owned device arrays, no allocation.

It serves callers that cannot let the library allocate device memory (a CUDA
Fortran / OpenACC host that owns FRD and S_GKUA on the device, or a process
whose device memory is reserved by another allocator).  The test plays such a
caller: it owns the device buffers (allocated here, by the test) and checks
the entry point's S_GKUA and CF against the context path's hyb_detfp output
for the same distribution, on two calls in a row, within the FP64 parity
tolerance of the other GPU tests (1e-12 relative), and its S_GKUA against the
oracle's DETFP of the same distribution.

Kept in its own file, collected last, so that a failure here cannot hide the
other GPU tests in a run that stops at the first failure.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_CELLS = 209715   # HYB_NOALLOC_MAX_CELLS in include/hyb_dvm.h


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            L = C.CDLL(name)
            L.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
            L.cudaFree.argtypes = [C.c_void_p]
            L.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            L.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
            L.cudaMemGetInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
            L.cudaDeviceSynchronize.argtypes = []
            return L
        except OSError:
            continue
    pytest.skip("CUDA runtime library not found")


class DevBuf:
    """Device buffer owned by the caller (this test)."""

    def __init__(self, rt, host):
        self.rt, self.n = rt, host.nbytes
        self.p = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.p), self.n) == 0
        assert rt.cudaMemcpy(self.p, host.ctypes.data, self.n, 1) == 0   # host -> device

    def get(self, like):
        out = np.empty_like(like)
        assert self.rt.cudaMemcpy(out.ctypes.data, self.p, self.n, 2) == 0   # device -> host
        return out

    def fill(self, byte):
        assert self.rt.cudaMemset(self.p, byte, self.n) == 0

    def free(self):
        self.rt.cudaFree(self.p)


def _interior(case, s_gkua):
    S = s_gkua.reshape(case.ny + 7, case.nx + 7, 11)
    return S[4:4 + case.ny - 1, 4:4 + case.nx - 1, :10]


def _cf_interior(case, cf):
    return cf.reshape(case.ny + 3, case.nx + 3)[2:2 + case.ny - 1, 2:2 + case.nx - 1]


@pytest.mark.parametrize("shape", [dict(ncy=32, nvx=16, nvy=16), dict(ncx=40, ncy=8, nvx=12, nvy=20)])
def test_detfp_noalloc_matches_context_path(pkg, shape):
    from hyb_gb300 import abi, cases
    rt = _cudart()
    c = cases.couette_small(dt=0.02, **shape)
    g = abi.Solver(c, precision=0)
    g.init_maxwellian()
    g.step(3)
    frd = g.download_f()
    s_ref, cf_ref = g.moments()          # the context path: hyb_detfp on the same f
    g.close()
    from oracle.oracle import Oracle
    o = Oracle(c)
    o.upload_f(frd)
    o.detfp()
    s_orc = o.s_gkua()
    vi, wi, vj, wj = (np.ascontiguousarray(a, dtype=np.float64) for a in c.vgrid())
    bufs = [DevBuf(rt, a) for a in (frd, vi, vj, wi, wj, np.zeros_like(s_ref), np.zeros_like(cf_ref))]
    dfrd, dvi, dvj, dwi, dwj, ds, dcf = bufs
    p = c.params()
    L = abi.load()
    try:
        for call in range(2):
            ds.fill(0xFF)                 # NaN pattern: every compared value must be written
            dcf.fill(0xFF)
            rc = L.hyb_detfp_noalloc(c.nx, c.ny, c.nvx, c.nvy, dfrd.p, dvi.p, dvj.p, dwi.p, dwj.p, C.byref(p),
                                     ds.p, dcf.p, None)
            assert rc == 0, (call, rc)
            s_out, cf_out = ds.get(s_ref), dcf.get(cf_ref)
            a, b = _interior(c, s_out), _interior(c, s_ref)
            for k in range(10):
                scale = max(np.abs(b[..., k]).max(), 1e-3)
                assert np.abs(a[..., k] - b[..., k]).max() <= 1e-12 * scale, (call, k)
            a, b = _interior(c, s_out), _interior(c, s_orc)
            for k in range(10):
                scale = max(np.abs(b[..., k]).max(), 1e-3)
                assert np.abs(a[..., k] - b[..., k]).max() <= 1e-12 * scale, ("oracle", call, k)
            ca, cb = _cf_interior(c, cf_out), _cf_interior(c, cf_ref)
            assert np.abs(ca - cb).max() <= 1e-12 * np.abs(cb).max(), call
    finally:
        for b in bufs:
            b.free()


def _free_bytes(rt):
    assert rt.cudaDeviceSynchronize() == 0
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def test_detfp_noalloc_allocates_nothing_up_to_its_limit(pkg):
    """Near HYB_NOALLOC_MAX_CELLS (409 x 512 cells) the scratch holds one
    velocity slice, so each slice sums several velocity rows; the result
    still matches the context path, and the device's free memory is the same
    before and after calls at the smallest and the largest accepted sizes."""
    from hyb_gb300 import abi, cases
    rt = _cudart()
    c = cases.couette_small(ncx=409, ncy=512, nvx=6, nvy=6, dt=0.02)
    assert c.cells <= MAX_CELLS and 2 * c.cells > MAX_CELLS
    g = abi.Solver(c, precision=0)
    g.init_maxwellian()
    g.step(1)
    frd = g.download_f()
    s_ref, cf_ref = g.moments()
    g.close()
    small = cases.couette_small(ncy=16, nvx=4, nvy=4)
    vi, wi, vj, wj = (np.ascontiguousarray(a, dtype=np.float64) for a in c.vgrid())
    bufs = [DevBuf(rt, a) for a in (frd, vi, vj, wi, wj, np.zeros_like(s_ref), np.zeros_like(cf_ref))]
    dfrd, dvi, dvj, dwi, dwj, ds, dcf = bufs
    p = c.params()
    L = abi.load()
    try:
        args = (c.nx, c.ny, c.nvx, c.nvy, dfrd.p, dvi.p, dvj.p, dwi.p, dwj.p, C.byref(p), ds.p, dcf.p, None)
        assert L.hyb_detfp_noalloc(*args) == 0            # first call on the device: set-up
        free0 = _free_bytes(rt)
        for call in range(2):
            ds.fill(0xFF)
            assert L.hyb_detfp_noalloc(*args) == 0
            # the small mesh reads the same (larger) buffers: any valid sub-range will do
            assert L.hyb_detfp_noalloc(small.nx, small.ny, 4, 4, dfrd.p, dvi.p, dvj.p, dwi.p, dwj.p, C.byref(p),
                                       dcf.p, None, None) == 0
            ds.fill(0xFF)
            assert L.hyb_detfp_noalloc(*args) == 0
            a, b = _interior(c, ds.get(s_ref)), _interior(c, s_ref)
            for k in range(10):
                scale = max(np.abs(b[..., k]).max(), 1e-3)
                assert np.abs(a[..., k] - b[..., k]).max() <= 1e-12 * scale, (call, k)
        assert _free_bytes(rt) == free0
    finally:
        for b in bufs:
            b.free()


def test_detfp_noalloc_rejects_sizes_beyond_its_scratch(pkg):
    from hyb_gb300 import abi, cases, hyb_types as T
    rt = _cudart()
    c = cases.couette_small(ncy=16, nvx=4, nvy=4)
    tiny = DevBuf(rt, np.zeros(16))
    p = c.params()
    L = abi.load()
    try:
        # 512 x 512 cells is beyond HYB_NOALLOC_MAX_CELLS; rejected before any launch
        rc = L.hyb_detfp_noalloc(513, 513, 4, 4, tiny.p, tiny.p, tiny.p, tiny.p, tiny.p, C.byref(p), tiny.p, None,
                                 None)
        assert rc == T.HYB_ERR_UNSUPPORTED
        assert 512 * 512 > MAX_CELLS
        rc = L.hyb_detfp_noalloc(513, 513, 4, 4, None, tiny.p, tiny.p, tiny.p, tiny.p, C.byref(p), tiny.p, None,
                                 None)
        assert rc == T.HYB_ERR_INVALID
    finally:
        tiny.free()
