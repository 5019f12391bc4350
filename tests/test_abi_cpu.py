"""C-ABI checks that need no GPU: exports, struct layout, argument errors."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hyb_dvm.h")


def _declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+char\s*\*|int)\s*(hyb_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib(pkg):
    from hyb_gb300 import build, abi
    build.build_all()
    return abi.load()


def test_header_and_binding_agree(pkg):
    from hyb_gb300 import abi
    assert _declared() == sorted(abi.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_version_string(lib):
    assert b"sm_103a" in lib.hyb_version()


def test_struct_layout_matches_c(pkg):
    from hyb_gb300 import hyb_types as T
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "hyb_dvm.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(hyb_mesh), sizeof(hyb_vgrid), sizeof(hyb_params),
         sizeof(hyb_residual), sizeof(hyb_gsis_params));
  printf("%zu %zu %zu %zu\n", offsetof(hyb_mesh, wall_t), offsetof(hyb_params, omega_ns),
         offsetof(hyb_params, device), offsetof(hyb_gsis_params, mlp_warm_after));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        cfile, exe = os.path.join(d, "p.c"), os.path.join(d, "p")
        open(cfile, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), cfile, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    sizes = [C.sizeof(T.HybMesh), C.sizeof(T.HybVgrid), C.sizeof(T.HybParams), C.sizeof(T.HybResidual),
             C.sizeof(T.HybGsisParams)]
    offs = [T.HybMesh.wall_t.offset, T.HybParams.omega_ns.offset, T.HybParams.device.offset,
            T.HybGsisParams.mlp_warm_after.offset]
    assert [int(x) for x in out] == sizes + offs


def test_invalid_arguments_are_rejected_without_a_device(lib, pkg):
    from hyb_gb300 import cases, hyb_types as T
    c = cases.couette_small(ncy=16, nvx=8, nvy=8)
    m, g, p, keep = c.c_structs()
    h = C.c_void_p()
    assert lib.hyb_create(None, C.byref(g), C.byref(p), C.byref(h)) == T.HYB_ERR_INVALID
    bad = T.HybParams.from_buffer_copy(p)
    bad.dt = -1.0
    assert lib.hyb_create(C.byref(m), C.byref(g), C.byref(bad), C.byref(h)) == T.HYB_ERR_INVALID
    bad = T.HybParams.from_buffer_copy(p)
    bad.precision = 7
    assert lib.hyb_create(C.byref(m), C.byref(g), C.byref(bad), C.byref(h)) == T.HYB_ERR_INVALID
    mm = T.HybMesh.from_buffer_copy(m)
    mm.bc[0] = 99
    assert lib.hyb_create(C.byref(mm), C.byref(g), C.byref(p), C.byref(h)) == T.HYB_ERR_UNSUPPORTED
    mm = T.HybMesh.from_buffer_copy(m)
    mm.bc[2] = T.HYB_BC_WALL       # periodic face without its partner
    assert lib.hyb_create(C.byref(mm), C.byref(g), C.byref(p), C.byref(h)) == T.HYB_ERR_INVALID
    # a valid request either needs a device or succeeds on one
    rc = lib.hyb_create(C.byref(m), C.byref(g), C.byref(p), C.byref(h))
    assert rc in (T.HYB_OK, T.HYB_ERR_NODEVICE)
    if rc == T.HYB_OK:
        lib.hyb_destroy(h)
    # null context calls fail cleanly
    assert lib.hyb_step(None, 1, None) == T.HYB_ERR_INVALID
    assert lib.hyb_destroy(None) == T.HYB_ERR_INVALID
    assert lib.hyb_last_error(None) == b"null context"


@pytest.mark.parametrize("ncy,ok", [(600, True), (602, False), (601, False), (256, True), (257, False), (255, True)])
def test_scan_axis_size_limits(lib, pkg, ncy, ok):
    """A sweep thread group must fit one 256-thread CTA: scan axes above 256
    cells need an even count, above 512 a multiple of 4 (checked before any
    device call)."""
    from hyb_gb300 import cases, hyb_types as T
    c = cases.couette_small(ncy=ncy, nvx=8, nvy=8)
    m, g, p, keep = c.c_structs()
    h = C.c_void_p()
    rc = lib.hyb_create(C.byref(m), C.byref(g), C.byref(p), C.byref(h))
    if ok:
        assert rc in (T.HYB_OK, T.HYB_ERR_NODEVICE)
        if rc == T.HYB_OK:
            lib.hyb_destroy(h)
    else:
        assert rc == T.HYB_ERR_UNSUPPORTED


def test_detfp_noalloc_rejects_misaligned_pointers_before_any_launch(lib, pkg):
    """hyb_detfp_noalloc reads and writes the caller's device arrays as
    doubles: a pointer that is not 8-byte aligned (an offset array section,
    say) is refused with HYB_ERR_INVALID before any CUDA call, so it never
    reaches a kernel.  The pointers here are never dereferenced."""
    from hyb_gb300 import cases, hyb_types as T
    p = cases.couette_small(ncy=16, nvx=4, nvy=4).params()
    good, odd = C.c_void_p(0x10000), C.c_void_p(0x10004)
    for k in range(6):
        ptrs = [good] * 6
        ptrs[k] = odd
        frd, vi, vj, wi, wj, s = ptrs
        rc = lib.hyb_detfp_noalloc(5, 17, 4, 4, frd, vi, vj, wi, wj, C.byref(p), s, None, None)
        assert rc == T.HYB_ERR_INVALID, k
    rc = lib.hyb_detfp_noalloc(5, 17, 4, 4, good, good, good, good, good, C.byref(p), good, odd, None)
    assert rc == T.HYB_ERR_INVALID
