"""ctypes driver of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker.  It is never imported by the product package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhyb_oracle.so")

_lib = None


def _sources():
    own = [os.path.join(HERE, n) for n in os.listdir(HERE) if n.endswith((".c", ".h")) or n == "Makefile"]
    return own + [os.path.join(os.path.dirname(HERE), "include", "hyb_dvm.h")]


def build(force=False):
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(p) for p in _sources() if os.path.exists(p)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, ip, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        L.orc_create.argtypes = [vp, vp, vp, C.POINTER(vp)]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_threads.argtypes = [ip]
        L.orc_init_maxwellian.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double]
        for fn in ("orc_exchange_f", "orc_phy_boundary", "orc_kinetic_step", "orc_detfp", "orc_convert_ns"):
            getattr(L, fn).argtypes = [vp]
        L.orc_detfp_res.argtypes = [vp, vp]
        L.orc_step.argtypes = [vp, ip, vp]
        for fn in ("orc_frd", "orc_frd00", "orc_s", "orc_cf"):
            getattr(L, fn).argtypes = [vp]
            getattr(L, fn).restype = dp
        L.orc_upload_f.argtypes = [vp, dp]
        L.orc_hot.argtypes = [vp, dp, dp, dp, dp]
        L.orc_hoq.argtypes = [vp, dp, dp]
        L.orc_nsf_in.argtypes = [vp, dp, dp, dp, dp]
        L.orc_err.argtypes = [vp]
        L.orc_err.restype = C.c_double
        L.orc_geometry.argtypes = [vp] + [dp] * 9
        L.orc_grid_gl.argtypes = [C.c_double, ip, C.c_double, ip, ip, dp, dp]
        L.orc_grid_nc.argtypes = [ip, C.c_double, C.c_double, ip, dp, dp]
        L.orc_cfc_vhs.argtypes = [C.c_double] * 10 + [dp]
        L.orc_cfc_vhs.restype = C.c_double
        L.orc_gsis_configure.argtypes = [vp, vp]
        L.orc_gsis_last_inner.argtypes = [vp]
        L.orc_gsis_skipped.argtypes = [vp]
        L.orc_ns_state.argtypes = [vp, dp]
        L.orc_ns_residual.argtypes = [vp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """One oracle instance for a cases.Case."""

    def __init__(self, case, threads=0):
        from_types = case.c_structs()
        self.case = case
        self._m, self._g, self._p, self._keep = from_types
        self.L = lib()
        if threads:
            self.L.orc_set_threads(threads)
        h = C.c_void_p()
        rc = self.L.orc_create(C.byref(self._m), C.byref(self._g), C.byref(self._p), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"orc_create failed: {rc}")
        self.h = h
        self.nx, self.ny, self.nv = case.nx, case.ny, case.nv
        self.P = (self.nx + 7) * (self.ny + 7)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # ---- stages ------------------------------------------------------------
    def init_maxwellian(self, rho=1.0, u=0.0, v=0.0, t=1.0):
        return self.L.orc_init_maxwellian(self.h, rho, u, v, t)

    def exchange_f(self):
        return self.L.orc_exchange_f(self.h)

    def phy_boundary(self):
        return self.L.orc_phy_boundary(self.h)

    def kinetic_step(self):
        return self.L.orc_kinetic_step(self.h)

    def detfp(self):
        return self.L.orc_detfp(self.h)

    def convert_ns(self):
        return self.L.orc_convert_ns(self.h)

    def residual(self):
        from importlib import import_module
        T = _types()
        r = T.HybResidual()
        self.L.orc_detfp_res(self.h, C.byref(r))
        return r.as_dict()

    def step(self, n=1):
        T = _types()
        r = T.HybResidual()
        rc = self.L.orc_step(self.h, n, C.byref(r))
        if rc != 0:
            raise RuntimeError(f"orc_step failed: {rc}")
        return r.as_dict()

    # ---- state -------------------------------------------------------------
    def frd(self):
        """FRD(NRD,-3:nx+3,-3:ny+3,NVI,NVJ) as a Fortran-ordered array view copy."""
        n = 2 * self.P * self.nv
        a = np.ctypeslib.as_array(self.L.orc_frd(self.h), shape=(n,)).copy()
        return a

    def frd00(self):
        n = 2 * self.P * self.nv
        return np.ctypeslib.as_array(self.L.orc_frd00(self.h), shape=(n,)).copy()

    def s_gkua(self):
        n = 11 * self.P
        return np.ctypeslib.as_array(self.L.orc_s(self.h), shape=(n,)).copy()

    def cf(self):
        return np.ctypeslib.as_array(self.L.orc_cf(self.h), shape=(self.P,)).copy()

    def upload_f(self, frd):
        frd = np.ascontiguousarray(frd, dtype=np.float64)
        return self.L.orc_upload_f(self.h, _dp(frd))

    def hot(self):
        nc = (self.nx + 3) * (self.ny + 3)
        ti, qi, tj, qj = np.zeros(4 * nc), np.zeros(2 * nc), np.zeros(4 * nc), np.zeros(2 * nc)
        self.L.orc_hot(self.h, _dp(ti), _dp(qi), _dp(tj), _dp(qj))
        return ti, qi, tj, qj

    def hoq(self):
        """HOT_GKUA(6, -3:nx+3, -3:ny+3), HOQ_GKUA(4, ...) of the current FRD."""
        hot, hoq = np.zeros(6 * self.P), np.zeros(4 * self.P)
        self.L.orc_hoq(self.h, _dp(hot), _dp(hoq))
        return hot, hoq

    def gsis(self, **kw):
        T = _types()
        gp = T.HybGsisParams()
        gp.enable = kw.get("enable", 1)
        gp.max_inner = kw.get("max_inner", 2000)
        gp.inner_tol = kw.get("inner_tol", 1e-6)
        gp.inner_rtol = kw.get("inner_rtol", 0.0)
        gp.cfl = kw.get("cfl", 20.0)
        gp.dtmax = kw.get("dtmax", 10.0)
        gp.dtmin = kw.get("dtmin", 1e-7)
        gp.flux = kw.get("flux", 5)
        gp.ns_scheme = kw.get("ns_scheme", 1)
        gp.mlp_warm_after = kw.get("mlp_warm_after", 0)
        gp.mlp_warm_inner = kw.get("mlp_warm_inner", 0)
        gp.mlp_warm_rtol = kw.get("mlp_warm_rtol", 0.0)
        gp.ns_solver = kw.get("ns_solver", 0)
        gp.lusgs_planes = kw.get("plane_order", 0)
        gp.no_mass_projection = kw.get("no_mass_projection", 0)
        gp.correct_f = kw.get("correct_f", 0)
        gp.wall_band = kw.get("wall_band", 0)
        gp.relax_pct = kw.get("relax_pct", 0)
        gp.line_mean = kw.get("line_mean", 0)
        rc = self.L.orc_gsis_configure(self.h, C.byref(gp))
        if rc != 0:
            raise RuntimeError(f"orc_gsis_configure failed: {rc}")

    def gsis_last_inner(self):
        return self.L.orc_gsis_last_inner(self.h)

    def gsis_skipped(self):
        return self.L.orc_gsis_skipped(self.h)

    def ns_state(self):
        nc = (self.nx + 3) * (self.ny + 3)
        U = np.zeros(4 * nc)
        self.L.orc_ns_state(self.h, _dp(U))
        return U

    def ns_residual(self, U):
        nc = (self.nx + 3) * (self.ny + 3)
        U = np.ascontiguousarray(U, dtype=np.float64)
        R = np.zeros(4 * nc)
        rc = self.L.orc_ns_residual(self.h, _dp(U), _dp(R))
        if rc != 0:
            raise RuntimeError(f"orc_ns_residual failed: {rc}")
        return R

    def err(self):
        return self.L.orc_err(self.h)


def _types():
    import sys
    return sys.modules["hyb_gb300.hyb_types"]


def grid_gl(dv, n, vdown, kgln, single_literals=1):
    m = n * kgln
    v, w = np.zeros(m), np.zeros(m)
    lib().orc_grid_gl(dv, n, vdown, kgln, single_literals, _dp(v), _dp(w))
    return v, w


def grid_nc(n, vdown, vup, rule=0):
    v, w = np.zeros(n), np.zeros(n)
    lib().orc_grid_nc(n, vdown, vup, rule, _dp(v), _dp(w))
    return v, w


def cfc_vhs(mole_mass, gamma, alp, omg, vis_ref, tref, ma, nd_inf, t_inf, lref):
    re = C.c_double()
    c = lib().orc_cfc_vhs(mole_mass, gamma, alp, omg, vis_ref, tref, ma, nd_inf, t_inf, lref, C.byref(re))
    return c, re.value
