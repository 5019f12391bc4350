"""ctypes binding of libhyb_gb300.so (the C ABI in include/hyb_dvm.h).

The library is the only compute path: if it is missing or cannot be loaded
every call raises; there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import hyb_types as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libhyb_gb300.so")

# every symbol declared in include/hyb_dvm.h
EXPORTS = [
    "hyb_create", "hyb_destroy", "hyb_last_error", "hyb_version", "hyb_set_precision",
    "hyb_init_maxwellian", "hyb_upload_f", "hyb_download_f", "hyb_download_moments",
    "hyb_download_hot", "hyb_download_hoq", "hyb_step", "hyb_phy_boundary", "hyb_kinetic_step", "hyb_detfp",
    "hyb_convert_ns", "hyb_detfp_res", "hyb_gsis_configure", "hyb_gsis_last_inner", "hyb_gsis_skipped",
    "hyb_launch_count", "hyb_last_step_ms", "hyb_stream", "hyb_set_walls",
    "hyb_profile_enable", "hyb_profile_read", "hyb_detfp_noalloc", "hyb_autotune", "hyb_test_stall",
    "hyb_batch_create", "hyb_batch_destroy", "hyb_batch_last_error", "hyb_batch_size",
    "hyb_batch_instance", "hyb_batch_init_maxwellian", "hyb_batch_autotune", "hyb_batch_step",
    "hyb_batch_last_step_ms", "hyb_batch_launch_count",
    "hyb_mlp_create", "hyb_mlp_destroy", "hyb_mlp_last_error", "hyb_mlp_param_count",
    "hyb_mlp_get_params", "hyb_mlp_set_params", "hyb_mlp_set_norm", "hyb_mlp_set_data",
    "hyb_mlp_train_epoch", "hyb_mlp_grad", "hyb_mlp_predict", "hyb_mlp_forward_dev",
    "hyb_mlp_last_ms", "hyb_mlp_launch_count", "hyb_gsis_attach_mlp", "hyb_gsis_warm_start",
    "hyb_closure_samples",
]
STAGES = ["wall", "sweep", "moments", "sghost", "convert_ns", "gsis", "residual"]

_lib = None


class HybError(RuntimeError):
    def __init__(self, rc, msg):
        super().__init__(f"hyb error {rc}: {msg}")
        self.rc = rc


def load(path=None):
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} not built: run __graft_entry__.build() first")
    L = C.CDLL(path)
    vp, ip, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
    L.hyb_create.argtypes = [vp, vp, vp, C.POINTER(vp)]
    L.hyb_destroy.argtypes = [vp]
    L.hyb_last_error.argtypes = [vp]
    L.hyb_last_error.restype = C.c_char_p
    L.hyb_version.restype = C.c_char_p
    L.hyb_init_maxwellian.argtypes = [vp] + [C.c_double] * 4
    L.hyb_upload_f.argtypes = [vp, dp]
    L.hyb_download_f.argtypes = [vp, dp]
    L.hyb_download_moments.argtypes = [vp, dp, dp]
    L.hyb_download_hot.argtypes = [vp, dp, dp, dp, dp]
    L.hyb_download_hoq.argtypes = [vp, dp, dp]
    L.hyb_step.argtypes = [vp, ip, vp]
    for fn in ("hyb_phy_boundary", "hyb_kinetic_step", "hyb_detfp", "hyb_convert_ns"):
        getattr(L, fn).argtypes = [vp]
    L.hyb_detfp_res.argtypes = [vp, vp]
    L.hyb_gsis_configure.argtypes = [vp, vp]
    L.hyb_gsis_last_inner.argtypes = [vp, C.POINTER(ip)]
    L.hyb_gsis_skipped.argtypes = [vp, C.POINTER(ip)]
    L.hyb_test_stall.argtypes = [vp, ip, C.c_longlong]
    L.hyb_set_precision.argtypes = [vp, ip]
    L.hyb_launch_count.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.hyb_last_step_ms.argtypes = [vp, dp]
    L.hyb_stream.argtypes = [vp, C.POINTER(vp)]
    L.hyb_set_walls.argtypes = [vp, ip, dp, dp, dp]
    L.hyb_autotune.argtypes = [vp, ip, C.POINTER(ip), C.POINTER(ip)]
    L.hyb_batch_create.argtypes = [ip, vp, vp, vp, C.POINTER(vp)]
    L.hyb_batch_destroy.argtypes = [vp]
    L.hyb_batch_last_error.argtypes = [vp]
    L.hyb_batch_last_error.restype = C.c_char_p
    L.hyb_batch_size.argtypes = [vp, C.POINTER(ip)]
    L.hyb_batch_instance.argtypes = [vp, ip, C.POINTER(vp)]
    L.hyb_batch_init_maxwellian.argtypes = [vp] + [C.c_double] * 4
    L.hyb_batch_autotune.argtypes = [vp, ip]
    L.hyb_batch_step.argtypes = [vp, ip, vp]
    L.hyb_batch_last_step_ms.argtypes = [vp, dp]
    L.hyb_batch_launch_count.argtypes = [vp, C.POINTER(C.c_longlong)]
    fp = C.POINTER(C.c_float)
    L.hyb_mlp_create.argtypes = [ip, C.c_ulonglong, C.POINTER(vp)]
    L.hyb_mlp_destroy.argtypes = [vp]
    L.hyb_mlp_last_error.argtypes = [vp]
    L.hyb_mlp_last_error.restype = C.c_char_p
    L.hyb_mlp_get_params.argtypes = [vp, fp]
    L.hyb_mlp_set_params.argtypes = [vp, fp]
    L.hyb_mlp_set_norm.argtypes = [vp, fp, fp, fp, fp]
    L.hyb_mlp_set_data.argtypes = [vp, fp, fp, ip]
    L.hyb_mlp_train_epoch.argtypes = [vp, C.POINTER(ip), ip, C.c_float, fp]
    L.hyb_mlp_grad.argtypes = [vp, fp, fp, ip, fp, fp]
    L.hyb_mlp_predict.argtypes = [vp, fp, ip, fp]
    L.hyb_mlp_forward_dev.argtypes = [vp, vp, ip, vp, vp]
    L.hyb_mlp_last_ms.argtypes = [vp, dp]
    L.hyb_mlp_launch_count.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.hyb_gsis_attach_mlp.argtypes = [vp, vp]
    L.hyb_gsis_warm_start.argtypes = [vp]
    L.hyb_closure_samples.argtypes = [vp, fp, fp, ip, C.POINTER(ip)]
    L.hyb_profile_enable.argtypes = [vp, ip]
    L.hyb_profile_read.argtypes = [vp, dp, C.POINTER(C.c_longlong), ip]
    L.hyb_detfp_noalloc.argtypes = [ip, ip, ip, ip, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Solver:
    """One device context for a cases.Case; methods follow the reference's
    subroutines (GKUA_Phy_boundary, Hybrid_GKUA_Comput_Block, DETFP,
    Convert_NS, DETFP_res, Hybrid_Time_advance_LU_SGS)."""

    def __init__(self, case, precision=None, device=0, handle=None):
        self.L = load()
        self.case = case
        self.owned = handle is None
        if handle is not None:      # an instance owned by a Batch
            self.h = handle
            self.nx, self.ny, self.nv = case.nx, case.ny, case.nv
            self.P = (self.nx + 7) * (self.ny + 7)
            return
        m, g, p, keep = case.c_structs()
        if precision is not None:
            p.precision = precision
        p.device = device
        self._keep = (m, g, p, keep)
        h = C.c_void_p()
        rc = self.L.hyb_create(C.byref(m), C.byref(g), C.byref(p), C.byref(h))
        if rc != 0:
            raise HybError(rc, "hyb_create failed")
        self.h = h
        self.nx, self.ny, self.nv = case.nx, case.ny, case.nv
        self.P = (self.nx + 7) * (self.ny + 7)

    def _ck(self, rc, what):
        if rc != 0:
            msg = self.L.hyb_last_error(self.h).decode() if self.h else ""
            raise HybError(rc, f"{what}: {msg}")

    def close(self):
        if getattr(self, "h", None) and getattr(self, "owned", True):
            self.L.hyb_destroy(self.h)
        self.h = None

    def attach_mlp(self, net):
        self._mlp = net
        self._ck(self.L.hyb_gsis_attach_mlp(self.h, net.h if net is not None else None), "gsis_attach_mlp")

    def warm_start(self):
        self._ck(self.L.hyb_gsis_warm_start(self.h), "gsis_warm_start")

    def closure_samples(self):
        """Closure-network inputs [n][8] and targets [n][4] of every j-face of
        the current kinetic state."""
        n = C.c_int(0)
        self._ck(self.L.hyb_closure_samples(self.h, None, None, 0, C.byref(n)), "closure_samples")
        x = np.zeros((n.value, 8), dtype=np.float32)
        y = np.zeros((n.value, 4), dtype=np.float32)
        self._ck(self.L.hyb_closure_samples(self.h, x.ctypes.data_as(C.POINTER(C.c_float)),
                                            y.ctypes.data_as(C.POINTER(C.c_float)), n.value, C.byref(n)),
                 "closure_samples")
        return x, y

    def autotune(self, reps=3):
        """Time every admissible sweep shape; returns the chosen (cpt, vpb)."""
        c, v = C.c_int(0), C.c_int(0)
        self._ck(self.L.hyb_autotune(self.h, reps, C.byref(c), C.byref(v)), "autotune")
        return c.value, v.value

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- the iteration -------------------------------------------------------
    def init_maxwellian(self, rho=1.0, u=0.0, v=0.0, t=1.0):
        self._ck(self.L.hyb_init_maxwellian(self.h, rho, u, v, t), "init_maxwellian")

    def step(self, n=1, residual=True):
        r = T.HybResidual()
        self._ck(self.L.hyb_step(self.h, n, C.byref(r) if residual else None), "step")
        return r.as_dict() if residual else None

    def phy_boundary(self):
        self._ck(self.L.hyb_phy_boundary(self.h), "phy_boundary")

    def kinetic_step(self):
        self._ck(self.L.hyb_kinetic_step(self.h), "kinetic_step")

    def detfp(self):
        self._ck(self.L.hyb_detfp(self.h), "detfp")

    def convert_ns(self):
        self._ck(self.L.hyb_convert_ns(self.h), "convert_ns")

    def residual(self):
        r = T.HybResidual()
        self._ck(self.L.hyb_detfp_res(self.h, C.byref(r)), "detfp_res")
        return r.as_dict()

    def gsis(self, **kw):
        gp = T.HybGsisParams()
        gp.enable = kw.get("enable", 1)
        gp.max_inner = kw.get("max_inner", 2000)
        gp.inner_tol = kw.get("inner_tol", 1e-6)
        gp.inner_rtol = kw.get("inner_rtol", 0.0)
        gp.lusgs_planes = kw.get("plane_order", 0)
        gp.cfl = kw.get("cfl", 20.0)
        gp.dtmax = kw.get("dtmax", 10.0)
        gp.dtmin = kw.get("dtmin", 1e-7)
        gp.flux = kw.get("flux", 5)
        gp.ns_scheme = kw.get("ns_scheme", 1)
        gp.mlp_warm_after = kw.get("mlp_warm_after", 0)
        gp.mlp_warm_inner = kw.get("mlp_warm_inner", 0)
        gp.mlp_warm_rtol = kw.get("mlp_warm_rtol", 0.0)
        gp.ns_solver = kw.get("ns_solver", 0)
        gp.no_mass_projection = kw.get("no_mass_projection", 0)
        gp.correct_f = kw.get("correct_f", 0)
        gp.wall_band = kw.get("wall_band", 0)
        gp.relax_pct = kw.get("relax_pct", 0)
        gp.line_mean = kw.get("line_mean", 0)
        self._ck(self.L.hyb_gsis_configure(self.h, C.byref(gp)), "gsis_configure")

    def gsis_last_inner(self):
        n = C.c_int(0)
        self._ck(self.L.hyb_gsis_last_inner(self.h, C.byref(n)), "gsis_last_inner")
        return n.value

    def set_precision(self, precision):
        """Promote a mixed context to FP64 on the device (hyb_set_precision)."""
        self._ck(self.L.hyb_set_precision(self.h, precision), "set_precision")

    def test_stall(self, site, spin_cycles):
        """Arm a planted wait that nothing completes for the next step."""
        self._ck(self.L.hyb_test_stall(self.h, site, spin_cycles), "test_stall")

    def gsis_skipped(self):
        n = C.c_int(0)
        self._ck(self.L.hyb_gsis_skipped(self.h, C.byref(n)), "gsis_skipped")
        return n.value

    # ---- state ---------------------------------------------------------------
    def download_f(self):
        a = np.zeros(2 * self.P * self.nv)
        self._ck(self.L.hyb_download_f(self.h, _dp(a)), "download_f")
        return a

    def upload_f(self, frd):
        frd = np.ascontiguousarray(frd, dtype=np.float64)
        self._ck(self.L.hyb_upload_f(self.h, _dp(frd)), "upload_f")

    def moments(self):
        s = np.zeros(11 * self.P)
        cf = np.zeros((self.nx + 3) * (self.ny + 3))
        self._ck(self.L.hyb_download_moments(self.h, _dp(s), _dp(cf)), "download_moments")
        return s, cf

    def hot(self):
        nc = (self.nx + 3) * (self.ny + 3)
        ti, qi, tj, qj = np.zeros(4 * nc), np.zeros(2 * nc), np.zeros(4 * nc), np.zeros(2 * nc)
        self._ck(self.L.hyb_download_hot(self.h, _dp(ti), _dp(qi), _dp(tj), _dp(qj)), "download_hot")
        return ti, qi, tj, qj

    def hoq(self):
        """HOT_GKUA(6, -3:nx+3, -3:ny+3) and HOQ_GKUA(4, ...) of the current f
        (flat, column-major; interior cells)."""
        hot, hoq = np.zeros(6 * self.P), np.zeros(4 * self.P)
        self._ck(self.L.hyb_download_hoq(self.h, _dp(hot), _dp(hoq)), "download_hoq")
        return hot, hoq

    def launches(self):
        n = C.c_longlong()
        self._ck(self.L.hyb_launch_count(self.h, C.byref(n)), "launch_count")
        return n.value

    def set_walls(self, face, u, v, t):
        u, v, t = (np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, t))
        self._ck(self.L.hyb_set_walls(self.h, face, _dp(u), _dp(v), _dp(t)), "set_walls")

    def profile(self, enable=True):
        self._ck(self.L.hyb_profile_enable(self.h, 1 if enable else 0), "profile_enable")

    def profile_read(self):
        n = len(STAGES)
        ms = np.zeros(n)
        ln = (C.c_longlong * n)()
        self._ck(self.L.hyb_profile_read(self.h, _dp(ms), ln, n), "profile_read")
        return {s: (float(ms[k]), int(ln[k])) for k, s in enumerate(STAGES)}

    def last_ms(self):
        x = C.c_double()
        self._ck(self.L.hyb_last_step_ms(self.h, C.byref(x)), "last_step_ms")
        return x.value


class Batch:
    """Many independent cases advanced together by one graph launch per outer
    iteration (hyb_batch_*)."""

    def __init__(self, case_list, precision=None, device=0):
        self.L = load()
        self.cases = list(case_list)
        n = len(self.cases)
        self._keep = []
        M = (T.HybMesh * n)()
        G = (T.HybVgrid * n)()
        P = (T.HybParams * n)()
        for k, c in enumerate(self.cases):
            m, g, p, keep = c.c_structs()
            if precision is not None:
                p.precision = precision
            p.device = device
            M[k], G[k], P[k] = m, g, p
            self._keep.append((m, g, p, keep))
        self._arrays = (M, G, P)
        h = C.c_void_p()
        rc = self.L.hyb_batch_create(n, M, G, P, C.byref(h))
        if rc != 0:
            raise HybError(rc, "hyb_batch_create failed")
        self.h = h
        self.n = n
        self._res = (T.HybResidual * n)()     # reused by every step

    def _ck(self, rc, what):
        if rc != 0:
            msg = self.L.hyb_batch_last_error(self.h).decode() if self.h else ""
            raise HybError(rc, f"{what}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.hyb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def instance(self, k):
        """Non-owning Solver view of instance k."""
        h = C.c_void_p()
        self._ck(self.L.hyb_batch_instance(self.h, k, C.byref(h)), "batch_instance")
        return Solver(self.cases[k], handle=h)

    def init_maxwellian(self, rho=1.0, u=0.0, v=0.0, t=1.0):
        self._ck(self.L.hyb_batch_init_maxwellian(self.h, rho, u, v, t), "batch_init_maxwellian")

    def autotune(self, reps=3):
        self._ck(self.L.hyb_batch_autotune(self.h, reps), "batch_autotune")

    def step(self, n=1, residual=True):
        self._ck(self.L.hyb_batch_step(self.h, n, self._res if residual else None), "batch_step")
        if not residual:
            return None
        # hyb_residual is 9 packed doubles: res_max[4], res_rms[4], max_rms
        rows = np.frombuffer(self._res, dtype=np.float64).reshape(self.n, 9).tolist()
        return [{"res_max": r[:4], "res_rms": r[4:8], "max_rms": r[8]} for r in rows]

    def last_ms(self):
        x = C.c_double()
        self._ck(self.L.hyb_batch_last_step_ms(self.h, C.byref(x)), "batch_last_step_ms")
        return x.value

    def launches(self):
        x = C.c_longlong()
        self._ck(self.L.hyb_batch_launch_count(self.h, C.byref(x)), "batch_launch_count")
        return x.value


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Mlp:
    """The learned closure network on the GPU (hyb_mlp_*)."""

    NPARAM = 9156

    def __init__(self, seed=0, device=0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.hyb_mlp_create(device, seed, C.byref(h))
        if rc != 0:
            raise HybError(rc, "hyb_mlp_create failed")
        self.h = h

    def _ck(self, rc, what):
        if rc != 0:
            msg = self.L.hyb_mlp_last_error(self.h).decode() if self.h else ""
            raise HybError(rc, f"{what}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.hyb_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        w = np.zeros(self.NPARAM, dtype=np.float32)
        self._ck(self.L.hyb_mlp_get_params(self.h, _fp(w)), "get_params")
        return w

    def set_params(self, w):
        w = _f32(w)
        assert w.size == self.NPARAM
        self._ck(self.L.hyb_mlp_set_params(self.h, _fp(w)), "set_params")

    def set_norm(self, in_mean, in_std, out_mean, out_std):
        a = [_f32(v) for v in (in_mean, in_std, out_mean, out_std)]
        self._norm = a
        self._ck(self.L.hyb_mlp_set_norm(self.h, *[_fp(v) for v in a]), "set_norm")

    def set_data(self, x, y):
        x, y = _f32(x), _f32(y)
        self._ck(self.L.hyb_mlp_set_data(self.h, _fp(x), _fp(y), x.shape[0]), "set_data")
        self.n = x.shape[0]

    def train_epoch(self, perm, batch=8192, lr=1e-3):
        perm = np.ascontiguousarray(perm, dtype=np.int32)
        out = C.c_float(0.0)
        self._ck(self.L.hyb_mlp_train_epoch(self.h, perm.ctypes.data_as(C.POINTER(C.c_int)), batch, lr,
                                            C.byref(out)), "train_epoch")
        return out.value

    def grad(self, x, y):
        x, y = _f32(x), _f32(y)
        g = np.zeros(self.NPARAM, dtype=np.float32)
        loss = C.c_float(0.0)
        self._ck(self.L.hyb_mlp_grad(self.h, _fp(x), _fp(y), x.shape[0], _fp(g), C.byref(loss)), "grad")
        return loss.value, g

    def predict(self, x):
        x = _f32(x)
        y = np.zeros((x.shape[0], 4), dtype=np.float32)
        self._ck(self.L.hyb_mlp_predict(self.h, _fp(x), x.shape[0], _fp(y)), "predict")
        return y

    def last_ms(self):
        v = C.c_double()
        self._ck(self.L.hyb_mlp_last_ms(self.h, C.byref(v)), "last_ms")
        return v.value

    def launches(self):
        v = C.c_longlong()
        self._ck(self.L.hyb_mlp_launch_count(self.h, C.byref(v)), "launch_count")
        return v.value
