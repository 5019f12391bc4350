"""ctypes mirrors of the structs in include/hyb_dvm.h.

Field order, types and constants must match the C header exactly; the
C-side tests load the library and compare sizeof() through hyb_abi_sizes.
"""
import ctypes as C

HYB_OK = 0
HYB_ERR_INVALID = -1
HYB_ERR_NOMEM = -2
HYB_ERR_CUDA = -3
HYB_ERR_NONFINITE = -4
HYB_ERR_TIMEOUT = -5
HYB_ERR_UNSUPPORTED = -6
HYB_ERR_TEMPERATURE = -7
HYB_ERR_NODEVICE = -8

HYB_BC_WALL = -2
HYB_BC_PERIODIC = 1

HYB_SCHEME_UP1 = 0
HYB_SCHEME_NND = 1
HYB_SCHEME_WENO3 = 3

HYB_PREC_FP64 = 0
HYB_PREC_MIXED = 1

HYB_STALL_NONE = 0
HYB_STALL_SWEEP_ROW = 1
HYB_STALL_NS_BARRIER = 2

HYB_SWEEP_REFERENCE = 0
HYB_SWEEP_UPWIND = 1

HYB_NSUM = 11
HYB_NRD = 2

_DP = C.POINTER(C.c_double)


class HybMesh(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int),
        ("x", _DP), ("y", _DP),
        ("bc", C.c_int * 4),
        ("wall_u", _DP * 4), ("wall_v", _DP * 4), ("wall_t", _DP * 4),
    ]


class HybVgrid(C.Structure):
    _fields_ = [
        ("nvi", C.c_int), ("nvj", C.c_int),
        ("vi", _DP), ("vj", _DP), ("wi", _DP), ("wj", _DP),
    ]


class HybParams(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("cfc", C.c_double), ("cpr", C.c_double), ("x1s", C.c_double),
        ("r00", C.c_double), ("t00", C.c_double),
        ("scheme", C.c_int), ("precision", C.c_int),
        ("gamma", C.c_double), ("ma", C.c_double), ("pr", C.c_double), ("re", C.c_double),
        ("omega_ns", C.c_double),
        ("device", C.c_int), ("sweep_order", C.c_int), ("mass_pin", C.c_int),
        ("reserved", C.c_int * 5),
    ]


class HybResidual(C.Structure):
    _fields_ = [
        ("res_max", C.c_double * 4), ("res_rms", C.c_double * 4), ("max_rms", C.c_double),
    ]

    def as_dict(self):
        return {"res_max": list(self.res_max), "res_rms": list(self.res_rms),
                "max_rms": float(self.max_rms)}


class HybGsisParams(C.Structure):
    _fields_ = [
        ("enable", C.c_int), ("max_inner", C.c_int), ("inner_tol", C.c_double),
        ("inner_rtol", C.c_double), ("cfl", C.c_double), ("dtmax", C.c_double), ("dtmin", C.c_double),
        ("flux", C.c_int), ("ns_scheme", C.c_int), ("mlp_warm_after", C.c_int),
        ("ns_solver", C.c_int), ("correct_f", C.c_int), ("no_mass_projection", C.c_int),
        ("lusgs_planes", C.c_int), ("mlp_warm_inner", C.c_int), ("mlp_warm_rtol", C.c_double),
        ("wall_band", C.c_int), ("relax_pct", C.c_int), ("line_mean", C.c_int),
    ]


def dptr(a):
    """double* view of a contiguous float64 numpy array (None -> NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(_DP)
