"""ctypes binding of the galaexi_gb300 C ABI (include/galaexi_gb300.h).

The library is built in-tree (galaexi_gb300/build.py).  There is no fallback: if the
shared library is missing or fails to load, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgalaexi_gb300.so")

DG_OK = 0
DG_ERR_ARG = -1
DG_ERR_ALLOC = -2
DG_ERR_CUDA = -3
DG_ERR_NAN = -4
DG_ERR_TIMEOUT = -5
DG_ERR_UNSUPPORTED = -6

DG_NODETYPE_GAUSS = 1
DG_NODETYPE_GAUSS_LOBATTO = 2
RIEMANN = {"lf": 0, "roe": 1, "roel2": 2, "roeentropyfix": 3, "hll": 4, "hllc": 5, "hlle": 6, "hllem": 7, "avg": 8}
SPLITDG = {"none": -1, "sd": 0, "mo": 1, "du": 2, "kg": 3, "pi": 4}
DG_PRECISION_FP64 = 0
DG_PRECISION_MIXED = 1
DG_EXACTFUNC_CONST = 1
DG_EXACTFUNC_SHU_VORTEX = 7
DG_EXACTFUNC_TGV = 100
DG_MAX_N = 9


class DGConfig(ctypes.Structure):
    """struct dg_config of include/galaexi_gb300.h."""
    _fields_ = [
        ("N", ctypes.c_int),
        ("node_type", ctypes.c_int),
        ("parabolic", ctypes.c_int),
        ("riemann", ctypes.c_int),
        ("split_dg", ctypes.c_int),
        ("lifting", ctypes.c_int),
        ("do_weak_lifting", ctypes.c_int),
        ("do_conservative_lifting", ctypes.c_int),
        ("eta_br2", ctypes.c_double),
        ("kappa", ctypes.c_double),
        ("R", ctypes.c_double),
        ("Pr", ctypes.c_double),
        ("mu0", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("filter_type", ctypes.c_int),
        ("n_filter", ctypes.c_int),
        ("hest_filter_param", ctypes.c_double * 3),
        ("laf_alpha", ctypes.c_double),
    ]


class DGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


_lib = None

_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)

_SIGS = {
    "dg_config_default": (None, [ctypes.POINTER(DGConfig)]),
    "dg_config_from_ini": (_I, [ctypes.c_char_p, ctypes.POINTER(DGConfig)]),
    "dg_ctx_create": (_I, [ctypes.POINTER(DGConfig), ctypes.POINTER(_P)]),
    "dg_ctx_destroy": (_I, [_P]),
    "dg_set_mesh": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "dg_rhs": (_I, [_P, _D, _P, _P, _P]),
    "dg_lserk_step": (_I, [_P, _D, _D, _P, _P, _P]),
    "dg_lserk_steps": (_I, [_P, _D, _D, _I, _P, _P, _P]),
    "dg_calc_timestep": (_I, [_P, _P, _D, _D, _DP, _P]),
    "dg_check_state": (_I, [_P, _P, ctypes.POINTER(ctypes.c_longlong), _P]),
    "dg_kernel_launch_count": (ctypes.c_longlong, [_P]),
    "dg_get_gradients": (_I, [_P, _P, _P, _P, _P]),
    "dg_set_boundaries": (_I, [_P, _P, _P, _I, _P]),
    "dg_laf_state": (_I, [_P, _P, _P, _P]),
    "dg_adjoint_scratch_bytes": (_I, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    "dg_mesh_hopr_sizes": (_I, [ctypes.c_char_p, _IP, _IP, _IP, _IP]),
    "dg_mesh_hopr": (_I, [ctypes.c_char_p, _I, _I] + [_P] * 12),
    "dg_mesh_hopr_bcs": (_I, [ctypes.c_char_p, _IP, _P, _I, _P]),
    "dg_h5_read": (_I, [ctypes.c_char_p, ctypes.c_char_p, _I, _IP, _P, _P, ctypes.c_longlong, _P, _I]),
    "dg_write_state": (_I, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _I, ctypes.c_char_p, _D, _I, _P]),
    "dg_integrals": (_I, [_P, _P, _P, _P]),
    "dg_kinetic_energy": (_I, [_P, _P, _P, _P, _P]),
    "dg_rhs_jvp": (_I, [_P, _D, _P, _P, _D, _P, _P, _P]),
    "dg_tlm_steps": (_I, [_P, _D, _D, _I, _P, _P, _D, _P, _P]),
    "dg_rhs_vjp": (_I, [_P, _D, _P, _P, _P, _P, _P]),
    "dg_adjoint_forward": (_I, [_P, _D, _D, _I, _P, _P, ctypes.c_size_t, _P, _P]),
    "dg_adjoint_reverse": (_I, [_P, _P, _P, _P]),
    "dg_adjoint_window": (_I, [_P, _D, _D, _I, _P, ctypes.c_size_t, _P, _P, _P, _P, _P]),
    "dg_last_error": (ctypes.c_char_p, []),
    "dg_basis": (_I, [_I, _I] + [_P] * 10),
    "dg_mesh_cartesian_sizes": (_I, [_I, _I, _I, _IP, _IP]),
    "dg_mesh_cartesian": (_I, [_I, _I, _I, _I, _I, _I, _P, _P, _D] + [_P] * 12),
    "dg_fill_ini": (_I, [_I, _P, _I, ctypes.c_longlong, _P, _D, _D, _D, _P]),
    "dg_profile_stage": (_I, [_P, _P, _P, _D, _I, _DP, _P]),
    "dg_measure_fma_peak": (_I, [_I, _DP]),
    "dg_selftest_bulk_wait": (_I, [ctypes.c_longlong, _DP]),
    "dg_set_pressure_offset": (_I, [_P, _D]),
    "dg_calc_timestep_noalloc": (_I, [_I, _I, _I, _I, _D, _D, _D, _P, _P, _P, _P, _P, _D, _D, _DP, _P]),
}


def lib():
    """Load the shared library once; raise if it is absent (no fallback path exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("galaexi_gb300 native library not built: %s (run galaexi_gb300/build.py)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, what):
    if rc != DG_OK:
        msg = lib().dg_last_error().decode(errors="replace")
        raise DGError(rc, "%s: %s" % (what, msg))


def exported_symbols():
    """Names of the C-ABI functions this binding expects the library to export."""
    return list(_SIGS.keys())
