"""TEST INFRASTRUCTURE: ctypes wrapper of the CPU oracle (oracle/dgsem_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the
checker.  The product (galaexi_gb300) never imports it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None
_P = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _b
            _b.build(verbose=False)
        L = ctypes.CDLL(LIB_PATH)
        L.orc_set_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_nodes_weights.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, _P]
        L.orc_derivative_matrix.argtypes = [ctypes.c_int, ctypes.c_int, _P]
        L.orc_dg_basis.argtypes = [ctypes.c_int, ctypes.c_int] + [_P] * 10
        L.orc_s2v2.argtypes = [ctypes.c_int, _P]
        L.orc_prolong_to_face_host.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, ctypes.c_int, _P,
                                               _P, _P]
        L.orc_surf_int_host.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P, _P]
        L.orc_create.restype = _P
        L.orc_create.argtypes = [_P, ctypes.c_int, ctypes.c_int] + [_P] * 10
        L.orc_destroy.argtypes = [_P]
        L.orc_set_boundaries.argtypes = [_P, ctypes.c_int, _P, _P, ctypes.c_int, _P]
        L.orc_rhs.argtypes = [_P, _P, _P]
        L.orc_get_work.argtypes = [_P, ctypes.c_int, _P]
        L.orc_lserk_steps.argtypes = [_P, ctypes.c_double, ctypes.c_double, ctypes.c_int, _P, _P]
        L.orc_calc_timestep.restype = ctypes.c_double
        L.orc_calc_timestep.argtypes = [_P, _P, ctypes.c_double, ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def set_threads(n):
    return lib().orc_set_threads(int(n))


def nodes_weights(N, node_type):
    x, w, wb = np.zeros(N + 1), np.zeros(N + 1), np.zeros(N + 1)
    lib().orc_nodes_weights(N, node_type, _p(x), _p(w), _p(wb))
    return x, w, wb


def derivative_matrix(N, node_type):
    """D(i,l) of the reference as a C-order array D[l, i] (Fortran column-major storage)."""
    D = np.zeros((N + 1) * (N + 1))
    lib().orc_derivative_matrix(N, node_type, _p(D))
    return D.reshape(N + 1, N + 1)


def dg_basis(N, node_type):
    n = N + 1
    out = {k: np.zeros(n) for k in ("xGP", "wGP", "wBary", "L_minus", "L_plus", "L_hat_minus", "L_hat_plus")}
    out.update({k: np.zeros(n * n) for k in ("D", "D_hat_T", "DVolSurf")})
    lib().orc_dg_basis(N, node_type, *[_p(out[k]) for k in (
        "xGP", "wGP", "wBary", "L_minus", "L_plus", "D", "D_hat_T", "L_hat_minus", "L_hat_plus", "DVolSurf")])
    return out


def s2v2(N):
    a = np.zeros(2 * (N + 1) ** 2 * 5 * 6, dtype=np.int32)
    lib().orc_s2v2(N, _p(a))
    return a


class Oracle:
    """CPU restatement of DGTimeDerivative_weakForm / TimeStepByLSERKW2 on one mesh."""

    def __init__(self, cfg, mesh, boundaries=None):
        """boundaries: (bc_type, bc_state, refstates) of the mesh's BC sides, as for the DG operator."""
        self.cfg, self.mesh = cfg, mesh
        m = mesh
        self._keep = [m.Metrics_fTilde, m.Metrics_gTilde, m.Metrics_hTilde, m.sJ, m.NormVec, m.TangVec1, m.TangVec2,
                      m.SurfElem, m.ElemToSide, m.SideToElem]
        self._h = lib().orc_create(ctypes.byref(cfg), m.nElems, m.nSides, *[_p(a) for a in self._keep])
        nb = getattr(m, "nBCSides", 0)
        if nb:
            if boundaries is None:
                raise ValueError("mesh has BC sides: pass boundaries=(bc_type, bc_state, refstates)")
            bt, bs, rs = boundaries
            bt = np.ascontiguousarray(bt, dtype=np.int32)
            bs = np.ascontiguousarray(bs, dtype=np.int32)
            rs = np.ascontiguousarray(rs, dtype=np.float64).reshape(-1, 5)
            rc = lib().orc_set_boundaries(self._h, nb, _p(bt), _p(bs), rs.shape[0], _p(rs))
            if rc != 0:
                raise ValueError(f"orc_set_boundaries failed ({rc})")

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rhs(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        Ut = np.zeros_like(U)
        lib().orc_rhs(self._h, _p(U), _p(Ut))
        return Ut

    def work(self, which, shape):
        out = np.zeros(shape)
        lib().orc_get_work(self._h, which, _p(out))
        return out

    def lserk_steps(self, U, dt, nSteps, Ut_tmp=None, t=0.0):
        U = np.array(U, dtype=np.float64, copy=True)
        Ut_tmp = np.zeros_like(U) if Ut_tmp is None else np.array(Ut_tmp, dtype=np.float64, copy=True)
        lib().orc_lserk_steps(self._h, float(t), float(dt), int(nSteps), _p(U), _p(Ut_tmp))
        return U, Ut_tmp

    def calc_timestep(self, U, cfl, dfl=0.0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        err = ctypes.c_int()
        dt = lib().orc_calc_timestep(self._h, _p(U), float(cfl), float(dfl), ctypes.byref(err))
        return dt, err.value
