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
        L.orc_laf_state.argtypes = [_P, _P, _P, _P]
        L.orc_get_vandermonde.argtypes = [ctypes.c_int] * 5 + [_P, _P]
        L.orc_change_basis_3d.argtypes = [ctypes.c_int] * 3 + [_P] * 5
        L.orc_rhs.argtypes = [_P, _P, _P]
        L.orc_get_work.argtypes = [_P, ctypes.c_int, _P]
        L.orc_lserk_steps.argtypes = [_P, ctypes.c_double, ctypes.c_double, ctypes.c_int, _P, _P]
        L.orc_calc_metrics.restype = ctypes.c_int
        L.orc_calc_metrics.argtypes = [ctypes.c_int] * 4 + [_P] * 12
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


def get_vandermonde(N_in, nt_in, N_out, nt_out, modal):
    """GetVandermonde: (Vdm_In_Out (N_out+1, N_in+1), Vdm_Out_In (N_in+1, N_out+1)), Fortran order."""
    a = np.zeros((N_out + 1, N_in + 1), order="F")
    b = np.zeros((N_in + 1, N_out + 1), order="F")
    lib().orc_get_vandermonde(N_in, nt_in, N_out, nt_out, int(modal), _p(a), _p(b))
    return a, b


def change_basis_3d(X, Vx, Vy=None, Vz=None):
    """ChangeBasis3D(_XYZ) of X(nVar,0:NIn,0:NIn,0:NIn) (Fortran order) with (0:NOut,0:NIn) matrices."""
    Vy = Vx if Vy is None else Vy
    Vz = Vx if Vz is None else Vz
    Vx, Vy, Vz = (np.asfortranarray(v, dtype=np.float64) for v in (Vx, Vy, Vz))
    X = np.asfortranarray(X, dtype=np.float64)
    nVar, NIn, NOut = X.shape[0], X.shape[1] - 1, Vx.shape[0] - 1
    out = np.zeros((nVar, NOut + 1, NOut + 1, NOut + 1), order="F")
    lib().orc_change_basis_3d(nVar, NIn, NOut, _p(Vx), _p(Vy), _p(Vz), _p(X), _p(out))
    return out


def calc_metrics(N, node_type, NGeo, NodeCoords, ElemToSide, nSides):
    """The oracle's own geometry (BuildCoords + CalcMetrics + CalcSurfMetrics) from the equidistant
    node coordinates NodeCoords (nElems, NGeo+1, NGeo+1, NGeo+1, 3) (C order of the Fortran
    (3,0:NGeo,0:NGeo,0:NGeo,nElems)) and ElemToSide (nElems, 6, 3).  Returns a dict with the mesh
    arrays of the reference (Elem_xGP, Metrics_f/g/hTilde, sJ, NormVec, TangVec1/2, SurfElem,
    Face_xGP) in the same shapes as galaexi_gb300.Mesh, and "bad_nodes" (scaled Jacobian < 0.01)."""
    NC = np.ascontiguousarray(NodeCoords, dtype=np.float64)
    E2S = np.ascontiguousarray(ElemToSide, dtype=np.int32)
    E, n = NC.shape[0], N + 1
    out = {"Elem_xGP": np.zeros((E, n, n, n, 3)), "Metrics_fTilde": np.zeros((E, n, n, n, 3)),
           "Metrics_gTilde": np.zeros((E, n, n, n, 3)), "Metrics_hTilde": np.zeros((E, n, n, n, 3)),
           "sJ": np.zeros((E, n, n, n)), "NormVec": np.zeros((nSides, n, n, 3)), "TangVec1": np.zeros((nSides, n, n, 3)),
           "TangVec2": np.zeros((nSides, n, n, 3)), "SurfElem": np.zeros((nSides, n, n)),
           "Face_xGP": np.zeros((nSides, n, n, 3))}
    keys = ("Elem_xGP", "Metrics_fTilde", "Metrics_gTilde", "Metrics_hTilde", "sJ", "NormVec", "TangVec1", "TangVec2",
            "SurfElem", "Face_xGP")
    out["bad_nodes"] = lib().orc_calc_metrics(int(N), int(node_type), int(NGeo), E, _p(NC), _p(E2S),
                                              *[_p(out[k]) for k in keys])
    return out


class _Geometry:
    """Mesh arrays from the oracle's own metric computation, with the connectivity of a mesh."""

    def __init__(self, mesh):
        g = calc_metrics(mesh.N, mesh.node_type, mesh.NGeo, mesh.NodeCoords, mesh.ElemToSide, mesh.nSides)
        if g["bad_nodes"] != 0:
            raise ValueError("oracle metrics: %d nodes with a bad Jacobian" % g["bad_nodes"])
        for k, v in g.items():
            setattr(self, k, v)
        for k in ("N", "node_type", "NGeo", "nElems", "nSides", "ElemToSide", "SideToElem", "NodeCoords"):
            setattr(self, k, getattr(mesh, k))
        self.nBCSides = getattr(mesh, "nBCSides", 0)

    @property
    def nDOF(self):
        return self.nElems * (self.N + 1) ** 3


class Oracle:
    """CPU restatement of DGTimeDerivative_weakForm / TimeStepByLSERKW2 on one mesh."""

    def __init__(self, cfg, mesh, boundaries=None, geometry="auto"):
        """boundaries: (bc_type, bc_state, refstates) of the mesh's BC sides, as for the DG operator.
        geometry: "own" computes the metric arrays here from the mesh's node coordinates
        (calc_metrics) and takes only its connectivity; "mesh" takes the metric arrays of the mesh
        object; "auto" is "own" for curved and file meshes and "mesh" for the affine generated box,
        whose metric terms are exact constants (the curl form of the reference reproduces them up
        to round-off, ~4e-14 relative, which the tests pin separately)."""
        if geometry == "auto":
            affine_box = getattr(mesh, "deform", None) == 0.0 and not hasattr(mesh, "path")
            geometry = "mesh" if (affine_box or not hasattr(mesh, "NodeCoords")) else "own"
        if geometry == "own":
            mesh = _Geometry(mesh)
        elif geometry != "mesh":
            raise ValueError("geometry: 'auto', 'mesh' or 'own'")
        self.cfg, self.mesh = cfg, mesh
        m = mesh
        self._keep = [m.Metrics_fTilde, m.Metrics_gTilde, m.Metrics_hTilde, m.sJ, m.NormVec, m.TangVec1, m.TangVec2,
                      m.SurfElem, m.ElemToSide, m.SideToElem]
        self._h = lib().orc_create(ctypes.byref(cfg), m.nElems, m.nSides, *[_p(a) for a in self._keep])
        if not self._h:
            raise ValueError("orc_create failed (filter configuration)")
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
        """Ut of the state U; with a filter configured U itself is filtered in place first (as the
        reference's DGTimeDerivative_weakForm does), so a numpy U receives the filtered state."""
        Uc = np.array(U, dtype=np.float64, copy=True, order="C")
        Ut = np.zeros_like(Uc)
        lib().orc_rhs(self._h, _p(Uc), _p(Ut))
        if self.cfg.filter_type and isinstance(U, np.ndarray):
            U[...] = Uc
        return Ut

    def laf_state(self):
        out = [np.zeros(self.mesh.nElems) for _ in range(3)]
        lib().orc_laf_state(self._h, *[_p(a) for a in out])
        return tuple(out)

    def work(self, which, shape):
        out = np.zeros(shape)
        lib().orc_get_work(self._h, which, _p(out))
        return out

    def lserk_steps(self, U, dt, nSteps, Ut_tmp=None, t=0.0):
        U = np.array(U, dtype=np.float64, copy=True)
        Ut_tmp = np.zeros_like(U) if Ut_tmp is None else np.array(Ut_tmp, dtype=np.float64, copy=True)
        lib().orc_lserk_steps(self._h, float(t), float(dt), int(nSteps), _p(U), _p(Ut_tmp))
        return U, Ut_tmp

    def lserk_steps_inplace(self, U, Ut_tmp, dt, nSteps, t=0.0):
        """lserk_steps on C-contiguous float64 arrays U and Ut_tmp, updated in place."""
        for a in (U, Ut_tmp):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
                raise ValueError("lserk_steps_inplace needs C-contiguous float64 arrays")
        lib().orc_lserk_steps(self._h, float(t), float(dt), int(nSteps), _p(U), _p(Ut_tmp))

    def calc_timestep(self, U, cfl, dfl=0.0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        err = ctypes.c_int()
        dt = lib().orc_calc_timestep(self._h, _p(U), float(cfl), float(dfl), ctypes.byref(err))
        return dt, err.value
