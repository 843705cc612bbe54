"""Host-side mirror of the reference's DG operator interface for this path.

The reference drives the operator through module procedures on module-global device arrays:
  InitDG / InitDGbasis              src/dg/dg.f90:67-242
  DGTimeDerivative_weakForm(t)      src/dg/dg.f90:255-425
  TimeStepByLSERKW2(t)              src/timedisc/timestep.f90:49-120
  CALCTIMESTEP(errType)             src/equations/navierstokes/calctimestep.f90:98-186
  FillIni                           src/dg/dg.f90:432-456
Here the same calls go through the C ABI of the GB300 library; device arrays are torch CUDA
tensors (plumbing only: the arithmetic runs in the library's own kernels).  Arrays use the
reference's Fortran layouts; a Fortran array A(5,0:N,0:N,0:N,nElems) is held as a C-order
array of shape (nElems, N+1, N+1, N+1, 5) with identical memory order.
"""
import ctypes

import numpy as np

from . import _native as nat


def config(N=3, NodeType="gauss-lobatto", Riemann="lf", SplitDG="none", parabolic=False, kappa=1.4, R=287.058,
           Pr=0.72, mu0=0.0, doWeakLifting=False, doConservativeLifting=False, etaBR2=2.0, precision="fp64",
           Lifting="br1", FilterType="none", NFilter=None, HestFilterParam=None, LAF_alpha=None):
    """Build a dg_config from the reference's ini key names (see dg_config_from_ini)."""
    cfg = nat.DGConfig()
    nat.lib().dg_config_default(ctypes.byref(cfg))
    text = "\n".join([
        "N = %d" % N, "NodeType = %s" % NodeType, "Riemann = %s" % Riemann, "SplitDG = %s" % SplitDG,
        "Parabolic = %s" % ("T" if parabolic else "F"), "kappa = %r" % kappa, "R = %r" % R, "Pr = %r" % Pr,
        "mu0 = %r" % mu0, "doWeakLifting = %s" % ("T" if doWeakLifting else "F"),
        "doConservativeLifting = %s" % ("T" if doConservativeLifting else "F"), "etaBR2 = %r" % etaBR2,
        "Precision = %s" % precision, "Lifting = %s" % Lifting, "FilterType = %s" % FilterType]
        + (["NFilter = %d" % NFilter] if NFilter is not None else [])
        + (["HestFilterParam = (/%r, %r, %r/)" % tuple(HestFilterParam)] if HestFilterParam is not None else [])
        + (["LAF_alpha = %r" % LAF_alpha] if LAF_alpha is not None else []))
    nat.check(nat.lib().dg_config_from_ini(text.encode(), ctypes.byref(cfg)), "dg_config_from_ini")
    return cfg


def config_from_ini(text, base=None):
    """Parse ini text (reference parameter-file syntax) into a dg_config."""
    cfg = nat.DGConfig()
    if base is None:
        nat.lib().dg_config_default(ctypes.byref(cfg))
    else:
        ctypes.pointer(cfg)[0] = base
    nat.check(nat.lib().dg_config_from_ini(text.encode(), ctypes.byref(cfg)), "dg_config_from_ini")
    return cfg


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _tp(t):
    """Device pointer of a torch tensor (None -> NULL)."""
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def basis(N, node_type):
    """InitInterpolationBasis + InitDGbasis: dict of the 1D operators (D, D_hat_T, ... column-major)."""
    n = N + 1
    out = {k: np.zeros(n) for k in ("xGP", "wGP", "wBary", "L_minus", "L_plus", "L_hat_minus", "L_hat_plus")}
    out.update({k: np.zeros(n * n) for k in ("D", "D_hat_T", "DVolSurf")})
    nat.check(nat.lib().dg_basis(N, node_type, *[_ptr(out[k]) for k in (
        "xGP", "wGP", "wBary", "L_minus", "L_plus", "D", "D_hat_T", "L_hat_minus", "L_hat_plus", "DVolSurf")]),
        "dg_basis")
    return out


def read_h5(path, name, attribute=False):
    """A dataset or root attribute of an HDF5 file (dg_h5_read): a numpy float64 array in the file's
    (C) shape, or a str for string data."""
    L = nat.lib()
    nd = ctypes.c_int()
    dims = np.zeros(8, dtype=np.int64)
    p, nm = str(path).encode(), str(name).encode()
    buf = ctypes.create_string_buffer(1024)
    nat.check(L.dg_h5_read(p, nm, int(attribute), ctypes.byref(nd), _ptr(dims), None, 0, buf, 1024), "dg_h5_read")
    shape = tuple(int(d) for d in dims[:nd.value])
    if buf.value:
        return buf.value.decode()
    out = np.zeros(shape if shape else (1,))
    nat.check(L.dg_h5_read(p, nm, int(attribute), ctypes.byref(nd), _ptr(dims), _ptr(out), out.size, None, 0),
              "dg_h5_read")
    return out


def write_state(path, U, N, node_type, time, mesh_file, project="galaexi_gb300"):
    """A FLEXI state file (dg_write_state): U of shape (nElems, n, n, n, 5) (host numpy or torch),
    node_type 1 (Gauss) / 2 (Gauss-Lobatto) or the reference's name."""
    if hasattr(U, "detach"):
        U = U.detach().cpu().numpy()
    U = np.ascontiguousarray(U, dtype=np.float64)
    if isinstance(node_type, int):
        node_type = "GAUSS" if node_type == 1 else "GAUSS-LOBATTO"
    nat.check(nat.lib().dg_write_state(str(path).encode(), str(project).encode(), str(mesh_file).encode(), int(N),
                                       str(node_type).encode(), float(time), U.shape[0], _ptr(U)), "dg_write_state")


def read_state(path):
    """(U, time, N, node_type, mesh_file) of a FLEXI state file."""
    U = read_h5(path, "DG_Solution")
    return (U, float(read_h5(path, "Time", True)[0]), int(read_h5(path, "N", True)[0]),
            read_h5(path, "NodeType", True), read_h5(path, "MeshFile", True))


class Mesh:
    """Periodic hexahedral box with the reference's connectivity and metric arrays.

    Stand-in for a HOPR mesh read by ReadMesh/InitMesh (src/mesh/mesh_readin.f90, mesh.f90) and
    CalcMetrics (src/mesh/metrics.f90).  Arrays (C order, Fortran layout reversed):
      Elem_xGP (nElems,n,n,n,3)   Metrics_f/g/hTilde (nElems,n,n,n,3)   sJ (nElems,n,n,n)
      NormVec/TangVec1/TangVec2 (nSides,n,n,3)   SurfElem (nSides,n,n)
      ElemToSide (nElems,6,3)   SideToElem (nSides,5)   (1-based IDs)
    """

    def __init__(self, N, node_type, nx, ny, nz, x0=(0.0, 0.0, 0.0), x1=(1.0, 1.0, 1.0), deform=0.0, NGeo=None):
        """NGeo: degree of the element mapping (node coordinates on NGeo+1 equidistant points per
        direction, displaced by `deform`); default 1 for the affine box, 2 for a displaced one."""
        L = nat.lib()
        ne, ns = ctypes.c_int(), ctypes.c_int()
        nat.check(L.dg_mesh_cartesian_sizes(nx, ny, nz, ctypes.byref(ne), ctypes.byref(ns)), "mesh sizes")
        self.N, self.node_type = N, node_type
        self.nElems, self.nSides = ne.value, ns.value
        self.nx, self.ny, self.nz = nx, ny, nz
        self.x0, self.x1, self.deform = tuple(x0), tuple(x1), deform
        self.NGeo = int(NGeo) if NGeo is not None else (2 if deform != 0.0 else 1)
        self.nBCSides = 0
        self._alloc()
        g = self.NGeo + 1
        self.NodeCoords = np.zeros((self.nElems, g, g, g, 3))
        a0 = np.asarray(x0, dtype=np.float64)
        a1 = np.asarray(x1, dtype=np.float64)
        nat.check(L.dg_mesh_cartesian(N, node_type, self.NGeo, nx, ny, nz, _ptr(a0), _ptr(a1), float(deform),
                                      _ptr(self.NodeCoords), _ptr(self.Elem_xGP), _ptr(self.Metrics_fTilde),
                                      _ptr(self.Metrics_gTilde),
                                      _ptr(self.Metrics_hTilde), _ptr(self.sJ), _ptr(self.NormVec),
                                      _ptr(self.TangVec1), _ptr(self.TangVec2), _ptr(self.SurfElem),
                                      _ptr(self.ElemToSide), _ptr(self.SideToElem)), "dg_mesh_cartesian")

    @classmethod
    def from_hopr(cls, path, N, node_type):
        """A HOPR mesh file (HDF5) read as ReadMesh + CalcMetrics do (dg_mesh_hopr); BC sides come
        first, BCIndex holds their index into the file's BCNames/BCType."""
        L = nat.lib()
        ne, ns, nb, ng = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        p = str(path).encode()
        nat.check(L.dg_mesh_hopr_sizes(p, ctypes.byref(ne), ctypes.byref(ns), ctypes.byref(nb), ctypes.byref(ng)),
                  "dg_mesh_hopr_sizes")
        self = cls.__new__(cls)
        self.N, self.node_type = N, node_type
        self.nElems, self.nSides, self.nBCSides, self.NGeo = ne.value, ns.value, nb.value, ng.value
        self.path = str(path)
        self._alloc()
        self.BCIndex = np.zeros(max(1, self.nBCSides), dtype=np.int32)
        nat.check(L.dg_mesh_hopr(p, N, node_type, _ptr(self.Elem_xGP), _ptr(self.Metrics_fTilde),
                                 _ptr(self.Metrics_gTilde), _ptr(self.Metrics_hTilde), _ptr(self.sJ), _ptr(self.NormVec),
                                 _ptr(self.TangVec1), _ptr(self.TangVec2), _ptr(self.SurfElem), _ptr(self.ElemToSide),
                                 _ptr(self.SideToElem), _ptr(self.BCIndex)), "dg_mesh_hopr")
        self.BCIndex = self.BCIndex[:self.nBCSides]
        g = self.NGeo + 1
        # the file's equidistant element node coordinates NodeCoords(3,0:NGeo,0:NGeo,0:NGeo,nElems)
        self.NodeCoords = read_h5(path, "NodeCoords").reshape(self.nElems, g, g, g, 3)
        nbc = ctypes.c_int()
        nat.check(L.dg_mesh_hopr_bcs(p, ctypes.byref(nbc), None, 0, None), "dg_mesh_hopr_bcs")
        NL = 256
        names = ctypes.create_string_buffer(max(1, nbc.value) * NL)
        self.BCType = np.zeros((max(1, nbc.value), 4), dtype=np.int32)
        nat.check(L.dg_mesh_hopr_bcs(p, ctypes.byref(nbc), names, NL, _ptr(self.BCType)), "dg_mesh_hopr_bcs")
        self.BCType = self.BCType[:nbc.value]
        self.BCNames = [names.raw[b * NL:(b + 1) * NL].split(b"\0", 1)[0].decode() for b in range(nbc.value)]
        return self

    def boundaries(self, refstates, boundary_types=None):
        """(bc_type, bc_state, refstates) for DG(..., boundaries=...): the file's BCType with the
        parameter file's BoundaryName / BoundaryType overrides (ReadBCs, mesh_readin.f90:98-169: an
        exact name match replaces type and state; an unknown name is an error), per BC side.
        refstates: the RefState rows (rho, u, v, w, p), type 27 rows (Tt, alpha, beta, -, pt)."""
        bct = self.BCType.copy()
        for name, (typ, state) in (boundary_types or {}).items():
            hit = [b for b, bn in enumerate(self.BCNames) if bn == name]
            if not hit:
                raise ValueError(f"Boundary condition specified in parameter file has not been found: {name}")
            for b in hit:
                if (typ == 1) != (bct[b, 0] == 1):
                    raise ValueError(f"boundary {name}: remapping between periodic and non-periodic is not supported")
                bct[b, 0], bct[b, 2] = typ, state
        idx = self.BCIndex - 1
        return bct[idx, 0].astype(np.int32), bct[idx, 2].astype(np.int32), np.asarray(refstates, dtype=np.float64)

    def _alloc(self):
        n = self.N + 1
        E, S = self.nElems, self.nSides
        self.Elem_xGP = np.zeros((E, n, n, n, 3))
        self.Metrics_fTilde = np.zeros((E, n, n, n, 3))
        self.Metrics_gTilde = np.zeros((E, n, n, n, 3))
        self.Metrics_hTilde = np.zeros((E, n, n, n, 3))
        self.sJ = np.zeros((E, n, n, n))
        self.NormVec = np.zeros((S, n, n, 3))
        self.TangVec1 = np.zeros((S, n, n, 3))
        self.TangVec2 = np.zeros((S, n, n, 3))
        self.SurfElem = np.zeros((S, n, n))
        self.ElemToSide = np.zeros((E, 6, 3), dtype=np.int32)
        self.SideToElem = np.zeros((S, 5), dtype=np.int32)

    @property
    def nDOF(self):
        return self.nElems * (self.N + 1) ** 3


def fill_ini(mesh, exactfunc, params, kappa=1.4, R=287.058, t=0.0):
    """FillIni (src/dg/dg.f90:432-456): conservative state at the nodes, shape (nElems,n,n,n,5)."""
    n = mesh.N + 1
    U = np.zeros((mesh.nElems, n, n, n, 5))
    p = np.asarray(params, dtype=np.float64)
    nat.check(nat.lib().dg_fill_ini(exactfunc, _ptr(p), len(p), mesh.nElems * n ** 3, _ptr(mesh.Elem_xGP),
                                    float(kappa), float(R), float(t), _ptr(U)), "dg_fill_ini")
    return U


def tgv_state(mesh, mach=0.1, kappa=1.4, R=287.058):
    """Taylor-Green vortex initial state (testcase/taylorgreenvortex/testcase.f90:220-262), rho0=U0=1, rho const."""
    return fill_ini(mesh, nat.DG_EXACTFUNC_TGV, [1.0, 1.0, mach, 1.0], kappa=kappa, R=R)


class DG:
    """The GB300 DG operator for one mesh: MOD_DG + MOD_TimeDisc for this path.

    U, Ut, Ut_tmp are torch float64 CUDA tensors of shape (nElems, n, n, n, 5) (reference layout).
    """

    def __init__(self, cfg, mesh, pressure_offset=None, boundaries=None):
        """pressure_offset: reference pressure of the mixed form (dg_set_pressure_offset); None picks
        the volume-mean pressure of the first state this operator sees (mixed form only).
        boundaries: for meshes with BC sides, (bc_type, bc_state, refstates): per BC side type and
        1-based RefState index, and the RefStates (n x 5 primitives) -- see dg_set_boundaries."""
        import torch  # device memory and streams only
        self._pref = pressure_offset
        self._torch = torch
        self.cfg = cfg
        self.mesh = mesh
        L = nat.lib()
        h = ctypes.c_void_p()
        nat.check(L.dg_ctx_create(ctypes.byref(cfg), ctypes.byref(h)), "dg_ctx_create")
        self._h = h
        m = mesh
        nat.check(L.dg_set_mesh(h, m.nElems, m.nSides, getattr(m, "nBCSides", 0), _ptr(m.Metrics_fTilde),
                                _ptr(m.Metrics_gTilde),
                                _ptr(m.Metrics_hTilde), _ptr(m.sJ), _ptr(m.NormVec), _ptr(m.TangVec1),
                                _ptr(m.TangVec2), _ptr(m.SurfElem), _ptr(m.ElemToSide), _ptr(m.SideToElem)),
                  "dg_set_mesh")
        if getattr(m, "nBCSides", 0):
            if boundaries is None:
                raise ValueError("mesh has BC sides: pass boundaries=(bc_type, bc_state, refstates)")
            bt, bs, rs = boundaries
            self._bc = (np.ascontiguousarray(bt, dtype=np.int32), np.ascontiguousarray(bs, dtype=np.int32),
                        np.ascontiguousarray(rs, dtype=np.float64).reshape(-1, 5))
            nat.check(L.dg_set_boundaries(h, _ptr(self._bc[0]), _ptr(self._bc[1]), self._bc[2].shape[0],
                                          _ptr(self._bc[2])), "dg_set_boundaries")
        if pressure_offset is not None:
            nat.check(L.dg_set_pressure_offset(h, float(pressure_offset)), "dg_set_pressure_offset")

    def _auto_offset(self, U):
        if self._pref is not None or self.cfg.precision != nat.DG_PRECISION_MIXED:
            return
        torch = self._torch
        m = self.mesh
        w = torch.from_numpy(basis(m.N, m.node_type)["wGP"]).to(U.device)
        W = w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
        J = W / torch.from_numpy(m.sJ).to(U.device)
        kin = 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2 + U[..., 3] ** 2) / U[..., 0]
        p = (self.cfg.kappa - 1.0) * (U[..., 4] - kin)
        self._pref = float((p * J).sum() / J.sum())
        nat.check(nat.lib().dg_set_pressure_offset(self._h, self._pref), "dg_set_pressure_offset")

    def close(self):
        if getattr(self, "_h", None):
            nat.lib().dg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- helpers ---------------------------------------------------------------------------
    def _stream(self, stream=None):
        torch = self._torch
        s = stream if stream is not None else torch.cuda.current_stream()
        return ctypes.c_void_p(s.cuda_stream)

    def _check_state(self, U):
        torch = self._torch
        n = self.mesh.N + 1
        if not (isinstance(U, torch.Tensor) and U.is_cuda and U.dtype == torch.float64 and U.is_contiguous()
                and tuple(U.shape) == (self.mesh.nElems, n, n, n, 5)):
            raise ValueError("state must be a contiguous float64 CUDA tensor of shape (nElems,n,n,n,5)")

    def new_state(self):
        n = self.mesh.N + 1
        return self._torch.zeros((self.mesh.nElems, n, n, n, 5), dtype=self._torch.float64, device="cuda")

    @property
    def kernel_launches(self):
        return nat.lib().dg_kernel_launch_count(self._h)

    # -- the reference's operator surface ----------------------------------------------------
    def DGTimeDerivative_weakForm(self, t, U, Ut=None, stream=None):
        """Ut = DGTimeDerivative_weakForm(U) (src/dg/dg.f90:255-425)."""
        self._check_state(U)
        if Ut is None:
            Ut = self._torch.empty_like(U)
        self._check_state(Ut)
        self._auto_offset(U)
        nat.check(nat.lib().dg_rhs(self._h, float(t), ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(Ut.data_ptr()),
                                   self._stream(stream)), "dg_rhs")
        return Ut

    def TimeStepByLSERKW2(self, t, dt, U, Ut_tmp, nSteps=1, stream=None):
        """nSteps Carpenter RK4-5 steps of size dt in place (src/timedisc/timestep.f90:49-120)."""
        self._check_state(U)
        self._check_state(Ut_tmp)
        self._auto_offset(U)
        nat.check(nat.lib().dg_lserk_steps(self._h, float(t), float(dt), int(nSteps), ctypes.c_void_p(U.data_ptr()),
                                           ctypes.c_void_p(Ut_tmp.data_ptr()), self._stream(stream)),
                  "dg_lserk_steps")

    def CalcTimeStep(self, U, CFLScale, DFLScale=0.0, stream=None):
        """dt from CFL/DFL (calctimestep.f90:98-296, FillCFL_DFL timedisc_func.f90:480-550).

        Returns (dt, errType); errType = 1 when the state holds NaN or non-positive rho/p."""
        self._check_state(U)
        dt = ctypes.c_double()
        rc = nat.lib().dg_calc_timestep(self._h, ctypes.c_void_p(U.data_ptr()), float(CFLScale), float(DFLScale),
                                        ctypes.byref(dt), self._stream(stream))
        if rc == nat.DG_ERR_NAN:
            return dt.value, 1
        nat.check(rc, "dg_calc_timestep")
        return dt.value, 0

    # -- integrals, tangent-linear and adjoint operators (FP64 form) ----------------------------
    def integrals(self, U, stream=None):
        """(mass, x-, y-, z-momentum, energy, kinetic energy) volume integrals of U in FP64."""
        self._check_state(U)
        out = (ctypes.c_double * 6)()
        nat.check(nat.lib().dg_integrals(self._h, _tp(U), out, self._stream(stream)), "dg_integrals")
        return list(out)

    def kinetic_energy(self, U, grad=False, stream=None):
        """J = integral of 0.5|m|^2/rho on the solution nodes; with grad=True also dJ/dU."""
        self._check_state(U)
        J = ctypes.c_double()
        G = self._torch.empty_like(U) if grad else None
        nat.check(nat.lib().dg_kinetic_energy(self._h, _tp(U), ctypes.byref(J), _tp(G), self._stream(stream)),
                  "dg_kinetic_energy")
        return (J.value, G) if grad else J.value

    def rhs_jvp(self, U, Udot, mu_dot=0.0, stream=None):
        """(Ut, Utdot): the operator and its exact directional derivative along (Udot, mu_dot)."""
        self._check_state(U)
        self._check_state(Udot)
        Ut, Utd = self._torch.empty_like(U), self._torch.empty_like(U)
        nat.check(nat.lib().dg_rhs_jvp(self._h, 0.0, _tp(U), _tp(Udot), float(mu_dot), _tp(Ut), _tp(Utd),
                                       self._stream(stream)), "dg_rhs_jvp")
        return Ut, Utd

    def tlm_steps(self, dt, U, Udot, Ut_tmp, nSteps=1, mu_dot=0.0, stream=None):
        """nSteps LSERK steps of U and its tangent Udot, in place."""
        for x in (U, Udot, Ut_tmp):
            self._check_state(x)
        nat.check(nat.lib().dg_tlm_steps(self._h, 0.0, float(dt), int(nSteps), _tp(U), _tp(Udot), float(mu_dot),
                                         _tp(Ut_tmp), self._stream(stream)), "dg_tlm_steps")

    def rhs_vjp(self, U, Utbar, stream=None):
        """(Ubar, mu_bar) = ((dR/dU)^T Utbar, <Utbar, dR/dmu>)."""
        self._check_state(U)
        self._check_state(Utbar)
        Ub = self._torch.empty_like(U)
        mb = ctypes.c_double()
        nat.check(nat.lib().dg_rhs_vjp(self._h, 0.0, _tp(U), _tp(Utbar), _tp(Ub), ctypes.byref(mb),
                                       self._stream(stream)), "dg_rhs_vjp")
        return Ub, mb.value

    def adjoint_scratch_bytes(self):
        """Device memory the adjoint still allocates besides its checkpoints (dg_adjoint_scratch_bytes)."""
        b = ctypes.c_size_t()
        nat.check(nat.lib().dg_adjoint_scratch_bytes(self._h, ctypes.byref(b)), "dg_adjoint_scratch_bytes")
        return b.value

    def adjoint_forward(self, dt, nSteps, U0, budget_bytes, stream=None, out=None):
        """Run and record nSteps steps from U0; returns (U_final, plan).  out: tensor for U_final
        (may be U0 itself)."""
        self._check_state(U0)
        Uf = self._torch.empty_like(U0) if out is None else out
        plan = ctypes.c_int()
        nat.check(nat.lib().dg_adjoint_forward(self._h, 0.0, float(dt), int(nSteps), _tp(U0), _tp(Uf),
                                               int(budget_bytes), ctypes.byref(plan), self._stream(stream)),
                  "dg_adjoint_forward")
        return Uf, plan.value

    def adjoint_reverse(self, Ubar, stream=None):
        """Ubar (in place): dJ/dU(t_end) -> dJ/dU(t0); returns dJ/dmu."""
        self._check_state(Ubar)
        mb = ctypes.c_double()
        nat.check(nat.lib().dg_adjoint_reverse(self._h, _tp(Ubar), ctypes.byref(mb), self._stream(stream)),
                  "dg_adjoint_reverse")
        return mb.value

    def adjoint_window(self, dt, nSteps, U0, budget_bytes, stream=None):
        """Kinetic-energy objective after nSteps: (J, dJ/dU0, dJ/dmu, U_final)."""
        self._check_state(U0)
        G, Uf = self._torch.empty_like(U0), self._torch.empty_like(U0)
        J, mb = ctypes.c_double(), ctypes.c_double()
        nat.check(nat.lib().dg_adjoint_window(self._h, 0.0, float(dt), int(nSteps), _tp(U0), int(budget_bytes),
                                              ctypes.byref(J), _tp(G), ctypes.byref(mb), _tp(Uf),
                                              self._stream(stream)), "dg_adjoint_window")
        return J.value, G, mb.value, Uf

    def laf_state(self):
        """(lim, eRatio, r) per element of the LAF filter after the last operator call (dg_laf_state)."""
        out = [np.zeros(self.mesh.nElems) for _ in range(3)]
        nat.check(nat.lib().dg_laf_state(self._h, *[_ptr(a) for a in out]), "dg_laf_state")
        return tuple(out)

    def gradients(self, stream=None):
        """Lifted gradients (GradUx, GradUy, GradUz) of the last RHS evaluation, each a float64 CUDA
        tensor (nElems, n, n, n, 5) over the lifting variables (rho, u, v, w, T)."""
        torch = self._torch
        m = self.mesh
        n = self.cfg.N + 1
        g = [torch.empty((m.nElems, n, n, n, 5), dtype=torch.float64, device="cuda") for _ in range(3)]
        nat.check(nat.lib().dg_get_gradients(self._h, *[ctypes.c_void_p(x.data_ptr()) for x in g],
                                             self._stream(stream)), "dg_get_gradients")
        return tuple(g)

    def check_state(self, U, stream=None):
        """Number of nodes holding NaN/Inf or non-positive density/pressure."""
        self._check_state(U)
        bad = ctypes.c_longlong()
        rc = nat.lib().dg_check_state(self._h, ctypes.c_void_p(U.data_ptr()), ctypes.byref(bad), self._stream(stream))
        if rc not in (nat.DG_OK, nat.DG_ERR_NAN):
            nat.check(rc, "dg_check_state")
        return bad.value
