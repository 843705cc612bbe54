"""Boundary conditions (GetBoundaryState / GetBoundaryFlux / Lifting_GetBoundaryFlux,
equations/navierstokes/idealgas/getboundaryflux.f90) on the reference's own mesh files.

Pins: the oracle reproduces the reference's lid-driven cavity regression (regressioncheck/checks/
parabolic/cavity_3D: isothermal walls, a Dirichlet lid, RoeEntropyFix, BR1, N = 2 Gauss, 353 CFL-
limited LSERK steps to t = 1) within that regression's own h5diff tolerance (1e-12 absolute on
DG_Solution).  The CUDA path is then checked against the oracle per evaluation on every BC type, on
flat and curved (NGeo = 2) meshes, and over the same 353-step cavity run.
"""
import os
import zlib

import numpy as np
import pytest

import galaexi_gb300 as gx
from oracle.oracle import Oracle
from tests.tgv_analysis import TimeControl

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CAVITY = os.path.join(GOLDEN, "cavity4x4x4_mesh.h5")
CAVITY_STATE = os.path.join(GOLDEN, "reggie_cavity_Re100_State_0000001.000000000.h5")
PLATE = os.path.join(GOLDEN, "CART_HEX2D_FlatPlateG_mesh.h5")
NACA = os.path.join(GOLDEN, "NACA0012_652_Ng2_mesh.h5")

# regressioncheck/checks/parabolic/cavity_3D/parameter.ini
CAVITY_REFSTATES = [[1.0, 1.0, 0.0, 0.0, 71.4285714286], [1.0, 0.0, 0.0, 0.0, 71.4285714286]]
CAVITY_BOUNDARIES = {"BC_wall_left": (4, 1), "BC_wall_right": (4, 1), "BC_free": (2, 1)}
CAVITY_ATOL = 1e-12  # the regression's h5diff_tolerance_value (absolute)

KAPPA, RGAS = 1.4, 1.0
P0 = 1.0 / KAPPA  # sound speed 1 at rho = 1
T0 = P0 / RGAS
MA = 0.3
# RefStates of the synthetic flow: 1 free stream, 2 outflow pressure, 3 subsonic inflow
# (Tt, alpha, beta, -, pt), 4 outflow Mach number (u = Mach), 5 a colder wall
FLOW_REFSTATES = [[1.0, MA, 0.0, 0.0, P0],
                  [1.0, MA, 0.0, 0.0, 0.98 * P0],
                  [T0 * (1 + 0.2 * MA * MA), 5.0, -3.0, 0.0, P0 * (1 + 0.2 * MA * MA) ** 3.5],
                  [1.0, 0.5, 0.0, 0.0, P0],
                  [1.2, 0.0, 0.0, 0.0, 0.95 * P0]]


def cavity_case(N=2, node_type=1):
    m = gx.Mesh.from_hopr(CAVITY, N, node_type)
    return m, m.boundaries(CAVITY_REFSTATES, CAVITY_BOUNDARIES)


def cavity_config(**kw):
    base = dict(N=2, NodeType="gauss", Riemann="roeentropyfix", parabolic=True, mu0=0.01, R=1.0, Pr=0.72,
                kappa=1.4)
    base.update(kw)
    return gx.config(**base)


def cavity_initial(m):
    # IniExactFunc = 1, IniRefState = 2: the fluid at rest
    n = m.N + 1
    U = np.zeros((m.nElems, n, n, n, 5))
    U[..., 0] = 1.0
    U[..., 4] = 71.4285714286 / (1.4 - 1.0)
    return U


def flow_state(m, seed):
    """A smooth subsonic flow (Mach ~0.3 in x) with a seeded perturbation, conservative variables."""
    x = m.Elem_xGP
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.5, 1.5, 6)
    rho = 1.0 + 0.05 * np.sin(a[0] * x[..., 0] + x[..., 1])
    u = MA + 0.05 * np.sin(a[1] * x[..., 2] + x[..., 1])
    v = 0.05 * np.cos(a[2] * x[..., 0])
    w = 0.02 * np.sin(a[3] * x[..., 1] - x[..., 2])
    p = P0 * (1.0 + 0.05 * np.cos(a[4] * x[..., 0] - a[5] * x[..., 2]))
    U = np.empty(x.shape[:-1] + (5,))
    U[..., 0] = rho
    U[..., 1], U[..., 2], U[..., 3] = rho * u, rho * v, rho * w
    U[..., 4] = p / (KAPPA - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return U


# flat-plate tutorial mesh: the tutorial's own BC set, and every other supported type
PLATE_TUTORIAL = {"BC_x-": (2, 1), "BC_x+": (24, 2), "BC_y-": (3, 0), "BC_y+": (2, 1), "BC_Euler_y-": (9, 0)}
PLATE_OTHERS = {"BC_x-": (27, 3), "BC_x+": (25, 2), "BC_y-": (91, 0), "BC_y+": (23, 4), "BC_Euler_y-": (4, 5)}
NACA_BCS = {"BC_wall": (3, 0), "BC_inflow": (2, 1), "BC_outflow": (2, 1)}


def roundoff(U, m):
    """Round-off scale of Ut for a state U on mesh m: 100 eps |U| max(sJ) (a wrong BC flux gives
    O(|U| sJ), e.g. 5.8e2 on the airfoil mesh against 2e-11 for the free stream)."""
    return 100 * np.finfo(float).eps * np.abs(U).max() * np.abs(m.sJ).max()


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ------------------------------------------------------------------------------------------------
# CPU: the oracle against the reference
# ------------------------------------------------------------------------------------------------
def run_cavity(stepper, calc_dt):
    tc = TimeControl(1.0)
    while True:
        dt = tc.update(calc_dt())
        stepper(tc.t, dt)
        tc.advance(dt)
        if tc.doFinalize:
            return tc.iter


def test_oracle_reproduces_cavity_regression():
    m, bnd = cavity_case()
    o = Oracle(cavity_config(), m, bnd)
    st = {"U": cavity_initial(m)}

    def calc_dt():
        dt, err = o.calc_timestep(st["U"], 0.99, 0.4)
        assert err == 0
        return dt

    def step(t, dt):
        st["U"], _ = o.lserk_steps(st["U"], dt, 1, t=t)

    iters = run_cavity(step, calc_dt)
    ref = gx.read_h5(CAVITY_STATE, "DG_Solution")
    assert float(gx.read_h5(CAVITY_STATE, "Time", attribute=True)[0]) == 1.0
    assert ref.shape == st["U"].shape and iters > 300
    err = np.abs(st["U"] - ref).max()
    assert err <= CAVITY_ATOL, err


def test_state_file_attributes():
    assert gx.read_h5(CAVITY_STATE, "NodeType", attribute=True) == "GAUSS"
    assert gx.read_h5(CAVITY_STATE, "MeshFile", attribute=True) == "cavity4x4x4_mesh.h5"
    assert int(gx.read_h5(CAVITY_STATE, "N", attribute=True)[0]) == 2


@pytest.mark.parametrize("wall", [3, 4, 9, 91])
def test_rest_state_is_steady(wall):
    """A fluid at rest between walls of its own temperature (and a Dirichlet side of the same state)
    stays at rest: the wall pressure of the local Riemann problem is the inner pressure."""
    m = gx.Mesh.from_hopr(CAVITY, 3, 2)
    bnd = m.boundaries(CAVITY_REFSTATES, {"BC_wall_left": (wall, 2), "BC_wall_right": (wall, 2),
                                          "BC_wall_lower": (wall, 2), "BC_zminus": (wall, 2),
                                          "BC_zplus": (wall, 2), "BC_free": (2, 2)})
    cfg = cavity_config(N=3, NodeType="gauss-lobatto", Riemann="roe", SplitDG="pi")
    U = cavity_initial(m)
    Ut = Oracle(cfg, m, bnd).rhs(U)
    assert np.abs(Ut).max() <= roundoff(U, m)


def test_freestream_on_curved_mesh_with_farfield():
    """Free-stream preservation on the curved airfoil mesh when every BC side is a Dirichlet side of
    the free stream (curl-form metrics satisfy the discrete metric identities)."""
    m = gx.Mesh.from_hopr(NACA, 3, 2)
    bnd = m.boundaries(FLOW_REFSTATES, {"BC_wall": (2, 1), "BC_inflow": (2, 1), "BC_outflow": (2, 1)})
    cfg = gx.config(N=3, Riemann="roe", SplitDG="pi", parabolic=True, mu0=1e-3, R=RGAS, kappa=KAPPA)
    n = m.N + 1
    U = np.zeros((m.nElems, n, n, n, 5))
    U[..., 0], U[..., 1], U[..., 4] = 1.0, MA, P0 / (KAPPA - 1) + 0.5 * MA * MA
    Ut = Oracle(cfg, m, bnd).rhs(U)
    assert np.abs(Ut).max() <= roundoff(U, m), np.abs(Ut).max()


def test_boundary_name_overrides():
    m = gx.Mesh.from_hopr(PLATE, 1, 2)
    bt, bs, rs = m.boundaries(FLOW_REFSTATES, PLATE_TUTORIAL)
    names = [m.BCNames[i - 1] for i in m.BCIndex]
    for name, (typ, state) in PLATE_TUTORIAL.items():
        sel = np.array([nm == name for nm in names])
        assert sel.any() and (bt[sel] == typ).all() and (bs[sel] == state).all()
    with pytest.raises(ValueError):
        m.boundaries(FLOW_REFSTATES, {"BC_nowhere": (2, 1)})
    with pytest.raises(ValueError):
        m.boundaries(FLOW_REFSTATES, {"BC_z-": (2, 1)})  # periodic in the file


def test_oracle_rejects_unknown_bc_type():
    m = gx.Mesh.from_hopr(PLATE, 1, 2)
    bt, bs, rs = m.boundaries(FLOW_REFSTATES, PLATE_TUTORIAL)
    bt = bt.copy()
    bt[0] = 12  # state-file BC: not part of this path
    with pytest.raises(ValueError):
        Oracle(gx.config(N=1), m, (bt, bs, rs))


# ------------------------------------------------------------------------------------------------
# GPU: the CUDA path against the oracle
# ------------------------------------------------------------------------------------------------
CONFIGS = [
    ("ns_gl_split_pi_roe_br1", dict(Riemann="roe", SplitDG="pi", parabolic=True, mu0=2e-3), 2),
    ("ns_gauss_roeef_br1_weaklift", dict(NodeType="gauss", Riemann="roeentropyfix", parabolic=True, mu0=2e-3,
                                         doWeakLifting=True), 1),
    ("ns_gl_lf_br2", dict(Riemann="lf", parabolic=True, mu0=2e-3, Lifting="br2"), 2),
    ("ns_gauss_hlle_conslift", dict(NodeType="gauss", Riemann="hlle", parabolic=True, mu0=2e-3,
                                    doConservativeLifting=True), 1),
    ("euler_gl_split_kg_roel2", dict(Riemann="roel2", SplitDG="kg"), 2),
    ("euler_gauss_hllc", dict(NodeType="gauss", Riemann="hllc"), 1),
]
MESHES = [
    ("plate_tutorial", PLATE, PLATE_TUTORIAL, 3),
    ("plate_other_types", PLATE, PLATE_OTHERS, 3),
    ("naca_curved", NACA, NACA_BCS, 2),
]


def _gpu_rhs(cfg, m, bnd, U):
    torch = pytest.importorskip("torch")
    op = gx.DG(cfg, m, boundaries=bnd)
    Ut = op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U).cuda())
    torch.cuda.synchronize()
    out = Ut.cpu().numpy()
    op.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("cname,ckw,nt", CONFIGS, ids=[c[0] for c in CONFIGS])
@pytest.mark.parametrize("mname,path,bcs,N", MESHES, ids=[m[0] for m in MESHES])
def test_bc_rhs_matches_oracle(cname, ckw, nt, mname, path, bcs, N):
    cfg = gx.config(N=N, R=RGAS, kappa=KAPPA, **ckw)
    m = gx.Mesh.from_hopr(path, N, nt)
    bnd = m.boundaries(FLOW_REFSTATES, bcs)
    U = flow_state(m, zlib.crc32((cname + mname).encode()))
    gpu = _gpu_rhs(cfg, m, bnd, U)
    ref = Oracle(cfg, m, bnd).rhs(U)
    assert np.isfinite(gpu).all()
    err = rel_l2(gpu, ref)
    assert err <= 1e-12, "%s/%s: relative L2 %.3e" % (cname, mname, err)


@pytest.mark.gpu
@pytest.mark.parametrize("mname,path,bcs,N", MESHES, ids=[m[0] for m in MESHES])
def test_bc_rhs_mixed_precision(mname, path, bcs, N):
    cfg = gx.config(N=N, R=RGAS, kappa=KAPPA, Riemann="roe", SplitDG="pi", parabolic=True, mu0=2e-3)
    cfgm = gx.config(N=N, R=RGAS, kappa=KAPPA, Riemann="roe", SplitDG="pi", parabolic=True, mu0=2e-3,
                     precision="mixed")
    m = gx.Mesh.from_hopr(path, N, 2)
    bnd = m.boundaries(FLOW_REFSTATES, bcs)
    U = flow_state(m, 11)
    gpu = _gpu_rhs(cfgm, m, bnd, U)
    ref = Oracle(cfg, m, bnd).rhs(U)
    err = rel_l2(gpu, ref)
    assert err <= 1e-5, err


@pytest.mark.gpu
def test_gpu_reproduces_cavity_regression():
    torch = pytest.importorskip("torch")
    m, bnd = cavity_case()
    op = gx.DG(cavity_config(), m, boundaries=bnd)
    U = torch.from_numpy(cavity_initial(m)).cuda()
    Ut_tmp = torch.zeros_like(U)

    def calc_dt():
        dt, err = op.CalcTimeStep(U, 0.99, 0.4)
        assert err == 0
        return dt

    def step(t, dt):
        op.TimeStepByLSERKW2(t, dt, U, Ut_tmp)

    run_cavity(step, calc_dt)
    torch.cuda.synchronize()
    ref = gx.read_h5(CAVITY_STATE, "DG_Solution")
    err = np.abs(U.cpu().numpy() - ref).max()
    op.close()
    assert err <= CAVITY_ATOL, err


# the adjoint's forms (BR1 in strong form, non-conservative or conservative; Euler)
ADJOINT_CONFIGS = [c for c in CONFIGS if "weaklift" not in c[0] and "br2" not in c[0]]


def _adjoint_state(m, seed):
    rng = np.random.default_rng(seed)
    U0 = flow_state(m, seed)
    # node noise: keeps the Lax-Friedrichs / Roe wave-speed maxima away from ties, where the operator
    # has one-sided derivatives only
    return U0 * (1.0 + 1e-3 * rng.standard_normal(U0.shape)), rng


@pytest.mark.gpu
@pytest.mark.parametrize("cname,ckw,nt", ADJOINT_CONFIGS, ids=[c[0] for c in ADJOINT_CONFIGS])
@pytest.mark.parametrize("mname,path,bcs,N", MESHES, ids=[m[0] for m in MESHES])
def test_bc_adjoint_dot_product(cname, ckw, nt, mname, path, bcs, N):
    """The discrete adjoint on meshes with boundary sides (the boundary flux and the lifting ghost
    state transposed through their local Jacobians) against the tangent-linear operator:
    <ybar, J v> = <J^T ybar, v> + mubar mu_dot per RHS evaluation, to round-off."""
    torch = pytest.importorskip("torch")
    cfg = gx.config(N=N, R=RGAS, kappa=KAPPA, **ckw)
    m = gx.Mesh.from_hopr(path, N, nt)
    bnd = m.boundaries(FLOW_REFSTATES, bcs)
    U0, rng = _adjoint_state(m, zlib.crc32((cname + mname + "adj").encode()))
    U = torch.from_numpy(U0).cuda()
    v = torch.from_numpy(rng.standard_normal(U0.shape)).cuda()
    ybar = torch.from_numpy(rng.standard_normal(U0.shape)).cuda()
    mu_dot = 0.7 if cfg.parabolic else 0.0
    op = gx.DG(cfg, m, boundaries=bnd)
    _, Jv = op.rhs_jvp(U, v, mu_dot)
    Ub, mub = op.rhs_vjp(U, ybar)
    op.close()
    lhs = float((ybar * Jv).sum())
    rhs = float((Ub * v).sum()) + mub * mu_dot
    scale = float(ybar.norm() * Jv.norm())
    assert abs(lhs - rhs) <= 1e-13 * scale, (cname, mname, lhs, rhs, scale)


@pytest.mark.gpu
def test_bc_adjoint_window_dot_product_cavity():
    """The adjoint of 10 LSERK steps of the cavity regression's operator (isothermal walls, a
    Dirichlet lid) from a perturbed moving state: <ybar, Udot(t_end)> of the tangent-linear steps
    equals <Ubar(t0), v> + mubar mu_dot of the reverse sweep to 1e-10."""
    torch = pytest.importorskip("torch")
    m, bnd = cavity_case()
    op = gx.DG(cavity_config(), m, boundaries=bnd)
    rng = np.random.default_rng(11)
    U0 = cavity_initial(m)
    U0[..., 1] = 0.1 * np.sin(m.Elem_xGP[..., 1] * np.pi)  # some x-momentum
    U0[..., 4] += 0.5 * U0[..., 1] ** 2
    U0 = torch.from_numpy(U0 * (1.0 + 1e-3 * rng.standard_normal(U0.shape))).cuda()
    dt, err = op.CalcTimeStep(U0, 0.99, 0.4)
    assert err == 0
    nSteps, mu_dot = 10, 0.3
    v = torch.from_numpy(rng.standard_normal(tuple(U0.shape))).cuda()
    ybar = torch.from_numpy(rng.standard_normal(tuple(U0.shape))).cuda()
    U, Ud, K = U0.clone(), v.clone(), torch.zeros_like(U0)
    op.tlm_steps(dt, U, Ud, K, nSteps=nSteps, mu_dot=mu_dot)
    Uf, plan = op.adjoint_forward(dt, nSteps, U0, budget_bytes=1 << 32)
    assert float((Uf - U).abs().max()) <= 1e-13 * float(U.abs().max())
    Ub = ybar.clone()
    mub = op.adjoint_reverse(Ub)
    op.close()
    lhs = float((ybar * Ud).sum())
    rhs = float((Ub * v).sum()) + mub * mu_dot
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs), (lhs, rhs)


@pytest.mark.gpu
@pytest.mark.parametrize("cname,ckw,nt", CONFIGS, ids=[c[0] for c in CONFIGS])
@pytest.mark.parametrize("mname,path,bcs,N", MESHES, ids=[m[0] for m in MESHES])
def test_bc_tangent_linear_vs_central_differences(cname, ckw, nt, mname, path, bcs, N):
    """The tangent-linear operator (the forward kernels on dual numbers, the boundary kernels
    included) on meshes with boundary sides: its primal equals the plain RHS, its tangent equals
    central differences of the plain RHS along a seeded direction and a viscosity change."""
    torch = pytest.importorskip("torch")
    cfg = gx.config(N=N, R=RGAS, kappa=KAPPA, **ckw)
    m = gx.Mesh.from_hopr(path, N, nt)
    bnd = m.boundaries(FLOW_REFSTATES, bcs)
    seed = zlib.crc32((cname + mname + "tlm").encode())
    rng = np.random.default_rng(seed)
    # node noise on top of the smooth flow: at nodes on y = z = 0 the smooth state's normal velocity on
    # the outflow boundary equals the reference state's exactly, a tie of the Lax-Friedrichs wave-speed
    # maximum where the operator has only one-sided derivatives (the dual numbers take one side,
    # central differences average the two)
    U0 = flow_state(m, seed)
    U = torch.from_numpy(U0 * (1.0 + 1e-3 * rng.standard_normal(U0.shape))).cuda()
    v = torch.from_numpy(rng.standard_normal(tuple(U.shape))).cuda()
    v = v * U.abs().mean(dim=(0, 1, 2, 3)) * 1e-2
    mu_dot = 1e-3 if cfg.parabolic else 0.0
    op = gx.DG(cfg, m, boundaries=bnd)
    Ut = op.DGTimeDerivative_weakForm(0.0, U.clone())
    Ut2, Jv = op.rhs_jvp(U, v, mu_dot)
    op.close()
    assert float((Ut2 - Ut).norm() / Ut.norm()) <= 1e-13
    eps = 1e-6
    fd = []
    for sgn in (1.0, -1.0):
        kw = dict(ckw, mu0=ckw["mu0"] + sgn * eps * mu_dot) if cfg.parabolic else ckw
        o2 = gx.DG(gx.config(N=N, R=RGAS, kappa=KAPPA, **kw), m, boundaries=bnd)
        fd.append(o2.DGTimeDerivative_weakForm(0.0, U + sgn * eps * v))
        o2.close()
    fd = (fd[0] - fd[1]) / (2 * eps)
    err = float((fd - Jv).norm() / Jv.norm())
    assert err <= 1e-6, (cname, mname, err)


@pytest.mark.gpu
def test_bc_mesh_needs_boundaries():
    m, _ = cavity_case()
    with pytest.raises(ValueError):
        gx.DG(cavity_config(), m)
