"""Every polynomial degree the library compiles (N = 1..9, one translation unit per N+1) against the
oracle, on meshes whose element counts leave partial element blocks (EPB elements per block for
N <= 4) and on a single self-periodic element (each face of the element is connected to its own
opposite face).

Bar: plain FP64 within 1e-12 relative L2 per RHS evaluation and 1e-10 after LSERK steps; the mixed
form within 1e-5.
"""
import math
import zlib

import numpy as np
import pytest

import galaexi_gb300 as gx
from oracle.oracle import Oracle

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

DIMS = [(1, 1, 1), (3, 2, 1)]


def state(m, seed, R):
    rng = np.random.default_rng(seed)
    U = gx.tgv_state(m, mach=0.3, R=R)
    return U + 1e-2 * rng.standard_normal(U.shape) * np.abs(U).mean(axis=(0, 1, 2, 3))


def rhs_pair(cfg, m, U):
    op = gx.DG(cfg, m)
    Ut = op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U.copy()).cuda())
    torch.cuda.synchronize()
    out = Ut.cpu().numpy()
    op.close()
    return out, Oracle(cfg, m).rhs(U)


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


SCHEMES = [
    ("euler_gauss_lf", dict(NodeType="gauss", Riemann="lf"), 1),
    ("euler_gl_roe", dict(Riemann="roe"), 1),
    ("ns_gauss_hllc_br1", dict(NodeType="gauss", Riemann="hllc", parabolic=True, mu0=2e-3), 1),
    ("ns_gl_split_pi_roe_br1", dict(Riemann="roe", SplitDG="pi", parabolic=True, mu0=2e-3), 2),
    ("ns_gl_split_kg_lf_br2", dict(Riemann="lf", SplitDG="kg", parabolic=True, mu0=2e-3, Lifting="br2"), 2),
]


@pytest.mark.parametrize("dims", DIMS, ids=["1x1x1", "3x2x1"])
@pytest.mark.parametrize("sname,skw,Nmin", SCHEMES, ids=[s[0] for s in SCHEMES])
@pytest.mark.parametrize("N", range(1, 10))
def test_rhs_every_degree(N, sname, skw, Nmin, dims):
    if N < Nmin:
        pytest.skip("split forms need N >= 2")
    R = 71.42857
    cfg = gx.config(N=N, R=R, **skw)
    nt = 1 if skw.get("NodeType") == "gauss" else 2
    m = gx.Mesh(N, nt, *dims, (-math.pi,) * 3, (math.pi,) * 3, deform=0.0 if dims == (1, 1, 1) else 0.03)
    U = state(m, zlib.crc32(("%s%d%s" % (sname, N, dims)).encode()), R)
    gpu, ref = rhs_pair(cfg, m, U)
    assert np.isfinite(gpu).all()
    assert rel(gpu, ref) <= 1e-12, (N, sname, dims, rel(gpu, ref))


@pytest.mark.parametrize("N", [1, 2, 6, 8, 9])
def test_lserk_steps_every_degree(N):
    R = 71.42857
    kw = dict(Riemann="roe", parabolic=True, mu0=2e-3)
    if N >= 2:
        kw["SplitDG"] = "pi"
    cfg = gx.config(N=N, R=R, **kw)
    m = gx.Mesh(N, 2, 3, 2, 1, (-math.pi,) * 3, (math.pi,) * 3)
    U = state(m, N, R)
    o = Oracle(cfg, m)
    dt, _ = o.calc_timestep(U, 0.9, 0.9)
    ref, _ = o.lserk_steps(U, dt, 10)
    op = gx.DG(cfg, m)
    Ud = torch.from_numpy(U.copy()).cuda()
    dt_gpu, _ = op.CalcTimeStep(Ud, 0.9, 0.9)
    assert abs(dt_gpu - dt) <= 1e-14 * dt
    op.TimeStepByLSERKW2(0.0, dt, Ud, torch.zeros_like(Ud), nSteps=10)
    torch.cuda.synchronize()
    err = rel(Ud.cpu().numpy(), ref)
    op.close()
    assert err <= 1e-10, (N, err)


@pytest.mark.parametrize("N", [1, 4, 9])
def test_mixed_every_degree(N):
    R = 71.42857
    kw = dict(Riemann="roe", parabolic=True, mu0=2e-3)
    if N >= 2:
        kw["SplitDG"] = "pi"
    m = gx.Mesh(N, 2, 3, 2, 1, (-math.pi,) * 3, (math.pi,) * 3)
    U = state(m, 100 + N, R)
    ref = Oracle(gx.config(N=N, R=R, **kw), m).rhs(U)
    op = gx.DG(gx.config(N=N, R=R, precision="mixed", **kw), m)
    Ut = op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U.copy()).cuda())
    torch.cuda.synchronize()
    err = rel(Ut.cpu().numpy(), ref)
    op.close()
    assert err <= 1e-5, (N, err)


@pytest.mark.parametrize("lift", ["br1", "br2"])
@pytest.mark.parametrize("N", [2, 5, 8, 9])
def test_mixed_gauss_curved(N, lift):
    """Mixed form on Gauss nodes (density and momenta interpolated to the faces in FP32, the energy in
    FP64; N = 9 interpolates all in FP64) on a curved mesh, HLLC, against the FP64 oracle."""
    R = 71.42857
    kw = dict(NodeType="gauss", Riemann="hllc", parabolic=True, mu0=2e-3, Lifting=lift)
    if lift == "br2":
        kw["etaBR2"] = 2.0
    m = gx.Mesh(N, 1, 3, 2, 2, (-math.pi,) * 3, (math.pi,) * 3, deform=0.05)
    U = state(m, 200 + N, R)
    ref = Oracle(gx.config(N=N, R=R, **kw), m).rhs(U)
    op = gx.DG(gx.config(N=N, R=R, precision="mixed", **kw), m)
    Ut = op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U.copy()).cuda())
    torch.cuda.synchronize()
    err = rel(Ut.cpu().numpy(), ref)
    op.close()
    assert err <= 1e-5, (N, lift, err)


@pytest.mark.parametrize("split", ["sd", "mo", "du", "kg", "pi"])
@pytest.mark.parametrize("N", [5, 6, 7])
def test_mixed_split_forms(N, split):
    """Mixed form of every split flux at the degrees whose FP32 split-form phase runs two threads per
    line and reads staged metric terms, Euler and Navier-Stokes, against the FP64 oracle."""
    R = 71.42857
    for parabolic in (False, True):
        kw = dict(Riemann="roe", SplitDG=split, parabolic=parabolic, mu0=2e-3)
        m = gx.Mesh(N, 2, 3, 2, 1, (-math.pi,) * 3, (math.pi,) * 3, deform=0.03)
        U = state(m, 300 + N, R)
        ref = Oracle(gx.config(N=N, R=R, **kw), m).rhs(U)
        op = gx.DG(gx.config(N=N, R=R, precision="mixed", **kw), m)
        Ut = op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U.copy()).cuda())
        torch.cuda.synchronize()
        err = rel(Ut.cpu().numpy(), ref)
        op.close()
        assert err <= 1e-5, (N, split, parabolic, err)


@pytest.mark.parametrize("N", [3, 4, 5, 6, 7])
def test_mixed_persistent_kernels_walk_several_elements(N):
    """The mixed form's persistent kernels on Gauss-Lobatto nodes (k_volume_lines at n = 4..8,
    k_prolong_gl at n = 6, 8) run one block per SM slot and let each block walk several elements,
    swapping its two shared-memory buffers; on a 12^3 mesh every block takes more than one element
    (n = 4, 6, 8 copy by bulk copies, n = 5, 7 by the threads).  The RHS and two LSERK steps against
    the oracle."""
    R = 71.42857
    kw = dict(Riemann="roe", parabolic=True, mu0=2e-3, SplitDG="pi")
    m = gx.Mesh(N, 2, 12, 12, 12, (-math.pi,) * 3, (math.pi,) * 3)
    U = state(m, 300 + N, R)
    o = Oracle(gx.config(N=N, R=R, **kw), m)
    ref = o.rhs(U)
    op = gx.DG(gx.config(N=N, R=R, precision="mixed", **kw), m)
    Ud = torch.from_numpy(U.copy()).cuda()
    Ut = op.DGTimeDerivative_weakForm(0.0, Ud)
    torch.cuda.synchronize()
    assert rel(Ut.cpu().numpy(), ref) <= 1e-5, N
    dt, _ = o.calc_timestep(U, 0.8, 0.8)
    ref2, _ = o.lserk_steps(U, dt, 2)
    op.TimeStepByLSERKW2(0.0, dt, Ud, torch.zeros_like(Ud), nSteps=2)
    torch.cuda.synchronize()
    assert rel(Ud.cpu().numpy(), ref2) <= 1e-6, N
    op.close()
