"""Parity of the CUDA path (through the C ABI) with the oracle, on seeded inputs.

Bar (from the reference path's specification): plain FP64 Ut within 1e-12 relative L2 of the oracle
per evaluation, and within 1e-10 after 100 LSERK steps; the mixed form within 1e-5 relative L2 of
the FP64 oracle per evaluation.
"""
import math
import zlib

import numpy as np
import pytest

import galaexi_gb300 as gx
from oracle.oracle import Oracle

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

RTOL_RHS = 1e-12
RTOL_STEPS = 1e-10


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def perturbed_state(mesh, base, seed, amp=1e-2):
    """Seeded smooth-plus-noise state around a base state (keeps rho, p positive)."""
    rng = np.random.default_rng(seed)
    U = base.copy()
    U += amp * rng.standard_normal(U.shape) * np.abs(U).mean(axis=(0, 1, 2, 3))
    return U


def tgv_case(N, nx, ny, nz, mach=0.1, R=71.42857):
    m = gx.Mesh(N, 2, nx, ny, nz, (-math.pi,) * 3, (math.pi,) * 3)
    return m, gx.tgv_state(m, mach=mach, kappa=1.4, R=R)


def run_rhs_pair(cfg, mesh, U):
    op = gx.DG(cfg, mesh)
    Ud = torch.from_numpy(U).cuda()
    Ut = op.DGTimeDerivative_weakForm(0.0, Ud)
    torch.cuda.synchronize()
    gpu = Ut.cpu().numpy()
    ref = Oracle(cfg, mesh).rhs(U)
    op.close()
    return gpu, ref


CASES = [
    # (name, config kwargs, N, node_type, mesh dims)
    ("euler_gauss_weak_lf", dict(NodeType="gauss", Riemann="lf"), 3, 1, (3, 2, 2)),
    ("euler_gl_weak_roe", dict(Riemann="roe"), 4, 2, (2, 3, 2)),
    ("euler_gl_split_pi_roe", dict(Riemann="roe", SplitDG="pi"), 5, 2, (2, 2, 3)),
    ("ns_gl_split_pi_roe_br1", dict(Riemann="roe", SplitDG="pi", parabolic=True, mu0=6.25e-4, R=71.42857), 7, 2, (2, 2, 2)),
    ("ns_gl_split_pi_roeef_br1", dict(Riemann="roeentropyfix", SplitDG="pi", parabolic=True, mu0=6.25e-4, R=71.42857), 7, 2, (3, 2, 2)),
    ("ns_gauss_weak_hllc_br1", dict(NodeType="gauss", Riemann="hllc", parabolic=True, mu0=1e-3), 5, 1, (2, 2, 3)),
    ("ns_gauss_weak_roe_br1_weaklift", dict(NodeType="gauss", Riemann="roe", parabolic=True, mu0=1e-3, doWeakLifting=True), 4, 1, (2, 3, 2)),
    ("ns_gl_weak_lf_br1_conslift", dict(Riemann="lf", parabolic=True, mu0=1e-3, doConservativeLifting=True), 4, 2, (3, 2, 2)),
]


@pytest.mark.parametrize("name,kw,N,nt,dims", CASES, ids=[c[0] for c in CASES])
def test_rhs_matches_oracle(name, kw, N, nt, dims):
    cfg = gx.config(N=N, **kw)
    m = gx.Mesh(N, nt, *dims, (-math.pi,) * 3, (math.pi,) * 3)
    U = perturbed_state(m, gx.tgv_state(m, mach=0.3, R=cfg.R), seed=zlib.crc32(name.encode()))
    gpu, ref = run_rhs_pair(cfg, m, U)
    assert np.isfinite(gpu).all()
    err = rel_l2(gpu, ref)
    assert err <= RTOL_RHS, "%s: relative L2 %.3e" % (name, err)


@pytest.mark.parametrize("riemann", ["lf", "roe", "roel2", "roeentropyfix", "hll", "hllc", "hlle", "hllem"])
def test_every_riemann_solver_weak(riemann):
    cfg = gx.config(N=3, NodeType="gauss", Riemann=riemann)
    m = gx.Mesh(3, 1, 2, 2, 2, (0, 0, 0), (1, 1, 1))
    U = perturbed_state(m, gx.fill_ini(m, 1, [1.0, 0.3, -0.2, 0.1, 1.0]), seed=7, amp=5e-2)
    gpu, ref = run_rhs_pair(cfg, m, U)
    assert rel_l2(gpu, ref) <= RTOL_RHS


@pytest.mark.parametrize("split", ["sd", "mo", "du", "kg", "pi"])
@pytest.mark.parametrize("riemann", ["lf", "roe", "roeentropyfix", "avg"])
def test_every_split_flux(split, riemann):
    cfg = gx.config(N=4, Riemann=riemann, SplitDG=split)
    m = gx.Mesh(4, 2, 2, 2, 2, (0, 0, 0), (1, 1, 1))
    U = perturbed_state(m, gx.fill_ini(m, 1, [1.0, 0.3, -0.2, 0.1, 1.0]), seed=11, amp=5e-2)
    gpu, ref = run_rhs_pair(cfg, m, U)
    assert rel_l2(gpu, ref) <= RTOL_RHS


def test_free_stream_preservation_curved():
    """Constant state on the curved (displaced) mesh: Ut vanishes to round-off."""
    cfg = gx.config(N=5, NodeType="gauss", Riemann="hllc", parabolic=True, mu0=1e-3)
    m = gx.Mesh(5, 1, 3, 3, 3, (0, 0, 0), (1, 1, 1), deform=0.05)
    U = gx.fill_ini(m, 1, [1.0, 0.3, 0.2, 0.1, 1 / 1.4])
    op = gx.DG(cfg, m)
    Ut = op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U).cuda()).cpu().numpy()
    assert np.abs(Ut).max() < 1e-11


def test_lserk_100_steps_matches_oracle():
    cfg = gx.config(N=5, Riemann="roe", SplitDG="pi", parabolic=True, mu0=6.25e-4, R=71.42857)
    m, U0 = tgv_case(5, 3, 3, 3)
    op = gx.DG(cfg, m)
    U = torch.from_numpy(U0).cuda()
    dt, err = op.CalcTimeStep(U, 0.5, 0.5)
    assert err == 0
    Ut_tmp = torch.zeros_like(U)
    op.TimeStepByLSERKW2(0.0, dt, U, Ut_tmp, nSteps=100)
    ref, _ = Oracle(cfg, m).lserk_steps(U0, dt, 100)
    assert rel_l2(U.cpu().numpy(), ref) <= RTOL_STEPS


def test_calc_timestep_matches_oracle():
    cfg = gx.config(N=7, Riemann="roeentropyfix", SplitDG="pi", parabolic=True, mu0=6.25e-4, R=71.42857)
    m, U0 = tgv_case(7, 3, 3, 3)
    op = gx.DG(cfg, m)
    dt, err = op.CalcTimeStep(torch.from_numpy(U0).cuda(), 0.8, 0.8)
    dref, eref = Oracle(cfg, m).calc_timestep(U0, 0.8, 0.8)
    assert err == 0 and eref == 0
    assert abs(dt - dref) <= 1e-14 * dref


def test_nan_is_reported_not_trapped():
    """A corrupted host state yields an error status from the C ABI; the context stays usable."""
    cfg = gx.config(N=3, Riemann="lf")
    m = gx.Mesh(3, 2, 2, 2, 2)
    U0 = gx.fill_ini(m, 1, [1.0, 0.1, 0.0, 0.0, 1.0])
    op = gx.DG(cfg, m)
    bad = U0.copy()
    bad[1, 2, 3, 1, 0] = np.nan
    bad[0, 0, 0, 0, 0] = -1.0
    assert op.check_state(torch.from_numpy(bad).cuda()) == 2
    _, err = op.CalcTimeStep(torch.from_numpy(bad).cuda(), 0.9)
    assert err == 1
    dt, err = op.CalcTimeStep(torch.from_numpy(U0).cuda(), 0.9)
    assert err == 0 and dt > 0


def kinetic_energy(mesh, U):
    """Volume-integrated kinetic energy on the solution nodes: sum w_i w_j w_k / sJ * 0.5 |m|^2 / rho."""
    w = gx.basis(mesh.N, mesh.node_type)["wGP"]
    W = w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    return float(np.sum(W / mesh.sJ * 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2 + U[..., 3] ** 2) / U[..., 0]))


def test_mixed_precision_run_close_to_fp64():
    """Mixed form (FP32 bulk, FP64 RK accumulation) vs the FP64 oracle after 30 TGV steps at
    CFL 0.5: relative kinetic-energy error <= 1e-6; relative L2 of U and total-mass drift stated."""
    kw = dict(Riemann="roe", SplitDG="pi", parabolic=True, mu0=6.25e-4, R=71.42857)
    m, U0 = tgv_case(7, 3, 3, 3)
    cfg = gx.config(N=7, **kw)
    dt, _ = Oracle(cfg, m).calc_timestep(U0, 0.5, 0.5)
    ref, _ = Oracle(cfg, m).lserk_steps(U0, dt, 30)
    op = gx.DG(gx.config(N=7, precision="mixed", **kw), m)
    U = torch.from_numpy(U0).cuda()
    op.TimeStepByLSERKW2(0.0, dt, U, torch.zeros_like(U), nSteps=30)
    Um = U.cpu().numpy()
    ke_err = abs(kinetic_energy(m, Um) - kinetic_energy(m, ref)) / kinetic_energy(m, ref)
    w = gx.basis(7, 2)["wGP"]
    W = w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    mass = lambda X: float(np.sum(W / m.sJ * X[..., 0]))
    print("mixed vs FP64: KE rel err %.2e, U rel L2 %.2e, mass drift %.2e" % (
        ke_err, rel_l2(Um, ref), abs(mass(Um) - mass(U0)) / mass(U0)))
    assert ke_err <= 1e-6
    assert rel_l2(Um, ref) < 1e-4


@pytest.mark.parametrize("lift", ["strong", "conservative", "weak"])
def test_lifted_gradients_match_oracle(lift):
    kw = dict(Riemann="roe", parabolic=True, mu0=1e-3, doWeakLifting=lift == "weak",
              doConservativeLifting=lift == "conservative")
    N, nt = (5, 1) if lift == "weak" else (5, 2)
    cfg = gx.config(N=N, NodeType="gauss" if nt == 1 else "gauss-lobatto", **kw)
    m = gx.Mesh(N, nt, 2, 3, 2, (-math.pi,) * 3, (math.pi,) * 3, deform=0.05)
    U = perturbed_state(m, gx.tgv_state(m, mach=0.3, R=cfg.R), seed=11)
    op = gx.DG(cfg, m)
    op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U).cuda())
    grads = [g.cpu().numpy() for g in op.gradients()]
    orc = Oracle(cfg, m)
    orc.rhs(U)
    for d, g in enumerate(grads):
        ref = orc.work(1 + d, g.shape)
        err = rel_l2(g, ref)
        assert err <= RTOL_RHS, "grad %s: relative L2 %.3e" % ("xyz"[d], err)
    op.close()


BR2_CASES = [
    # the curved-box Gauss case of the BR2 workload (weak form, HLLC, etaBR2 = 2)
    ("gauss_weak_hllc_br2_curved", dict(NodeType="gauss", Riemann="hllc", Lifting="br2", etaBR2=2.0), 5, 1, 0.05),
    ("gl_split_pi_roe_br2_conslift", dict(Riemann="roe", SplitDG="pi", Lifting="br2", etaBR2=3.0,
                                          doConservativeLifting=True), 4, 2, 0.0),
    ("gauss_weak_lf_br2_curved_n3", dict(NodeType="gauss", Riemann="lf", Lifting="br2", etaBR2=2.0), 3, 1, 0.05),
]


@pytest.mark.parametrize("name,kw,N,nt,deform", BR2_CASES, ids=[c[0] for c in BR2_CASES])
def test_br2_rhs_and_gradients_match_oracle(name, kw, N, nt, deform):
    cfg = gx.config(N=N, parabolic=True, mu0=1e-3, **kw)
    m = gx.Mesh(N, nt, 3, 2, 2, (0.0,) * 3, (1.0,) * 3, deform=deform)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    U = gx.fill_ini(m, 1, [1.0, 0.3, 0.2, 0.1, 1.0 / 1.4])
    U = U + 1e-2 * rng.standard_normal(U.shape) * np.abs(U).mean(axis=(0, 1, 2, 3))
    op = gx.DG(cfg, m)
    Ut = op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U).cuda()).cpu().numpy()
    grads = [g.cpu().numpy() for g in op.gradients()]
    op.close()
    orc = Oracle(cfg, m)
    ref = orc.rhs(U)
    err = rel_l2(Ut, ref)
    assert err <= RTOL_RHS, "%s: Ut relative L2 %.3e" % (name, err)
    for d, g in enumerate(grads):
        e = rel_l2(g, orc.work(1 + d, g.shape))
        assert e <= RTOL_RHS, "%s: grad %s relative L2 %.3e" % (name, "xyz"[d], e)
