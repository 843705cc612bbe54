"""Tangent-linear and discrete adjoint operators (dg_rhs_jvp, dg_tlm_steps, dg_rhs_vjp, dg_adjoint_*).

Checks, through the C ABI:
  * the dual-number operator reproduces the plain operator's values;
  * the tangent-linear operator against central finite differences of the plain operator;
  * the adjoint against the tangent-linear operator by the dot-product test
    <ybar, J v> = <J^T ybar, v> (both exact linearisations, so the test holds to round-off);
  * over LSERK windows: the dot-product test to 1e-10, the checkpoint plans against each other, and
    the kinetic-energy gradient (w.r.t. the initial state and the viscosity) against central finite
    differences (eps = 1e-6) to 1e-6;
  * a torch.autograd.Function around dg_rhs / dg_rhs_vjp passes torch's gradcheck.
"""
import math
import zlib

import numpy as np
import pytest

import galaexi_gb300 as gx

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

CASES = [
    # name, config kwargs, N, node type, mesh dims, deform
    ("gl_split_pi_roe_ns", dict(Riemann="roe", SplitDG="pi", parabolic=True, mu0=2e-3, R=71.42857), 4, 2, (2, 2, 3), 0.0),
    ("gauss_weak_lf_euler", dict(Riemann="lf"), 3, 1, (3, 2, 2), 0.05),
    ("gauss_weak_hllc_ns_conslift", dict(Riemann="hllc", parabolic=True, mu0=1e-3, doConservativeLifting=True), 3, 1,
     (2, 3, 2), 0.05),
    ("gl_split_kg_roeef_ns", dict(Riemann="roeentropyfix", SplitDG="kg", parabolic=True, mu0=2e-3, R=71.42857), 5, 2,
     (2, 2, 2), 0.0),
    ("gl_weak_roe_ns_curved", dict(Riemann="roe", parabolic=True, mu0=1e-3), 3, 2, (2, 2, 3), 0.05),
]


def setup_case(name, kw, N, nt, dims, deform):
    cfg = gx.config(N=N, NodeType="gauss" if nt == 1 else "gauss-lobatto", **kw)
    m = gx.Mesh(N, nt, *dims, (-math.pi,) * 3, (math.pi,) * 3, deform=deform)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    U = gx.tgv_state(m, mach=0.3, R=cfg.R)
    U = U + 1e-2 * rng.standard_normal(U.shape) * np.abs(U).mean(axis=(0, 1, 2, 3))
    return cfg, m, torch.from_numpy(U).cuda(), rng


def rand_like(rng, U):
    return torch.from_numpy(rng.standard_normal(tuple(U.shape))).cuda()


def dot(a, b):
    return float((a * b).sum())


@pytest.mark.parametrize("name,kw,N,nt,dims,deform", CASES, ids=[c[0] for c in CASES])
def test_jvp_values_and_fd(name, kw, N, nt, dims, deform):
    cfg, m, U, rng = setup_case(name, kw, N, nt, dims, deform)
    op = gx.DG(cfg, m)
    Ut = op.DGTimeDerivative_weakForm(0.0, U)
    v = rand_like(rng, U) * U.abs().mean(dim=(0, 1, 2, 3))
    mu_dot = 1e-3 if cfg.parabolic else 0.0
    Ut2, Jv = op.rhs_jvp(U, v, mu_dot)
    assert float((Ut2 - Ut).norm() / Ut.norm()) <= 1e-13
    # central differences of the plain operator along (v, mu_dot)
    eps = 1e-6
    fd = []
    for sgn in (1.0, -1.0):
        c2 = gx.config(N=N, NodeType="gauss" if nt == 1 else "gauss-lobatto",
                       **dict(kw, mu0=kw.get("mu0", 0.0) + sgn * eps * mu_dot)) if cfg.parabolic else cfg
        o2 = gx.DG(c2, m)
        fd.append(o2.DGTimeDerivative_weakForm(0.0, U + sgn * eps * v))
        o2.close()
    fd = (fd[0] - fd[1]) / (2 * eps)
    err = float((fd - Jv).norm() / Jv.norm())
    assert err <= 1e-6, err
    op.close()


@pytest.mark.parametrize("name,kw,N,nt,dims,deform", CASES, ids=[c[0] for c in CASES])
def test_rhs_dot_product(name, kw, N, nt, dims, deform):
    cfg, m, U, rng = setup_case(name, kw, N, nt, dims, deform)
    op = gx.DG(cfg, m)
    v = rand_like(rng, U)
    ybar = rand_like(rng, U)
    mu_dot = 0.7 if cfg.parabolic else 0.0
    _, Jv = op.rhs_jvp(U, v, mu_dot)
    Ub, mub = op.rhs_vjp(U, ybar)
    lhs = dot(ybar, Jv)
    rhs = dot(Ub, v) + mub * mu_dot
    scale = float(ybar.norm() * Jv.norm())
    assert abs(lhs - rhs) <= 1e-13 * scale, (lhs, rhs, scale)
    op.close()


class RHSFunction(torch.autograd.Function):
    """Ut = R(U) with the hand-written adjoint as its backward (test harness only)."""

    @staticmethod
    def forward(ctx, U, op):
        ctx.save_for_backward(U)
        ctx.op = op
        return op.DGTimeDerivative_weakForm(0.0, U.detach().contiguous())

    @staticmethod
    def backward(ctx, gout):
        (U,) = ctx.saved_tensors
        Ub, _ = ctx.op.rhs_vjp(U.detach().contiguous(), gout.contiguous())
        return Ub, None


def test_autograd_function_gradcheck():
    cfg = gx.config(N=2, Riemann="roe", SplitDG="pi", parabolic=True, mu0=2e-3, R=71.42857)
    m = gx.Mesh(2, 2, 2, 2, 2, (-math.pi,) * 3, (math.pi,) * 3)
    rng = np.random.default_rng(3)
    U = gx.tgv_state(m, mach=0.3, R=cfg.R)
    U = U + 1e-2 * rng.standard_normal(U.shape) * np.abs(U).mean(axis=(0, 1, 2, 3))
    op = gx.DG(cfg, m)
    Ut = torch.from_numpy(U).cuda().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: RHSFunction.apply(x, op), (Ut,), eps=1e-6, atol=1e-5, rtol=1e-5,
                                    fast_mode=True)
    op.close()


def window_case():
    cfg = gx.config(N=3, Riemann="roe", SplitDG="pi", parabolic=True, mu0=5e-3, R=71.42857)
    m = gx.Mesh(3, 2, 2, 2, 2, (-math.pi,) * 3, (math.pi,) * 3)
    rng = np.random.default_rng(11)
    U = gx.tgv_state(m, mach=0.3, R=cfg.R)
    U = U + 1e-3 * rng.standard_normal(U.shape) * np.abs(U).mean(axis=(0, 1, 2, 3))
    op = gx.DG(cfg, m)
    U0 = torch.from_numpy(U).cuda()
    dt, _ = op.CalcTimeStep(U0, 0.5, 0.5)
    return cfg, m, op, U0, dt, rng


def test_window_dot_product():
    cfg, m, op, U0, dt, rng = window_case()
    nSteps = 10
    v = rand_like(rng, U0)
    ybar = rand_like(rng, U0)
    mu_dot = 0.3
    U, Ud, K = U0.clone(), v.clone(), torch.zeros_like(U0)
    op.tlm_steps(dt, U, Ud, K, nSteps=nSteps, mu_dot=mu_dot)
    Uf, plan = op.adjoint_forward(dt, nSteps, U0, budget_bytes=1 << 34)
    assert plan == 1
    # the recorded forward end state equals the tangent-linear primal
    assert float((Uf - U).abs().max()) <= 1e-13 * float(U.abs().max())
    Ub = ybar.clone()
    mub = op.adjoint_reverse(Ub)
    lhs = dot(ybar, Ud)
    rhs = dot(Ub, v) + mub * mu_dot
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs), (lhs, rhs)
    op.close()


@pytest.mark.parametrize("nSteps", [12, 13])
def test_window_checkpoint_plans_agree(nSteps):
    """Plans 2 and 3 give the bits of plan 1; 13 steps leave a short first segment (plan 2: k = 2,
    plan 3: k = 3, one step in the first segment)."""
    cfg, m, op, U0, dt, rng = window_case()
    state = U0.numel() * 8
    ybar = rand_like(rng, U0)
    out = {}
    for budget in (state * 5 * nSteps, state * 20, state * 13):
        _, plan = op.adjoint_forward(dt, nSteps, U0, budget_bytes=budget)
        Ub = ybar.clone()
        mub = op.adjoint_reverse(Ub)
        out[plan] = (Ub, mub)
    assert sorted(out) == [1, 2, 3]
    for p in (2, 3):
        assert torch.equal(out[p][0], out[1][0])
        assert out[p][1] == out[1][1]
    op.close()


def test_window_end_state_over_start_state_and_scratch_size():
    """The end state may be written over the start state; the scratch estimate covers what the
    adjoint allocates besides its checkpoints.  The memory check reads the device's free memory, so
    it needs the GPU to itself: with other processes allocating on the same device (a parallel
    pytest run, for instance) their allocations count as used."""
    cfg, m, op, U0, dt, rng = window_case()
    nSteps = 6
    state = U0.numel() * 8
    free0 = torch.cuda.mem_get_info()[0]
    scratch = op.adjoint_scratch_bytes()
    Uf_ref, plan = op.adjoint_forward(dt, nSteps, U0, budget_bytes=state * 5 * nSteps)
    assert plan == 1
    ybar = rand_like(rng, U0)
    Ub_ref = ybar.clone()
    mub_ref = op.adjoint_reverse(Ub_ref)
    torch.cuda.synchronize()
    used = free0 - torch.cuda.mem_get_info()[0]
    # what stays allocated (work states, scratch and the recorded tape) plus the torch tensors of this
    # test fit the estimate up to allocator granularity
    assert scratch >= 3 * state and used <= scratch + (5 * nSteps + 4) * state + (64 << 20)
    U = U0.clone()
    Uf, _ = op.adjoint_forward(dt, nSteps, U, budget_bytes=state * 5 * nSteps, out=U)
    assert Uf.data_ptr() == U.data_ptr() and torch.equal(Uf, Uf_ref)
    Ub = ybar.clone()
    mub = op.adjoint_reverse(Ub)
    assert torch.equal(Ub, Ub_ref) and mub == mub_ref
    op.close()


def test_window_kinetic_energy_gradient_vs_fd():
    cfg, m, op, U0, dt, rng = window_case()
    nSteps = 20
    J, G, dJdmu, _ = op.adjoint_window(dt, nSteps, U0, budget_bytes=1 << 34)

    def J_of(U, mu):
        c2 = gx.config(N=3, Riemann="roe", SplitDG="pi", parabolic=True, mu0=mu, R=71.42857)
        o2 = gx.DG(c2, m)
        U = U.clone()
        K = torch.zeros_like(U)
        o2.TimeStepByLSERKW2(0.0, dt, U, K, nSteps=nSteps)
        val = o2.kinetic_energy(U)
        o2.close()
        return val

    assert abs(J_of(U0, cfg.mu0) - J) <= 1e-14 * abs(J)
    eps = 1e-6
    for d in range(4):
        v = rand_like(rng, U0)
        v = v / v.norm()
        fd = (J_of(U0 + eps * v, cfg.mu0) - J_of(U0 - eps * v, cfg.mu0)) / (2 * eps)
        ad = dot(G, v)
        assert abs(fd - ad) <= 1e-6 * abs(ad), (d, fd, ad)
    fd = (J_of(U0, cfg.mu0 + eps) - J_of(U0, cfg.mu0 - eps)) / (2 * eps)
    assert abs(fd - dJdmu) <= 1e-6 * abs(dJdmu), (fd, dJdmu)
    op.close()
