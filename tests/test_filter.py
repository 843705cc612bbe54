"""Solution filter at the start of the operator (DGTimeDerivative_weakForm step 1, src/dg/dg.f90:330;
src/filter/filter.f90): cut-off and modal (Hesthaven) filters through FilterMat = Vdm_Leg diag(sigma)
sVdm_Leg, and the adaptive LAF filter with its per-element state.

The oracle's building blocks are pinned to the reference's golden vectors (Vandermonde.bin for the
modal Vandermonde, ChangeBasis.bin for the sweeps; tests/test_oracle_golden.py); here the filter's own
properties are checked on the CPU and the CUDA path against the oracle on the GPU: the filtered state
(the filter writes U in place, as the reference does), Ut, LSERK steps and the LAF state.
"""
import math
import zlib

import numpy as np
import pytest

import galaexi_gb300 as gx
from oracle.oracle import Oracle


def box(N, node_type=2, dims=(2, 2, 2)):
    return gx.Mesh(N, node_type, *dims, (-math.pi,) * 3, (math.pi,) * 3)


def noisy_tgv(m, seed, amp=1e-2, R=71.42857):
    rng = np.random.default_rng(seed)
    U = gx.tgv_state(m, mach=0.3, R=R)
    U += amp * rng.standard_normal(U.shape) * np.abs(U).mean(axis=(0, 1, 2, 3))
    return U


def legendre_mode(x, k):
    """Legendre polynomial P_k on [-1, 1] (unnormalised)."""
    return np.polynomial.legendre.legval(x, [0] * k + [1])


def ns_cfg(N, **kw):
    base = dict(N=N, Riemann="roe", SplitDG="pi", parabolic=True, mu0=1e-3, R=71.42857)
    base.update(kw)
    return gx.config(**base)


# ------------------------------------------------------------------------------------------------
# CPU: the oracle's filter
# ------------------------------------------------------------------------------------------------
def test_cutoff_at_N_is_identity():
    N = 5
    m = box(N)
    U = noisy_tgv(m, 1)
    U0 = U.copy()
    Ut = Oracle(ns_cfg(N, FilterType="cutoff", NFilter=N), m).rhs(U)
    ref = Oracle(ns_cfg(N), m).rhs(U0)
    assert np.abs(U - U0).max() <= 1e-13 * np.abs(U0).max()
    assert np.linalg.norm(Ut - ref) <= 1e-11 * np.linalg.norm(ref)


@pytest.mark.parametrize("nfilter", [1, 3])
def test_cutoff_is_modal_projection(nfilter):
    """Per element and direction the cut-off filter keeps the Legendre modes up to NFilter and
    removes the others; applying it twice equals applying it once."""
    N = 5
    m = box(N, dims=(1, 1, 1))
    x = gx.basis(N, 2)["xGP"]
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")  # (i, j, k)
    low = legendre_mode(X, nfilter) * legendre_mode(Y, 1) + 0.3 * legendre_mode(Z, min(nfilter, 2))
    high = legendre_mode(X, nfilter + 1) * legendre_mode(Y, 2)
    U = np.zeros((1, N + 1, N + 1, N + 1, 5))
    U[..., 0] = 1.0 + 0.01 * (low + high).transpose(2, 1, 0)  # layout (e, k, j, i)
    U[..., 4] = 2.5
    o = Oracle(ns_cfg(N, FilterType="cutoff", NFilter=nfilter), m)
    o.rhs(U)
    expect = 1.0 + 0.01 * low.transpose(2, 1, 0)
    assert np.abs(U[0, ..., 0] - expect).max() <= 1e-13
    U1 = U.copy()
    o.rhs(U)
    assert np.abs(U - U1).max() <= 1e-13


def test_modal_filter_damps_high_modes():
    """Hesthaven's filter with the default HestFilterParam (36, 12, 1): mode 0 is kept, mode N is
    damped by exp(-36)."""
    N = 4
    m = box(N, dims=(1, 1, 1))
    x = gx.basis(N, 2)["xGP"]
    X = np.meshgrid(x, x, x, indexing="ij")[0]
    U = np.zeros((1, N + 1, N + 1, N + 1, 5))
    U[..., 0] = (1.0 + 0.1 * legendre_mode(X, N)).transpose(2, 1, 0)
    U[..., 4] = 2.5
    Oracle(ns_cfg(N, FilterType="modal"), m).rhs(U)
    eta = (N + 1) / (N + 1)
    etac = 1.0 / (N + 1)
    sigma = math.exp(-36.0 * ((eta - etac) / (1 - etac)) ** 12)
    expect = (1.0 + 0.1 * sigma * legendre_mode(X, N)).transpose(2, 1, 0)
    assert np.abs(U[0, ..., 0] - expect).max() <= 1e-13


def growing_noise(m, seed, calls, nfilter=3):
    """States with the same smooth part and growing noise in the modes above NFilter only: the
    fluctuation energy rises while the resolved field stays, which is when LAF filters."""
    rng = np.random.default_rng(seed)
    base = gx.tgv_state(m, mach=0.3, R=71.42857)
    noise = rng.standard_normal(base.shape) * np.abs(base).mean(axis=(0, 1, 2, 3))
    noise[..., 0] = noise[..., 4] = 0.0  # momentum only: LAF measures velocity fluctuations
    cut = Oracle(ns_cfg(m.N, FilterType="cutoff", NFilter=nfilter), m)
    s1, s0 = base + noise, base.copy()
    cut.rhs(s1)
    cut.rhs(s0)
    high = noise - (s1 - s0)  # noise minus its modes up to NFilter (the filter is linear)
    return [base + 0.1 * (1 + 3 * c) * high for c in range(calls)]


def test_laf_filters_when_fluctuations_grow():
    """First call: the fluctuation energy jumps from its initial 1e-16, lim takes eRatio and nothing
    is filtered.  Later calls with more node noise raise eRatio above lim: every element is filtered
    (r counts it) and its state is replaced by the filtered one."""
    N = 5
    m = box(N)
    o = Oracle(ns_cfg(N, FilterType="laf", NFilter=3, LAF_alpha=1.0), m)
    states = growing_noise(m, 3, 3)
    U = states[0].copy()
    o.rhs(U)
    assert np.array_equal(U, states[0])
    lim1, eRatio1, r1 = o.laf_state()
    assert r1.sum() == 0 and np.array_equal(lim1, eRatio1)
    U = states[1].copy()
    o.rhs(U)
    lim, eRatio, r = o.laf_state()
    assert (r == 1).all() and (eRatio > eRatio1).all()
    assert np.abs(U - states[1]).max() > 1e-4  # filtered
    Uf = states[1].copy()
    Oracle(ns_cfg(N, FilterType="cutoff", NFilter=3), m).rhs(Uf)
    assert np.abs(U - Uf).max() <= 1e-13 * np.abs(Uf).max()


def test_filter_rejects_bad_nfilter():
    with pytest.raises(ValueError):
        Oracle(ns_cfg(3, FilterType="cutoff", NFilter=7), box(3))


# ------------------------------------------------------------------------------------------------
# GPU: the CUDA path against the oracle
# ------------------------------------------------------------------------------------------------
FILTERS = [
    ("cutoff_n3", dict(FilterType="cutoff", NFilter=3)),
    ("modal_default", dict(FilterType="modal")),
    ("modal_params", dict(FilterType="modal", HestFilterParam=(20.0, 4.0, 2.0))),
    ("laf", dict(FilterType="laf", NFilter=3, LAF_alpha=1.0)),
]
SCHEMES = [
    ("ns_gl_split_pi", dict(Riemann="roe", SplitDG="pi", parabolic=True, mu0=1e-3, R=71.42857), 5, 2),
    ("ns_gauss_weak", dict(NodeType="gauss", Riemann="roeentropyfix", parabolic=True, mu0=1e-3, R=71.42857), 4, 1),
    ("euler_gl_weak", dict(Riemann="lf", R=71.42857), 7, 2),
]


@pytest.mark.gpu
@pytest.mark.parametrize("fname,fkw", FILTERS, ids=[f[0] for f in FILTERS])
@pytest.mark.parametrize("sname,skw,N,nt", SCHEMES, ids=[s[0] for s in SCHEMES])
def test_filtered_rhs_matches_oracle(fname, fkw, sname, skw, N, nt):
    torch = pytest.importorskip("torch")
    cfg = gx.config(N=N, **skw, **fkw)
    m = box(N, nt, (3, 2, 2))
    o = Oracle(cfg, m)
    op = gx.DG(cfg, m)
    for call, U in enumerate(growing_noise(m, zlib.crc32((fname + sname).encode()), 3)):  # LAF keeps state
        Ud = torch.from_numpy(U.copy()).cuda()
        Ut = op.DGTimeDerivative_weakForm(0.0, Ud)
        ref = o.rhs(U)
        torch.cuda.synchronize()
        Ug, Utg = Ud.cpu().numpy(), Ut.cpu().numpy()
        assert np.linalg.norm(Ug - U) <= 1e-13 * np.linalg.norm(U), (fname, call)
        err = np.linalg.norm(Utg - ref) / np.linalg.norm(ref)
        assert err <= 1e-12, (fname, sname, call, err)
        if fkw["FilterType"] == "laf":
            for a, b in zip(op.laf_state(), o.laf_state()):
                assert np.allclose(a, b, rtol=1e-10, atol=0.0), call
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("fname,fkw", FILTERS, ids=[f[0] for f in FILTERS])
def test_filtered_lserk_steps(fname, fkw):
    torch = pytest.importorskip("torch")
    N = 5
    cfg = ns_cfg(N, **fkw)
    m = box(N, 2, (2, 3, 2))
    U = noisy_tgv(m, 17)
    dt, _ = Oracle(cfg, m).calc_timestep(U, 0.9, 0.9)
    ref, _ = Oracle(cfg, m).lserk_steps(U, dt, 20)
    op = gx.DG(cfg, m)
    Ud = torch.from_numpy(U.copy()).cuda()
    tmp = torch.zeros_like(Ud)
    op.TimeStepByLSERKW2(0.0, dt, Ud, tmp, nSteps=20)
    torch.cuda.synchronize()
    err = np.linalg.norm(Ud.cpu().numpy() - ref) / np.linalg.norm(ref)
    op.close()
    assert err <= 1e-10, err


@pytest.mark.gpu
def test_filter_mixed_precision():
    torch = pytest.importorskip("torch")
    N = 5
    m = box(N, 2, (3, 2, 2))
    U = noisy_tgv(m, 5)
    ref = Oracle(ns_cfg(N, FilterType="modal"), m).rhs(U.copy())
    op = gx.DG(ns_cfg(N, FilterType="modal", precision="mixed"), m)
    Ut = op.DGTimeDerivative_weakForm(0.0, torch.from_numpy(U.copy()).cuda())
    torch.cuda.synchronize()
    err = np.linalg.norm(Ut.cpu().numpy() - ref) / np.linalg.norm(ref)
    op.close()
    assert err <= 1e-5, err


@pytest.mark.gpu
def test_filter_rejected_by_tangent_and_adjoint():
    torch = pytest.importorskip("torch")
    m = box(3)
    op = gx.DG(ns_cfg(3, FilterType="modal"), m)
    U = torch.from_numpy(noisy_tgv(m, 2)).cuda()
    with pytest.raises(gx.DGError):
        op.rhs_jvp(U, torch.zeros_like(U))
    op.close()
