"""The oracle against the reference's own golden vectors (unitTests/*.bin, copied to tests/golden).

Tolerances follow the reference's unit tests: ALMOSTEQUALABSORREL(..., 50*PP_RealTolerance) for nodes
(unitTests/NodesAndWeights.f90:46-50) and for ChangeBasis (ChangeBasis.f90), 100*PP_RealTolerance for
D, ProlongToFace, SurfInt and the Vandermonde matrices (unitTests/DerivativeMatrix.f90:76,
SurfInt.f90:151-153, Vandermonde.f90).
"""
import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests.fortran_records import Cursor, records

GOLD = os.path.join(os.path.dirname(__file__), "golden")
EPS = np.finfo(np.float64).eps


def almost_equal_abs_or_rel(a, b, tol):
    # ALMOSTEQUALABSORREL (src/globals/globals.f90): |a-b| <= tol or |a-b| <= tol*|b|
    d = np.abs(a - b)
    return np.all((d <= tol) | (d <= tol * np.abs(b)))


def element_data():
    c = Cursor(records(os.path.join(GOLD, "UnittestElementData3D.bin"))[0])
    d = {}
    d["nElems"] = c.take("<i4", 1)[0]
    d["SideToElem"] = c.take("<i4", 30)
    d["firstMPISide_YOUR"], d["lastMPISide_MINE"], d["nSides"] = c.take("<i4", 3)
    d["S2V2"] = c.take("<i4", 2 * 10 * 10 * 5 * 6)
    d["L_Minus"], d["L_Plus"] = c.take("<f8", 10), c.take("<f8", 10)
    d["L_HatPlus"], d["L_HatMinus"] = c.take("<f8", 10), c.take("<f8", 10)
    d["sJ"] = c.take("<f8", 2000)
    return d


def test_nodes_and_weights_golden():
    a = np.frombuffer(records(os.path.join(GOLD, "NodesAndWeights.bin"))[0], "<f8").reshape(3, 4, 10, 11)
    for t in range(4):
        for N in range(1, 11):
            x, w, wb = orc.nodes_weights(N, t + 1)
            assert almost_equal_abs_or_rel(x, a[0, t, N - 1, :N + 1], 50 * EPS), (t, N)
            assert almost_equal_abs_or_rel(w, a[1, t, N - 1, :N + 1], 50 * EPS), (t, N)
            assert almost_equal_abs_or_rel(wb, a[2, t, N - 1, :N + 1], 50 * EPS), (t, N)


def test_derivative_matrix_golden():
    D = np.frombuffer(records(os.path.join(GOLD, "DerivativeMatrix.bin"))[0], "<f8").reshape(40, 11, 11)
    k = 0
    for t in range(4):
        for N in range(1, 11):
            mine = orc.derivative_matrix(N, t + 1)
            assert almost_equal_abs_or_rel(mine, D[k, :N + 1, :N + 1], 100 * EPS), (t, N)
            k += 1


def test_s2v2_golden():
    d = element_data()
    assert np.array_equal(orc.s2v2(9), d["S2V2"])


def test_gauss_face_vectors_golden():
    d = element_data()
    b = orc.dg_basis(9, 1)
    assert almost_equal_abs_or_rel(b["L_minus"], d["L_Minus"], 100 * EPS)
    assert almost_equal_abs_or_rel(b["L_plus"], d["L_Plus"], 100 * EPS)
    assert almost_equal_abs_or_rel(b["L_hat_minus"], d["L_HatMinus"], 100 * EPS * 100)
    assert almost_equal_abs_or_rel(b["L_hat_plus"], d["L_HatPlus"], 100 * EPS * 100)


@pytest.mark.parametrize("node_type,name", [(1, "G"), (2, "GL")])
def test_prolong_to_face_golden(node_type, name):
    d = element_data()
    uvol = np.frombuffer(records(os.path.join(GOLD, "ProlongToFaceUvol.bin"))[0], "<f8").copy()
    ref = np.frombuffer(records(os.path.join(GOLD, "ProlongToFace_%s3D.bin" % name))[0], "<f8")
    out = np.zeros(600)
    p = orc._p
    orc.lib().orc_prolong_to_face_host(9, 1, node_type, p(d["L_Minus"]), p(d["L_Plus"]), p(d["SideToElem"]), 6,
                                       p(d["S2V2"]), p(uvol), p(out))
    assert almost_equal_abs_or_rel(out, ref, 100 * EPS)


@pytest.mark.parametrize("node_type,name", [(1, "G"), (2, "GL")])
def test_surf_int_golden(node_type, name):
    d = element_data()
    flux = np.frombuffer(records(os.path.join(GOLD, "SurfIntFlux.bin"))[0], "<f8").copy()
    ref = np.frombuffer(records(os.path.join(GOLD, "SurfInt_%s3D.bin" % name))[0], "<f8")
    ut = np.zeros(1000)
    p = orc._p
    orc.lib().orc_surf_int_host(9, 1, node_type, p(d["L_HatMinus"]), p(d["L_HatPlus"]), p(d["SideToElem"]), 6,
                                p(d["S2V2"]), p(flux), p(ut))
    assert almost_equal_abs_or_rel(ut, ref, 100 * EPS)


@pytest.mark.parametrize("N", [1, 2, 3, 5, 7, 9])
@pytest.mark.parametrize("node_type", [1, 2])
def test_product_basis_matches_oracle(N, node_type):
    import galaexi_gb300 as gx
    a = gx.basis(N, node_type)
    b = orc.dg_basis(N, node_type)
    for k in a:
        scale = max(1.0, np.abs(b[k]).max())
        assert np.abs(a[k] - b[k]).max() <= 1e-14 * scale, k


def test_sbp_property():
    """M D + (M D)^T = B for Gauss-Lobatto nodes (summation-by-parts), and D x^k exact."""
    for N in range(1, 10):
        b = orc.dg_basis(N, 2)
        D = b["D"].reshape(N + 1, N + 1).T
        M = np.diag(b["wGP"])
        B = np.zeros((N + 1, N + 1)); B[0, 0] = -1; B[N, N] = 1
        assert np.abs(M @ D + (M @ D).T - B).max() < 1e-12
        x = b["xGP"]
        for k in range(N + 1):
            assert np.abs(D @ x ** k - (k * x ** (k - 1) if k else 0 * x)).max() < 1e-11


def _lifting_pair(N, node_type, deform, U_fn, **kw):
    import galaexi_gb300 as gx
    m = gx.Mesh(N, node_type, 3, 2, 2, (0.0,) * 3, (1.0,) * 3, deform=deform)
    U = U_fn(m)
    out = {}
    for lift in ("br1", "br2"):
        cfg = gx.config(N=N, NodeType="gauss" if node_type == 1 else "gauss-lobatto", parabolic=True, mu0=1e-3,
                        Riemann="lf", Lifting=lift, **kw)
        o = orc.Oracle(cfg, m)
        Ut = o.rhs(U)
        out[lift] = (Ut, [o.work(1 + d, U.shape) for d in range(3)])
    return out


@pytest.mark.parametrize("node_type,deform,cons", [(1, 0.05, False), (2, 0.0, True), (2, 0.05, False)])
def test_br2_volume_gradients_equal_br1(node_type, deform, cons):
    """BR2 changes only the face traces: the volume gradients equal BR1's (lifting_br2.t90:43-310)."""
    import galaexi_gb300 as gx

    def noisy(m):
        rng = np.random.default_rng(3)
        U = gx.fill_ini(m, 1, [1.0, 0.3, 0.2, 0.1, 1.0 / 1.4])
        return U + 1e-2 * rng.standard_normal(U.shape) * np.abs(U).mean(axis=(0, 1, 2, 3))

    out = _lifting_pair(4, node_type, deform, noisy, doConservativeLifting=cons)
    for g1, g2 in zip(out["br1"][1], out["br2"][1]):
        assert np.abs(g1 - g2).max() <= 1e-12 * np.abs(g1).max()
    # the jumps of the noisy state make the BR2 face traces, hence Ut, differ from BR1
    assert np.abs(out["br1"][0] - out["br2"][0]).max() > 1e-6 * np.abs(out["br1"][0]).max()


def test_br2_equals_br1_for_continuous_data():
    """On Gauss-Lobatto nodes a state sampled from one smooth periodic field has no jumps at the
    faces, so the BR2 penalty vanishes and the operator equals BR1."""
    import galaexi_gb300 as gx

    def smooth(m):
        x = m.Elem_xGP
        s = np.sin(2 * np.pi * x[..., 0]) * np.cos(2 * np.pi * x[..., 1]) + 0.5 * np.sin(2 * np.pi * x[..., 2])
        U = np.empty(x.shape[:-1] + (5,))
        rho = 1.0 + 0.1 * s
        U[..., 0] = rho
        U[..., 1] = rho * (0.3 + 0.05 * s)
        U[..., 2] = rho * 0.2
        U[..., 3] = rho * (0.1 - 0.05 * s)
        U[..., 4] = (1.0 + 0.05 * s) / 0.4 + 0.5 * (U[..., 1] ** 2 + U[..., 2] ** 2 + U[..., 3] ** 2) / rho
        return U

    out = _lifting_pair(5, 2, 0.0, smooth)
    a, b = out["br1"][0], out["br2"][0]
    assert np.abs(a - b).max() <= 1e-11 * np.abs(a).max()


def test_vandermonde_golden():
    """GetVandermonde (interpolation.f90:324-395) for N_in = 2..5, N_out = 3..6, the four node sets in
    and out, nodal and modal (the modal branches use buildLegendreVdm, basis.f90:100-160)."""
    a = np.frombuffer(records(os.path.join(GOLD, "Vandermonde.bin"))[0], "<f8")
    voi = a[:6 * 7 * 512].reshape(512, 7, 6).transpose(2, 1, 0)   # Vdm_Out_In(0:5,0:6,k)
    vio = a[6 * 7 * 512:].reshape(512, 6, 7).transpose(2, 1, 0)   # Vdm_In_Out(0:6,0:5,k)
    k = 0
    for nin in range(2, 6):
        for nout in range(3, 7):
            for tin in range(1, 5):
                for tout in range(1, 5):
                    for modal in (False, True):
                        io, oi = orc.get_vandermonde(nin, tin, nout, tout, modal)
                        assert almost_equal_abs_or_rel(io, vio[:nout + 1, :nin + 1, k], 100 * EPS), (nin, nout, tin, tout, modal)
                        assert almost_equal_abs_or_rel(oi, voi[:nin + 1, :nout + 1, k], 100 * EPS), (nin, nout, tin, tout, modal)
                        k += 1
    assert k == 512


def test_change_basis_golden():
    """ChangeBasis3D and ChangeBasis3D_XYZ (changeBasis.t90) on the unit test's fixed field: the
    sweeps the solution filter applies."""
    nVar, NIn, NOut, nElems = 3, 4, 5, 6
    a = np.frombuffer(records(os.path.join(GOLD, "ChangeBasis.bin"))[0], "<f8")
    n3 = nVar * (NOut + 1) ** 3
    uout = a[:n3 * nElems * 4].reshape(4, nElems, n3)
    Vdm = np.zeros((NOut + 1, NIn + 1), order="F")
    Vdm2, Vdm3 = np.zeros_like(Vdm), np.zeros_like(Vdm)
    z = 1
    for q in range(NIn + 1):
        for p in range(NOut + 1):
            z += 1
            Vdm[p, q], Vdm2[p, q], Vdm3[p, q] = 1.0 + 1.0 / z, 1.0 - 1.0 / z, 1.0 + 0.1 * z
    cnt = nVar * (NIn + 1) ** 3
    uin = (1.0 + 0.1 * (2 + np.arange(cnt, dtype=np.float64))).reshape((nVar, NIn + 1, NIn + 1, NIn + 1), order="F")
    for slot, mats in ((2, (Vdm, Vdm, Vdm)), (3, (Vdm, Vdm2, Vdm3))):
        out = orc.change_basis_3d(uin, *mats).ravel(order="F")
        assert almost_equal_abs_or_rel(out, uout[slot, 0], 50 * EPS), slot
