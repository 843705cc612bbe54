"""The oracle against the reference's own golden vectors (unitTests/*.bin, copied to tests/golden).

Tolerances follow the reference's unit tests: ALMOSTEQUALABSORREL(..., 50*PP_RealTolerance) for nodes
(unitTests/NodesAndWeights.f90:46-50) and 100*PP_RealTolerance for D, ProlongToFace and SurfInt
(unitTests/DerivativeMatrix.f90:76, SurfInt.f90:151-153).
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
