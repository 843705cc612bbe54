"""The geometry of the mesh arrays against the oracle's own restatement of the reference's metric
computation (BuildCoords + CalcMetrics + CalcSurfMetrics, src/mesh/metrics.f90:85-789).

The oracle computes Elem_xGP, Metrics_f/g/hTilde, sJ, NormVec, TangVec1/2 and SurfElem from the
element node coordinates alone (the equidistant NGeo nodes a HOPR file holds) and the connectivity;
the product's mesh code (dg_mesh_hopr, dg_mesh_cartesian) must give the same arrays to <= 1e-13
relative (max |difference| / max |value| per array) on the reference's own mesh files and on the
curved boxes.  The oracle's metric path is pinned independently by volume conservation (the modal
projection of the Jacobian keeps the element volumes, so the curved periodic box keeps the volume of
the undeformed one) and, on the reference's regression mesh, by the end-to-end TGV reproduction.
"""
import os

import numpy as np
import pytest

import galaexi_gb300 as gx
from oracle.oracle import calc_metrics, dg_basis

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KEYS = ("Elem_xGP", "Metrics_fTilde", "Metrics_gTilde", "Metrics_hTilde", "sJ", "NormVec", "TangVec1", "TangVec2",
        "SurfElem")
TOL = 1e-13


def compare(mesh, tol=TOL, keys=KEYS):
    o = calc_metrics(mesh.N, mesh.node_type, mesh.NGeo, mesh.NodeCoords, mesh.ElemToSide, mesh.nSides)
    assert o["bad_nodes"] == 0
    errs = {k: float(np.abs(getattr(mesh, k) - o[k]).max() / np.abs(o[k]).max()) for k in keys}
    bad = {k: e for k, e in errs.items() if not e <= tol}
    assert not bad, bad
    return o


FILES = [
    ("CART_HEX_PERIODIC_008_mesh.h5", 7, 2),   # the TGV regression run's mesh (NGeo = 1)
    ("NACA0012_652_Ng2_mesh.h5", 5, 1),        # curved, NGeo = 2, N < 3 NGeo (modal Jacobian projection)
    ("NACA0012_652_Ng2_mesh.h5", 2, 2),
    ("NACA0012_652_Ng2_mesh.h5", 7, 2),        # N > 3 NGeo: interpolation of the Jacobian
    ("CART_HEX2D_FlatPlateG_mesh.h5", 3, 1),   # BC sides
    ("cavity4x4x4_mesh.h5", 2, 1),
]


@pytest.mark.parametrize("name,N,node_type", FILES, ids=["%s_N%d_%d" % f for f in FILES])
def test_hopr_file_metrics_equal_oracle(name, N, node_type):
    path = os.path.join(GOLD, name)
    if not os.path.exists(path):
        pytest.skip("fixture %s not present" % name)
    compare(gx.Mesh.from_hopr(path, N, node_type))


BOXES = [
    # (N, node type, elements per direction, NGeo, displacement amplitude)
    (5, 1, 4, 2, 0.05),   # the curved box of the mixed-precision / BR2 workload, smaller
    (2, 2, 3, 2, 0.05),   # N < 3 NGeo - 1: the modal projection differs from interpolation here
    (3, 1, 3, 3, 0.08),
    (5, 1, 3, 5, 0.05),
    (1, 2, 3, 2, 0.05),   # N < NGeo: metrics differentiated on the CL(N) points
]


@pytest.mark.parametrize("N,nt,ne,NGeo,amp", BOXES, ids=["N%d_nt%d_ne%d_ngeo%d" % b[:4] for b in BOXES])
def test_curved_box_metrics_equal_oracle(N, nt, ne, NGeo, amp):
    m = gx.Mesh(N, nt, ne, ne, ne, (0.0,) * 3, (1.0,) * 3, deform=amp, NGeo=NGeo)
    compare(m)


def test_curved_box_node_coordinates():
    """The box's node coordinates are the equidistant NGeo nodes displaced by
    0.05 sin(2 pi x) sin(2 pi y) sin(2 pi z) (restated here in numpy)."""
    ne, NGeo, amp = 3, 2, 0.05
    m = gx.Mesh(5, 1, ne, ne, ne, (0.0,) * 3, (1.0,) * 3, deform=amp, NGeo=NGeo)
    xi = np.array([2.0 * i / NGeo - 1.0 for i in range(NGeo + 1)])
    ref = np.zeros_like(m.NodeCoords)
    for e in range(m.nElems):
        e3 = (e % ne, (e // ne) % ne, e // (ne * ne))
        for k in range(NGeo + 1):
            for j in range(NGeo + 1):
                for i in range(NGeo + 1):
                    X = np.array([(e3[d] + 0.5 * ((xi[i], xi[j], xi[k])[d] + 1.0)) / ne for d in range(3)])
                    s = np.prod(np.sin(2 * np.pi * X))
                    ref[e, k, j, i] = X + amp * s
    assert np.abs(m.NodeCoords - ref).max() <= 1e-15


def test_affine_box_metrics_equal_oracle_to_round_off():
    """The affine box carries the exact constant metric terms; the reference's curl form on the node
    coordinates reproduces them up to its round-off."""
    m = gx.Mesh(7, 2, 3, 3, 3, (-np.pi,) * 3, (np.pi,) * 3)
    compare(m, tol=1e-13)
    h = 2 * np.pi / 3
    assert np.allclose(m.Metrics_fTilde[..., 0], h * h / 4, rtol=0, atol=1e-15)
    assert np.all(m.sJ == 8.0 / h ** 3)


@pytest.mark.parametrize("N,nt,NGeo", [(5, 1, 2), (2, 2, 2), (3, 1, 3), (1, 2, 2)])
def test_oracle_volume_conservation(N, nt, NGeo):
    """Sum of w_i w_j w_k / sJ over the curved periodic box = the box volume: the displacement leaves
    the box faces in their planes, the elements tile the box (shared face nodes), and the Jacobian's
    projection to N keeps its integral."""
    ne = 3
    m = gx.Mesh(N, nt, ne, ne, ne, (0.0,) * 3, (1.0,) * 3, deform=0.05, NGeo=NGeo)
    o = calc_metrics(N, nt, NGeo, m.NodeCoords, m.ElemToSide, m.nSides)
    w = dg_basis(N, nt)["wGP"]
    W = w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    # sum over the elements of the quadrature of det(dX/dxi) over [-1,1]^3: exact, since the projected
    # Jacobian has degree <= N per direction and the N+1-point quadrature integrates that exactly
    vol = float((W / o["sJ"]).sum())
    assert abs(vol - 1.0) <= 1e-13, vol
