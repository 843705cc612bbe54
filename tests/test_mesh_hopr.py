"""HOPR mesh files (HDF5) read through dg_mesh_hopr, checked on the reference's own TGV regression
mesh (regressioncheck/checks/tgv/split/CART_HEX_PERIODIC_008_mesh.h5, a fixture copied by
tests/golden/fetch_reference_fixtures.py).

The file's 8^3 periodic box on [0, 2 pi]^3 is the box `gx.Mesh` generates, with HOPR's own element
order, side numbering and orientations (every element of this file is slave on some sides and
master on others).  The oracle's RHS on the file's mesh must equal the RHS on the generated box,
node by node at the same physical points: that checks the HDF5 reading, the connectivity (sides,
flips, master/slave) and the metrics together.
"""
import math
import os

import numpy as np
import pytest

import galaexi_gb300 as gx
from oracle.oracle import Oracle

MESH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "CART_HEX_PERIODIC_008_mesh.h5")


def test_reads_reference_mesh_file():
    m = gx.Mesh.from_hopr(MESH, 3, 2)
    assert (m.nElems, m.nSides, m.nBCSides, m.NGeo) == (512, 1536, 0, 1)
    h = math.pi / 4
    assert np.allclose(m.Elem_xGP.min(axis=(0, 1, 2, 3)), 0.0) and np.allclose(m.Elem_xGP.max(axis=(0, 1, 2, 3)), 2 * math.pi)
    assert np.abs(m.sJ / (8 / h ** 3) - 1).max() < 1e-13
    for d, M in enumerate((m.Metrics_fTilde, m.Metrics_gTilde, m.Metrics_hTilde)):
        ref = np.zeros(3)
        ref[d] = h * h / 4
        assert np.abs(M - ref).max() < 1e-13 * h * h  # curl-form metrics: round-off of the X dX products
    assert np.abs(m.SurfElem - h * h / 4).max() < 1e-13 * h * h
    assert np.allclose(np.linalg.norm(m.NormVec, axis=-1), 1.0)
    # every side: exactly one master (flip 0) and one slave
    cnt = np.zeros((m.nSides, 2), int)
    for e in range(m.nElems):
        for ls in range(6):
            s, flip, master = m.ElemToSide[e, ls]
            cnt[s - 1, 0 if master else 1] += 1
            assert (flip == 0) == bool(master)
    assert (cnt == 1).all()
    # HOPR orientations: this file has masters on minus sides too
    assert (m.ElemToSide[:, :, 2] == 0).any(axis=1).sum() > 0


def _node_map(mesh, values):
    """{(element barycentre, node position) -> value} with positions rounded for matching."""
    out = {}
    bc = mesh.Elem_xGP.mean(axis=(1, 2, 3))
    for e in range(mesh.nElems):
        kb = tuple(np.round(bc[e], 9))
        X = mesh.Elem_xGP[e].reshape(-1, 3)
        V = values[e].reshape(X.shape[0], -1)
        for x, v in zip(X, V):
            out[kb + tuple(np.round(x, 9))] = v
    return out


@pytest.mark.parametrize("kw,N", [(dict(Riemann="roe", SplitDG="pi", parabolic=True, mu0=6.25e-4, R=71.42857), 3),
                                  (dict(NodeType="gauss", Riemann="lf", parabolic=True, mu0=1e-3), 2)])
def test_rhs_on_file_mesh_equals_generated_box(kw, N):
    nt = 1 if kw.get("NodeType") == "gauss" else 2
    cfg = gx.config(N=N, **kw)
    mf = gx.Mesh.from_hopr(MESH, N, nt)
    mg = gx.Mesh(N, nt, 8, 8, 8, (0.0,) * 3, (2 * math.pi,) * 3)

    def state(m):
        U = gx.tgv_state(m, mach=0.3, R=cfg.R)
        x = m.Elem_xGP
        # a smooth non-symmetric perturbation, a function of position only
        s = np.sin(x[..., 0] + 0.3) * np.cos(2 * x[..., 1]) + 0.5 * np.sin(x[..., 2] - 0.7)
        U = U.copy()
        U[..., 0] *= 1 + 0.02 * s
        U[..., 4] *= 1 + 0.01 * s
        return U

    Uf, Ug = state(mf), state(mg)
    rf = Oracle(cfg, mf).rhs(Uf)
    rg = Oracle(cfg, mg).rhs(Ug)
    a, b = _node_map(mf, rf), _node_map(mg, rg)
    assert a.keys() == b.keys()
    diff = max(np.abs(a[k] - b[k]).max() for k in a)
    scale = max(np.abs(v).max() for v in b.values())
    # The file's metrics come from the curl form (round-off ~2e-14 relative), the generated box's are
    # exact; the background pressure p0 ~ 8 of this state turns that into ~1e-11 in Ut.  A wrong side,
    # flip or orientation would give O(1) differences.
    assert diff <= 1e-10 * scale, (diff, scale)
