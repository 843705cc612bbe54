"""CPU checks of the C-ABI library: it loads, exports every function include/galaexi_gb300.h declares,
and its host-side set-up (ini parsing, mesh, metrics, initial states) is consistent.  No kernel runs here."""
import ctypes
import math
import os
import re
import subprocess

import numpy as np
import pytest

import galaexi_gb300 as gx
from galaexi_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "galaexi_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    names = header_functions()
    assert len(names) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", nat.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (dg_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    L = nat.lib()
    for n in names:
        assert getattr(L, n) is not None
    assert set(nat.exported_symbols()) <= set(names)


def test_config_from_ini_uses_reference_keys():
    ini = """
    ! parameter file in the reference's syntax
    N             = 7 ! Polynomial degree
    NodeType      = Gauss-Lobatto
    Riemann       = RoeEntropyFix
    SplitDG       = PI
    Parabolic     = T
    mu0           = 6.25E-04
    R             = 71.42857
    doWeakLifting = F
    Precision     = mixed
    """
    cfg = gx.config_from_ini(ini)
    assert cfg.N == 7 and cfg.node_type == 2 and cfg.riemann == 3 and cfg.split_dg == 4
    assert cfg.parabolic == 1 and abs(cfg.mu0 - 6.25e-4) < 1e-18 and abs(cfg.R - 71.42857) < 1e-12
    assert cfg.precision == 1 and cfg.kappa == 1.4 and cfg.Pr == 0.72
    with pytest.raises(nat.DGError):
        gx.config_from_ini("Riemann = nonsense")


def test_context_rejects_invalid_combinations():
    for kw in [dict(NodeType="gauss", SplitDG="pi"), dict(SplitDG="pi", Riemann="hllc"), dict(Riemann="avg"),
               dict(parabolic=True, mu0=1e-3, Lifting="br2", doWeakLifting=True)]:
        cfg = gx.config(N=3, **kw)
        h = ctypes.c_void_p()
        rc = nat.lib().dg_ctx_create(ctypes.byref(cfg), ctypes.byref(h))
        assert rc == nat.DG_ERR_ARG, kw
        assert nat.lib().dg_last_error()


@pytest.mark.parametrize("node_type", [1, 2])
def test_mesh_connectivity_and_metrics(node_type):
    N = 3
    m = gx.Mesh(N, node_type, 3, 2, 4, (0, 0, 0), (3.0, 2.0, 4.0))
    assert m.nElems == 24 and m.nSides == 72
    # every side has exactly one master (flip 0) and one slave (flip 1..4)
    cnt = np.zeros((m.nSides, 2), int)
    for e in range(m.nElems):
        for ls in range(6):
            s, flip, master = m.ElemToSide[e, ls]
            cnt[s - 1, 0 if flip == 0 else 1] += 1
            assert master == (1 if flip == 0 else 0)
    assert (cnt == 1).all()
    # unit spacing h=1: Ja = h^2/4, sJ = 8/h^3, |n| = 1, SurfElem = h^2/4
    assert np.allclose(m.Metrics_fTilde[..., 0], 0.25) and np.allclose(m.Metrics_fTilde[..., 1:], 0)
    assert np.allclose(m.sJ, 8.0)
    assert np.allclose(np.linalg.norm(m.NormVec, axis=-1), 1.0) and np.allclose(m.SurfElem, 0.25)
    # master and slave face points coincide (periodically) under the S2V2 orientation
    n = N + 1
    from oracle import oracle as orc
    s2v2 = orc.s2v2(N).reshape(6, 5, n, n, 2)  # [loc-1][flip][q][p][c]
    L = np.array([3.0, 2.0, 4.0])
    for s in range(m.nSides):
        e, nb, loc, nbloc, flip = m.SideToElem[s]
        for q in range(n):
            for p in range(n):
                def pt(elem, lside, fl):
                    a, b = s2v2[lside - 1, fl, q, p]
                    i, j, k = {5: (0, a, b), 3: (N, a, b), 2: (a, 0, b), 4: (a, N, b), 1: (a, b, 0), 6: (a, b, N)}[lside]
                    return m.Elem_xGP[elem - 1, k, j, i]
                d = pt(e, loc, 0) - pt(nb, nbloc, flip)
                d = d - L * np.round(d / L)
                if node_type == 1:  # Gauss face points are off the nodes in the normal direction
                    d[{5: 0, 3: 0, 2: 1, 4: 1, 1: 2, 6: 2}[loc]] = 0.0
                assert np.abs(d).max() < 1e-12


def test_curved_mesh_metric_identities():
    """Conservative curl-form metrics satisfy the discrete metric identities (free-stream preservation):
    sum_i D (Ja^i)_d = 0 at every node."""
    N = 4
    m = gx.Mesh(N, 2, 2, 2, 2, (0, 0, 0), (1, 1, 1), deform=0.05)
    b = gx.basis(N, 2)
    D = b["D"].reshape(N + 1, N + 1).T  # D[i, l]
    div = (np.einsum("il,elkjd->eikjd".replace("eikjd", "ekjid").replace("elkjd", "ekjld"), D, m.Metrics_fTilde)
           + np.einsum("jl,ekljd->ekjd".replace("ekjd", "ekjid").replace("ekljd", "eklid"), D, m.Metrics_gTilde)
           + np.einsum("kl,eljid->ekjid", D, m.Metrics_hTilde))
    assert np.abs(div).max() < 1e-11
    assert (m.sJ > 0).all()


def test_fill_ini_tgv_and_vortex():
    m = gx.Mesh(3, 2, 2, 2, 2, (-math.pi,) * 3, (math.pi,) * 3)
    U = gx.tgv_state(m, mach=0.1, kappa=1.4, R=71.42857)
    assert np.allclose(U[..., 0], 1.0)
    x = m.Elem_xGP
    assert np.allclose(U[..., 1], np.sin(x[..., 0]) * np.cos(x[..., 1]) * np.cos(x[..., 2]))
    prm = [1, 1, 1, 0, 1, 5, 5, 0, 0, 0, 1, 5, 1]
    mv = gx.Mesh(3, 1, 2, 2, 1, (0, 0, 0), (10, 10, 10))
    V = gx.fill_ini(mv, nat.DG_EXACTFUNC_SHU_VORTEX, prm)
    xv = mv.Elem_xGP
    r2 = (xv[..., 0] - 5) ** 2 + (xv[..., 1] - 5) ** 2
    du = -5 / (2 * math.pi) * np.exp((1 - r2) / 2) * (xv[..., 1] - 5)
    assert np.allclose(V[..., 1] / V[..., 0], 1 + du)


def test_ctypes_signatures_match_header():
    """The ctypes argtypes/restype of every entry point agree with the C declaration: same count,
    scalars with the matching ctypes type, pointers as pointers (c_void_p, c_char_p or POINTER(...))."""
    import ctypes
    import re
    from galaexi_gb300 import _native as nat
    text = re.sub(r"/\*.*?\*/", " ", open(os.path.join(ROOT, "include", "galaexi_gb300.h")).read(), flags=re.S)
    decls = {}
    for m in re.finditer(r"\b([A-Za-z_][\w\s\*]*?)\b(dg_\w+)\s*\(([^;{}]*?)\)\s*;", text):
        args = [a.strip() for a in m.group(3).split(",") if a.strip() and a.strip() != "void"]
        decls[m.group(2)] = (m.group(1).splitlines()[-1].replace("const", "").strip(), args)
    assert sorted(decls) == sorted(nat._SIGS)
    scalar = {"int": ctypes.c_int, "double": ctypes.c_double, "size_t": ctypes.c_size_t,
              "long long": ctypes.c_longlong}

    def is_pointer(t):
        return t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(t, ctypes._Pointer))

    for name, (res, args) in nat._SIGS.items():
        ret, cargs = decls[name]
        if ret == "void":
            assert res is None, name
        elif "*" in ret:
            assert is_pointer(res), name
        else:
            assert res is scalar[ret], (name, ret)
        assert len(args) == len(cargs), name
        for a, c in zip(args, cargs):
            words = [w for w in re.split(r"[\s\*]+", c) if w and w != "const"]
            base = " ".join(words[:-1])
            if "*" in c:
                assert is_pointer(a), (name, c, a)
            else:
                assert a is scalar[base], (name, c, a)
