"""TEST INFRASTRUCTURE: inputs for the oracle built without the product library.

The CPU baseline (bench.py's reference arm and its cpu_baseline leg) times the oracle on the
benchmark workload.  Everything it needs is made here from the oracle and numpy alone, so that the
baseline loads no part of galaexi_gb300:

  OracleConfig / config()   struct dg_config of include/galaexi_gb300.h, filled from keyword values
  PeriodicBox               a periodic hexahedral box as a HOPR mesh describes it: equidistant NGeo = 1
                            node coordinates, ElemToSide / SideToElem (mesh_vars.f90:92-129 layout,
                            1-based IDs), and the mesh arrays from the oracle's own BuildCoords +
                            CalcMetrics + CalcSurfMetrics (calc_metrics)
  tgv_state                 the Taylor-Green vortex initial state (testcase/taylorgreenvortex/
                            testcase.f90:145-149, 220-262; rho0 = U0 = 1, constant density) and
                            PrimToCons (idealgas/eos.f90:467-489)
"""
import ctypes

import numpy as np

from .oracle import calc_metrics


class OracleConfig(ctypes.Structure):
    """struct dg_config (include/galaexi_gb300.h)."""
    _fields_ = [
        ("N", ctypes.c_int), ("node_type", ctypes.c_int), ("parabolic", ctypes.c_int), ("riemann", ctypes.c_int),
        ("split_dg", ctypes.c_int), ("lifting", ctypes.c_int), ("do_weak_lifting", ctypes.c_int),
        ("do_conservative_lifting", ctypes.c_int), ("eta_br2", ctypes.c_double), ("kappa", ctypes.c_double),
        ("R", ctypes.c_double), ("Pr", ctypes.c_double), ("mu0", ctypes.c_double), ("precision", ctypes.c_int),
        ("filter_type", ctypes.c_int), ("n_filter", ctypes.c_int), ("hest_filter_param", ctypes.c_double * 3),
        ("laf_alpha", ctypes.c_double),
    ]


RIEMANN = {"lf": 0, "roe": 1, "roel2": 2, "roeentropyfix": 3, "hll": 4, "hllc": 5, "hlle": 6, "hllem": 7, "avg": 8}
SPLIT = {"none": -1, "sd": 0, "mo": 1, "du": 2, "kg": 3, "pi": 4}
NODETYPE = {"gauss": 1, "gauss-lobatto": 2}


def config(N, node_type="gauss-lobatto", riemann="lf", split="none", parabolic=False, kappa=1.4, R=287.058, Pr=0.72,
           mu0=0.0):
    """A dg_config with the reference's defaults for everything not given (BR1, strong
    non-conservative lifting, etaBR2 = 2, FP64, no filter)."""
    c = OracleConfig()
    c.N, c.node_type, c.parabolic = int(N), NODETYPE[node_type], int(bool(parabolic))
    c.riemann, c.split_dg, c.lifting = RIEMANN[riemann], SPLIT[split], 1
    c.do_weak_lifting = c.do_conservative_lifting = 0
    c.eta_br2, c.kappa, c.R, c.Pr, c.mu0 = 2.0, kappa, R, Pr, mu0
    c.precision, c.filter_type, c.n_filter, c.laf_alpha = 0, 0, 0, 0.0
    return c


# local sides (flexi.h:98-103)
ZETA_MINUS, ETA_MINUS, XI_PLUS, ETA_PLUS, XI_MINUS, ZETA_PLUS = 1, 2, 3, 4, 5, 6


class PeriodicBox:
    """Periodic box [x0,x1]^3 of ne^3 affine hexahedra.  Element e = ix + ne (iy + ne iz); side
    3e + d (d = 0, 1, 2) is the XI_PLUS / ETA_PLUS / ZETA_PLUS side of element e (its master, flip 0)
    and the XI_MINUS / ETA_MINUS / ZETA_MINUS side of the next element in direction d, whose flips
    follow from the CGNS orientation of the local sides (mappings.f90:376-409): 1 for XI_MINUS and
    ZETA_MINUS (their side axes are swapped against the plus side), 2 for ETA_MINUS (its first axis
    runs backwards)."""

    def __init__(self, N, node_type, ne, x0, x1):
        self.N, self.node_type, self.NGeo = N, node_type, 1
        E = ne ** 3
        self.nElems, self.nSides, self.nBCSides = E, 3 * E, 0
        eid = lambda ix, iy, iz: (ix % ne) + ne * ((iy % ne) + ne * (iz % ne))
        E2S = np.zeros((E, 6, 3), dtype=np.int32)
        S2E = np.zeros((3 * E, 5), dtype=np.int32)
        nodes = np.zeros((E, 2, 2, 2, 3))
        h = [(x1[d] - x0[d]) / ne for d in range(3)]
        for iz in range(ne):
            for iy in range(ne):
                for ix in range(ne):
                    e = eid(ix, iy, iz)
                    for d, (plus, minus, flip) in enumerate(((XI_PLUS, XI_MINUS, 1), (ETA_PLUS, ETA_MINUS, 2),
                                                             (ZETA_PLUS, ZETA_MINUS, 1))):
                        nb = eid(ix + (d == 0), iy + (d == 1), iz + (d == 2))
                        s = 3 * e + d
                        E2S[e, plus - 1] = (s + 1, 0, 1)
                        E2S[nb, minus - 1] = (s + 1, flip, 0)
                        S2E[s] = (e + 1, nb + 1, plus, minus, flip)
                    for k in range(2):
                        for j in range(2):
                            for i in range(2):
                                nodes[e, k, j, i] = (x0[0] + (ix + i) * h[0], x0[1] + (iy + j) * h[1],
                                                     x0[2] + (iz + k) * h[2])
        self.ElemToSide, self.SideToElem, self.NodeCoords = E2S, S2E, nodes
        g = calc_metrics(N, node_type, 1, nodes, E2S, self.nSides)
        if g["bad_nodes"] != 0:
            raise ValueError("PeriodicBox: bad Jacobian")
        for k in ("Elem_xGP", "Metrics_fTilde", "Metrics_gTilde", "Metrics_hTilde", "sJ", "NormVec", "TangVec1",
                  "TangVec2", "SurfElem"):
            setattr(self, k, g[k])

    @property
    def nDOF(self):
        return self.nElems * (self.N + 1) ** 3


def tgv_state(xgp, mach=0.1, kappa=1.4, R=287.058, rho0=1.0, U0=1.0):
    """TGV conservative state at the nodes xgp (..., 3); same layout with 5 variables."""
    x, y, z = xgp[..., 0], xgp[..., 1], xgp[..., 2]
    p0 = (U0 / mach) ** 2 / kappa * rho0
    u = U0 * np.sin(x) * np.cos(y) * np.cos(z)
    v = -U0 * np.cos(x) * np.sin(y) * np.cos(z)
    w = np.zeros_like(u)
    p = p0 + (rho0 * U0 * U0) / 16.0 * (np.cos(2 * x) * np.cos(2.0 * z) + 2.0 * np.cos(2.0 * y) + 2.0 * np.cos(2.0 * x)
                                         + np.cos(2 * y) * np.cos(2.0 * z))
    rho = np.full_like(u, rho0)
    out = np.empty(xgp.shape[:-1] + (5,))
    out[..., 0] = rho
    out[..., 1], out[..., 2], out[..., 3] = u * rho, v * rho, w * rho
    out[..., 4] = p / (kappa - 1.0) + 0.5 * (out[..., 1] * u + out[..., 2] * v + out[..., 3] * w)
    return out
