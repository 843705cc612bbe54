"""galaexi_gb300: GB300-native DGSEM right-hand side and low-storage RK stepper.

A drop-in for the DGTimeDerivative_weakForm / TimeStepByLSERKW2 path of GALAEXI, built as
hand-written sm_103a CUDA kernels behind a C ABI (include/galaexi_gb300.h).  This package
holds the in-tree build (build.py), the ctypes binding (_native.py) and the host-side mirror
of the reference's operator interface (dg.py).
"""
from . import _native
from ._native import DGError, DGConfig, RIEMANN, SPLITDG
from .dg import DG, Mesh, basis, config, config_from_ini, fill_ini, read_h5, read_state, tgv_state, write_state

__all__ = ["DG", "Mesh", "DGError", "DGConfig", "RIEMANN", "SPLITDG", "basis", "config", "config_from_ini",
           "fill_ini", "tgv_state"]
