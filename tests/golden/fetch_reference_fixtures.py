"""Copy the reference's golden unit-test data into tests/golden/.

The GALAEXI reference keeps golden vectors for its basis and face operators as
Fortran sequential-unformatted files (4-byte record markers, float64/int32
little endian) under unitTests/.  They are data, not code.  This script copies
the ones that pin the DGSEM path so that the tests also run where the reference
tree is absent:

  NodesAndWeights.bin          x, w, wBary for N=1..10, 4 node sets   (unitTests/NodesAndWeights.f90)
  DerivativeMatrix.bin         D for N=1..10, 4 node sets             (unitTests/DerivativeMatrix.f90)
  UnittestElementData3D.bin    one curved element, NRef=9             (unitTests/unittest.f90:50,97)
  ProlongToFaceUvol.bin        random volume data                     (unitTests/ProlongToFace.f90)
  ProlongToFace_{G,GL}3D.bin   prolonged face data
  SurfIntFlux.bin              random face flux                       (unitTests/SurfInt.f90)
  SurfInt_{G,GL}3D.bin         surface-integral result
  Vandermonde.bin              nodal and modal Vandermonde matrices, 4 node sets  (unitTests/Vandermonde.f90)
  ChangeBasis.bin              ChangeBasis3D / ChangeBasis3D_XYZ of a fixed field (unitTests/ChangeBasis.f90)
  TGV_Re1600_Split_TGVAnalysis_Reference.csv
                               Taylor-Green vortex analysis of the split-form regression run
                               (regressioncheck/checks/tgv/split/), one row every 10 time steps
  CART_HEX_PERIODIC_008_mesh.h5  the HOPR mesh of that run (8^3 periodic hexahedra on [0,2pi]^3)
  cavity4x4x4_mesh.h5          the lid-driven cavity regression (regressioncheck/checks/parabolic/
                               cavity_3D/): 4^3 elements, isothermal walls and a Dirichlet lid
  reggie_cavity_Re100_State_0000001.000000000.h5
                               that regression's reference state at t = 1 (DG_Solution, N = 2)
  CART_HEX2D_FlatPlateG_mesh.h5  flat-plate tutorial mesh (tutorials/flatPlate/meshes/): Dirichlet,
                               pressure-outflow, adiabatic-wall and slip-wall sides
  NACA0012_652_Ng2_mesh.h5     curved (NGeo = 2) airfoil mesh of regressioncheck/checks/naca/3D/:
                               adiabatic wall, far-field and periodic sides

Usage:  python tests/golden/fetch_reference_fixtures.py [/path/to/reference]
"""
import os
import shutil
import sys

FILES = [
    "NodesAndWeights.bin",
    "DerivativeMatrix.bin",
    "UnittestElementData3D.bin",
    "ProlongToFaceUvol.bin",
    "ProlongToFace_G3D.bin",
    "ProlongToFace_GL3D.bin",
    "SurfIntFlux.bin",
    "SurfInt_G3D.bin",
    "SurfInt_GL3D.bin",
    "Vandermonde.bin",
    "ChangeBasis.bin",
]


REGRESSION = [
    ("regressioncheck/checks/tgv/split", "TGV_Re1600_Split_TGVAnalysis_Reference.csv"),
    ("regressioncheck/checks/tgv/split", "CART_HEX_PERIODIC_008_mesh.h5"),
    ("regressioncheck/checks/parabolic/cavity_3D", "cavity4x4x4_mesh.h5"),
    ("regressioncheck/checks/parabolic/cavity_3D", "reggie_cavity_Re100_State_0000001.000000000.h5"),
    ("tutorials/flatPlate/meshes", "CART_HEX2D_FlatPlateG_mesh.h5"),
    ("regressioncheck/checks/naca/3D", "NACA0012_652_Ng2_mesh.h5"),
]


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    for name in FILES:
        src = os.path.join(ref_root, "unitTests", name)
        shutil.copyfile(src, os.path.join(here, name))
        print("copied", name)
    for sub, name in REGRESSION:
        shutil.copyfile(os.path.join(ref_root, sub, name), os.path.join(here, name))
        print("copied", name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
