"""gcchem: GB300-native KPP fullchem Rosenbrock chemistry solve.

A drop-in for the per-cell chemistry loop of GEOS-Chem's Do_FullChem
(GeosCore/fullchem_mod.F90:528-1551): rate evaluation, the Rodas3
Rosenbrock integration with sparse analytic Jacobian and unrolled sparse LU,
all in FP64, as hand-written CUDA for sm_103a behind a C ABI
(include/gckpp_gb300.h).  The Python modules here are the host-side mirror
of that interface, the build step, the code generator and the synthetic
input generator.
"""
import os

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
