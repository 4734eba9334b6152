"""Mechanism IR for the KPP fullchem mechanism.

``fullchem.json`` is produced by ``extract_kpp.py`` from the KPP-3.2.0
generated Fortran of GEOS-Chem (KPP/fullchem/gckpp_*.F90) and holds, with
0-based indices:

* ``dims``: NSPEC/NVAR/NFIX/NREACT/LU_NONZERO (gckpp_Parameters.F90:34-54)
* ``species``: species names in KPP order (variable species first, then fixed)
* ``fun``: Fun_SPLIT statements (gckpp_Function.F90:2172-5059)
* ``jac``: Jac_SP statements (gckpp_Jacobian.F90:48-20887)
* ``lu``: LU_IROW/LU_ICOL/LU_CROW/LU_DIAG (gckpp_JacobianSP.F90:525-1093)
* ``solve``: KppSolve statement order (gckpp_LinearAlgebra.F90:644-2309)
* ``rconst``: Update_RCONST expressions (gckpp_Rates.F90:441-1502)
"""
import functools
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


@functools.lru_cache(maxsize=None)
def load_ir(name="fullchem"):
    with open(os.path.join(HERE, name + ".json")) as fh:
        return json.load(fh)


def species_index(ir, name):
    return ir["species"].index(name)
