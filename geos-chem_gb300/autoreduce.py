"""Host side of auto-reduction: the per-cell controls and the keep-active mask
that GEOS-Chem's fullchem driver hands the integrator when it runs with
``Input_Opt%USE_AUTOREDUCE``.

* ``HALOGEN_KEEP`` / ``keep_mask``: the species of
  fullchem_AR_KeepHalogensActive (KPP/fullchem/fullchem_AutoReduceFuncs.F90:
  47-110), never frozen when keepActive is on.  Do_FullChem turns keepActive
  on for every grid box (GeosCore/fullchem_mod.F90:585-587) and fills the mask
  when AutoReduce_Is_KeepActive is set (:510-515).
* ``integrator_options``: the auto-reduce part of
  fullchem_AR_SetIntegratorOptions (fullchem_AutoReduceFuncs.F90:274-343) for
  a batch of cells -- ICNTRL(12), and per cell RCNTRL(12) (optionally scaled
  by the pressure ratio to the surface level), or a target species
  ICNTRL(14) with ratio RCNTRL(14): OH by day, NO2 when SUNCOSmid is at most
  cos(98 deg).

The arrays go to ``Solver.set_autoreduce`` (C ABI gc_kpp_ctx_set_autoreduce).
"""
import numpy as np

# fullchem_AutoReduceFuncs.F90:69-108 (KPP species names; Fortran is
# case-insensitive, so SALACl is the mechanism's SALACL)
HALOGEN_KEEP = (
    "AERI", "Br", "Br2", "BrCl", "BrNO2", "BrNO3", "BrO", "BrSALA", "BrSALC", "HBr", "HOBr",
    "Cl", "Cl2", "Cl2O2", "ClNO2", "ClNO3", "ClO", "ClOO", "OClO", "HCl", "HOCl",
    "I", "I2", "IO", "I2O2", "HI", "ISALA", "ISALC", "I2O4", "I2O3", "INO", "IONO", "IONO2", "ICl", "IBr", "HOI",
    "SALACl", "SALCCl", "SALAAL", "SALCAL",
)

# cos(98 deg): the night test of fullchem_AutoReduceFuncs.F90:337
NIGHT_SUNCOS = -0.1391731e0


def _index(ir, name):
    low = [s.lower() for s in ir["species"]]
    return low.index(name.lower())


def keep_mask(ir, names=HALOGEN_KEEP):
    """keepSpcActive as a [NVAR] uint8 mask (1 = never frozen)."""
    nvar = ir["dims"]["nvar"]
    m = np.zeros(nvar, np.uint8)
    for n in names:
        i = _index(ir, n)
        if i >= nvar:
            raise ValueError("%s is not a variable species" % n)
        m[i] = 1
    return m


def integrator_options(ir, ncell, threshold=1.0e2, pmid=None, pmid_sfc=None, suncos_mid=None,
                       is_prs_threshold=False, is_key_threshold=False, tuning_oh=0.0, tuning_no2=0.0):
    """Per-cell auto-reduce controls of fullchem_AR_SetIntegratorOptions.

    Returns (thr, target, ratio), each [ncell]: RCNTRL(12), ICNTRL(14)
    (1-based species index, 0 = threshold mode) and RCNTRL(14).  With the
    key-species method the threshold array is left at 0 (RCNTRL(12) is not
    set there, and the integrator ignores it when ICNTRL(14) > 0)."""
    thr = np.zeros(ncell, np.float64)
    target = np.zeros(ncell, np.int32)
    ratio = np.zeros(ncell, np.float64)
    if not is_key_threshold:
        if is_prs_threshold:
            thr[:] = threshold * np.asarray(pmid, np.float64) / np.asarray(pmid_sfc, np.float64)
        else:
            thr[:] = threshold
        return thr, target, ratio
    oh = _index(ir, "OH") + 1
    no2 = _index(ir, "NO2") + 1
    night = np.asarray(suncos_mid, np.float64) <= NIGHT_SUNCOS
    target[:] = np.where(night, no2, oh)
    ratio[:] = np.where(night, tuning_no2, tuning_oh)
    return thr, target, ratio
