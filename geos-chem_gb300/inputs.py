"""Seeded synthetic cell states for the fullchem workloads.

GEOS-Chem restart and meteorology files are not available, so cell states are
generated (numpy PCG64, ``default_rng(seed)``) with the shapes and value
ranges of the benchmark configurations:

* box model (``box_cells``): T ~ U(190, 310) K, P ~ logU(1, 1013) hPa,
  H2O vmr ~ logU(1e-6, 3e-2), half the cells at night (all J = 0), the others
  with J = s * J_noon, s ~ logU(1e-3, 1);
* global grids (``grid_cells``): nlon x nlat x nlev cells ordered like the
  reference's I (fastest), J, L loop; T and P follow a standard atmosphere on
  72 levels with N(0, 15 K) temperature noise; night or day from the solar
  zenith angle at a seeded UTC hour and day of year (night: SZA > 98 deg,
  fullchem_mod.F90:621-642); daytime J = J_noon scaled by
  (cos SZA - cos 98deg) / (1 - cos 98deg).

Initial concentrations are logU(1e2, 1e12) molec/cm3 per variable species;
fixed species are O2 = 0.2095, N2 = 0.7808, H2 = 5e-7 times the air number
density; the prod/loss family dummies are zero (fullchem_mod.F90:943-946).
Heterogeneous state, K_MT/K_CLD and SRHOCl/SRHOBr are zero.

J_noon (``noon_j_profile``) is a fabricated clear-sky noon profile: Cloud-J
data is not available, so each photolysis slot gets a typical magnitude for
the species it photolyses (NO2 ~ 8e-3 1/s, O3 ~ 3e-5 ... , 1e-5 1/s
otherwise).
"""
import re

import numpy as np

from . import mechanism
from .rates_program import MET_FIELDS

KB = 1.380649e-23  # J/K
NPHOTOL = 200

# typical clear-sky noon J-values [1/s] by photolysed species (fabricated)
_J_TYPICAL = {
    "NO2": 8.0e-3, "NO3": 1.5e-1, "O3": 3.0e-5, "HNO2": 1.5e-3, "HONO": 1.5e-3, "H2O2": 7.0e-6, "HNO3": 5.0e-7,
    "HNO4": 5.0e-6, "N2O5": 3.0e-5, "CH2O": 3.0e-5, "MP": 5.0e-6, "Cl2": 2.0e-3, "Br2": 3.0e-2, "BrO": 3.0e-2,
    "ClO": 1.0e-4, "OClO": 6.0e-2, "Cl2O2": 1.0e-3, "HOBr": 1.0e-3, "HOCl": 2.0e-4, "BrNO3": 1.0e-3,
    "ClNO3": 5.0e-5, "ClNO2": 3.0e-4, "BrNO2": 1.0e-3, "BrCl": 1.0e-2, "I2": 1.0e-1, "IO": 1.0e-1, "OIO": 1.0e-1,
    "HOI": 1.0e-2, "IONO": 1.0e-2, "IONO2": 1.0e-2, "INO": 1.0e-2, "IBr": 5.0e-2, "ICl": 2.0e-2, "CH3I": 1.0e-6,
    "CH2I2": 5.0e-3, "CH2IBr": 5.0e-4, "CH2ICl": 1.0e-4, "ALD2": 5.0e-6, "ACET": 5.0e-7, "MGLY": 1.0e-4,
    "GLYX": 1.0e-4, "PAN": 5.0e-7, "MEK": 1.0e-6, "HAC": 1.0e-6, "GLYC": 5.0e-6, "MVK": 1.0e-6, "MACR": 2.0e-6,
    "O2": 1.0e-11, "N2O": 1.0e-12, "OCS": 1.0e-11, "H2O": 1.0e-12,
}
J_DEFAULT = 1.0e-5


def photolysis_slots(ir=None):
    """{PHOTOL slot (0-based): photolysed species name} from Update_RCONST."""
    ir = ir or mechanism.load_ir()
    out = {}
    for r, e in enumerate(ir["rconst"]):
        m = re.fullmatch(r"\(PHOTOL\[(\d+)\]\)", e)
        if not m:
            continue
        slot = int(m.group(1))
        vars_ = [t for t in ir["fun"]["A"][r] if t.startswith("V")]
        if vars_:
            out.setdefault(slot, ir["species"][int(vars_[0][1:])])
    return out


def noon_j_profile(ir=None):
    j = np.zeros(NPHOTOL)
    for slot, sp in photolysis_slots(ir).items():
        j[slot] = _J_TYPICAL.get(sp, J_DEFAULT)
    return j


def _log_uniform(rng, lo, hi, size):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size))


def _fill_concentrations(rng, ir, numden, n):
    d = ir["dims"]
    sp = ir["species"]
    c = _log_uniform(rng, 1e2, 1e12, (d["nspec"], n))
    fixed = {"O2": 0.2095, "N2": 0.7808, "H2": 5.0e-7}
    for name, frac in fixed.items():
        if name in sp:
            c[sp.index(name)] = frac * numden
    for fam in ir["families"]:
        c[sp.index(fam)] = 0.0
    return c


def tolerances(ir=None):
    """ATOL/RTOL(NVAR) as Do_FullChem sets them from the species database
    (fullchem_mod.F90:485-487, 2899-2905)."""
    ir = ir or mechanism.load_ir()
    tol = ir["tolerances"]
    nvar = ir["dims"]["nvar"]
    names = ir["species"][:nvar]
    atol = np.array([tol["atol"].get(s, tol["atol_default"]) for s in names])
    rtol = np.array([tol["rtol"].get(s, tol["rtol_default"]) for s in names])
    return atol, rtol


def box_cells(n=1024, seed=0, ir=None):
    """Box-model cells: returns dict(met [NMET,n], photol [200,n], c [NSPEC,n])."""
    ir = ir or mechanism.load_ir()
    rng = np.random.default_rng(seed)
    temp = rng.uniform(190.0, 310.0, n)
    press = _log_uniform(rng, 1.0, 1013.0, n)
    vmr = _log_uniform(rng, 1e-6, 3e-2, n)
    night = np.zeros(n, bool)
    night[rng.permutation(n)[: n // 2]] = True
    scale = _log_uniform(rng, 1e-3, 1.0, n)
    return _assemble(rng, ir, temp, press, vmr, np.where(night, 0.0, scale), {"night": night})


def _assemble(rng, ir, temp, press, vmr, jscale, extra):
    n = temp.size
    numden = press * 100.0 / (KB * temp) * 1e-6
    met = np.zeros((len(MET_FIELDS), n))
    met[MET_FIELDS.index("TEMP")] = temp
    met[MET_FIELDS.index("NUMDEN")] = numden
    met[MET_FIELDS.index("H2O")] = vmr * numden
    met[MET_FIELDS.index("PRESS")] = press
    photol = noon_j_profile(ir)[:, None] * jscale[None, :]
    c = _fill_concentrations(rng, ir, numden, n)
    out = {"met": met, "photol": np.ascontiguousarray(photol), "c": c, "temp": temp, "press": press}
    out.update(extra)
    return out


# --- standard atmosphere on 72 levels -------------------------------------------

_US76 = [(0.0, 288.15, -6.5), (11.0, 216.65, 0.0), (20.0, 216.65, 1.0), (32.0, 228.65, 2.8),
         (47.0, 270.65, 0.0), (51.0, 270.65, -2.8), (71.0, 214.65, -2.0), (84.852, 186.946, 0.0)]


def _std_atmosphere(z_km):
    """(T [K], P [hPa]) of the 1976 US standard atmosphere at altitude z."""
    g0, M, R = 9.80665, 0.0289644, 8.3144598
    t = np.empty_like(z_km)
    p = np.empty_like(z_km)
    for i, z in enumerate(z_km):
        pb, k = 1013.25, 0
        while k + 1 < len(_US76) and z > _US76[k + 1][0]:
            hb, tb, lr = _US76[k]
            h1 = _US76[k + 1][0]
            if lr == 0:
                pb = pb * np.exp(-g0 * M * (h1 - hb) * 1e3 / (R * tb))
            else:
                pb = pb * (tb / (tb + lr * (h1 - hb))) ** (g0 * M / (R * lr * 1e-3))
            k += 1
        hb, tb, lr = _US76[k]
        t[i] = tb + lr * (z - hb)
        if lr == 0:
            p[i] = pb * np.exp(-g0 * M * (z - hb) * 1e3 / (R * tb))
        else:
            p[i] = pb * (tb / t[i]) ** (g0 * M / (R * lr * 1e-3))
    return t, p


def level_profile(nlev=72):
    """Mid-level altitude/temperature/pressure of an nlev grid from the surface
    to ~0.01 hPa, finer near the surface like the GEOS 72-level grid."""
    s = (np.arange(nlev) + 0.5) / nlev
    z = 80.0 * s ** 1.6
    t, p = _std_atmosphere(z)
    return z, t, p


def _cos_sza(lat_deg, lon_deg, hour_utc, doy):
    dec = np.deg2rad(23.44) * np.sin(2 * np.pi * (284 + doy) / 365.0)
    ha = np.deg2rad((hour_utc + lon_deg / 15.0 - 12.0) * 15.0)
    lat = np.deg2rad(lat_deg)
    return np.sin(lat) * np.sin(dec) + np.cos(lat) * np.cos(dec) * np.cos(ha)


def grid_cells(nlon=72, nlat=46, nlev=72, seed=0, ir=None, nox_boundary_layer=False):
    """Global-grid cells, cell index = i + nlon*(j + nlat*l) (I fastest)."""
    ir = ir or mechanism.load_ir()
    rng = np.random.default_rng(seed)
    z, t_prof, p_prof = level_profile(nlev)
    lon = -180.0 + (np.arange(nlon) + 0.5) * 360.0 / nlon
    lat = -90.0 + (np.arange(nlat) + 0.5) * 180.0 / nlat
    L, J, I = np.meshgrid(np.arange(nlev), np.arange(nlat), np.arange(nlon), indexing="ij")
    L, J, I = L.ravel(), J.ravel(), I.ravel()
    n = L.size
    temp = np.clip(t_prof[L] + rng.normal(0.0, 15.0, n), 180.0, 330.0)
    press = p_prof[L]
    vmr_sfc = _log_uniform(rng, 3e-3, 3e-2, n)
    vmr = np.maximum(vmr_sfc * np.exp(-z[L] / 2.5), 3e-6)
    hour = rng.uniform(0.0, 24.0)
    doy = int(rng.integers(1, 366))
    mu = _cos_sza(lat[J], lon[I], hour, doy)
    cos98 = np.cos(np.deg2rad(98.0))
    night = mu <= cos98
    jscale = np.where(night, 0.0, (mu - cos98) / (1.0 - cos98))
    out = _assemble(rng, ir, temp, press, vmr, jscale, {"night": night, "level": L, "lat": lat[J], "lon": lon[I]})
    if nox_boundary_layer:
        sp = ir["species"]
        bl = L < 10
        for name in ("NO", "NO2"):
            out["c"][sp.index(name), bl] = _log_uniform(rng, 1e8, 1e12, int(bl.sum()))
    return out


def default_controls():
    """ICNTRL/RCNTRL as fullchem_AR_SetIntegratorOptions sets them
    (KPP/fullchem/fullchem_AutoReduceFuncs.F90:240-287): autonomous, Rodas3,
    no adjoint, no rate updates inside the integrator; RCNTRL(3) = Hstart."""
    icntrl = np.zeros(20, np.int32)
    icntrl[0] = 1
    icntrl[2] = 4
    icntrl[6] = 1
    icntrl[14] = -1
    rcntrl = np.zeros(20)
    return icntrl, rcntrl
