"""The HetState of a cell as rows of a cell-interleaved array.

Update_RCONST's heterogeneous rate laws read the per-cell HetState that
fullchem_SetStateHet fills (KPP/fullchem/commonIncludeVars.H:111-201,
KPP/fullchem/fullchem_HetStateFuncs.F90:48).  The batch boundary takes it as
``het[f * ldh + cell]``, one row per scalar field and one row per element of
the array fields, in the order of FIELDS below (the order of the Fortran
type, then SUNCOS).  Logical fields are 0.0 (false) or 1.0 (true).
``emit_c`` gives the row offsets of csrc/het_layout.h (and of the oracle's
copy), which a test keeps equal to this list.

``het_cells`` draws a seeded synthetic HetState per cell: aerosol surface
areas, radii and water of the 14 aerosol types, cloud liquid/ice areas and
radii, halide and sulfite concentrations, pH values and the stratospheric
flags, with magnitudes of tropospheric/stratospheric conditions.  No restart
or aerosol model output is available here, so these stand in for the fields
fullchem_SetStateHet computes from State_Chm and State_Met.
"""
import numpy as np

# (name, length); length 1 = scalar.  Logical fields are marked in LOGICAL.
FIELDS = [
    ("AVO", 1), ("natSurface", 1), ("pscBox", 1), ("stratBox", 1), ("NAEROTYPE", 1),
    ("aClArea", 1), ("aClRadi", 1), ("aClVol", 1), ("aIce", 1), ("aLiq", 1), ("aWater", 2),
    ("Br_conc_CldA", 1), ("Br_conc_CldC", 1), ("Br_conc_CldG", 1), ("Br_conc_Cld", 1),
    ("Br_conc_SSA", 1), ("Br_conc_SSC", 1), ("Br_over_Cl_Cld", 1), ("Br_over_Cl_SSA", 1),
    ("Br_over_Cl_SSC", 1), ("Cl_conc_CldA", 1), ("Cl_conc_CldC", 1), ("Cl_conc_CldG", 1),
    ("Cl_conc_Cld", 1), ("Cl_conc_SSA", 1), ("Cl_conc_SSC", 1), ("cldFr", 1), ("clearFr", 1),
    ("frac_Br_CldA", 1), ("frac_Br_CldC", 1), ("frac_Br_CldG", 1), ("frac_Cl_CldA", 1),
    ("frac_Cl_CldC", 1), ("frac_Cl_CldG", 1), ("frac_HSO3_aq", 1), ("frac_SALACL", 1),
    ("frac_SO3_aq", 1), ("fupdateHOBr", 1), ("fupdateHOCl", 1), ("gamma_HO2", 1), ("H2O", 1),
    ("HBr_theta", 1), ("HCl_theta", 1), ("H_conc_ICl", 1), ("H_conc_LCl", 1), ("H_conc_SSA", 1),
    ("H_conc_SSC", 1), ("H_conc_Sul", 1), ("HNO3_theta", 1), ("HSO3_aq", 1), ("SO3_aq", 1),
    ("HSO3m", 1), ("SO3mm", 1), ("TSO3_aq", 1), ("H_plus", 1), ("KHETI_SLA", 11), ("HSO4_molal", 1),
    ("NO3_molal", 1), ("SO4_molal", 1), ("NIT_conc_SSA", 1), ("NIT_conc_SSC", 1), ("PI", 1),
    ("pHCloud", 1), ("pHSSA", 2), ("OMOC_POA", 1), ("OMOC_OPOA", 1), ("qIce", 1), ("qLiq", 1),
    ("rIce", 1), ("rLiq", 1), ("f_Acid_SSA", 1), ("f_Acid_SSC", 1), ("f_Alk_SSA", 1), ("f_Alk_SSC", 1),
    ("SSA_is_Alk", 1), ("SSA_is_Acid", 1), ("SSC_is_Alk", 1), ("SSC_is_Acid", 1), ("vAir", 1),
    ("vIce", 1), ("vLiq", 1), ("wetArea", 14), ("xArea", 14), ("xH2O", 14), ("xRadi", 14), ("xVol", 14),
    ("cloudBox", 1), ("fracOrgAer", 1), ("fracInorgAer", 1), ("TurnOffHetRates", 1),
    # not a HetState field: the cosine of the solar zenith angle that
    # Set_Kpp_GridBox_Values stores in SUNCOS (GeosCore/fullchem_mod.F90:2141),
    # read by GLYXuptk1stOrd
    ("SUNCOS", 1),
]
LOGICAL = {"natSurface", "pscBox", "stratBox", "SSA_is_Alk", "SSA_is_Acid", "SSC_is_Alk", "SSC_is_Acid",
           "cloudBox", "TurnOffHetRates"}

OFFSET = {}
_o = 0
for _name, _len in FIELDS:
    OFFSET[_name] = _o
    _o += _len
NFIELD = _o

# aerosol types of xArea/xRadi/... (KPP/fullchem/fullchem_RateLawFuncs.F90:27-40), 1-based
DU1, SUL, BKC, ORC, SSA, SSC, SLA, IIC = 1, 8, 9, 10, 11, 12, 13, 14


# Grid-box inputs of the per-cell producers before Update_RCONST --
# fullchem_SetStateHet (KPP/fullchem/fullchem_HetStateFuncs.F90:48-244),
# fullchem_SulfurAqChem, fullchem_SulfurCldChem / SET_SO2 and
# fullchem_HetDropChem (KPP/fullchem/fullchem_SulfurChemFuncs.F90:120-305,
# 414-790, 865-1620) -- per cell,
# as rows of a cell-interleaved array ``hetin[f * ldi + cell]``: the State_Met
# and State_Chm fields they read, in their units (State_Met: T [K], CLDF [1],
# QI/QL [kg/kg], AIRVOL [m3], AIRDEN [kg/m3], AD [kg], FRLAND/FROCEAN [1],
# InStratosphere 0/1, PMID_DRY [hPa], OMEGA [Pa/s], U/V [m/s], IsWater 0/1;
# State_Chm: aerosol areas [cm2/cm3],
# radii [cm], AeroH2O [cm3/m3], ISORROPIA/HETP water, molalities, H+ and pH,
# cloud pH, HSO3_aq/SO3_aq [mol/L], fupdateHOBr/HOCl, KHETI_SLA, STATE_PSC,
# and the concentrations [molec/cm3] of the species that are not KPP
# species: sea salt SALA, SALAAL, SALC, SALCAL, NH4, NH3, the seven dust
# bins, pFe), and SUNCOS, which is copied to the HetState array's last row.
# The KPP species they read come from C.  SET_SO2 writes HSO3_aq, SO3_aq and
# pHCloud, and Set_Sulfur_Chem_Rates sets fupdateHOBr/HOCl to 1, before
# fullchem_SetStateHet reads them (GeosCore/fullchem_mod.F90:861-936).
HETIN_FIELDS = [
    ("T", 1), ("CLDF", 1), ("QI", 1), ("QL", 1), ("AIRVOL", 1), ("AIRDEN", 1), ("AD", 1), ("FRLAND", 1),
    ("FROCEAN", 1), ("InStratosphere", 1), ("aClArea", 1), ("aClRadi", 1), ("IsorropAeroH2O", 2),
    ("AeroArea", 14), ("AeroRadi", 14), ("WetAeroArea", 14), ("AeroH2O", 14), ("OMOC_POA", 1), ("OMOC_OPOA", 1),
    ("HSO3_aq", 1), ("SO3_aq", 1), ("IsorropBisulfate", 1), ("IsorropNitrate", 1), ("IsorropSulfate", 1),
    ("IsorropHplus", 1), ("pHCloud", 1), ("IsorropAeropH", 2), ("SALA", 1), ("SALAAL", 1), ("SALC", 1),
    ("SALCAL", 1), ("fupdateHOBr", 1), ("fupdateHOCl", 1), ("KHETI_SLA", 11), ("STATE_PSC", 1), ("SUNCOS", 1),
    # read by SET_SO2 only
    ("PMID_DRY", 1), ("NH4", 1), ("NH3", 1), ("DSTbin", 7), ("pFe", 1),
    # read by fullchem_HetDropChem only: pressure velocity [Pa/s], winds
    # [m/s], State_Met%IsWater 0/1
    ("OMEGA", 1), ("U", 1), ("V", 1), ("IsWater", 1),
]
HETIN_OFFSET = {}
_o = 0
for _name, _len in HETIN_FIELDS:
    HETIN_OFFSET[_name] = _o
    _o += _len
NHETIN = _o
# KPP species that fullchem_SetStateHet and fullchem_SulfurAqChem read
# through C(ind_X)
SETSTATE_SPECIES = ["SO2", "HNO3", "HCl", "HBr", "BrSALA", "BrSALC", "SALACL", "SALCCL", "NIT", "NITs", "SO4",
                    "SALAAL", "SALCAL", "O3", "H2O2", "CH2O", "SO4s", "HMS", "HCOOH", "ACTA", "HOCl", "HOBr"]
# MW_g of the species whose mass SET_SO2 and HetDropChem convert
# (run/shared/species_database.yml: DSTbin1, pFe, SALA, SALC, SO4)
NONKPP_MW = {"DSTbin1": 29.0, "pFe": 55.85, "SALA": 31.4, "SALC": 31.4, "SO4": 96.06}


def emit_c():
    lines = ["// Generated by gcchem.hetstate (emit_c). Do not edit.", "#pragma once",
             "// rows of the cell-interleaved HetState array (order of the Fortran type)",
             "#define HET_NFIELD %d" % NFIELD]
    for name, n in FIELDS:
        lines.append("#define HET_%s %d%s" % (name, OFFSET[name], "  /* %d rows */" % n if n > 1 else ""))
    lines += ["// rows of the cell-interleaved fullchem_SetStateHet input array",
              "#define HETIN_NFIELD %d" % NHETIN]
    for name, n in HETIN_FIELDS:
        lines.append("#define HETIN_%s %d%s" % (name, HETIN_OFFSET[name], "  /* %d rows */" % n if n > 1 else ""))
    lines.append("// KPP species read by fullchem_SetStateHet and fullchem_SulfurAqChem, in the order of the "
                 "index table")
    for k, name in enumerate(SETSTATE_SPECIES):
        lines.append("#define HSS_%s %d" % (name, k))
    lines.append("#define HSS_N %d" % len(SETSTATE_SPECIES))
    lines.append("// MW_g of the non-KPP species SET_SO2 reads (species database)")
    for name, mw in NONKPP_MW.items():
        lines.append("#define HSS_MW_%s %r" % (name, mw))
    return "\n".join(lines) + "\n"


def zero_cells(n):
    """The zeroed HetState (no aerosol, no cloud: ClearFr 1, PI, AVO set)."""
    h = np.zeros((NFIELD, n))
    h[OFFSET["AVO"]] = 6.022140857e23
    h[OFFSET["PI"]] = np.pi
    h[OFFSET["clearFr"]] = 1.0
    h[OFFSET["NAEROTYPE"]] = 14.0
    return h


def het_cells(n, seed=0, strat_fraction=0.15, cloud_fraction=0.5):
    """Seeded synthetic HetState for n cells (see the module docstring)."""
    rng = np.random.default_rng(seed)
    h = zero_cells(n)
    o = OFFSET
    lu = lambda lo, hi, size=n: np.exp(rng.uniform(np.log(lo), np.log(hi), size))
    strat = rng.uniform(size=n) < strat_fraction
    h[o["stratBox"]] = strat
    h[o["natSurface"]] = strat & (rng.uniform(size=n) < 0.3)
    h[o["pscBox"]] = strat & (rng.uniform(size=n) < 0.3)
    # aerosol areas [cm2/cm3], radii [cm], water and volume per type
    for t in range(14):
        area = lu(1e-9, 1e-5)
        radi = lu(2e-6, 2e-4)
        h[o["xArea"] + t] = area
        h[o["wetArea"] + t] = area * rng.uniform(1.0, 2.0, n)
        h[o["xRadi"] + t] = radi
        h[o["xVol"] + t] = area * radi / 3.0
        h[o["xH2O"] + t] = area * radi / 3.0 * rng.uniform(0.0, 0.8, n)
    # the stratospheric liquid aerosol and ice only where strat
    for t in (SLA, IIC):
        h[o["xArea"] + t - 1] *= strat
    h[o["aClArea"]] = h[o["xArea"] + SUL - 1] + h[o["xArea"] + SSA - 1]
    h[o["aClRadi"]] = lu(5e-6, 5e-5)
    h[o["aClVol"]] = h[o["aClArea"]] * h[o["aClRadi"]] / 3.0
    h[o["aWater"]] = lu(1e-12, 1e-9)
    h[o["aWater"] + 1] = lu(1e-12, 1e-9)
    # cloud: fraction, liquid/ice areas and radii (Cld_Params magnitudes)
    cloudy = (rng.uniform(size=n) < cloud_fraction) & ~strat
    cldf = np.where(cloudy, rng.uniform(0.01, 1.0, n), 0.0)
    h[o["cldFr"]] = cldf
    h[o["clearFr"]] = 1.0 - cldf
    h[o["cloudBox"]] = cloudy
    h[o["rLiq"]] = np.where(rng.uniform(size=n) < 0.5, 6.0e-4, 10.0e-4)
    h[o["rIce"]] = lu(1e-3, 5e-3)
    h[o["aLiq"]] = np.where(cloudy, lu(1e-6, 1e-3), 0.0)
    h[o["aIce"]] = np.where(cloudy, lu(1e-7, 1e-4), 0.0)
    h[o["vLiq"]] = h[o["aLiq"]] * h[o["rLiq"]] / 3.0
    h[o["vIce"]] = h[o["aIce"]] * h[o["rIce"]] / 3.0 / 2.25
    h[o["vAir"]] = lu(1e13, 1e15)
    h[o["qLiq"]] = np.where(cloudy, lu(1e-6, 1e-3), 0.0)
    h[o["qIce"]] = np.where(cloudy, lu(1e-7, 1e-4), 0.0)
    # halides [mol/L or mol/kg], fractions, ratios
    for f in ("Br_conc_CldA", "Br_conc_CldC", "Br_conc_CldG", "Br_conc_SSA", "Br_conc_SSC"):
        h[o[f]] = lu(1e-9, 1e-3)
    for f in ("Cl_conc_CldA", "Cl_conc_CldC", "Cl_conc_CldG", "Cl_conc_SSA", "Cl_conc_SSC",
              "NIT_conc_SSA", "NIT_conc_SSC"):
        h[o[f]] = lu(1e-6, 5.0)
    h[o["Br_conc_Cld"]] = h[o["Br_conc_CldA"]] + h[o["Br_conc_CldC"]] + h[o["Br_conc_CldG"]]
    h[o["Cl_conc_Cld"]] = h[o["Cl_conc_CldA"]] + h[o["Cl_conc_CldC"]] + h[o["Cl_conc_CldG"]]
    for x in ("Br", "Cl"):
        parts = rng.dirichlet([1.0, 1.0, 1.0], n).T
        for k, s in enumerate("ACG"):
            h[o["frac_%s_Cld%s" % (x, s)]] = parts[k]
    h[o["Br_over_Cl_Cld"]] = h[o["Br_conc_Cld"]] / h[o["Cl_conc_Cld"]]
    h[o["Br_over_Cl_SSA"]] = h[o["Br_conc_SSA"]] / h[o["Cl_conc_SSA"]]
    h[o["Br_over_Cl_SSC"]] = h[o["Br_conc_SSC"]] / h[o["Cl_conc_SSC"]]
    h[o["frac_SALACL"]] = rng.uniform(0.0, 1.0, n)
    # sulfite in cloud
    h[o["HSO3_aq"]] = lu(1e-9, 1e-4)
    h[o["SO3_aq"]] = lu(1e-12, 1e-6)
    h[o["TSO3_aq"]] = h[o["HSO3_aq"]] + h[o["SO3_aq"]]
    h[o["frac_HSO3_aq"]] = h[o["HSO3_aq"]] / h[o["TSO3_aq"]]
    h[o["frac_SO3_aq"]] = h[o["SO3_aq"]] / h[o["TSO3_aq"]]
    h[o["HSO3m"]] = lu(1e-3, 1.0)
    h[o["SO3mm"]] = lu(1e-6, 1e-2)
    h[o["fupdateHOBr"]] = rng.uniform(0.5, 1.0, n)
    h[o["fupdateHOCl"]] = rng.uniform(0.5, 1.0, n)
    h[o["gamma_HO2"]] = rng.uniform(0.0, 0.2, n)
    h[o["H2O"]] = lu(1e14, 5e17)
    for f in ("HBr_theta", "HCl_theta", "HNO3_theta"):
        h[o[f]] = rng.uniform(0.0, 1.0, n)
    for f in ("H_conc_ICl", "H_conc_LCl", "H_conc_SSA", "H_conc_SSC", "H_conc_Sul", "H_plus"):
        h[o[f]] = lu(1e-8, 1e-1)
    h[o["KHETI_SLA"]:o["KHETI_SLA"] + 11] = lu(1e-12, 1e-5, (11, n)) * strat
    for f in ("HSO4_molal", "NO3_molal", "SO4_molal"):
        h[o[f]] = lu(1e-4, 5.0)
    h[o["pHCloud"]] = rng.uniform(3.0, 6.5, n)
    h[o["pHSSA"]] = rng.uniform(1.0, 8.0, n)
    h[o["pHSSA"] + 1] = rng.uniform(1.0, 8.0, n)
    h[o["OMOC_POA"]] = rng.uniform(1.4, 2.1, n)
    h[o["OMOC_OPOA"]] = rng.uniform(1.4, 2.1, n)
    alk_a = h[o["pHSSA"]] >= 5.0
    alk_c = h[o["pHSSA"] + 1] >= 5.0
    h[o["SSA_is_Alk"]] = alk_a
    h[o["SSA_is_Acid"]] = ~alk_a
    h[o["SSC_is_Alk"]] = alk_c
    h[o["SSC_is_Acid"]] = ~alk_c
    h[o["f_Alk_SSA"]] = np.where(alk_a, rng.uniform(0.5, 1.0, n), 0.0)
    h[o["f_Acid_SSA"]] = 1.0 - h[o["f_Alk_SSA"]]
    h[o["f_Alk_SSC"]] = np.where(alk_c, rng.uniform(0.5, 1.0, n), 0.0)
    h[o["f_Acid_SSC"]] = 1.0 - h[o["f_Alk_SSC"]]
    h[o["fracOrgAer"]] = rng.uniform(0.0, 1.0, n)
    h[o["fracInorgAer"]] = 1.0 - h[o["fracOrgAer"]]
    h[o["SUNCOS"]] = np.where(rng.uniform(size=n) < 0.5, rng.uniform(0.0, 1.0, n), -rng.uniform(0.0, 1.0, n))
    return h


def hetin_cells(n, seed=0, strat_fraction=0.15, cloud_fraction=0.5):
    """Seeded synthetic inputs of fullchem_SetStateHet for n cells
    ([NHETIN, n]): grid-box air volume, density and mass of a 4x5 column,
    cloud fraction and condensate where cloudy, land/ocean split, aerosol
    areas/radii/water of the 14 types (the stratospheric liquid and ice
    types only in the stratosphere), ISORROPIA/HETP water and molalities,
    pH values, sulfite, sea-salt alkalinity, KHETI_SLA and the PSC state."""
    rng = np.random.default_rng(seed)
    h = np.zeros((NHETIN, n))
    o = HETIN_OFFSET
    lu = lambda lo, hi, size=n: np.exp(rng.uniform(np.log(lo), np.log(hi), size))
    strat = rng.uniform(size=n) < strat_fraction
    h[o["T"]] = np.where(strat, rng.uniform(185.0, 240.0, n), rng.uniform(200.0, 310.0, n))
    cloudy = (rng.uniform(size=n) < cloud_fraction) & ~strat
    h[o["CLDF"]] = np.where(cloudy, rng.uniform(1e-4, 1.0, n), 0.0)
    h[o["QL"]] = np.where(cloudy & (rng.uniform(size=n) < 0.8), lu(1e-7, 1e-3), 0.0)
    h[o["QI"]] = np.where(cloudy & (rng.uniform(size=n) < 0.5), lu(1e-8, 1e-4), 0.0)
    h[o["AIRVOL"]] = lu(2e12, 3e14)
    h[o["AIRDEN"]] = np.where(strat, lu(1e-3, 0.2), lu(0.1, 1.3))
    h[o["AD"]] = h[o["AIRDEN"]] * h[o["AIRVOL"]]
    land = rng.uniform(size=n)
    h[o["FRLAND"]] = land
    h[o["FROCEAN"]] = 1.0 - land
    h[o["InStratosphere"]] = strat
    for t in range(14):
        area = lu(1e-9, 1e-5)
        radi = lu(2e-6, 2e-4)
        if t + 1 in (SLA, IIC):
            area = area * strat
        h[o["AeroArea"] + t] = area
        h[o["WetAeroArea"] + t] = area * rng.uniform(1.0, 2.0, n)
        h[o["AeroRadi"] + t] = radi
        h[o["AeroH2O"] + t] = area * radi / 3.0 * 1e6 * rng.uniform(0.0, 0.8, n)
    h[o["aClArea"]] = h[o["AeroArea"] + SUL - 1] + h[o["AeroArea"] + SSA - 1]
    h[o["aClRadi"]] = lu(5e-6, 5e-5)
    h[o["IsorropAeroH2O"]] = lu(1e-12, 1e-9)
    h[o["IsorropAeroH2O"] + 1] = lu(1e-12, 1e-9)
    h[o["OMOC_POA"]] = rng.uniform(1.4, 2.1, n)
    h[o["OMOC_OPOA"]] = rng.uniform(1.4, 2.1, n)
    h[o["HSO3_aq"]] = np.where(cloudy, lu(1e-9, 1e-4), 0.0)
    h[o["SO3_aq"]] = np.where(cloudy, lu(1e-12, 1e-6), 0.0)
    for f in ("IsorropBisulfate", "IsorropNitrate", "IsorropSulfate"):
        h[o[f]] = lu(1e-4, 5.0)
    h[o["IsorropHplus"]] = lu(1e-8, 1e-1)
    h[o["pHCloud"]] = np.where(cloudy, rng.uniform(3.0, 6.5, n), 0.0)
    h[o["IsorropAeropH"]] = rng.uniform(1.0, 8.0, n)
    h[o["IsorropAeropH"] + 1] = rng.uniform(1.0, 8.0, n)
    h[o["SALA"]] = lu(1e5, 1e11)
    h[o["SALAAL"]] = h[o["SALA"]] * np.where(rng.uniform(size=n) < 0.5, rng.uniform(0.0, 1.2, n), 0.0)
    h[o["SALC"]] = np.where(rng.uniform(size=n) < 0.9, lu(1e5, 1e11), 0.0)
    h[o["SALCAL"]] = h[o["SALC"]] * rng.uniform(0.0, 0.05, n)
    h[o["fupdateHOBr"]] = rng.uniform(0.5, 1.0, n)
    h[o["fupdateHOCl"]] = rng.uniform(0.5, 1.0, n)
    h[o["KHETI_SLA"]:o["KHETI_SLA"] + 11] = lu(1e-12, 1e-5, (11, n)) * strat
    h[o["STATE_PSC"]] = np.where(strat, rng.integers(0, 4, n), 0)
    h[o["SUNCOS"]] = rng.uniform(-1.0, 1.0, n)
    # dry pressure from density and temperature (R_dry = 287.05 J/kg/K)
    h[o["PMID_DRY"]] = h[o["AIRDEN"]] * 287.05 * h[o["T"]] / 100.0
    h[o["NH4"]] = lu(1e6, 1e11)
    h[o["NH3"]] = lu(1e6, 1e11)
    h[o["DSTbin"]:o["DSTbin"] + 7] = lu(1e2, 1e8, (7, n)) * (rng.uniform(size=n) < 0.7)
    h[o["pFe"]] = lu(1e1, 1e6)
    h[o["OMEGA"]] = rng.normal(0.0, 0.3, n)
    h[o["U"]] = rng.normal(0.0, 10.0, n)
    h[o["V"]] = rng.normal(0.0, 8.0, n)
    h[o["IsWater"]] = 1.0 - land.round()
    return h
