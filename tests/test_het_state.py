"""fullchem_SetStateHet (KPP/fullchem/fullchem_HetStateFuncs.F90:48-244): the
producer of the HetState rows that Update_RCONST's heterogeneous laws read.

* CPU: the oracle's C restatement (oracle/het_state.c) against an
  independent numpy restatement of the same Fortran (Cld_Params,
  Get_Theta_Ice, Halide_Conc with Get_Halide_CldConc / Get_Halide_SsaConc /
  CALC_KH / CALC_HEFF, the pH and alkalinity fields, the PSC flags), on seeded
  synthetic grid-box fields.
* GPU: gc_kpp_set_state_het_batch against the oracle, field by field; then
  a chemistry step whose HetState comes from the GPU producer, against the
  oracle's loop body fed by the oracle's producer.
"""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
AVO = 6.022140857e23


def _case(n, seed):
    import gcchem.hetstate as hs
    import gcchem.inputs as inputs
    from gcchem.mechanism import load_ir

    ir = load_ir()
    cells = inputs.box_cells(n, seed=seed)
    hin = hs.hetin_cells(n, seed=seed + 100)
    # sea-salt halides and nitrate with magnitudes that reach every branch
    rng = np.random.default_rng(seed)
    sp = ir["species"]
    for name in ("BrSALA", "BrSALC", "SALACL", "SALCCL", "NIT", "NITs", "SO4"):
        v = np.exp(rng.uniform(np.log(1e2), np.log(1e10), n))
        v[rng.uniform(size=n) < 0.1] = 0.0
        cells["c"][sp.index(name)] = v
    return ir, cells, hin


def _numpy_state(ir, hin, c, gamma_ho2, lpscchem, turn_off):
    """The Fortran restated in numpy, field by field."""
    import gcchem.hetstate as hs

    o = hs.HETIN_OFFSET
    sp = ir["species"]
    C = lambda name: c[sp.index(name)]
    T = hin[o["T"]]
    cldf = hin[o["CLDF"]]
    ql, qi = hin[o["QL"]], hin[o["QI"]]
    out = {}
    out["cldFr"] = np.clip(cldf, 0.0, 1.0)
    vair = hin[o["AIRVOL"]] * 1e6
    # Cld_Params
    cloudy = ~((ql + qi <= 0.0) | (cldf <= 0.0))
    rliq = np.where(hin[o["FRLAND"]] > hin[o["FROCEAN"]], 6.0e-4, 10.0e-4)
    vliq = ql * hin[o["AD"]] / 0.001 / vair
    vice = qi * hin[o["AD"]] / 0.91e-3 / vair
    alpha = np.where(T < 202.0, 83.3, np.where(T < 217.0, 9.1744e4, 308.4))
    beta = np.where(T < 202.0, 0.0184, np.where(T < 217.0, 0.117, 0.0152))
    rice = 0.5 * alpha * np.exp(beta * (T - 273.15)) / 1e4
    out["rLiq"] = np.where(cloudy, rliq, 6.0e-4)
    out["rIce"] = np.where(cloudy, rice, 38.5e-4)
    out["vLiq"] = np.where(cloudy, vliq, 0.0)
    out["vIce"] = np.where(cloudy, vice, 0.0)
    out["aLiq"] = np.where(cloudy, 3.0 * vliq / rliq, 0.0)
    out["aIce"] = np.where(cloudy, 3.0 * vice / rice * 2.25, 0.0)
    # Get_Theta_Ice
    k1 = 7.5e-5 * np.exp(4585.0 / T) / 2.7e14
    k2 = 1.3e-5 * np.exp(4600.0 / T) / 3.0e14
    den = 1.0 + k1 * C("HNO3") + k2 * C("HCl")
    out["HNO3_theta"] = k1 * C("HNO3") / den
    out["HCl_theta"] = k2 * C("HCl") / den
    out["HBr_theta"] = np.minimum(4.14e-10 * C("HBr") ** 0.88, 1.0)
    # pH and alkalinity
    ph1 = hin[o["IsorropAeropH"]]
    out["H_conc_Sul"] = 10.0 ** (-ph1)
    out["H_conc_LCl"] = 10.0 ** (-hin[o["pHCloud"]])
    with np.errstate(divide="ignore", invalid="ignore"):
        fa = np.where(hin[o["SALA"]] != 0.0, hin[o["SALAAL"]] / hin[o["SALA"]], 0.0)
        fc = np.where(hin[o["SALC"]] != 0.0, hin[o["SALCAL"]] / hin[o["SALC"]], 0.0)
    out["f_Alk_SSA"] = np.clip(fa, 0.0, 1.0)
    out["f_Alk_SSC"] = np.clip(fc, 0.0, 1.0)
    out["SSA_is_Alk"] = (out["f_Alk_SSA"] > 0.01).astype(float)
    out["SSC_is_Acid"] = (out["f_Alk_SSC"] <= 0.01).astype(float)
    # Halide_Conc: cloud water
    hbr = C("HBr") + C("BrSALA") * 0.7 + C("BrSALC")
    hcl = C("HCl") + C("SALACL") * 0.7 + C("SALCCL")
    with np.errstate(divide="ignore", invalid="ignore"):
        vtot = np.where(out["cldFr"] != 0.0, out["vLiq"] / out["cldFr"], 0.0)
        ph = hin[o["pHCloud"]]

        def l2g(k0, cr, pka):
            kh = k0 * np.exp(cr * (1.0 / T - 1.0 / 298.15)) * 8.3144598 * T / 101.325
            heff = np.where((ph > 0.0) & (pka > -100.0), kh * (1.0 + 10.0 ** (ph - pka)), kh)
            return heff * vtot

        lc = l2g(1.0, 9000.0, -6.3)
        lb = l2g(0.75, 10200.0, -9.0)
        cl = np.where(vtot < 1e-20, 0.0, lc / (1.0 + lc) * hcl / (vtot * AVO * 1e-3))
        br = np.where(vtot < 1e-20, 0.0, lb / (1.0 + lb) * hbr / (vtot * AVO * 1e-3))
        out["Br_conc_Cld"] = np.where(hbr > 0.0, br, 0.0)
        out["Cl_conc_Cld"] = np.where(hcl > 0.0, cl, 0.0)
        out["frac_Cl_CldG"] = np.where(out["Cl_conc_Cld"] > 0.0, C("HCl") / hcl, 0.0)
    # sea-salt halides
    a12, r12 = hin[o["AeroArea"] + 11], hin[o["AeroRadi"] + 11]

    def ssa(nx, area, r):
        v = area * r / 3.0 * 1e-3
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(v <= 1e-20, 0.0, np.maximum(nx / AVO / v, 0.0))

    out["Br_conc_SSA"] = ssa(C("BrSALA"), hin[o["aClArea"]], hin[o["aClRadi"]])
    out["Cl_conc_SSC"] = ssa(C("SALCCL"), a12, r12)
    out["NIT_conc_SSA"] = ssa(C("NIT"), hin[o["aClArea"]], hin[o["aClRadi"]])
    s = C("SALACL") + C("NIT") + C("SO4")
    with np.errstate(divide="ignore", invalid="ignore"):
        out["frac_SALACL"] = np.where(s > 0.0, C("SALACL") / s, 0.0)
    # sulfite over SO2
    with np.errstate(divide="ignore", invalid="ignore"):
        num = hin[o["HSO3_aq"]] * 1e-3 * AVO * ql * hin[o["AIRDEN"]] * 1e-3
        x = np.where(cldf != 0.0, num / cldf, 0.0)
        out["HSO3m"] = np.where(C("SO2") != 0.0, x / C("SO2"), 0.0)
    # flags
    strat = hin[o["InStratosphere"]] != 0.0
    psc = bool(lpscchem) & (hin[o["STATE_PSC"]] >= 2.0) & strat
    out["stratBox"] = strat.astype(float)
    out["pscBox"] = psc.astype(float)
    out["natSurface"] = (psc & (C("NIT") > 0.0)).astype(float)
    out["TurnOffHetRates"] = np.full(c.shape[1], float(bool(turn_off)))
    out["gamma_HO2"] = np.full(c.shape[1], gamma_ho2)
    out["xH2O"] = hin[o["AeroH2O"]:o["AeroH2O"] + 14] * 1e-6
    out["SUNCOS"] = hin[o["SUNCOS"]]
    return out


def test_setstatehet_layout_in_public_header():
    import gcchem.hetstate as hs

    with open(os.path.join(ROOT, "include", "gckpp_gb300.h")) as fh:
        text = fh.read()
    assert "#define GC_KPP_NHETIN %d" % hs.NHETIN in text
    assert hs.NHETIN == 115


@pytest.mark.parametrize("lpscchem,turn_off", [(1, 0), (0, 1)])
def test_oracle_setstatehet_matches_numpy_restatement(orc, lpscchem, turn_off):
    import gcchem.hetstate as hs

    n = 2048
    ir, cells, hin = _case(n, 7)
    h = orc.set_state_het(hin, cells["c"], gamma_ho2=0.2, lpscchem=lpscchem, turn_off_het_rates=turn_off)
    ref = _numpy_state(ir, hin, cells["c"], 0.2, lpscchem, turn_off)
    assert np.all(np.isfinite(h))
    for name, want in ref.items():
        got = h[hs.OFFSET[name]] if name != "xH2O" else h[hs.OFFSET["xH2O"]:hs.OFFSET["xH2O"] + 14]
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=0, err_msg=name)
    # both branches of every test are reached
    for name in ("aLiq", "Br_conc_Cld", "Br_conc_SSA", "HSO3m", "frac_SALACL"):
        v = h[hs.OFFSET[name]]
        assert (v == 0).any() and (v > 0).any(), name
    assert (h[hs.OFFSET["pscBox"]] > 0).any() == bool(lpscchem)
    # fields the routine leaves alone
    for name in ("H2O", "cloudBox", "fracOrgAer", "fracInorgAer"):
        assert np.all(h[hs.OFFSET[name]] == 0.0)
    assert np.all(h[hs.OFFSET["NAEROTYPE"]] == 14.0)


# rows that are copies, flags or set arithmetic without libm calls: equal bit
# for bit between the GPU and the oracle (both without FMA contraction)
_LIBM_FIELDS = {"H_conc_Sul", "H_conc_LCl", "H_conc_ICl", "H_conc_SSA", "H_conc_SSC", "rIce", "aIce",
                "HNO3_theta", "HCl_theta", "HBr_theta", "Br_conc_CldA", "Br_conc_CldC", "Br_conc_CldG",
                "Br_conc_Cld", "Cl_conc_CldA", "Cl_conc_CldC", "Cl_conc_CldG", "Cl_conc_Cld", "frac_Br_CldA",
                "frac_Br_CldC", "frac_Br_CldG", "frac_Cl_CldA", "frac_Cl_CldC", "frac_Cl_CldG", "Br_over_Cl_Cld"}


@pytest.mark.gpu
def test_gpu_setstatehet_matches_oracle(orc):
    import gcchem.capi as capi
    import gcchem.hetstate as hs

    n = 4096
    _, cells, hin = _case(n, 8)
    ref = orc.set_state_het(hin, cells["c"], gamma_ho2=0.1, lpscchem=1, turn_off_het_rates=0)
    s = capi.Solver(0)
    got = np.full_like(ref, -1.0)
    s.set_state_het(hin, cells["c"], got, gamma_ho2=0.1, lpscchem=1, turn_off_het_rates=0)
    s.close()
    for name, k in hs.FIELDS:
        a = got[hs.OFFSET[name]:hs.OFFSET[name] + k]
        b = ref[hs.OFFSET[name]:hs.OFFSET[name] + k]
        if name in _LIBM_FIELDS:
            # CUDA's exp/pow against glibc's: a few ulp
            rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
            assert np.array_equal(a == 0, b == 0), name
            assert rel.max() < 1e-13, (name, rel.max())
        else:
            assert np.array_equal(a, b), name


@pytest.mark.gpu
def test_gpu_chemistry_step_from_produced_hetstate(orc):
    """SetStateHet on the GPU -> gc_kpp_ctx_set_hetstate -> one chemistry
    step (strict arithmetic), against the oracle's SetStateHet, Update_RCONST
    with that HetState and loop body, on cells with cloud and aerosol."""
    import torch

    import gcchem.capi as capi
    import gcchem.inputs as inputs

    n = 192
    ir, cells, hin = _case(n, 9)
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    c = cells["c"].copy()
    for fam in ir["families"]:
        c[ir["species"].index(fam)] = 0.0
    dev = torch.device("cuda", 0)
    s = capi.Solver(0, arith="strict", schedule="queue")
    hin_d = torch.tensor(hin, device=dev)
    c_d = torch.tensor(c, device=dev)
    het_d = torch.zeros((168, n), dtype=torch.float64, device=dev)
    s.set_state_het(hin_d, c_d, het_d, gamma_ho2=0.2, lpscchem=1, turn_off_het_rates=0)
    torch.cuda.synchronize()
    h_gpu = het_d.cpu().numpy()
    h_ref = orc.set_state_het(hin, c, gamma_ho2=0.2, lpscchem=1, turn_off_het_rates=0)
    assert np.allclose(h_gpu, h_ref, rtol=1e-13, atol=0)
    # the step's rates come from the GPU's HetState; the oracle integrates
    # with the GPU's rates (the rates' own parity is tested elsewhere)
    r = np.zeros((len(ir["rconst"]), n))
    s.update_rconst(cells["met"], cells["photol"], c, r, het=h_gpu)
    r_o = orc.update_rconst(cells["met"], cells["photol"], c, het=h_ref)
    nz = r_o != 0
    assert np.array_equal(r == 0, r_o == 0)
    assert np.median(np.abs(r[nz] - r_o[nz]) / np.abs(r_o[nz])) < 1e-14
    c_ref, ist_ref, _, ierr_ref = orc.integrate(c, r, atol, rtol, 0.0, 600.0, ic, rc)
    bad = ierr_ref < 0
    if bad.any():
        c2, ist2, _, ierr2 = orc.integrate(c[:, bad], r[:, bad], atol, rtol, 0.0, 600.0, ic, rc)
        c_ref[:, bad], ist_ref[:, bad], ierr_ref[bad] = c2, ist2, ierr2
    c_ref = np.maximum(c_ref, 0.0)
    s.set_hetstate(het_d)
    cg = torch.tensor(cells["c"], device=dev)
    ist = torch.zeros((20, n), dtype=torch.int32, device=dev)
    rst = torch.zeros((20, n), dtype=torch.float64, device=dev)
    ierr = torch.zeros(n, dtype=torch.int32, device=dev)
    met = torch.tensor(cells["met"], device=dev)
    ph = torch.tensor(cells["photol"], device=dev)
    s.fullchem_step(600.0, met, ph, cg, torch.tensor(atol, device=dev), torch.tensor(rtol, device=dev), ic, rc,
                    None, ist, rst, ierr)
    torch.cuda.synchronize()
    s.set_hetstate(None)
    s.close()
    cg, ist, ierr = cg.cpu().numpy(), ist.cpu().numpy(), ierr.cpu().numpy()
    assert np.array_equal(ierr, ierr_ref)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.99
    big = np.abs(c_ref) > 1e4
    rel = np.abs(cg - c_ref) / np.maximum(np.abs(c_ref), 1e-300)
    assert np.max(np.where(big, rel, 0.0)[:, same]) < 1e-9


def _numpy_kmt(ir, hin, c, temp, numden):
    """fullchem_SulfurAqChem restated in numpy (Ars_L1K, kIIR1Ltd)."""
    import json

    import gcchem.hetstate as hs

    sp = ir["species"]
    with open(os.path.join(ROOT, "geos-chem_gb300", "mechanism", "fullchem_species.json")) as fh:
        mw = json.load(fh)["mw"]
    srmw = lambda name: np.sqrt(mw[sp.index(name)])
    C = lambda name: c[sp.index(name)]
    o = hs.HETIN_OFFSET
    sr_t = np.sqrt(temp)

    def ars(area, radius, gamma, s):
        dfkg = (9.45e17 / numden) * sr_t * np.sqrt(3.472e-2 + 1.0 / (s * s))
        return np.where((gamma < 1e-30) | (radius < 1e-30), 0.0,
                        area / ((radius / dfkg) + 2.749064e-4 * s / (gamma * sr_t)))

    def kiir(gas, educt, k):
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            kii = np.where(educt < 1.0, 0.0, k / educt)
            life_a = np.where(k > 0, 1.0 / k, 0.0)
            k_educt = k * gas / educt
            life_b = np.where(k_educt != 0, 1.0 / k_educt, 0.0)
            lim_a = (k > 0) & (life_a < life_b) & (life_a < 1e-3)
            lim_b = (k > 0) & ~lim_a & (life_b < 1e-3)
            kii = np.where(lim_a, 1e3 / educt, np.where(lim_b, 1e3 / gas, kii))
            return np.where(educt < 1.0, 0.0, kii)

    out = np.zeros((6, c.shape[1]))
    o3 = C("O3") > 1e10
    for t, (educt, typ) in enumerate((("SALAAL", 11), ("SALCAL", 12))):
        alk = C(educt) > 0.1
        area = hin[o["WetAeroArea"] + typ - 1]
        radius = hin[o["AeroRadi"] + typ - 1]
        with np.errstate(divide="ignore", invalid="ignore"):
            k = kiir(C("SO2"), C(educt), ars(area, radius, 0.11, srmw("SO2"))) / C("O3")
        out[3 * t] = np.where(alk & o3, k, 0.0)
        out[3 * t + 1] = np.where(alk, kiir(C("HCl"), C(educt), ars(area, radius, 0.07, srmw("HCl"))), 0.0)
        out[3 * t + 2] = np.where(alk, kiir(C("HNO3"), C(educt), ars(area, radius, 0.5, srmw("HNO3"))), 0.0)
    return out


def _kmt_case(n, seed):
    ir, cells, hin = _case(n, seed)
    rng = np.random.default_rng(seed + 7)
    sp = ir["species"]
    # alkaline sea salt above and below the 0.1 molec/cm3 switch, O3 around 1e10
    for name in ("SALAAL", "SALCAL"):
        cells["c"][sp.index(name)] = np.where(rng.uniform(size=n) < 0.2, 0.05,
                                              np.exp(rng.uniform(np.log(1.0), np.log(1e9), n)))
    cells["c"][sp.index("O3")] = np.exp(rng.uniform(np.log(1e9), np.log(1e13), n))
    return ir, cells, hin


def test_oracle_sulfur_aq_matches_numpy_restatement(orc):
    from gcchem.rates_program import MET_FIELDS

    n = 2048
    ir, cells, hin = _kmt_case(n, 17)
    temp = cells["met"][MET_FIELDS.index("TEMP")]
    numden = cells["met"][MET_FIELDS.index("NUMDEN")]
    k = orc.sulfur_aq_rates(hin, cells["c"], temp, numden)
    ref = _numpy_kmt(ir, hin, cells["c"], temp, numden)
    np.testing.assert_allclose(k, ref, rtol=1e-12, atol=0)
    for r in range(6):
        assert (k[r] == 0).any() and (k[r] > 0).any(), r


@pytest.mark.gpu
def test_gpu_sulfur_aq_matches_oracle(orc):
    import gcchem.capi as capi
    from gcchem.rates_program import MET_FIELDS

    n = 4096
    ir, cells, hin = _kmt_case(n, 18)
    met = cells["met"].copy()
    met[MET_FIELDS.index("K_MT0"):MET_FIELDS.index("K_MT0") + 6] = -1.0
    s = capi.Solver(0)
    s.sulfur_aq_rates(hin, cells["c"], met)
    s.close()
    ref = orc.sulfur_aq_rates(hin, cells["c"], met[MET_FIELDS.index("TEMP")], met[MET_FIELDS.index("NUMDEN")])
    k = met[MET_FIELDS.index("K_MT0"):MET_FIELDS.index("K_MT0") + 6]
    assert np.array_equal(k == 0, ref == 0)
    rel = np.abs(k - ref) / np.maximum(np.abs(ref), 1e-300)
    assert rel.max() < 1e-14, rel.max()
    # the other met rows are untouched
    others = [i for i, f in enumerate(MET_FIELDS) if not f.startswith("K_MT")]
    assert np.array_equal(met[others], cells["met"][others])


# ---------------------------------------------------------------------------
# SET_SO2 (fullchem_SulfurCldChem), KPP/fullchem/fullchem_SulfurChemFuncs.F90:
# 865-1620 with GET_HPLUS (:1635-1853), the equilibrium functions
# (:1867-3156) and AQCHEM_SO2 (:3171-3549).  The Python restatement below is
# written from the Fortran independently of oracle/het_state.c: the nine
# Henry/dissociation pairs as data, evaluated by two generic functions.

def _f32(x):
    return float(np.float32(x))


# (Henry constant, its temperature coefficient, K1, its coefficient[, K2, its
# coefficient]) of the species of GET_HPLUS, with the Fortran's literal kinds
_SO2_DI = {"CO2": (_f32(3.4e-2), 2.44e+3, _f32(4.3e-7), _f32(-1000.0), _f32(4.68e-11), _f32(-1760.0)),
           "SO2": (_f32(1.23), 3.14e+3, _f32(1.3e-2), _f32(1960.0), _f32(6.6e-8), _f32(1500.0))}
_SO2_MONO = {"HNO3": (_f32(2.1e5), _f32(0.0), _f32(15.4), _f32(8700.0)),
             "HCl": (1.5e+3, 2.3e+3, 1.74e+6, 6900.0),
             "FA": (8800.0, 6100.0, 1.8e-4, 151.0),
             "AA": (4100.0, 6200.0, 1.75e-5, 50.0)}


def _py_set_so2(hin_col, cvec, sp, lmetal, mw):
    """One cell of SET_SO2: (kcld[6], HSO3_aq, SO3_aq, pHCloud, size_res, niter)."""
    import math

    import gcchem.hetstate as hs

    o = hs.HETIN_OFFSET
    X = lambda f, k=0: float(hin_col[o[f] + k])
    C = lambda name: float(cvec[sp.index(name)])
    AIRMW, AVO_, ATM = 28.9644, 6.022140857e+23, 1.01325e+5
    RL = 0.08205
    tf = lambda D, T: math.exp(D * ((1.0 / T) - (1.0 / 298.0)))
    kcld = [0.0] * 6
    rho = X("AIRDEN")
    cnv = 1.0e3 * AIRMW / (rho * AVO_)
    so2 = C("SO2") * cnv
    h2o2 = C("H2O2") * cnv
    patm = X("PMID_DRY") / (ATM * 1.e-2)
    T = X("T")
    fc = X("CLDF")
    lwc = max(0.0, X("QL") * X("AIRDEN") * 1e-3)
    e = lambda v: 0 if v == 0 else math.frexp(v)[1]
    if fc == 0.0 or e(lwc) - e(fc) > 1023:
        lwc = 0.0
    elif e(lwc) - e(fc) < -1020:
        lwc = 0.0
    else:
        lwc = lwc / fc
    if not (fc > 1.0e-4 and so2 > 1e-20 and T > 258.0 and lwc > 1.0e-20):
        return kcld, 1.0e-32, 1.0e-32, 0.0, 0, 0
    so4nss = 1.e+3 * (C("SO4") * 0.7 + C("SO4s")) / (lwc * AVO_)
    tnh3 = ((X("NH4") * 0.7) + X("NH3")) * cnv
    cl = ((C("SALACL") * 0.7) + C("SALCCL") + C("HCl")) * cnv
    tfa, taa = C("HCOOH") * cnv, C("ACTA") * cnv
    tna = 1.e3 * (X("SALA") * 0.7 + X("SALC")) * (31.6 * 0.359 / 23.0) / (lwc * AVO_)
    dsum = 0.0
    for b in range(7):
        dsum = X("DSTbin", b) if b == 0 else dsum + X("DSTbin", b)
    dust = dsum * 1.e+15 * mw["DSTbin1"] / AVO_
    tdca = dust * 2.22e-15 / lwc
    tno3 = (C("HNO3") + (C("NIT") * 0.7) + C("NITs")) * cnv
    amount = {"CO2": 390.0e-6, "SO2": so2, "HNO3": tno3, "HCl": cl, "FA": tfa, "AA": taa}

    def di(name, H):
        Hc, Dh, K1, D1, K2, D2 = _SO2_DI[name]
        H_T, K1_T, K2_T = Hc * tf(Dh, T), K1 * tf(D1, T), K2 * tf(D2, T)
        heff = H_T * (1.0 + (K1_T / H) + ((K1_T * K2_T) / (H * H)))
        p = amount[name] * patm * (1.0 / (1.0 + (heff * RL * T * lwc)))
        if name == "CO2":
            f1 = H_T / H * K1_T * p
        else:
            f1 = H_T * K1_T * p / H
        f2 = K1_T * K2_T * H_T / H / H * p
        den = (K1_T * K2_T * H_T * RL * T * lwc + K1_T * H_T * RL * T * lwc * H + H_T * RL * T * lwc * H * H
               + H * H) ** 2
        d1 = K1_T * H_T * amount[name] * patm * (K1_T * K2_T * H_T * RL * T * lwc - H_T * RL * T * lwc * H * H
                                                - H * H) / den
        d2 = -1.0 * K1_T * K2_T * H_T * amount[name] * patm * (K1_T * H_T * RL * T * lwc + 2.0 * H_T * RL * T * lwc * H
                                                               + 2.0 * H) / den
        return f1, f2, d1, d2

    def mono(name, H):
        Hc, Dh, K, D = _SO2_MONO[name]
        H_T, K_T = Hc * tf(Dh, T), K * tf(D, T)
        heff = H_T * (1.0 + (K_T / H))
        p = amount[name] * patm * (1.0 / (1.0 + (heff * RL * T * lwc)))
        f = H_T * K_T * p / H
        d = (-1.0 * K_T * H_T * amount[name] * patm * (1.0 + H_T * RL * T * lwc)
             / (K_T * H_T * RL * T * lwc + H_T * RL * T * lwc * H + H) ** 2)
        return f, d

    Kw = 1.0e-14
    Kw_T = Kw * math.exp(-6710.0 * ((1.0 / T) - (1.0 / 298.0)))
    Hn, Kn = 60.0 * tf(4200.0, T), _f32(1.7e-5) * tf(_f32(-450.0), T)
    ca_den = 4.3e-7 * tf(-1000.0, T) * 4.68e-11 * tf(-1760.0, T)
    ca_den = (4.3e-7 * tf(-1000.0, T)) * (4.68e-11 * tf(-1760.0, T)) * (3.4e-2 * tf(2.44e+3, T)) * 390.0e-6 * patm
    ksp = 3.3e-9 * tf(-1200.0, T)
    ipH, newpH, count = -math.log10(3.16227766016837953e-5), 0.0, 0
    while abs(ipH - newpH) > _f32(0.01):
        count += 1
        if count > 1:
            ipH = newpH
        H = 10.0 ** (-ipH)
        fHCO3, fCO3, dHCO3, dCO3 = di("CO2", H)
        fHSO3, fSO3, dHSO3, dSO3 = di("SO2", H)
        (fHNO3, dHNO3), (fHCl, dHCl), (fFA, dFA), (fAA, dAA) = (mono(k, H) for k in ("HNO3", "HCl", "FA", "AA"))
        heff = Hn * (1.0 + ((Kn * H) / Kw_T))
        fNH4 = H * Hn * Kn * (tnh3 * patm * (1.0 / (1.0 + (heff * RL * T * lwc)))) / Kw_T
        dNH4 = (Kn * Hn * tnh3 * Kw_T * patm * (1.0 + Hn * RL * T * lwc)
                / (Hn * RL * T * lwc * (Kw_T + Kn * H) + Kw_T) ** 2)
        fCa, dCa = ksp * H * H / ca_den, 2.0 * ksp * H / ca_den
        if fCa >= tdca:
            D = (2.0 * so4nss) - (tna + 2.0 * tdca)
            fca_t, dca_t = 0.0, 0.0
        else:
            D = (2.0 * so4nss) - tna
            fca_t, dca_t = 2.0 * fCa, 2.0 * dCa
        f = D - H + Kw / H + fHCO3 + 2.0 * fCO3 + fHSO3 + 2.0 * fSO3 + fHNO3 - fNH4 + fHCl + fFA + fAA
        df = -1.0 - Kw / H / H + dHCO3 + 2.0 * dCO3 + dHSO3 + 2.0 * dSO3 + dHNO3 - dNH4 + dHCl + dFA + dAA
        if fca_t:
            f, df = f - fca_t, df - dca_t
        nn = min(max(H - f / df, 1.0e-14), 1.0e-1)
        if count > 50:
            newpH = ((-math.log10(nn)) + (-math.log10(H))) / 2.0
            break
        newpH = -math.log10(nn)
    hplus = 10.0 ** (-newpH)
    ph = -1.0 * math.log10(hplus)
    mn, fe = 0.0, 0.0
    if lmetal:
        fe_nat = dust * 35e-3
        fe_ant = X("pFe") * cnv * 1.e+12 * X("AD") / (AIRMW / mw["pFe"]) / X("AIRVOL")
        mn = ((fe_ant / 10.0) + (fe_nat / 50.0)) * 1e-9 / 54.94 / lwc * 1e-3 * 0.5
        fe_d = (fe_ant * 1e-9 / mw["pFe"] / lwc * 1e-3) * 0.1 + (fe_nat * 1e-9 / mw["pFe"] / lwc * 1e-3) * 0.01
        fe = fe_d * (0.1 if X("SUNCOS") > 0.0 else 0.9)
    # AQCHEM_SO2
    ex = lambda a, b: a * math.exp(b * (298.15 / T - 1.0))
    Ks1, Ks2 = ex(1.30e-2, 6.75), ex(6.31e-8, 5.05)
    xso2aq = 1.0 / (1.0 + Ks1 / hplus + Ks1 * Ks2 / (hplus * hplus))
    xhso3 = 1.0 / (1.0 + hplus / Ks1 + Ks2 / hplus)
    xso3 = 1.0 / (1.0 + hplus / Ks2 + hplus * hplus / (Ks1 * Ks2))
    hcso2 = ex(1.22, 10.55)
    fhcso2 = hcso2 * (1.0 + (Ks1 / hplus) + (Ks1 * Ks2 / (hplus * hplus)))
    xso2g = 1.0 / (1.0 + (fhcso2 * RL * T * lwc))
    siv = fhcso2 * xso2g * so2 * patm
    fhch2o2 = ex(7.45e+4, 22.21) * (1.0 + (ex(2.20e-12, -12.52) / hplus))
    xh2o2g = 1.0 / (1.0 + (fhch2o2 * RL * T * lwc))
    kaq_h2o2 = 6.31e+14 * math.exp(-4.76e+3 / T) * Ks1 * fhch2o2 * hcso2 * xh2o2g * xso2g * patm * lwc * RL * T
    hco3 = ex(1.13e-2, 8.51)
    xo3g = 1.0 / (1.0 + (hco3 * RL * T * lwc))
    ko1, ko2 = 3.49e+12 * math.exp(-4.83e+3 / T), 7.32e+14 * math.exp(-4.03e+3 / T)
    kaq_o3 = (2.40e+4 * xso2aq + ko1 * xhso3 + ko2 * xso3) * fhcso2 * xso2g * patm * hco3 * xo3g * lwc * RL * T
    kaq_o2 = fhcso2 * xso2g * ((750.0 * mn) + (2600.0 * fe) + (1e+10 * mn * fe)) * lwc * RL * T
    hchcho = ex(2.5, 21.6)
    xhchog = 1.0 / (1.0 + (hchcho * (1.0 + ex(2.53e+3, 13.48)) * RL * T * lwc))
    kaq_hcho = ((ex(7.9e+2, -16.44) * xhso3 + ex(2.5e+7, -6.04) * xso3) * fhcso2 * xso2g * patm * hchcho * xhchog
                * lwc * RL * T)
    kaq_hms = ex(3.6e+3, -15.09) * (ex(1e-14, -22.51) / hplus) * 0.7
    kaq_hms2 = ex(2.65e+8, -5.03) * 1.0e-19 * 0.7
    kcld = [kaq_h2o2 * fc * cnv, kaq_o3 * fc * cnv, kaq_o2 * fc, kaq_hcho * fc * cnv, kaq_hms * fc,
            kaq_hms2 * fc / C("SO2")]
    size_res = 1 if (not (h2o2 > so2 + 1e-9) and lwc < 0.1e-6) else 0
    return kcld, siv * xhso3, siv * xso3, ph, size_res, count


def _cld_case(n, seed):
    ir, cells, hin = _case(n, seed)
    rng = np.random.default_rng(seed + 11)
    sp = ir["species"]
    lu = lambda lo, hi: np.exp(rng.uniform(np.log(lo), np.log(hi), n))
    for name, lo, hi in (("SO2", 1e7, 1e12), ("H2O2", 1e7, 1e12), ("HCOOH", 1e6, 1e11), ("ACTA", 1e6, 1e11),
                         ("HMS", 1e3, 1e9), ("CH2O", 1e8, 1e12), ("SO4s", 1e2, 1e8), ("HNO3", 1e6, 1e11)):
        cells["c"][sp.index(name)] = lu(lo, hi)
    return ir, cells, hin


@pytest.mark.parametrize("lmetal", [1, 0])
def test_oracle_set_so2_matches_python_restatement(orc, lmetal):
    import gcchem.hetstate as hs

    n = 1024
    ir, cells, hin = _cld_case(n, 31)
    hout, kcld, sr, it = orc.sulfur_cld_rates(hin, cells["c"], lmetal)
    o = hs.HETIN_OFFSET
    cloud = 0
    for j in range(n):
        k, hso3, so3, ph, s_, nit = _py_set_so2(hin[:, j], cells["c"][:, j], ir["species"], lmetal, hs.NONKPP_MW)
        cloud += nit > 0
        assert nit == it[j] and s_ == sr[j], j
        got = [kcld[r, j] for r in range(6)] + [hout[o["HSO3_aq"], j], hout[o["SO3_aq"], j], hout[o["pHCloud"], j]]
        np.testing.assert_allclose(got, k + [hso3, so3, ph], rtol=1e-12, atol=0, err_msg=str(j))
    assert cloud > 100 and sr.sum() > 0 and (sr == 0).sum() > 0, (cloud, sr.sum())
    assert np.all(hout[o["fupdateHOBr"]] == 1.0) and np.all(hout[o["fupdateHOCl"]] == 1.0)
    # the rows SET_SO2 does not write are untouched
    others = [r for r in range(hs.NHETIN)
              if r not in (o["HSO3_aq"], o["SO3_aq"], o["pHCloud"], o["fupdateHOBr"], o["fupdateHOCl"])]
    assert np.array_equal(hout[others], hin[others])


@pytest.mark.gpu
def test_gpu_set_so2_matches_oracle(orc):
    import torch
    import gcchem.capi as capi
    import gcchem.hetstate as hs
    from gcchem.rates_program import MET_FIELDS

    n = 8192
    ir, cells, hin = _cld_case(n, 32)
    hout, kcld, sr, it = orc.sulfur_cld_rates(hin, cells["c"], 1)
    o = hs.HETIN_OFFSET
    k0 = MET_FIELDS.index("K_CLD0")
    s = capi.Solver(0)
    # host memory (numpy) and device memory (torch) give the same bits
    met_h, hin_h = cells["met"].copy(), hin.copy()
    met_h[k0:k0 + 6] = -1.0
    sr_h = np.zeros(n, np.int32)
    s.sulfur_cld_rates(hin_h, cells["c"], met_h, 1, sr_h)
    T = lambda a: torch.tensor(a, device="cuda").contiguous()
    met_d, hin_d, sr_d = T(met_h), T(hin), torch.zeros(n, dtype=torch.int32, device="cuda")
    s.sulfur_cld_rates(hin_d, T(cells["c"]), met_d, 1, sr_d)
    torch.cuda.synchronize()
    assert np.array_equal(met_d.cpu().numpy(), met_h) and np.array_equal(hin_d.cpu().numpy(), hin_h)
    assert np.array_equal(sr_d.cpu().numpy(), sr_h)
    s.close()
    others = [i for i, f in enumerate(MET_FIELDS) if not f.startswith("K_CLD")]
    assert np.array_equal(met_h[others], cells["met"][others])
    got = np.vstack([met_h[k0:k0 + 6], hin_h[[o["HSO3_aq"], o["SO3_aq"], o["pHCloud"]]]])
    ref = np.vstack([kcld, hout[[o["HSO3_aq"], o["SO3_aq"], o["pHCloud"]]]])
    cloud = it > 0
    assert cloud.sum() > 1000
    # CUDA's exp/log10/pow against glibc's: a Newton step whose |dpH| lands
    # within rounding of the 0.01 stopping test may stop one iteration apart
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    same = np.all(rel < 1e-11, axis=0)
    print("SET_SO2 GPU vs oracle: %d cloudy cells, worst %.2e, %d cells off by a Newton step"
          % (cloud.sum(), rel[:, same].max(), (~same).sum()))
    assert (~same).sum() <= 0.005 * n
    assert np.all(np.abs(got[8, ~same] - ref[8, ~same]) <= 0.011)  # pHCloud within one stopping tolerance
    assert np.array_equal(sr_h[same], sr[same])


@pytest.mark.gpu
def test_gpu_sulfur_and_hetstate_producers_drive_a_step(orc):
    """The producers in Do_FullChem's order on the GPU -- SulfurAqChem (K_MT),
    SET_SO2 (K_CLD, cloud pH, HSO3/SO3 into the grid-box rows),
    SetStateHet (HetState from those rows) -- then one chemistry step on
    them; against the oracle's producers in the same order and its loop body
    integrating the GPU's rates."""
    import torch

    import gcchem.capi as capi
    import gcchem.inputs as inputs
    from gcchem.rates_program import MET_FIELDS

    n = 256
    ir, cells, hin = _cld_case(n, 41)
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    c = cells["c"].copy()
    for fam in ir["families"]:
        c[ir["species"].index(fam)] = 0.0
    dev = torch.device("cuda", 0)
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    s = capi.Solver(0, arith="strict", schedule="queue")
    hin_d, c_d, met_d = T(hin), T(c), T(cells["met"])
    het_d = torch.zeros((168, n), dtype=torch.float64, device=dev)
    sr_d = torch.zeros(n, dtype=torch.int32, device=dev)
    s.sulfur_aq_rates(hin_d, c_d, met_d)
    s.sulfur_cld_rates(hin_d, c_d, met_d, 1, sr_d)
    s.set_state_het(hin_d, c_d, het_d, gamma_ho2=0.2, lpscchem=1, turn_off_het_rates=0)
    s.het_drop_chem(600.0, hin_d, c_d, het_d, sr_d, met_d)
    torch.cuda.synchronize()
    # oracle chain
    kmt = orc.sulfur_aq_rates(hin, c, cells["met"][MET_FIELDS.index("TEMP")], cells["met"][MET_FIELDS.index("NUMDEN")])
    hin_o, kcld, sr_o, it = orc.sulfur_cld_rates(hin, c, 1)
    h_ref = orc.set_state_het(hin_o, c, gamma_ho2=0.2, lpscchem=1, turn_off_het_rates=0)
    met_o = cells["met"].copy()
    met_o[6:12], met_o[12:18] = kmt, kcld
    met_o = orc.het_drop_chem(600.0, hin_o, c, h_ref, sr_o, met_o)
    met_g = met_d.cpu().numpy()
    assert np.array_equal(sr_d.cpu().numpy(), sr_o)
    sr_g, sr_ref = met_g[4:6], met_o[4:6]
    assert np.array_equal(sr_g == 0, sr_ref == 0)
    if (sr_ref != 0).any():
        rel = np.abs(sr_g - sr_ref)[sr_ref != 0] / np.abs(sr_ref[sr_ref != 0])
        assert np.median(rel) < 1e-12 and rel.max() < 1e-3
    km, kc = MET_FIELDS.index("K_MT0"), MET_FIELDS.index("K_CLD0")
    assert (it > 0).sum() > 30
    np.testing.assert_allclose(met_g[km:km + 6], kmt, rtol=1e-13, atol=0)
    # cells whose cloud pH agrees (a Newton step may stop one iteration
    # apart where |dpH| is within rounding of 0.01: see the SET_SO2 test)
    import gcchem.hetstate as hs
    ph_g, ph_o = hin_d.cpu().numpy()[hs.HETIN_OFFSET["pHCloud"]], hin_o[hs.HETIN_OFFSET["pHCloud"]]
    ok = np.abs(ph_g - ph_o) <= 1e-10 * np.abs(ph_o)
    assert ok.mean() >= 0.98
    np.testing.assert_allclose(met_g[kc:kc + 6, ok], kcld[:, ok], rtol=1e-10, atol=0)
    np.testing.assert_allclose(het_d.cpu().numpy()[:, ok], h_ref[:, ok], rtol=1e-10, atol=0)
    # one step on the GPU's rates and HetState
    r = np.zeros((len(ir["rconst"]), n))
    s.update_rconst(met_g, cells["photol"], c, r, het=het_d.cpu().numpy())
    assert np.any(r[:, :] != orc.update_rconst(cells["met"], cells["photol"], c, het=h_ref))  # K_MT/K_CLD enter
    c_ref, ist_ref, _, ierr_ref = orc.integrate(c, r, atol, rtol, 0.0, 600.0, ic, rc)
    bad = ierr_ref < 0
    if bad.any():
        c2, ist2, _, ierr2 = orc.integrate(c[:, bad], r[:, bad], atol, rtol, 0.0, 600.0, ic, rc)
        c_ref[:, bad], ist_ref[:, bad], ierr_ref[bad] = c2, ist2, ierr2
    c_ref = np.maximum(c_ref, 0.0)
    s.set_hetstate(het_d)
    cg = T(cells["c"])
    ist = torch.zeros((20, n), dtype=torch.int32, device=dev)
    rst = torch.zeros((20, n), dtype=torch.float64, device=dev)
    ierr = torch.zeros(n, dtype=torch.int32, device=dev)
    s.fullchem_step(600.0, met_d, T(cells["photol"]), cg, T(atol), T(rtol), ic, rc, None, ist, rst, ierr)
    torch.cuda.synchronize()
    s.set_hetstate(None)
    s.close()
    cg, ist, ierr = cg.cpu().numpy(), ist.cpu().numpy(), ierr.cpu().numpy()
    assert np.array_equal(ierr, ierr_ref)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.99
    big = np.abs(c_ref) > 1e4
    rel = np.abs(cg - c_ref) / np.maximum(np.abs(c_ref), 1e-300)
    assert np.max(np.where(big, rel, 0.0)[:, same]) < 1e-9


# ---------------------------------------------------------------------------
# fullchem_HetDropChem (KPP/fullchem/fullchem_SulfurChemFuncs.F90:414-790)
# under Do_FullChem's call conditions (GeosCore/fullchem_mod.F90:913-934).

def _py_het_drop(hin_col, cvec, met_col, up, size_res, dt, sp, mw):
    """One cell: (SRHOCl, SRHOBr), given the four sulfite uptake rates up."""
    import math

    import gcchem.hetstate as hs

    o = hs.HETIN_OFFSET
    X = lambda f: float(hin_col[o[f]])
    C = lambda name: float(cvec[sp.index(name)])
    AIRMW, AVO_ = 28.9644, 6.022140857e+23
    fc, temp = X("CLDF"), float(met_col[0])
    if not fc > 1.0e-4:
        return 0.0, 0.0
    lwc = X("QL") * X("AIRDEN") * 1.0e-3 / fc
    if not (size_res and X("IsWater") != 0.0 and temp > 268.15 and lwc > 1.0e-20):
        return 0.0, 0.0

    def loss(r1, r2, k):
        arg = (r1 - r2) * (k * dt)
        if abs(arg) < 709.0 and abs(arg) > 0.0:
            xx = math.exp(arg)
            return (r1 * r2) * (xx - 1.0) / ((r1 * xx) - r2)
        d = r1 - r2
        return r1 if d < 0 else (r2 if d > 0 else r1 - 1.0 / (k * dt + (1.0 / r1)))

    cvf = 1.0e3 * AIRMW / (X("AIRDEN") * AVO_)
    so2 = C("SO2") * cvf
    xx = [loss(so2, C("H2O2") * cvf, float(met_col[12]) / cvf / fc),
          loss(so2, C("O3") * cvf, float(met_col[13]) / cvf / fc)]
    a3 = (-float(met_col[14]) / fc) * dt
    xx.append(so2 * (1.0 - math.exp(a3)) if abs(a3) < 709.0 else 0.0)
    rh, rs = C("SO2") * cvf * X("HSO3_aq"), C("SO2") * cvf * X("SO3_aq")
    hocl, hobr = C("HOCl") * cvf, C("HOBr") * cvf
    xx.append(loss(rh, hocl, up[0] / cvf) + loss(rs, hocl, up[1] / cvf))
    xx.append(loss(rh, hobr, up[2] / cvf) + loss(rs, hobr, up[3] / cvf))
    lst = xx[0] + xx[1] + xx[2] + xx[3] + xx[4]
    if lst > rs:
        xx = [(rs * v) / lst for v in xx]
        lst = xx[0] + xx[1] + xx[2] + xx[3] + xx[4]
    vpp = lambda v: v * 1.0e12
    nh3, so2p = vpp(X("NH3") * cvf), max(C("SO2") * cvf - (lst * fc), 1.0e-20) * 1.0e+12
    h2o2, hno3 = vpp(C("H2O2") * cvf), vpp(C("HNO3") * cvf)
    ad, vol, rho = X("AD"), X("AIRVOL"), X("AIRDEN")
    so4 = (C("SO4") * cvf * ad * 1.0e+9) / ((AIRMW / mw["SO4"]) * vol)
    b = (lst * ad * 1.0e+9) / ((AIRMW / mw["SO4"]) * vol)
    cnss = X("SALC") * cvf * ad / ((AIRMW / mw["SALC"]) * vol)
    rg3 = float.fromhex("0x1.2e3b40a0e9b4fp-64")  # (0.4e-6)**3 rounded once
    arg = 4.5 * (math.log(1.8) * math.log(1.8))
    cn = (0.75 * cnss) / (3.14159265358979323 * 2200.0 * rg3 * math.exp(arg)) * 1.e-6
    table = [(200.0, (0.5318, -1.67e-7, 2.59e-6, -1.77e-7, -1.72e-7, 1.22e-6, 4.58e-6, -1.00e-5)),
             (500.0, (0.5591, 3.62e-6, 1.66e-6, 1.06e-7, -5.45e-7, -5.79e-7, 1.63e-5, -7.40e-6)),
             (999.0, (1.1547, -4.28e-8, -1.23e-7, -9.05e-7, 1.73e-7, 7.22e-6, 2.44e-5, 3.25e-5))]
    al = (1.1795, 2.57e-7, -5.54e-7, -1.08e-6, 1.95e-6, 6.14e-6, 1.64e-5, 2.48e-6)
    for hi, coef in table:
        if so2p <= hi or (hi == 999.0 and so2p < 1000.0):
            al = coef
            break
    aB, aNH3, aSO2, aH2O2, aHNO3, aW, aCN, aSO4 = al
    w = -X("OMEGA") / (rho * 9.80665) * 100.0
    h = dt * (math.sqrt(X("U") * X("U") + X("V") * X("V")) + (w * w * 1.0e-4))
    dsvi = (aB * b) + (((aCN * cn) + (aW * w) + (aSO4 * so4)
                        + ((aNH3 * nh3) + (aSO2 * so2p) + (aH2O2 * h2o2) + (aHNO3 * hno3))) * h)
    sr = 0.0
    if w > 0.0 and C("SO2") > 0.0:
        sr = max(dsvi - b, 0.0)
        if sr > 0.0:
            sr = min(sr * (AIRMW / mw["SO4"]) * 1.e-9 / rho, so2p / 1.0e12)
    sr = sr / cvf / dt
    denom = xx[1] + xx[3] + xx[4]
    sdiv = lambda a, d: 0.0 if d == 0.0 else a / d
    return (sdiv(sr * sdiv(xx[3], denom), C("SO2") * C("HOCl")), sdiv(sr * sdiv(xx[4], denom), C("SO2") * C("HOBr")))


def _drop_case(n, seed):
    """Grid-box rows after SET_SO2 and SetStateHet, with clouds thin enough
    for size_res and warm enough, ascending and descending air."""
    import gcchem.hetstate as hs
    from gcchem.rates_program import MET_FIELDS

    ir, cells, hin = _cld_case(n, seed)
    rng = np.random.default_rng(seed + 3)
    o = hs.HETIN_OFFSET
    sp = ir["species"]
    hin[o["QL"]] = np.exp(rng.uniform(np.log(1e-9), np.log(1e-5), n))
    hin[o["T"]] = np.where(hin[o["CLDF"]] > 0, rng.uniform(262.0, 300.0, n), hin[o["T"]])
    hin[o["IsWater"]] = (rng.uniform(size=n) < 0.9).astype(float)
    hin[o["OMEGA"]] = np.abs(hin[o["OMEGA"]]) * np.where(rng.uniform(size=n) < 0.85, -1.0, 1.0)
    cells["met"][MET_FIELDS.index("TEMP")] = np.maximum(cells["met"][MET_FIELDS.index("TEMP")], hin[o["T"]])
    for name in ("HOCl", "HOBr"):
        cells["c"][sp.index(name)] = np.exp(rng.uniform(np.log(1e4), np.log(1e9), n))
    return ir, cells, hin


def test_oracle_het_drop_matches_python_restatement(orc):
    import gcchem.hetstate as hs

    n = 2048
    ir, cells, hin = _drop_case(n, 51)
    hin2, kcld, sr, _ = orc.sulfur_cld_rates(hin, cells["c"], 1)
    met = cells["met"].copy()
    met[12:18] = kcld
    het = orc.set_state_het(hin2, cells["c"])
    up = orc.sulfite_uptakes(met, cells["c"], het)
    out = orc.het_drop_chem(1200.0, hin2, cells["c"], het, sr, met)
    called = 0
    for j in range(n):
        a, b = _py_het_drop(hin2[:, j], cells["c"][:, j], met[:, j], up[:, j], sr[j], 1200.0, ir["species"],
                            hs.NONKPP_MW)
        called += a > 0 or b > 0
        np.testing.assert_allclose([out[4, j], out[5, j]], [a, b], rtol=1e-12, atol=0, err_msg=str(j))
    assert called > 20, called
    others = [r for r in range(18) if r not in (4, 5)]
    assert np.array_equal(out[others], met[others])


@pytest.mark.gpu
def test_gpu_het_drop_matches_oracle(orc):
    import torch
    import gcchem.capi as capi

    n = 8192
    ir, cells, hin = _drop_case(n, 52)
    hin2, kcld, sr, _ = orc.sulfur_cld_rates(hin, cells["c"], 1)
    met = cells["met"].copy()
    met[12:18] = kcld
    het = orc.set_state_het(hin2, cells["c"])
    ref = orc.het_drop_chem(1200.0, hin2, cells["c"], het, sr, met)
    s = capi.Solver(0)
    met_h = met.copy()
    s.het_drop_chem(1200.0, hin2, cells["c"], het, sr, met_h)
    T = lambda a: torch.tensor(a, device="cuda").contiguous()
    met_d = T(met)
    s.het_drop_chem(1200.0, T(hin2), T(cells["c"]), T(het), T(sr), met_d)
    torch.cuda.synchronize()
    s.close()
    assert np.array_equal(met_d.cpu().numpy(), met_h)
    others = [r for r in range(18) if r not in (4, 5)]
    assert np.array_equal(met_h[others], met[others])
    got, want = met_h[4:6], ref[4:6]
    assert np.array_equal(got == 0, want == 0)
    nz = want != 0
    assert nz.sum() > 100, nz.sum()
    rel = np.abs(got[nz] - want[nz]) / np.abs(want[nz])
    print("HetDropChem GPU vs oracle: %d nonzero rates, median %.1e, max %.1e" % (nz.sum(), np.median(rel), rel.max()))
    # the sulfite uptake laws go through CloudHet, whose few-ulp libm
    # differences the oracle's own conditioning amplifies on a few cells
    assert np.median(rel) < 1e-13 and np.mean(rel < 1e-9) >= 0.99 and rel.max() < 1e-3
