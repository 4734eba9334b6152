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
    assert hs.NHETIN == 100


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
