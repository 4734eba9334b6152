"""Heterogeneous rates of Update_RCONST with a real HetState
(gc_kpp_update_rconst_het_batch): the GPU rate laws of csrc/het_rates.cuh
against the oracle's restatement (oracle/het_laws.h) of
KPP/fullchem/fullchem_RateLawFuncs.F90:795-3460, on seeded synthetic
HetStates; plus the interface tables and a few laws recomputed here from
their Fortran formulas."""
import math
import os
import re
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "geos-chem_gb300", "csrc")


def test_het_layout_header_matches_field_list():
    import gcchem.hetstate as hs

    with open(os.path.join(CSRC, "het_layout.h")) as fh:
        assert fh.read() == hs.emit_c()
    assert hs.NFIELD == 168
    with open(os.path.join(ROOT, "include", "gckpp_gb300.h")) as fh:
        assert "#define GC_KPP_NHET %d" % hs.NFIELD in fh.read()


def test_het_law_tables_agree():
    """rates_program.HET_LAWS is the het_law switch of het_rates.cuh, its
    HET_SPECIES the HetSpc enum, and the oracle generator knows every law."""
    import gcchem.rates_program as rp

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import gen_oracle

    src = open(os.path.join(CSRC, "het_rates.cuh")).read()
    cases = re.findall(r"case (\d+): return .*;  // (\w+)", src)
    assert [(int(i), n) for i, n in cases] == [(i, n) for i, (n, _) in enumerate(rp.HET_LAWS)]
    enum = re.search(r"enum HetSpc : int \{([^}]*)\}", src).group(1)
    names = [x.strip().split("=")[0].strip()[3:] for x in enum.split(",") if x.strip()]
    assert names[:-1] == rp.HET_SPECIES and names[-1] == "N"
    assert rp.HET_SPECIES == gen_oracle.HET_SPECIES
    assert {n: k for n, k in rp.HET_LAWS} == gen_oracle.HET_FUNCS
    # every heterogeneous call of the fullchem Update_RCONST is one of them
    from gcchem.mechanism import load_ir

    calls = set()
    for e in load_ir()["rconst"]:
        calls |= {m for m in re.findall(r"([A-Za-z_]\w*)\(", e) if "(H)" in e or ",H)" in e}
    het_calls = {c for c in calls if c not in {n for n, _ in rp.LAWS} and c not in ("exp", "log10")}
    assert het_calls <= set(gen_oracle.HET_FUNCS)
    assert len(het_calls) == 60


def test_species_database_constants():
    from gcchem.mechanism import species_db

    d = species_db.load("fullchem")
    i = d["species"].index
    assert d["mw"][i("BrNO3")] == 141.91 and d["mw"][i("NO")] == 30.01
    assert d["henry_k0"][i("HOBr")] == 1300.0 and d["henry_cr"][i("HOCl")] == 5900.0
    assert all(m > 0 for m in d["mw"])


def _oracle_rates(n, seed):
    import gcchem.hetstate as hs
    import gcchem.inputs as inputs
    import oracle

    cells = inputs.box_cells(n, seed=seed)
    h = hs.het_cells(n, seed=seed + 100)
    r = oracle.update_rconst(cells["met"], cells["photol"], cells["c"], het=h)
    r0 = oracle.update_rconst(cells["met"], cells["photol"], cells["c"])
    return cells, h, r, r0


def test_oracle_het_rates_are_finite_and_switch_on():
    from gcchem.mechanism import load_ir

    ir = load_ir()
    cells, h, r, r0 = _oracle_rates(256, 1)
    het_rows = [i for i, e in enumerate(ir["rconst"]) if "H)" in e]
    other = np.setdiff1d(np.arange(len(ir["rconst"])), het_rows)
    assert np.array_equal(r[other], r0[other])  # gas-phase rates do not see the HetState
    assert np.all(np.isfinite(r)) and np.all(r[het_rows] >= 0.0)
    assert np.all(r0[het_rows] == 0.0)
    on = (r[het_rows] > 0).mean(axis=1)
    assert (on > 0).mean() > 0.9  # nearly every heterogeneous reaction is active somewhere


def test_oracle_laws_against_fortran_formulas():
    """A few laws recomputed here from the Fortran text (Ars_L1k,
    kIIR1Ltd without its minimum-lifetime clamp, HBrUptkBySALA,
    VOCuptk1stOrd, MGLYuptk1stOrd)."""
    import gcchem.hetstate as hs
    from gcchem.mechanism import load_ir, species_db

    ir = load_ir()
    cells, h, r, _ = _oracle_rates(64, 2)
    sp = species_db.load("fullchem")
    T = cells["met"][0]
    nd = cells["met"][1]
    h2o = cells["met"][2]
    o = hs.OFFSET
    srt = np.sqrt(T)

    def ars(area, radius, gamma, srmw):
        dfkg = (9.45e17 / nd) * srt * math.sqrt(3.472e-2 + 1.0 / (srmw * srmw))
        k = area / ((radius / dfkg) + 2.749064e-4 * srmw / (gamma * srt))
        return np.where((gamma < 1e-30) | (radius < 1e-30), 0.0, k)

    def row(expr):
        return ir["rconst"].index(expr)

    strat = h[o["stratBox"]] != 0
    srmw_hbr = math.sqrt(sp["mw"][sp["species"].index("HBr")])
    area = h[o["clearFr"]] * h[o["aClArea"]]
    ref = np.where(strat, 0.0, ars(area, h[o["aClRadi"]], 1.3e-8 * np.exp(4290.0 / T), srmw_hbr))
    got = r[[i for i, e in enumerate(ir["rconst"]) if e == "(HBrUptkBySALA(H))"][0]]
    assert np.allclose(got, ref, rtol=1e-13, atol=0)
    # RELHUM of Set_Kpp_GridBox_Values
    consvap = 6.1078e3 / (1.38064852e-23 * 1e7)
    relhum = h2o / (consvap * np.exp(17.2693882 * (T - 273.16) / (T - 35.86)) / T) * 100.0
    for i, e in enumerate(ir["rconst"]):
        m = re.fullmatch(r"\(VOCuptk1stOrd\(SR_MW\[(\d+)\],([0-9.eE+-]+),H\)\)", e)
        if m:
            srmw = math.sqrt(sp["mw"][int(m.group(1))])
            g = float(m.group(2))
            k = sum(ars(h[o["xArea"] + t - 1], h[o["xRadi"] + t - 1], g, srmw) for t in (8, 9, 10, 11, 12, 13, 14))
            assert np.allclose(r[i], np.where(relhum >= 35.0, k, 0.0), rtol=1e-12, atol=0), e
        m = re.fullmatch(r"\(MGLYuptk1stOrd\(SR_MW\[(\d+)\],H\)\)", e)
        if m:
            srmw = math.sqrt(sp["mw"][int(m.group(1))])
            k = ars(h[o["xArea"] + 7], h[o["xRadi"] + 7], 3.6e-7, srmw)
            assert np.allclose(r[i], np.where(relhum >= 35.0, k, 0.0), rtol=1e-13, atol=0), e


def _het_calls(ir):
    """(rconst row, law id, numeric arguments) of every heterogeneous call; a
    concentration argument C(i) is encoded as -1-i."""
    import gcchem.rates_program as rp
    from gcchem.mechanism import species_db

    sp = species_db.load(ir.get("mechanism", "fullchem"))
    out = []
    for i, e in enumerate(ir["rconst"]):
        for m in re.finditer(r"(\w+)\(([^()]*)\)", e):
            if m.group(1) not in rp.HET_ID:
                continue
            vals = []
            for a in m.group(2).split(",")[:-1]:
                mm = re.fullmatch(r"SR_MW\[(\d+)\]", a)
                mc = re.fullmatch(r"C\[(\d+)\]", a)
                vals.append(math.sqrt(sp["mw"][int(mm.group(1))]) if mm else
                            -1.0 - int(mc.group(1)) if mc else float(a))
            out.append((i, rp.HET_ID[m.group(1)][0], vals + [0.0] * (3 - len(vals))))
    return out


def test_gpu_laws_equal_oracle_on_the_same_libm(tmp_path):
    """The GPU laws of csrc/het_rates.cuh, built for the host (g++, glibc's
    math), give the oracle's rates bit for bit: the two restatements perform
    the same arithmetic, so every GPU/oracle difference comes from CUDA's
    libm (checked on the GPU below)."""
    import shutil
    import subprocess

    import gcchem.rates_program as rp
    from gcchem.mechanism import load_ir

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    ir = load_ir()
    n = 1024
    cells, h, r_ref, _ = _oracle_rates(n, 3)
    prog = rp.build_program(ir)
    (tmp_path / "fake").mkdir()
    (tmp_path / "fake" / "cuda_runtime.h").write_text("#pragma once\n")
    exe = str(tmp_path / "harness")
    subprocess.check_call([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(tmp_path / "fake"), "-I", CSRC,
                           os.path.join(ROOT, "tests", "host", "het_laws_host.cpp"), "-o", exe])
    for name, arr in (("met", cells["met"]), ("c", cells["c"]), ("het", h)):
        np.ascontiguousarray(arr, np.float64).tofile(str(tmp_path / (name + ".bin")))
    for name, key in (("hsind", "hs_ind"), ("hsmw", "hs_mw"), ("hssr", "hs_srmw"), ("hsk0", "hs_hk0"),
                      ("hscr", "hs_hcr")):
        np.array(prog[key], np.float64).tofile(str(tmp_path / (name + ".bin")))
    calls = _het_calls(ir)
    np.array([[k] + v for _, k, v in calls], np.float64).tofile(str(tmp_path / "calls.bin"))
    subprocess.check_call([exe, str(n), str(len(ir["species"])), str(len(calls))], cwd=str(tmp_path))
    out = np.fromfile(str(tmp_path / "out.bin")).reshape(len(calls), n)
    met = cells["met"]
    for k, (i, _, _) in enumerate(calls):
        e = ir["rconst"][i]
        if "+" in e:  # (HOClUptkByHSO3m(H)+HOClUptkBySO3mm(H)+SRHOCl): check the sum
            ks = [q for q, c in enumerate(calls) if c[0] == i]
            if k != ks[0]:
                continue
            extra = met[4] if "SRHOCl" in e else met[5]
            got = out[ks[0]] + out[ks[1]] + extra
        else:
            got = out[k]
        assert np.array_equal(got, r_ref[i]), e


def _ulp_sensitivity(cells, h, r_ref):
    """How much the oracle's rates move when TEMP or NUMDEN move by a few
    ulp (the largest of three such changes): the conditioning of the
    reference's formulas at each cell."""
    import oracle

    out = np.zeros_like(r_ref)
    for row, fac in ((0, 1.0 + 4.4e-16), (0, 1.0 - 4.4e-16), (1, 1.0 + 4.4e-16)):
        met = cells["met"].copy()
        met[row] *= fac
        r2 = oracle.update_rconst(met, cells["photol"], cells["c"], het=h)
        out = np.maximum(out, np.abs(r2 - r_ref) / np.maximum(np.abs(r_ref), 1e-300))
    return out


@pytest.mark.gpu
def test_gpu_het_rates_match_oracle():
    import gcchem.capi as capi

    n = 4096
    cells, h, r_ref, _ = _oracle_rates(n, 3)
    s = capi.Solver(0, arith="fast")
    r = np.zeros_like(r_ref)
    s.update_rconst(cells["met"], cells["photol"], cells["c"], r, het=h)
    assert np.array_equal(r == 0, r_ref == 0)
    rel = np.abs(r - r_ref) / np.maximum(np.abs(r_ref), 1e-300)
    # CUDA's exp/log10/pow differ from glibc's in the last bit (the host
    # build of these laws equals the oracle bit for bit, test above).  A few
    # rates are ill-conditioned in the reference's own formulas (CloudHet's
    # (ff-kk-1)/2 + sqrt(...)/2 cancels when kk >> ff), where those bits grow
    # to ~1e-3: the GPU's spread must stay within what a few-ulp change of
    # TEMP or NUMDEN does to the oracle itself.
    sens = _ulp_sensitivity(cells, h, r_ref)
    for thr in (1e-12, 1e-9, 1e-6):
        assert (rel > thr).mean() <= 3.0 * (sens > thr).mean() + 1e-5, (thr, (rel > thr).mean(), (sens > thr).mean())
    assert rel.max() <= 10.0 * sens.max() + 1e-9, (rel.max(), sens.max())
    # NULL HetState: the heterogeneous rates are 0, the rest unchanged
    r0 = np.zeros_like(r_ref)
    s.update_rconst(cells["met"], cells["photol"], cells["c"], r0)
    from gcchem.mechanism import load_ir

    het_rows = [i for i, e in enumerate(load_ir()["rconst"]) if "H)" in e]
    assert np.all(r0[het_rows] == 0.0)
    other = np.setdiff1d(np.arange(r.shape[0]), het_rows)
    assert np.array_equal(r0[other], r[other])
    s.close()


@pytest.mark.gpu
def test_gpu_step_with_het_rates_matches_oracle():
    """Integration with the heterogeneous rates switched on: GPU (fast
    arithmetic) against the oracle at the parity bar of the gas-phase case."""
    import gcchem.capi as capi
    import gcchem.inputs as inputs
    import oracle

    n = 256
    cells, h, r_ref, _ = _oracle_rates(n, 4)
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    s = capi.Solver(0, arith="fast", schedule="queue")
    r = np.zeros_like(r_ref)
    s.update_rconst(cells["met"], cells["photol"], cells["c"], r, het=h)
    # the same rates on both sides (the rates' own parity is the test above)
    c_ref, ist_ref, _, ierr_ref = oracle.integrate(cells["c"], r, atol, rtol, 0.0, 600.0, ic, rc)
    c = cells["c"].copy()
    ist = np.zeros((20, n), np.int32)
    ierr = np.zeros(n, np.int32)
    s.integrate(c, r, atol, rtol, 0.0, 600.0, ic, rc, istatus=ist, ierr=ierr)
    assert np.array_equal(ierr, ierr_ref)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.97
    big = np.abs(c_ref[:353]) > 1e4
    rel = np.abs(c[:353] - c_ref[:353]) / np.maximum(np.abs(c_ref[:353]), 1e-300)
    assert np.max(np.where(big, rel, 0.0)[:, same]) < 1e-8
    s.close()


@pytest.mark.gpu
def test_gpu_chemistry_step_with_hetstate_matches_oracle():
    """gc_kpp_ctx_set_hetstate: the one-call chemistry step (family zeroing,
    rates with the HetState, integration, retry, clamp) against the oracle's
    Do_FullChem loop body with the same heterogeneous rates (strict
    arithmetic: the parity bar of the gas-phase step)."""
    import gcchem.capi as capi
    import gcchem.hetstate as hs
    import gcchem.inputs as inputs
    import oracle
    from gcchem.mechanism import load_ir

    ir = load_ir()
    n = 192
    cells = inputs.box_cells(n, seed=21)
    h = hs.het_cells(n, seed=22)
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    c = cells["c"].copy()
    for fam in ir["families"]:
        c[ir["species"].index(fam)] = 0.0
    s = capi.Solver(0, arith="strict", schedule="queue")
    # the step's rates are the GPU's (compared with the oracle's above); the
    # oracle integrates with the same rates
    r = np.zeros((len(ir["rconst"]), n))
    s.update_rconst(cells["met"], cells["photol"], c, r, het=h)
    r_o = oracle.update_rconst(cells["met"], cells["photol"], c, het=h)
    assert np.allclose(r, r_o, rtol=1e-2, atol=0)
    c_ref, ist_ref, _, ierr_ref = oracle.integrate(c, r, atol, rtol, 0.0, 600.0, ic, rc)
    bad = ierr_ref < 0
    if bad.any():
        c2, ist2, _, ierr2 = oracle.integrate(c[:, bad], r[:, bad], atol, rtol, 0.0, 600.0, ic, rc)
        c_ref[:, bad], ist_ref[:, bad], ierr_ref[bad] = c2, ist2, ierr2
    c_ref = np.maximum(c_ref, 0.0)

    s.set_hetstate(h)
    cg = cells["c"].copy()
    ist = np.zeros((20, n), np.int32)
    rst = np.zeros((20, n))
    ierr = np.zeros(n, np.int32)
    s.fullchem_step(600.0, cells["met"], cells["photol"], cg, atol, rtol, ic, rc, None, ist, rst, ierr)
    assert np.array_equal(ierr, ierr_ref)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.99
    big = np.abs(c_ref) > 1e4
    rel = np.abs(cg - c_ref) / np.maximum(np.abs(c_ref), 1e-300)
    assert np.max(np.where(big, rel, 0.0)[:, same]) < 1e-9
    # a step over another number of cells is refused while the HetState is set
    with pytest.raises(capi.GcKppError):
        s.fullchem_step(600.0, cells["met"][:, :8].copy(), cells["photol"][:, :8].copy(), cg[:, :8].copy(),
                        atol, rtol, ic, rc)
    s.set_hetstate(None)
    s.close()


@pytest.mark.gpu
def test_direct_rates_kernel_equals_interpreter():
    """GC_KPP_OPT_RATES_DIRECT: the generated straight-line Update_RCONST
    gives the rate-program interpreter's results to rounding, with and
    without a HetState: the same operations in the same order, but the
    literal constants of the straight-line code let the compiler specialise
    some libm calls (a power or exponential of a known argument), which moves
    the last bit of a few rates; the parity bar against the oracle (1e-13
    relative) holds for both."""
    import gcchem.capi as capi

    n = 2048
    cells, h, _, _ = _oracle_rates(n, 5)
    s = capi.Solver(0, arith="fast")
    out = {}
    for direct in (False, True):
        s.set(rates_direct=direct)
        for het in (None, h):
            r = np.zeros((1058, n))
            s.update_rconst(cells["met"], cells["photol"], cells["c"], r, het=het)
            out[(direct, het is None)] = r
    for key in (True, False):
        a, b = out[(True, key)], out[(False, key)]
        assert np.array_equal(a == 0, b == 0)
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
        assert np.max(rel) <= 1e-13, np.max(rel)
    s.close()
