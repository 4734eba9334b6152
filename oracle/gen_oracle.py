"""Generate the oracle's mechanism C code from the mechanism IR.

TEST INFRASTRUCTURE (the CPU oracle).  Emits ``_gen/kpp_mech_oracle.c``: one
C statement per statement of the KPP-generated Fortran, in the same order and
with the same infix evaluation order, so that compiled with
``-ffp-contract=off`` it performs the reference's arithmetic exactly:

* oracle_fun_split   KPP/fullchem/gckpp_Function.F90:2172-5059 (Fun_SPLIT)
* oracle_jac_sp      KPP/fullchem/gckpp_Jacobian.F90:48-20887 (Jac_SP)
* oracle_kpp_solve   KPP/fullchem/gckpp_LinearAlgebra.F90:644-2309 (KppSolve)
* LU_CROW/LU_DIAG/LU_ICOL tables for oracle_kpp_decomp
  (KPP/fullchem/gckpp_JacobianSP.F90:525-1093)

Literals are written as C hexadecimal floats, i.e. the correctly rounded
double of the Fortran literal (the reference compiles with
-fdefault-real-8, KPP/fullchem/CMakeLists.txt:88-92).

This generator is deliberately independent of the product's table lowering
(gcchem.tables): it reads the IR JSON directly.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
MECH_DIR = os.path.join(HERE, "..", "geos-chem_gb300", "mechanism")


def _ir(mech):
    with open(os.path.join(MECH_DIR, mech + ".json")) as fh:
        return json.load(fh)


def _lit(tok):
    return float(tok.replace("d", "e").replace("D", "e")).hex()


def _fac(tok):
    m = re.fullmatch(r"([RVFAB])(\d+)", tok)
    if m:
        name = {"R": "RCT", "V": "V", "F": "F", "A": "A", "B": "B"}[m.group(1)]
        return "%s[%s]" % (name, m.group(2))
    return _lit(tok)


def _prod(toks):
    # an empty product is a reaction KPP leaves uncomputed (never referenced)
    return "*".join(_fac(t) for t in toks) if toks else "0.0"


def _signed(terms, render):
    if not terms:
        return "0.0"
    out = ""
    for k, (sign, payload) in enumerate(terms):
        body = render(payload)
        if k == 0:
            out += ("-" if sign == "-" else "") + body
        else:
            out += " %s %s" % (sign, body)
    return out


def _coef_ref(arr):
    def r(p):
        coef, idx = p
        return ("%s*" % _lit(coef) if coef is not None else "") + "%s[%d]" % (arr, idx)
    return r


def generate(ir):
    d = ir["dims"]
    nvar, nreact, lunz = d["nvar"], d["nreact"], d["lu_nonzero"]
    nb = len(ir["jac"]["B"])
    L = ["/* Generated by oracle/gen_oracle.py from the mechanism IR. Do not edit. */",
         "#include \"kpp_oracle.h\"",
         ""]
    lu = ir["lu"]
    for name in ("crow", "diag", "icol", "irow"):
        vals = lu[name]
        L.append("const int ORACLE_LU_%s[%d] = {%s};" % (name.upper(), len(vals), ",".join(map(str, vals))))
    L.append("")
    L.append("void oracle_fun_split(const double* V, const double* F, const double* RCT, double* Vdot) {")
    L.append("  double A[%d], P_VAR[%d], D_VAR[%d];" % (nreact, nvar, nvar))
    for r, f in enumerate(ir["fun"]["A"]):
        L.append("  A[%d] = %s;" % (r, _prod(f)))
    for i, terms in enumerate(ir["fun"]["P"]):
        L.append("  P_VAR[%d] = %s;" % (i, _signed([(s, (c, a)) for s, c, a in terms], _coef_ref("A"))))
    for i, terms in enumerate(ir["fun"]["D"]):
        L.append("  D_VAR[%d] = %s;" % (i, _signed([(s, f) for s, f in terms], _prod)))
    L.append("  for (int i = 0; i < %d; ++i) Vdot[i] = P_VAR[i] - D_VAR[i]*V[i];" % nvar)
    L.append("}")
    L.append("")
    # Fun_SPLITF (gckpp_Function.F90:5081-7260) has the same A, P_VAR and D_VAR
    # statements as Fun_SPLIT and returns P_VAR and D_VAR themselves
    L.append("void oracle_fun_pd(const double* V, const double* F, const double* RCT, double* P, double* D) {")
    L.append("  double A[%d];" % nreact)
    for r, f in enumerate(ir["fun"]["A"]):
        L.append("  A[%d] = %s;" % (r, _prod(f)))
    for i, terms in enumerate(ir["fun"]["P"]):
        L.append("  P[%d] = %s;" % (i, _signed([(s_, (c, a_)) for s_, c, a_ in terms], _coef_ref("A"))))
    for i, terms in enumerate(ir["fun"]["D"]):
        L.append("  D[%d] = %s;" % (i, _signed([(s_, f) for s_, f in terms], _prod)))
    L.append("}")
    L.append("")
    L.append("void oracle_jac_sp(const double* V, const double* F, const double* RCT, double* JVS) {")
    L.append("  double B[%d];" % nb)
    for b, f in enumerate(ir["jac"]["B"]):
        if f is not None:
            L.append("  B[%d] = %s;" % (b, _prod(f)))
    for k, terms in enumerate(ir["jac"]["JVS"]):
        L.append("  JVS[%d] = %s;" % (k, _signed([(s, (c, b)) for s, c, b in terms], _coef_ref("B"))))
    L.append("}")
    L.append("")
    for name, guarded in (("oracle_kpp_solve", False), ("oracle_kpp_solve_slv", True)):
        # the guarded form is KppSolve's IF (DO_SLV(i)) statements
        # (gckpp_LinearAlgebra.F90:644-2309) under auto-reduction
        L.append("void %s(const double* JVS, double* X%s) {" % (name, ", const unsigned char* DO_SLV" if guarded else ""))
        for st in ir["solve"]:
            i = st["row"]
            e = "X[%d]" % i + "".join(" - JVS[%d]*X[%d]" % (k, j) for k, j in st["terms"])
            if st["kind"] == "B":
                e = "(%s)/(JVS[%d])" % (e, st["diag"]) if st["terms"] else "X[%d]/JVS[%d]" % (i, st["diag"])
            L.append("  %sX[%d] = %s;" % ("if (DO_SLV[%d]) " % i if guarded else "", i, e))
        L.append("}")
        L.append("")
    return "\n".join(L) + "\n", {"nvar": nvar, "nreact": nreact, "lu_nonzero": lunz, "nb": nb,
                                 "nspec": d["nspec"], "nfix": d["nfix"]}


def write(outdir, mech="fullchem"):
    ir = _ir(mech)
    text, dims = generate(ir)
    os.makedirs(outdir, exist_ok=True)
    path = os.path.join(outdir, "kpp_mech_oracle.c")
    old = open(path).read() if os.path.exists(path) else None
    if old != text:
        with open(path, "w") as fh:
            fh.write(text)
    hdr = os.path.join(outdir, "kpp_dims.h")
    htxt = "".join("#define ORACLE_%s %d\n" % (k.upper(), v) for k, v in sorted(dims.items()))
    old = open(hdr).read() if os.path.exists(hdr) else None
    if old != htxt:
        with open(hdr, "w") as fh:
            fh.write(htxt)
    write_rates(outdir, mech)
    return path



# --- Update_RCONST -----------------------------------------------------------

GAS_LAWS = {
    "GCARR_ab", "GCARR_ac", "GCARR_abc", "ARRPLUS_ade", "ARRPLUS_abde", "TUNPLUS_abcde", "GC_ISO1", "GC_ISO2",
    "GC_EPO_a", "GC_PAN_abab", "GC_PAN_acac", "GC_NIT", "GC_ALK", "GC_HO2HO2_acac", "GC_TBRANCH_1_acac",
    "GC_RO2HO2_aca", "GC_DMSOH_acac", "GC_GLYXNO3_ac", "GC_GLYCOH_A_a", "GC_GLYCOH_B_a", "GC_HACOH_A_ac",
    "GC_HACOH_B_ac", "GC_RO2NO_A1_ac", "GC_RO2NO_B1_ac", "GC_RO2NO_A2_aca", "GC_RO2NO_B2_aca", "GCJPLEQ_acabab",
    "GCJPLPR_aa", "GCJPLPR_aba", "GCJPLPR_abab", "GCJPLPR_abcabc", "GCJPLAC_ababac",
}

# per-cell meteorology/state fields of the rate evaluation (cell-interleaved)
MET_FIELDS = ["TEMP", "NUMDEN", "H2O", "PRESS", "SRHOCl", "SRHOBr"] + \
    ["K_MT%d" % i for i in range(6)] + ["K_CLD%d" % i for i in range(6)]


# heterogeneous rate functions restated in het_laws.h (o_<name>), with the
# number of numeric arguments before the HetState argument H
HET_FUNCS = {
    "IuptkBySulf1stOrd": 2, "IuptkBySALA1stOrd": 2, "IuptkByAlkSALA1stOrd": 2, "IuptkBySALC1stOrd": 2,
    "IuptkByAlkSALC1stOrd": 2, "IbrkdnByAcidBrSALA": 3, "IbrkdnByAcidBrSALC": 3, "IbrkdnByAcidSALACl": 3,
    "IbrkdnByAcidSALCCl": 3, "GLYXuptk1stOrd": 1, "IEPOXuptk1stOrd": 2, "MGLYuptk1stOrd": 1, "VOCuptk1stOrd": 2,
}
for _n in ("BrNO3uptkByH2O BrNO3uptkByHCl ClNO2uptkByBrSALA ClNO2uptkByBrSALC ClNO2uptkByHBr ClNO2uptkBySALACL "
           "ClNO2uptkBySALCCL ClNO2uptkByHCl ClNO3uptkByH2O ClNO3uptkByHCl ClNO3uptkByHBr ClNO3uptkByBrSALA "
           "ClNO3uptkByBrSALC ClNO3uptkBySALACL ClNO3uptkBySALCCL HBrUptkBySALA HBrUptkBySALC HO2uptk1stOrd "
           "HOBrUptkByHBr HOBrUptkByHCl HOBrUptkByBrSALA HOBrUptkByBrSALC HOBrUptkBySALACL HOBrUptkBySALCCL "
           "HOBrUptkByHSO3m HOBrUptkBySO3mm HOClUptkByHCl HOClUptkByHBr HOClUptkBySALACL HOClUptkBySALCCL "
           "HOClUptkByHSO3m HOClUptkBySO3mm IONO2uptkByH2O N2O5uptkByH2O N2O5uptkBySALACl N2O5uptkBySALCCl "
           "N2O5uptkByCloud N2O5uptkByStratHCl NO2uptk1stOrdAndCloud NO3uptk1stOrdAndCloud NO3hypsisClonSALA "
           "NO3hypsisClonSALC O3uptkByHBr O3uptkByBrSALA O3uptkByBrSALC OHuptkBySALACl OHuptkBySALCCl").split():
    HET_FUNCS[_n] = 0
HET_SPECIES = ["BrNO3", "H2O", "HCl", "ClNO2", "BrSALA", "BrSALC", "HBr", "SALACL", "SALCCL", "ClNO3", "HOBr",
               "SO2", "HOCl", "HO2", "IONO2", "N2O5", "NIT", "NITs", "NO2", "NO3", "O3", "OH"]


def _split_args(text):
    out, depth, cur = [], 0, ""
    for ch in text:
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
            continue
        depth += ch == "("
        depth -= ch == ")"
        cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _rate_c(expr, het_calls, het_laws=False):
    """Rate expression (C-like IR text) -> oracle C text."""
    out = ""
    i = 0
    while i < len(expr):
        m = re.match(r"[A-Za-z_][A-Za-z_0-9]*", expr[i:])
        if m and not re.match(r"\d", expr[i - 1:i] or " "):
            name = m.group(0)
            j = i + len(name)
            if j < len(expr) and expr[j] == "(" and name not in ("exp", "log10"):
                # find the matching parenthesis
                depth, k = 0, j
                while True:
                    if expr[k] == "(":
                        depth += 1
                    elif expr[k] == ")":
                        depth -= 1
                        if depth == 0:
                            break
                    k += 1
                args = expr[j + 1:k]
                if name in GAS_LAWS:
                    out += "%s(&E, %s)" % (name, _rate_c(args, het_calls, het_laws))
                elif het_laws and name in HET_FUNCS:
                    parts = _split_args(args)
                    assert parts[-1] == "H" and len(parts) == HET_FUNCS[name] + 1, (name, parts)
                    num = "".join(", " + _rate_c(a, het_calls, het_laws) for a in parts[:-1])
                    out += "(het ? o_%s(&X%s) : 0.0)" % (name, num)
                else:
                    het_calls.add(name)
                    out += "HET_ZERO"
                i = k + 1
                continue
            if name in ("TEMP", "NUMDEN", "SRHOCl", "SRHOBr"):
                out += "E.%s" % name
            else:
                out += name
            i = j
            continue
        out += expr[i]
        i += 1
    return out


def _species_consts(ir):
    """SR_MW of every species and the MW/SR_MW/HENRY table of HET_SPECIES
    (species database values, mechanism/<mech>_species.json)."""
    import math

    path = os.path.join(MECH_DIR, ir.get("mechanism", "fullchem") + "_species.json")
    with open(path) as fh:
        spc = json.load(fh)
    assert spc["species"] == ir["species"]
    L = ["static const double SR_MW[%d] = {%s};" % (len(spc["mw"]),
                                                   ",".join(math.sqrt(m).hex() for m in spc["mw"]))]
    ind = [ir["species"].index(n) if n in ir["species"] else -1 for n in HET_SPECIES]
    for k, (n, i) in enumerate(zip(HET_SPECIES, ind)):
        L.append("#define OHS_%s %d" % (n, i))
        L.append("#define OHSI_%s %d" % (n, k))
    for name, key in (("O_MW", "mw"), ("O_HK0", "henry_k0"), ("O_HCR", "henry_cr")):
        L.append("static const double %s[%d] = {%s};" % (name, len(ind), ",".join(
            (spc[key][i] if i >= 0 else 0.0).hex() for i in ind)))
    L.append("static const double O_SRMW[%d] = {%s};" % (len(ind), ",".join(
        (math.sqrt(spc["mw"][i]) if i >= 0 else 0.0).hex() for i in ind)))
    return L


def generate_rates(ir):
    het_laws = ir.get("mechanism", "fullchem") == "fullchem"
    L = ["/* Generated by oracle/gen_oracle.py: Update_RCONST (KPP/fullchem/gckpp_Rates.F90:408-1503). */",
         "#include \"kpp_oracle.h\"",
         "#include \"rate_laws.h\""]
    L += _species_consts(ir)
    L += ["#include \"het_laws.h\"",
          "/* Heterogeneous rates without a HetState, and those that het_laws.h does not",
          " * restate (other mechanisms), are 0: no aerosol surface and no cloud, where the",
          " * Ars_L1k/CloudHet terms vanish. */",
          "#define HET_ZERO 0.0",
          "void oracle_update_rconst_het(const double* met, const double* PHOTOL, const double* C, const double* het,",
          "                              long long ldh, double* RCONST) {",
          "  rate_env_t E;",
          "  rate_env_init(&E, met[0], met[1], met[2], met[3], met[4], met[5]);",
          "  const double* K_MT = met + 6;",
          "  const double* K_CLD = met + 12;",
          "  het_cell_t X;",
          "  if (het) het_cell_load(&X, &E, het, ldh, C);",
          "  (void)C;",
          "  (void)X;"]
    het = set()
    for i, e in enumerate(ir["rconst"]):
        L.append("  RCONST[%d] = %s;" % (i, _rate_c(e, het, het_laws)))
    L.append("}")
    L.append("void oracle_update_rconst(const double* met, const double* PHOTOL, const double* C, double* RCONST) {")
    L.append("  oracle_update_rconst_het(met, PHOTOL, C, 0, 0, RCONST);")
    L.append("}")
    # the four sulfite uptake laws that fullchem_HetDropChem calls
    # (KPP/fullchem/fullchem_SulfurChemFuncs.F90:565-640)
    L += ["void oracle_sulfite_uptakes(const double* met, const double* C, const double* het, long long ldh,",
          "                            double* out) {"]
    if het_laws:
        L += ["  rate_env_t E;",
              "  rate_env_init(&E, met[0], met[1], met[2], met[3], met[4], met[5]);",
              "  het_cell_t X;",
              "  het_cell_load(&X, &E, het, ldh, C);",
              "  out[0] = o_HOClUptkByHSO3m(&X);",
              "  out[1] = o_HOClUptkBySO3mm(&X);",
              "  out[2] = o_HOBrUptkByHSO3m(&X);",
              "  out[3] = o_HOBrUptkBySO3mm(&X);"]
    else:
        L += ["  (void)met; (void)C; (void)het; (void)ldh;",
              "  out[0] = out[1] = out[2] = out[3] = 0.0;"]
    L.append("}")
    return "\n".join(L) + "\n", sorted(het)


def write_het_layout(outdir, mech="fullchem"):
    """oracle_het_layout.h: OHET_* row offsets of the HetState array, OHIN_*
    row offsets of fullchem_SetStateHet's inputs, and OSS_* the KPP indices
    (-1 when absent) of the species fullchem_SetStateHet reads."""
    sys.path.insert(0, os.path.join(HERE, "..", "geos-chem_gb300"))
    import hetstate  # the field lists of the batch interface (data only)

    import math

    species = _ir(mech)["species"]
    with open(os.path.join(HERE, "..", "geos-chem_gb300", "mechanism", mech + "_species.json")) as fh:
        mw = json.load(fh)["mw"]
    lines = ["/* Generated by oracle/gen_oracle.py from the HetState field list. */", "#pragma once"]
    for name, n in hetstate.FIELDS:
        lines.append("#define OHET_%s %d" % (name, hetstate.OFFSET[name]))
    for name, n in hetstate.HETIN_FIELDS:
        lines.append("#define OHIN_%s %d" % (name, hetstate.HETIN_OFFSET[name]))
    for name in hetstate.SETSTATE_SPECIES:
        k = species.index(name) if name in species else -1
        lines.append("#define OSS_%s %d" % (name, k))
        lines.append("#define OSS_SRMW_%s %s" % (name, repr(math.sqrt(mw[k])) if k >= 0 else "0.0"))
    for name, v in hetstate.NONKPP_MW.items():
        lines.append("#define OSS_MW_%s %r" % (name, v))
    text = "\n".join(lines) + "\n"
    path = os.path.join(outdir, "oracle_het_layout.h")
    old = open(path).read() if os.path.exists(path) else None
    if old != text:
        with open(path, "w") as fh:
            fh.write(text)
    return path


def write_rates(outdir, mech="fullchem"):
    write_het_layout(outdir, mech)
    text, het = generate_rates(_ir(mech))
    path = os.path.join(outdir, "kpp_rates_oracle.c")
    old = open(path).read() if os.path.exists(path) else None
    if old != text:
        with open(path, "w") as fh:
            fh.write(text)
    return path, het


if __name__ == "__main__":
    mech = sys.argv[2] if len(sys.argv) > 2 else "fullchem"
    print(write(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "_gen", mech), mech))
