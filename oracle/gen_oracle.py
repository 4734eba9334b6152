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
    for name in ("crow", "diag", "icol"):
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
    L.append("void oracle_jac_sp(const double* V, const double* F, const double* RCT, double* JVS) {")
    L.append("  double B[%d];" % nb)
    for b, f in enumerate(ir["jac"]["B"]):
        if f is not None:
            L.append("  B[%d] = %s;" % (b, _prod(f)))
    for k, terms in enumerate(ir["jac"]["JVS"]):
        L.append("  JVS[%d] = %s;" % (k, _signed([(s, (c, b)) for s, c, b in terms], _coef_ref("B"))))
    L.append("}")
    L.append("")
    L.append("void oracle_kpp_solve(const double* JVS, double* X) {")
    for st in ir["solve"]:
        i = st["row"]
        e = "X[%d]" % i + "".join(" - JVS[%d]*X[%d]" % (k, j) for k, j in st["terms"])
        if st["kind"] == "B":
            e = "(%s)/(JVS[%d])" % (e, st["diag"]) if st["terms"] else "X[%d]/JVS[%d]" % (i, st["diag"])
        L.append("  X[%d] = %s;" % (i, e))
    L.append("}")
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


def _rate_c(expr, het_calls):
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
                    out += "%s(&E, %s)" % (name, _rate_c(args, het_calls))
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


def generate_rates(ir):
    L = ["/* Generated by oracle/gen_oracle.py: Update_RCONST (KPP/fullchem/gckpp_Rates.F90:408-1503). */",
         "#include \"kpp_oracle.h\"",
         "#include \"rate_laws.h\"",
         "/* Heterogeneous rates with the zeroed HetState of the synthetic cells: every het",
         " * rate function of fullchem_RateLawFuncs.F90 sums Ars_L1k/CloudHet terms that are 0",
         " * for zero aerosol area/radius and zero cloud fraction. */",
         "#define HET_ZERO 0.0",
         "void oracle_update_rconst(const double* met, const double* PHOTOL, const double* C, double* RCONST) {",
         "  rate_env_t E;",
         "  rate_env_init(&E, met[0], met[1], met[2], met[3], met[4], met[5]);",
         "  const double* K_MT = met + 6;",
         "  const double* K_CLD = met + 12;",
         "  (void)C;"]
    het = set()
    for i, e in enumerate(ir["rconst"]):
        L.append("  RCONST[%d] = %s;" % (i, _rate_c(e, het)))
    L.append("}")
    return "\n".join(L) + "\n", sorted(het)


def write_rates(outdir, mech="fullchem"):
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
