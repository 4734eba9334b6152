"""Lower the Update_RCONST expressions to a stack program for the GPU.

Each of the 1058 rate expressions of Update_RCONST
(KPP/fullchem/gckpp_Rates.F90:441-1502, normalised in the mechanism IR) is
parsed with ordinary precedence and left associativity (the Fortran
evaluation order) and emitted as postfix code for ``csrc/kpp_rates.cu``:
every lane of a warp runs the same opcode for its own cell.

Heterogeneous rate functions (those taking the HetState ``H``) of
KPP/fullchem/fullchem_RateLawFuncs.F90 are emitted as HET calls of the laws
in csrc/het_rates.cuh (HET_LAWS order), their numeric arguments first
(``SR_MW[i]`` becomes the constant SQRT(MW) of the species database, as
GeosCore/fullchem_mod.F90:2915 sets it).  Without a HetState array the
heterogeneous rates are 0 (no aerosol surface, no cloud: the sums of
Ars_L1k/CloudHet terms vanish, KPP/fullchem/rateLawUtilFuncs.F90:77-96,
:141-230; evaluating the laws on an all-zero HetState gives the same zeros
except N2O5 uptake, which the Fortran arithmetic turns into NaN there).
Heterogeneous functions of other mechanisms stay HETZERO.
"""
import os
import re

from . import mechanism

OPS = ["END", "CONST", "VAR", "PHOTOL", "CONC", "ADD", "SUB", "MUL", "DIV", "NEG", "EXP", "LOG10", "CALL",
       "HETZERO", "HET"]
OP = {n: i for i, n in enumerate(OPS)}

# Per-cell met/state fields, in the order of GC_KPP_MET_* in the C ABI.
MET_FIELDS = ["TEMP", "NUMDEN", "H2O", "PRESS", "SRHOCl", "SRHOBr"] + \
    ["K_MT%d" % i for i in range(6)] + ["K_CLD%d" % i for i in range(6)]

# Gas-phase rate laws implemented in csrc/rate_laws.cuh: name -> (id, nargs)
LAWS = [
    ("GCARR_ab", 2), ("GCARR_ac", 2), ("GCARR_abc", 3), ("ARRPLUS_ade", 3), ("ARRPLUS_abde", 4),
    ("TUNPLUS_abcde", 5), ("GC_ISO1", 7), ("GC_ISO2", 7), ("GC_EPO_a", 3), ("GC_PAN_abab", 5),
    ("GC_PAN_acac", 5), ("GC_NIT", 6), ("GC_ALK", 6), ("GC_HO2HO2_acac", 4), ("GC_TBRANCH_1_acac", 4),
    ("GC_RO2HO2_aca", 3), ("GC_DMSOH_acac", 4), ("GC_GLYXNO3_ac", 2), ("GC_GLYCOH_A_a", 1),
    ("GC_GLYCOH_B_a", 1), ("GC_HACOH_A_ac", 2), ("GC_HACOH_B_ac", 2), ("GC_RO2NO_A1_ac", 2),
    ("GC_RO2NO_B1_ac", 2), ("GC_RO2NO_A2_aca", 3), ("GC_RO2NO_B2_aca", 3), ("GCJPLEQ_acabab", 7),
    ("GCJPLPR_aa", 3), ("GCJPLPR_aba", 4), ("GCJPLPR_abab", 5), ("GCJPLPR_abcabc", 7), ("GCJPLAC_ababac", 7),
]
LAW_ID = {n: (i, k) for i, (n, k) in enumerate(LAWS)}

# Heterogeneous rate laws of csrc/het_rates.cuh (het_law switch order):
# name -> number of numeric arguments (the HetState argument H is implicit)
HET_LAWS = [
    ("BrNO3uptkByH2O", 0), ("BrNO3uptkByHCl", 0), ("ClNO2uptkByBrSALA", 0), ("ClNO2uptkByBrSALC", 0),
    ("ClNO2uptkByHBr", 0), ("ClNO2uptkBySALACL", 0), ("ClNO2uptkBySALCCL", 0), ("ClNO2uptkByHCl", 0),
    ("ClNO3uptkByH2O", 0), ("ClNO3uptkByHCl", 0), ("ClNO3uptkByHBr", 0), ("ClNO3uptkByBrSALA", 0),
    ("ClNO3uptkByBrSALC", 0), ("ClNO3uptkBySALACL", 0), ("ClNO3uptkBySALCCL", 0), ("HBrUptkBySALA", 0),
    ("HBrUptkBySALC", 0), ("HO2uptk1stOrd", 0), ("HOBrUptkByHBr", 0), ("HOBrUptkByHCl", 0),
    ("HOBrUptkByBrSALA", 0), ("HOBrUptkByBrSALC", 0), ("HOBrUptkBySALACL", 0), ("HOBrUptkBySALCCL", 0),
    ("HOBrUptkByHSO3m", 0), ("HOBrUptkBySO3mm", 0), ("HOClUptkByHCl", 0), ("HOClUptkByHBr", 0),
    ("HOClUptkBySALACL", 0), ("HOClUptkBySALCCL", 0), ("HOClUptkByHSO3m", 0), ("HOClUptkBySO3mm", 0),
    ("IuptkBySulf1stOrd", 2), ("IuptkBySALA1stOrd", 2), ("IuptkByAlkSALA1stOrd", 2), ("IuptkBySALC1stOrd", 2),
    ("IuptkByAlkSALC1stOrd", 2), ("IbrkdnByAcidBrSALA", 3), ("IbrkdnByAcidBrSALC", 3), ("IbrkdnByAcidSALACl", 3),
    ("IbrkdnByAcidSALCCl", 3), ("IONO2uptkByH2O", 0), ("N2O5uptkByH2O", 0), ("N2O5uptkBySALACl", 0),
    ("N2O5uptkBySALCCl", 0), ("N2O5uptkByCloud", 0), ("N2O5uptkByStratHCl", 0), ("NO2uptk1stOrdAndCloud", 0),
    ("NO3uptk1stOrdAndCloud", 0), ("NO3hypsisClonSALA", 0), ("NO3hypsisClonSALC", 0), ("O3uptkByHBr", 0),
    ("O3uptkByBrSALA", 0), ("O3uptkByBrSALC", 0), ("OHuptkBySALACl", 0), ("OHuptkBySALCCl", 0),
    ("GLYXuptk1stOrd", 1), ("IEPOXuptk1stOrd", 2), ("MGLYuptk1stOrd", 1), ("VOCuptk1stOrd", 2),
]
HET_ID = {n: (i, k) for i, (n, k) in enumerate(HET_LAWS)}
# species the heterogeneous laws reference (csrc/het_rates.cuh HetSpc order)
HET_SPECIES = ["BrNO3", "H2O", "HCl", "ClNO2", "BrSALA", "BrSALC", "HBr", "SALACL", "SALCCL", "ClNO3", "HOBr",
               "SO2", "HOCl", "HO2", "IONO2", "N2O5", "NIT", "NITs", "NO2", "NO3", "O3", "OH"]

_TOKEN = re.compile(r"\s*(?:(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+(?:[eE][+-]?\d+)?)|"
                    r"([A-Za-z_][A-Za-z_0-9]*)|(.))")


def _tokens(s):
    out = []
    pos = 0
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if m.group(1):
            out.append(("num", m.group(1)))
        elif m.group(2):
            out.append(("id", m.group(2)))
        elif m.group(3).strip():
            out.append(("op", m.group(3)))
        pos = m.end()
    return out


class _Parser:
    def __init__(self, text, consts, srmw=None, het_laws=True):
        self.t = _tokens(text)
        self.i = 0
        self.code = []
        self.consts = consts
        self.het = 0
        self.srmw = srmw
        self.het_laws = het_laws

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.t[self.i]
        if val is not None and tok[1] != val:
            raise ValueError("expected %r got %r" % (val, tok))
        self.i += 1
        return tok

    def const(self, v):
        if v not in self.consts:
            self.consts[v] = len(self.consts)
        self.code += [OP["CONST"], self.consts[v]]

    def expr(self):
        self.term()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            self.term()
            self.code.append(OP["ADD"] if op == "+" else OP["SUB"])

    def term(self):
        self.unary()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            self.unary()
            self.code.append(OP["MUL"] if op == "*" else OP["DIV"])

    def unary(self):
        if self.peek()[1] == "-":
            self.take()
            self.unary()
            self.code.append(OP["NEG"])
        elif self.peek()[1] == "+":
            self.take()
            self.unary()
        else:
            self.atom()

    def _args(self):
        self.take("(")
        n = 0
        if self.peek()[1] != ")":
            while True:
                self.expr()
                n += 1
                if self.peek()[1] == ",":
                    self.take()
                    continue
                break
        self.take(")")
        return n

    def _het_args(self):
        """Numeric arguments of a heterogeneous law; the HetState H is implicit."""
        self.take("(")
        n = 0
        while True:
            if self.peek() == ("id", "H") and self.t[self.i + 1][1] in (",", ")"):
                self.take()
            else:
                self.expr()
                n += 1
            if self.peek()[1] == ",":
                self.take()
                continue
            break
        self.take(")")
        return n

    def _skip_call(self):
        depth = 0
        while True:
            tok = self.take()
            if tok[1] == "(":
                depth += 1
            elif tok[1] == ")":
                depth -= 1
                if depth == 0:
                    return

    def atom(self):
        kind, val = self.peek()
        if kind == "num":
            self.take()
            self.const(float(val))
        elif kind == "op" and val == "(":
            self.take()
            self.expr()
            self.take(")")
        elif kind == "id":
            self.take()
            nxt = self.peek()[1]
            if nxt == "[":
                self.take()
                idx = int(self.take()[1])
                self.take("]")
                if val == "PHOTOL":
                    self.code += [OP["PHOTOL"], idx]
                elif val == "K_MT":
                    self.code += [OP["VAR"], MET_FIELDS.index("K_MT%d" % idx)]
                elif val == "K_CLD":
                    self.code += [OP["VAR"], MET_FIELDS.index("K_CLD%d" % idx)]
                elif val == "C":
                    self.code += [OP["CONC"], idx]
                elif val == "SR_MW" and self.srmw is not None:
                    self.const(self.srmw[idx])
                else:
                    raise ValueError("array %s" % val)
            elif nxt == "(":
                if val in ("exp", "log10"):
                    n = self._args()
                    assert n == 1
                    self.code.append(OP["EXP"] if val == "exp" else OP["LOG10"])
                elif val in LAW_ID:
                    lid, k = LAW_ID[val]
                    n = self._args()
                    assert n == k, (val, n, k)
                    self.code += [OP["CALL"], lid]
                elif val in HET_ID and self.het_laws:
                    hid, k = HET_ID[val]
                    n = self._het_args()
                    assert n == k, (val, n, k)
                    self.code += [OP["HET"], hid]
                    self.het += 1
                else:
                    self._skip_call()
                    self.code.append(OP["HETZERO"])
                    self.het += 1
            elif val in MET_FIELDS:
                self.code += [OP["VAR"], MET_FIELDS.index(val)]
            else:
                raise ValueError("unknown identifier %s" % val)
        else:
            raise ValueError("unexpected %r" % (val,))


def build_program(ir=None):
    import math

    from .mechanism import species_db

    ir = ir or mechanism.load_ir()
    mech = ir.get("mechanism", "fullchem")
    spc = species_db.load(mech)
    assert spc["species"] == ir["species"], "species constants out of date for %s" % mech
    srmw = [math.sqrt(m) for m in spc["mw"]]
    het_laws = mech == "fullchem"
    consts = {}
    code = []
    start = [0]
    nhet = 0
    for e in ir["rconst"]:
        p = _Parser(e, consts, srmw, het_laws)
        p.expr()
        assert p.i == len(p.t), e
        code += p.code + [OP["END"]]
        start.append(len(code))
        nhet += p.het
    pool = [0.0] * len(consts)
    for v, i in consts.items():
        pool[i] = v
    # species table of the heterogeneous laws (KPP index or -1, MW, SR_MW, HENRY_K0, HENRY_CR)
    ind = [ir["species"].index(n) if n in ir["species"] else -1 for n in HET_SPECIES]
    pick = lambda arr: [arr[i] if i >= 0 else 0.0 for i in ind]
    # KPP indices of the species fullchem_SetStateHet reads (order of hetstate.SETSTATE_SPECIES)
    from .hetstate import SETSTATE_SPECIES

    hss = [ir["species"].index(n) if n in ir["species"] else -1 for n in SETSTATE_SPECIES]
    photol_rows = sorted({int(k) for e in ir["rconst"] for k in re.findall(r"PHOTOL\[(\d+)\]", e)})
    return {"code": code, "start": start, "consts": pool, "nhet": nhet, "photol_rows": photol_rows,
            "hs_ind": ind, "hs_mw": pick(spc["mw"]),
            "hs_srmw": pick(srmw), "hs_hk0": pick(spc["henry_k0"]), "hs_hcr": pick(spc["henry_cr"]),
            "hss_ind": hss, "hss_srmw": [srmw[i] if i >= 0 else 0.0 for i in hss]}


def _runs(rows):
    """Sorted row indices as contiguous runs [(first, last + 1), ...]."""
    runs = []
    for r in rows:
        if runs and runs[-1][1] == r:
            runs[-1][1] = r + 1
        else:
            runs.append([r, r + 1])
    return [tuple(x) for x in runs]


def emit_c(prog):
    lines = ["// Generated by gcchem.rates_program from the mechanism IR. Do not edit.",
             "#pragma once",
             "namespace gcrates_tables {",
             "constexpr int NMET = %d;" % len(MET_FIELDS),
             "static const int code[%d] = {%s};" % (len(prog["code"]), ",".join(map(str, prog["code"]))),
             "static const int start[%d] = {%s};" % (len(prog["start"]), ",".join(map(str, prog["start"]))),
             "static const double consts[%d] = {%s};" % (len(prog["consts"]),
                                                       ",".join(float(v).hex() for v in prog["consts"])),
             "static const int law_nargs[%d] = {%s};" % (len(LAWS), ",".join(str(k) for _, k in LAWS)),
             "static const int het_nargs[%d] = {%s};" % (len(HET_LAWS), ",".join(str(k) for _, k in HET_LAWS)),
             "static const int hs_ind[%d] = {%s};" % (len(HET_SPECIES), ",".join(map(str, prog["hs_ind"]))),
             "static const int hss_ind[%d] = {%s};" % (len(prog["hss_ind"]), ",".join(map(str, prog["hss_ind"]))),
             "static const double hss_srmw[%d] = {%s};" % (len(prog["hss_srmw"]),
                                                          ",".join(float(v).hex() for v in prog["hss_srmw"])),
             "// PHOTOL rows that the rate program reads, as runs [first, last + 1)",
             "constexpr int NPHOTOL_RUNS = %d;" % len(_runs(prog["photol_rows"])),
             "static const int photol_runs[%d] = {%s};" % (
                 max(1, 2 * len(_runs(prog["photol_rows"]))),
                 ",".join("%d,%d" % r for r in _runs(prog["photol_rows"])) or "0")]
    for key in ("hs_mw", "hs_srmw", "hs_hk0", "hs_hcr"):
        lines.append("static const double %s[%d] = {%s};" % (key, len(HET_SPECIES),
                                                            ",".join(float(v).hex() for v in prog[key])))
    lines.append("}  // namespace gcrates_tables")
    return "\n".join(lines) + "\n"


def write_generated(outdir, ir=None):
    prog = build_program(ir)
    os.makedirs(outdir, exist_ok=True)
    for name, text in (("rates_program.inc", emit_c(prog)), ("rates_direct.inc", emit_direct(prog))):
        path = os.path.join(outdir, name)
        old = open(path).read() if os.path.exists(path) else None
        if old != text:
            with open(path, "w") as fh:
                fh.write(text)
    return os.path.join(outdir, "rates_program.inc")


def emit_direct(prog):
    """Straight-line CUDA statements of the same postfix program (one
    expression per rate, operations in the program's order, additions and
    multiplications through the round-to-nearest intrinsics so that nothing
    is contracted): the body of the per-mechanism rates_direct_kernel
    (rates_direct.cu), which gives the interpreter's results to rounding
    without its dispatch and local-memory stack.  Uses the kernel's macros
    M(f) (met row), PH(j), CC(i), OUT(r) and the functions lawv/hetv."""
    code, start, consts = prog["code"], prog["start"], prog["consts"]
    nargs = {i: k for i, (_, k) in enumerate(LAWS)}
    hnargs = {i: k for i, (_, k) in enumerate(HET_LAWS)}
    lines = ["// Generated by gcchem.rates_program (emit_direct). Do not edit."]
    ntmp = 0
    for r in range(len(start) - 1):
        st = []
        pc = start[r]
        while True:
            op = OPS[code[pc]]
            pc += 1
            if op == "END":
                break
            if op == "CONST":
                st.append(float(consts[code[pc]]).hex())
                pc += 1
            elif op == "VAR":
                st.append("M(%d)" % code[pc])
                pc += 1
            elif op == "PHOTOL":
                st.append("PH(%d)" % code[pc])
                pc += 1
            elif op == "CONC":
                st.append("CC(%d)" % code[pc])
                pc += 1
            elif op in ("ADD", "SUB", "MUL", "DIV"):
                b, a = st.pop(), st.pop()
                if op == "DIV":
                    st.append("(%s / %s)" % (a, b))
                else:
                    st.append("__d%s_rn(%s, %s)" % ({"ADD": "add", "SUB": "sub", "MUL": "mul"}[op], a, b))
            elif op == "NEG":
                st.append("(-%s)" % st.pop())
            elif op in ("EXP", "LOG10"):
                st.append("%s(%s)" % (op.lower(), st.pop()))
            elif op == "CALL":
                lid = code[pc]
                pc += 1
                k = nargs[lid]
                args = st[len(st) - k:]
                del st[len(st) - k:]
                lines.append("  const double x%d = lawv(%d, E, %s);" % (ntmp, lid, ", ".join(args)))
                st.append("x%d" % ntmp)
                ntmp += 1
            elif op == "HETZERO":
                st.append("0.0")
            elif op == "HET":
                hid = code[pc]
                pc += 1
                k = hnargs[hid]
                args = st[len(st) - k:] if k else []
                if k:
                    del st[len(st) - k:]
                lines.append("  const double x%d = hetv(%d, has_het, X%s);" % (
                    ntmp, hid, "".join(", " + a for a in args)))
                st.append("x%d" % ntmp)
                ntmp += 1
            else:
                raise ValueError(op)
        assert len(st) == 1, r
        lines.append("  OUT(%d) = %s;" % (r, st[0]))
    return "\n".join(lines) + "\n"
