"""Extract the fullchem mechanism IR from KPP-3.2.0 generated Fortran.

This is the build step that turns GEOS-Chem's KPP-generated mechanism files
into ``fullchem.json``, the data every other part of this package is
generated from (the CUDA kernels, the C oracle, the parity tests).  It is run
once, in a checkout that has the GEOS-Chem source tree, and its output is
committed; nothing at run time reads the Fortran.

What is extracted (paths relative to the GEOS-Chem source root):

* dimensions and species order   KPP/fullchem/gckpp_Parameters.F90:34-54, 59-431
* Fun_SPLIT statements           KPP/fullchem/gckpp_Function.F90:2172-5059
    A(r)   = product of factors (rate, variable/fixed species, literal)
    P_VAR  = signed sum of [coef*]A(r)
    D_VAR  = signed sum of products of factors
* Jac_SP statements              KPP/fullchem/gckpp_Jacobian.F90:48-20887
    B(b)   = product of factors;  JVS(k) = signed sum of [coef*]B(b)
* sparse LU structure            KPP/fullchem/gckpp_JacobianSP.F90:525-1093
* KppSolve statement order       KPP/fullchem/gckpp_LinearAlgebra.F90:644-2309
* Update_RCONST expressions      KPP/fullchem/gckpp_Rates.F90:441-1502
  and the two constant rates     KPP/fullchem/gckpp_Initialize.F90:57-58

Every statement is parsed into a compact structured form and then rendered
back to Fortran text; the extraction fails unless the rendering reproduces the
original statement exactly (modulo whitespace), so the IR holds the same
arithmetic in the same evaluation order as the generated code.

Usage: python extract_kpp.py <geos-chem-root> [out.json]
"""
import json
import os
import re
import sys

MECH = ["fullchem"]  # the KPP mechanism directory being read (KPP/<mech>)


def _read(root, name):
    with open(os.path.join(root, "KPP", MECH[0], name)) as fh:
        return fh.read()


def _join_continuations(text):
    # Fortran free-form continuation: trailing '&' + optional leading '&'.
    text = re.sub(r"&[ \t]*\n[ \t]*&", "", text)
    text = re.sub(r"&[ \t]*\n[ \t]*", "", text)
    return text


def _body(text, start_pat, end_pat):
    s = text.index(start_pat)
    e = text.index(end_pat, s)
    return text[s:e]


def _statements(body, lhs_names):
    """Return [(name, 1-based index, rhs)] for assignment statements."""
    out = []
    pat = re.compile(r"^\s*(%s)\((\d+)\)\s*=\s*(.+?)\s*$" % "|".join(lhs_names))
    for line in body.split("\n"):
        line = line.split("!", 1)[0] if not line.strip().startswith("IF") else line
        line = re.sub(r"^\s*IF \(DO_\w+\(\d+\)\)\s*", "", line)
        m = pat.match(line)
        if m:
            out.append((m.group(1), int(m.group(2)), m.group(3).replace(" ", "")))
    return out


NUM = r"(?:\d+\.\d*(?:[eEdD][+-]?\d+)?|\d+(?:[eEdD][+-]?\d+)?)"
REF = r"(?:RCT|V|F|A|B|JVS|X)\(\d+\)"


def _factor_tok(f):
    """Fortran factor -> IR token: R<i>, V<i>, F<i>, A<i>, B<i>, J<i>, X<i> (0-based) or a literal."""
    m = re.fullmatch(r"(RCT|V|F|A|B|JVS|X)\((\d+)\)", f)
    if m:
        tag = {"RCT": "R", "JVS": "J"}.get(m.group(1), m.group(1))
        return "%s%d" % (tag, int(m.group(2)) - 1)
    if re.fullmatch(NUM, f):
        return f
    raise ValueError("bad factor %r" % f)


def _tok_fortran(t):
    m = re.fullmatch(r"([RVFABJX])(\d+)", t)
    if m:
        name = {"R": "RCT", "J": "JVS"}.get(m.group(1), m.group(1))
        return "%s(%d)" % (name, int(m.group(2)) + 1)
    return t


def _split_terms(rhs):
    """Split a sum of products into [(sign, product_text)] at top level."""
    terms = []
    cur = ""
    depth = 0
    sign = "+"
    i = 0
    while i < len(rhs):
        c = rhs[i]
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        if depth == 0 and c in "+-" and i > 0 and not re.search(r"\d[eEdD]$", cur):
            terms.append((sign, cur))
            sign = c
            cur = ""
        elif depth == 0 and c in "+-" and i == 0:
            sign = c
        else:
            cur += c
        i += 1
    terms.append((sign, cur))
    return terms


def _product(text):
    return [_factor_tok(f) for f in text.split("*")]


def _render_product(toks):
    return "*".join(_tok_fortran(t) for t in toks)


def _render_sum(terms, render_one):
    out = ""
    for k, (sign, payload) in enumerate(terms):
        body = render_one(payload)
        if k == 0:
            out += ("-" if sign == "-" else "") + body
        else:
            out += sign + body
    return out


def _coef_ref_terms(rhs, refname):
    """Sum of [coef*]REF terms -> [[sign, coef or None, index]]."""
    if rhs == "0":
        return []
    out = []
    for sign, t in _split_terms(rhs):
        parts = t.split("*")
        if len(parts) == 1:
            coef, ref = None, parts[0]
        elif len(parts) == 2:
            coef, ref = parts
            if not re.fullmatch(NUM, coef):
                raise ValueError(t)
        else:
            raise ValueError(t)
        m = re.fullmatch(r"%s\((\d+)\)" % refname, ref)
        if not m:
            raise ValueError(t)
        out.append([sign, coef, int(m.group(1)) - 1])
    return out


def _render_coef_ref(terms, refname):
    if not terms:
        return "0"
    return _render_sum(
        [(s, (c, i)) for s, c, i in terms],
        lambda p: ("%s*" % p[0] if p[0] is not None else "") + "%s(%d)" % (refname, p[1] + 1),
    )


def _prod_terms(rhs):
    if rhs == "0":
        return []
    return [[sign, _product(t)] for sign, t in _split_terms(rhs)]


def _render_prod_terms(terms):
    if not terms:
        return "0"
    return _render_sum([(s, f) for s, f in terms], _render_product)


def _check(orig, rendered, what):
    if orig != rendered:
        raise AssertionError("round trip failed for %s:\n  %s\n  %s" % (what, orig, rendered))


def parse_parameters(root):
    txt = _read(root, "gckpp_Parameters.F90")
    dims = {}
    for key in ["NSPEC", "NVAR", "NFAM", "NVARACT", "NFIX", "NREACT", "NONZERO", "LU_NONZERO"]:
        dims[key.lower()] = int(re.search(r"\b%s\s*=\s*(\d+)" % key, txt).group(1))
    species = [None] * dims["nspec"]
    for name, idx in re.findall(r"INTEGER, PARAMETER :: ind_(\w+) = (\d+)", txt):
        species[int(idx) - 1] = name
    assert all(s is not None for s in species)
    return dims, species


def parse_fun(root, dims):
    txt = _join_continuations(_read(root, "gckpp_Function.F90"))
    body = _body(txt, "SUBROUTINE Fun_SPLIT", "END SUBROUTINE Fun_SPLIT")
    st = _statements(body, ["A", "P_VAR", "D_VAR"])
    A = [None] * dims["nreact"]
    P = [None] * dims["nvar"]
    D = [None] * dims["nvar"]
    for name, idx, rhs in st:
        if name == "A":
            A[idx - 1] = _product(rhs)
            _check(rhs, _render_product(A[idx - 1]), "A(%d)" % idx)
        elif name == "P_VAR":
            P[idx - 1] = [] if rhs.strip() == "0" else _coef_ref_terms(rhs, "A")
            if P[idx - 1]:
                _check(rhs, _render_coef_ref(P[idx - 1], "A"), "P_VAR(%d)" % idx)
        else:
            D[idx - 1] = [] if rhs.strip() == "0" else _prod_terms(rhs)
            if D[idx - 1]:
                _check(rhs, _render_prod_terms(D[idx - 1]), "D_VAR(%d)" % idx)
    assert all(x is not None for x in P + D)
    # KPP leaves out A(r) of reactions that change no variable species; such
    # a rate is never referenced, and is kept as an empty product
    used = {t[2] for terms in P for t in terms}
    for r, a in enumerate(A):
        if a is None:
            assert r not in used, "A(%d) referenced but not computed" % (r + 1)
            A[r] = []
    assert "Vdot = P_VAR - D_VAR*V" in body
    return {"A": A, "P": P, "D": D}


def parse_jac(root, dims):
    txt = _join_continuations(_read(root, "gckpp_Jacobian.F90"))
    body = _body(txt, "SUBROUTINE Jac_SP ", "END SUBROUTINE Jac_SP")
    nb = int(re.search(r"REAL\(kind=dp\) :: B\((\d+)\)", body).group(1))
    st = _statements(body, ["B", "JVS"])
    B = [None] * nb
    J = [None] * dims["lu_nonzero"]
    order_b = []
    for name, idx, rhs in st:
        if name == "B":
            B[idx - 1] = _product(rhs)
            order_b.append(idx - 1)
            _check(rhs, _render_product(B[idx - 1]), "B(%d)" % idx)
        else:
            J[idx - 1] = _coef_ref_terms(rhs, "B")
            _check(rhs, _render_coef_ref(J[idx - 1], "B"), "JVS(%d)" % idx)
    # KPP sizes B by its own count but leaves a few slots unassigned; they
    # must never be read.
    assert all(x is not None for x in J)
    used = {i for terms in J for _, _, i in terms}
    assert all(B[i] is not None for i in used)
    assert order_b == sorted(order_b)
    return {"B": B, "JVS": J}


def _int_array(txt, name):
    # concatenated DATA chunks NAME_0, NAME_1, ... (or a single NAME)
    chunks = re.findall(r"DIMENSION\(\d+\) :: %s(?:_\d+)? = \(/(.*?)/\)" % name, txt, re.S)
    vals = []
    for ch in chunks:
        ch = re.sub(r"!.*", "", ch)
        if re.search(r"[A-Za-z]", ch):
            continue  # the concatenation of the chunks, not data
        vals += [int(v) for v in re.findall(r"\d+", ch)]
    return vals


def parse_lu(root, dims):
    txt = _read(root, "gckpp_JacobianSP.F90")
    irow = _int_array(txt, "LU_IROW")
    icol = _int_array(txt, "LU_ICOL")
    crow = _int_array(txt, "LU_CROW")
    diag = _int_array(txt, "LU_DIAG")
    n, nnz = dims["nvar"], dims["lu_nonzero"]
    assert len(irow) == nnz and len(icol) == nnz, (len(irow), len(icol))
    assert len(crow) == n + 1 and len(diag) == n + 1
    return {
        "irow": [v - 1 for v in irow],
        "icol": [v - 1 for v in icol],
        "crow": [v - 1 for v in crow],
        "diag": [v - 1 for v in diag],
    }


def parse_solve(root, dims):
    txt = _join_continuations(_read(root, "gckpp_LinearAlgebra.F90"))
    body = _body(txt, "SUBROUTINE KppSolve ", "END SUBROUTINE KppSolve")
    st = _statements(body, ["X"])
    out = []
    for _, idx, rhs in st:
        i = idx - 1
        m = re.fullmatch(r"\((.*)\)/\(JVS\((\d+)\)\)", rhs)
        m2 = re.fullmatch(r"X\((\d+)\)/JVS\((\d+)\)", rhs)
        if m:
            inner, d = m.group(1), int(m.group(2)) - 1
            kind = "B"
        elif m2:
            inner, d = "X(%s)" % m2.group(1), int(m2.group(2)) - 1
            kind = "B"
        else:
            inner, d = rhs, None
            kind = "F"
        terms = _split_terms(inner)
        assert terms[0] == ("+", "X(%d)" % idx), (idx, terms[0])
        pairs = []
        for sign, t in terms[1:]:
            mm = re.fullmatch(r"JVS\((\d+)\)\*X\((\d+)\)", t)
            assert sign == "-" and mm, t
            pairs.append([int(mm.group(1)) - 1, int(mm.group(2)) - 1])
        rendered = "X(%d)" % idx + "".join("-JVS(%d)*X(%d)" % (k + 1, j + 1) for k, j in pairs)
        if kind == "B":
            if pairs:
                rendered = "(%s)/(JVS(%d))" % (rendered, d + 1)
            else:
                rendered = "X(%d)/JVS(%d)" % (idx, d + 1)
        _check(rhs, rendered, "X(%d)" % idx)
        out.append({"row": i, "kind": kind, "terms": pairs, "diag": d})
    return out


# --- Update_RCONST -------------------------------------------------------------

def _norm_rate_expr(rhs, species):
    """Normalise a Fortran rate expression to a C-like expression text.

    Literals lose their Fortran kind suffix and 'd' exponents; ind_<SPC> is
    replaced by its 0-based species index; C(i), SR_MW(i) become C[i], SR_MW[i];
    PHOTOL(j), K_MT(j), K_CLD(j) become 0-based array reads; State_Het becomes H;
    .TRUE./.FALSE. become 1/0; EXP/exp become exp.
    """
    sp = {s: i for i, s in enumerate(species)}
    e = rhs
    e = re.sub(r"ind_(\w+)", lambda m: str(sp[m.group(1)] + 1), e)
    e = re.sub(r"(\d+\.\d*|\d+|\.\d+)[dD]([+-]?\d+)", r"\1e\2", e)
    e = re.sub(r"_dp\b", "", e)
    e = e.replace(".TRUE.", "1").replace(".FALSE.", "0")
    e = re.sub(r"\bEXP\(", "exp(", e)
    e = re.sub(r"\bLOG10\(", "log10(", e)
    e = re.sub(r"\b(C|SR_MW|PHOTOL|K_MT|K_CLD)\((\d+)\)", lambda m: "%s[%d]" % (m.group(1), int(m.group(2)) - 1), e)
    e = e.replace("State_Het", "H")
    return e


def parse_rates(root, dims, species):
    txt = _join_continuations(_read(root, "gckpp_Rates.F90"))
    body = _body(txt, "SUBROUTINE Update_RCONST", "END SUBROUTINE UPDATE_RCONST")
    exprs = [None] * dims["nreact"]
    raw = [None] * dims["nreact"]
    for line in body.split("\n"):
        m = re.match(r"^\s*RCONST\((\d+)\)\s*=\s*(.+?)\s*$", line)
        if m:
            i = int(m.group(1)) - 1
            raw[i] = m.group(2)
            exprs[i] = _norm_rate_expr(m.group(2).replace(" ", ""), species)
    init = _read(root, "gckpp_Initialize.F90")
    for idx, val in re.findall(r"RCONST\((\d+)\)\s*=\s*([0-9.eEdD+-]+)", init):
        i = int(idx) - 1
        assert exprs[i] is None
        exprs[i] = "(%s)" % _norm_rate_expr(val, species)
        raw[i] = "constant (gckpp_Initialize.F90) " + val
    assert all(e is not None for e in exprs)
    return exprs


def parse_families(root):
    """Prod/loss family dummy species (KPP/fullchem/fullchem.kpp:13-20); their
    concentrations are zeroed before each integration
    (GeosCore/fullchem_mod.F90:943-946)."""
    txt = _read(root, MECH[0] + ".kpp")
    if "#FAMILIES" not in txt:
        return []
    block = txt.split("#FAMILIES", 1)[1].split("#INLINE", 1)[0]
    return re.findall(r"^\s*(\w+)\s*:", block, re.M)


def parse_tolerances(root, species):
    """KPP_AbsTol/KPP_RelTol from run/shared/species_database.yml for the
    mechanism's species, and the defaults applied where the database has none
    (GeosCore/fullchem_mod.F90:2899-2905)."""
    path = os.path.join(root, "run", "shared", "species_database.yml")
    atol, rtol = {}, {}
    cur = None
    with open(path) as fh:
        for line in fh:
            m = re.match(r"^(\S[^:]*):\s*$", line)
            if m:
                cur = m.group(1).strip()
                continue
            m = re.match(r"^\s+KPP_(AbsTol|RelTol):\s*([0-9.eE+-]+)", line)
            if m and cur in species:
                (atol if m.group(1) == "AbsTol" else rtol)[cur] = float(m.group(2))
    return {"atol_default": 1.0e-2, "rtol_default": 0.5e-2, "atol": atol, "rtol": rtol}


def extract(root, mech="fullchem"):
    MECH[0] = mech
    dims, species = parse_parameters(root)
    ir = {
        "mechanism": mech,
        "generator": "KPP-3.2.0",
        "dims": dims,
        "species": species,
        "fixed": species[dims["nvar"]:],
        "fun": parse_fun(root, dims),
        "jac": parse_jac(root, dims),
        "lu": parse_lu(root, dims),
        "solve": parse_solve(root, dims),
        "rconst": parse_rates(root, dims, species),
        "families": parse_families(root),
        "tolerances": parse_tolerances(root, set(species)),
    }
    return ir


def main(argv):
    root = argv[1]
    mech = argv[3] if len(argv) > 3 else "fullchem"
    out = argv[2] if len(argv) > 2 else os.path.join(os.path.dirname(os.path.abspath(__file__)), mech + ".json")
    ir = extract(root, mech)
    with open(out, "w") as fh:
        json.dump(ir, fh, separators=(",", ":"))
        fh.write("\n")
    d = ir["dims"]
    print("wrote %s: nvar=%d nreact=%d lu_nonzero=%d nB=%d nsolve=%d" % (
        out, d["nvar"], d["nreact"], d["lu_nonzero"], len(ir["jac"]["B"]), len(ir["solve"])))


if __name__ == "__main__":
    main(sys.argv)
