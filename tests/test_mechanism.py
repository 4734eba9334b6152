"""CPU checks of the mechanism IR, the oracle's generated code and the
product's table lowering, against each other and against mathematics.

The reference ships no golden vectors for this path, so the oracle is pinned
by internal invariants of KPP's generated code:
* Fun_SPLIT / Jac_SP / KppDecomp / KppSolve of the oracle reproduce a
  statement-by-statement Python evaluation of the IR bit for bit;
* Jac_SP equals the complex-step derivative of Fun_SPLIT;
* KppDecomp + KppSolve equal a dense LU solve of the same matrix.
"""
import json
import os

import numpy as np
import pytest

import ir_eval
import gcchem.tables as tables

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def point(ir):
    rng = np.random.default_rng(42)
    d = ir["dims"]
    V = np.exp(rng.uniform(np.log(1e2), np.log(1e12), d["nvar"]))
    F = np.array([5e-7, 0.7808, 0.2095]) * 2.5e19
    RCT = np.exp(rng.uniform(np.log(1e-16), np.log(1e-9), d["nreact"]))
    return V, F, RCT


def test_ir_dimensions(ir):
    d = ir["dims"]
    assert (d["nspec"], d["nvar"], d["nfix"], d["nreact"], d["lu_nonzero"]) == (356, 353, 3, 1058, 5683)
    assert len(ir["species"]) == 356 and ir["species"][353:] == ["H2", "N2", "O2"]
    lu = ir["lu"]
    assert len(lu["crow"]) == 354 and lu["crow"][-1] == 5683
    for k in range(d["nvar"]):
        row = lu["icol"][lu["crow"][k]:lu["crow"][k + 1]]
        assert row == sorted(row) and lu["icol"][lu["diag"][k]] == k
        assert all(lu["irow"][kk] == k for kk in range(lu["crow"][k], lu["crow"][k + 1]))


def test_ir_matches_reference_sources():
    # the GEOS-Chem source tree, where one is checked out (GEOSCHEM_SRC)
    ref = os.environ.get("GEOSCHEM_SRC", "")
    if not ref or not os.path.isdir(os.path.join(ref, "KPP", "fullchem")):
        pytest.skip("GEOS-Chem source tree not present (set GEOSCHEM_SRC)")
    import importlib.util

    path = os.path.join(ROOT, "geos-chem_gb300", "mechanism", "extract_kpp.py")
    spec = importlib.util.spec_from_file_location("extract_kpp", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    fresh = json.loads(json.dumps(mod.extract(ref)))
    with open(os.path.join(ROOT, "geos-chem_gb300", "mechanism", "fullchem.json")) as fh:
        committed = json.load(fh)
    assert fresh == committed


def test_oracle_fun_jac_bitwise_vs_ir(ir, orc, point):
    V, F, RCT = point
    f_ir = np.array(ir_eval.fun_split(ir, list(V), list(F), list(RCT)))
    f_or = orc.fun_split(V, F, RCT)
    assert np.array_equal(f_ir, f_or)
    j_ir = np.array(ir_eval.jac_sp(ir, list(V), list(F), list(RCT)))
    j_or = orc.jac_sp(V, F, RCT)
    assert np.array_equal(j_ir, j_or)


def test_jacobian_is_derivative_of_fun(ir, orc, point):
    V, F, RCT = point
    n = ir["dims"]["nvar"]
    J = ir_eval.dense_from_lu(ir, orc.jac_sp(V, F, RCT))
    rng = np.random.default_rng(1)
    cols = rng.choice(n, 24, replace=False)
    for j in cols:
        h = V[j] * 1e-20
        Vc = V.astype(complex)
        Vc[j] += 1j * h
        d = np.array(ir_eval.fun_split(ir, list(Vc), list(F.astype(complex)), list(RCT.astype(complex)))).imag / h
        scale = np.maximum(np.abs(d), np.abs(J[:, j])) + 1e-300
        assert np.max(np.abs(d - J[:, j]) / scale) < 1e-9, j


def test_lu_solve_matches_dense(ir, orc, point):
    V, F, RCT = point
    jvs = orc.jac_sp(V, F, RCT)
    G = -jvs.copy()
    ghinv = 1.0 / (30.0 * 0.5)
    G[ir["lu"]["diag"][:-1]] += ghinv
    Gd = ir_eval.dense_from_lu(ir, G)
    lu, ier = orc.decomp(G)
    assert ier == 0
    lu_py, ier_py = ir_eval.decomp(ir, list(G))
    assert ier_py == 0 and np.array_equal(np.array(lu_py), lu)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(ir["dims"]["nvar"])
    x = orc.solve(lu, b)
    assert np.array_equal(x, np.array(ir_eval.solve(ir, list(lu), list(b))))
    xd = np.linalg.solve(Gd, b)
    assert np.max(np.abs(x - xd)) / np.max(np.abs(xd)) < 1e-10


def test_singular_row_detected(ir, orc, point):
    V, F, RCT = point
    G = -orc.jac_sp(V, F, RCT)
    G[ir["lu"]["diag"][:-1]] += 1.0
    k = 17
    G[ir["lu"]["diag"][k]] = 0.0
    _, ier = orc.decomp(G)
    assert ier == k + 1


def _tables_fun(t, V, F, RCT):
    """Interpret the product's lowered tables (STRICT semantics) in Python."""
    aux = list(F) + list(RCT)
    lit = t.literals

    def operand(code):
        if code < t.nvar:
            return V[code]
        if code < t.lit0:
            return aux[code - t.nvar]
        return lit[code - t.lit0]

    Y = list(V) + list(F)
    auxp = list(RCT) + list(t.pre_literals)

    def product(p):
        # packed form used by the CUDA engine: pre [* 2] * s1 * s2 * s3
        x, y = (int(v) for v in t.prod_packed[p])
        a = auxp[x & 0xFFF]
        if x & 0x1000:
            a = a * 2.0
        for k, s in enumerate((x >> 16, y & 0xFFFF, y >> 16)):
            if k < ((x >> 13) & 3):
                a = a * Y[s]
        # the generic factor-list form agrees bit for bit
        s0, e0 = t.prod_start[p], t.prod_start[p + 1]
        if e0 > s0:
            acc = operand(t.prod_fac[s0])
            for i in range(s0 + 1, e0):
                acc = acc * operand(t.prod_fac[i])
            assert acc == a or (acc != acc and a != a)
        return a

    def csum(terms, s, e, X):
        acc = None
        for u in terms[s:e].view(np.uint32):
            c = (int(u) >> 20) & 0x7FF
            x = X[int(u) & 0xFFFFF]
            v = x if c == tables.NOCOEF else lit[c] * x
            neg = (int(u) >> 31) != 0
            acc = (-v if neg else v) if acc is None else (acc - v if neg else acc + v)
        return 0.0 if acc is None else acc

    A = [product(r) for r in range(t.nreact)]
    B = [product(t.nreact + b) if t.prod_start[t.nreact + b + 1] > t.prod_start[t.nreact + b] else 0.0
         for b in range(t.nb)]
    out = []
    for i in range(t.nvar):
        p = csum(t.p_term, t.p_start[i], t.p_start[i + 1], A)
        d = csum(t.d_term, t.d_start[i], t.d_start[i + 1], B)
        out.append(p - d * V[i])
    jac = [csum(t.j_term, t.j_start[k], t.j_start[k + 1], B) for k in range(t.lu_nonzero)]
    return np.array(out), np.array(jac)


def test_product_tables_reproduce_oracle(ir, orc, point):
    V, F, RCT = point
    t = tables.Tables(ir)
    f, j = _tables_fun(t, list(V), list(F), list(RCT))
    assert np.array_equal(f, orc.fun_split(V, F, RCT))
    assert np.array_equal(j, orc.jac_sp(V, F, RCT))
    # LU program: replay lop/uop against KppDecomp
    G = -orc.jac_sp(V, F, RCT)
    G[ir["lu"]["diag"][:-1]] += 0.25
    ref, _ = orc.decomp(G)
    g = list(G)
    for k in range(t.nvar):
        for l in range(t.lrow_start[k], t.lrow_start[k + 1]):
            kk, dj = t.lop_kk[l], t.lop_dj[l]
            a = -g[kk] / g[dj]
            g[kk] = -a
            for u in t.uop[t.lop_u[l]:t.lop_u[l + 1]].view(np.uint32):
                tt, ss = int(u) >> 16, int(u) & 0xFFFF
                g[tt] = g[tt] + a * g[ss]
    assert np.array_equal(np.array(g), ref)
    # row-wise dot-product form (decomp_rows): same updates, same order
    h = [0.0] * t.lu_nonzero
    for k in range(t.nvar):
        for e in range(t.crow[k], t.crow[k + 1]):
            acc = G[e]
            for u in t.dot_term[t.dot_start[e]:t.dot_start[e + 1]].view(np.uint32):
                acc = acc - h[int(u) >> 16] * h[int(u) & 0xFFFF]
            if e < t.diag[k]:
                acc = acc / h[t.diag[t.icol[e]]]
            h[e] = acc
    assert np.array_equal(np.array(h), ref)


def test_flop_counts(ir):
    f = tables.Tables(ir).flops()
    # per-call FP64 operation counts of the generated routines
    assert 9000 < f["fun"] < 13000
    assert 8000 < f["jac"] < 16000
    assert f["decomp"] == 2 * 20790 + 2773 + 353
    assert f["solve"] == 2 * 5330 + 353
