"""Plain-Python evaluation of the mechanism IR, for the CPU tests.

Independent of both the oracle's C code generator and the product's table
lowering: it walks the IR statements directly, with Python floats (IEEE
double, no contraction) in the statements' left-to-right order, so its
results are bit-for-bit those of the KPP-generated Fortran's arithmetic.
Works with complex numbers too (complex-step derivatives).
"""
import numpy as np


def _val(tok, V, F, RCT, lit=float):
    k = tok[0]
    if k == "V":
        return V[int(tok[1:])]
    if k == "F":
        return F[int(tok[1:])]
    if k == "R":
        return RCT[int(tok[1:])]
    return lit(tok.replace("d", "e"))


def _prod(toks, V, F, RCT):
    if not toks:  # a rate KPP leaves uncomputed (never referenced)
        return 0.0
    acc = _val(toks[0], V, F, RCT)
    for t in toks[1:]:
        acc = acc * _val(t, V, F, RCT)
    return acc


def _coef_sum(terms, X):
    if not terms:
        return 0.0
    acc = None
    for sign, coef, idx in terms:
        v = X[idx] if coef is None else float(coef) * X[idx]
        if acc is None:
            acc = -v if sign == "-" else v
        else:
            acc = acc - v if sign == "-" else acc + v
    return acc


def _prod_sum(terms, V, F, RCT):
    if not terms:
        return 0.0
    acc = None
    for sign, fac in terms:
        v = _prod(fac, V, F, RCT)
        if acc is None:
            acc = -v if sign == "-" else v
        else:
            acc = acc - v if sign == "-" else acc + v
    return acc


def fun_split(ir, V, F, RCT):
    A = [_prod(f, V, F, RCT) for f in ir["fun"]["A"]]
    out = []
    for i in range(ir["dims"]["nvar"]):
        p = _coef_sum(ir["fun"]["P"][i], A)
        d = _prod_sum(ir["fun"]["D"][i], V, F, RCT)
        out.append(p - d * V[i])
    return out


def jac_sp(ir, V, F, RCT):
    B = [(_prod(f, V, F, RCT) if f is not None else None) for f in ir["jac"]["B"]]
    return [_coef_sum(t, B) for t in ir["jac"]["JVS"]]


def dense_from_lu(ir, jvs):
    n = ir["dims"]["nvar"]
    M = np.zeros((n, n), dtype=np.asarray(jvs).dtype)
    M[ir["lu"]["irow"], ir["lu"]["icol"]] = jvs
    return M


def decomp(ir, jvs):
    """KppDecomp (KPP/fullchem/gckpp_LinearAlgebra.F90:46-83) in Python."""
    lu = ir["lu"]
    crow, diag, icol = lu["crow"], lu["diag"], lu["icol"]
    J = list(jvs)
    W = [0.0] * ir["dims"]["nvar"]
    for k in range(ir["dims"]["nvar"]):
        if abs(J[diag[k]]) < np.finfo(float).tiny:
            return J, k + 1
        for kk in range(crow[k], crow[k + 1]):
            W[icol[kk]] = J[kk]
        for kk in range(crow[k], diag[k]):
            j = icol[kk]
            a = -W[j] / J[diag[j]]
            W[j] = -a
            for jj in range(diag[j] + 1, crow[j + 1]):
                W[icol[jj]] = W[icol[jj]] + a * J[jj]
        for kk in range(crow[k], crow[k + 1]):
            J[kk] = W[icol[kk]]
    return J, 0


def solve(ir, jvs, x):
    """KppSolve statement order (KPP/fullchem/gckpp_LinearAlgebra.F90:644-2309)."""
    X = list(x)
    for st in ir["solve"]:
        i = st["row"]
        v = X[i]
        for k, j in st["terms"]:
            v = v - jvs[k] * X[j]
        if st["kind"] == "B":
            v = v / jvs[st["diag"]]
        X[i] = v
    return X
