"""The Rosenbrock method tables pinned by mathematics: the coefficients of
Ros2, Ros3, Ros4, Rodas3, Rodas4 and Rang3 (KPP/fullchem/gckpp_Integrator.F90
:2060-2480, in KPP's transformed form A, C, M, E with the diagonal gamma =
ros_Gamma(1)) are converted back to the standard Rosenbrock form
(alpha_ij, gamma_ij, b_i; Hairer & Wanner, Solving ODEs II, IV.7, eq. 7.3')
and must satisfy the order conditions of their published order (ibid. Table
7.1), their embedded error estimators those of order ELO - 1, and
ros_Alpha / ros_Gamma must be the row sums of alpha / gamma.  The kernels'
tables (csrc/ros_methods.h) and the oracle's (oracle/kpp_oracle.c) are read
from their sources and must be the same numbers."""
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORDER = {1: 2, 2: 3, 3: 4, 4: 3, 5: 4, 6: 3}  # Ros2, Ros3, Ros4, Rodas3, Rodas4, Rang3
FIELDS = ("S", "A", "C", "M", "E", "Alpha", "Gamma", "NewF", "ELO")


class _Method:
    def __init__(self):
        self.S, self.ELO = 0, 0.0
        self.A, self.C = [0.0] * 15, [0.0] * 15
        self.M, self.E, self.Alpha, self.Gamma = [0.0] * 6, [0.0] * 6, [0.0] * 6, [0.0] * 6
        self.NewF = [0] * 6


def _run(code):
    """Executes C assignments to the method record r as Python."""
    code = re.sub(r"//[^\n]*|/\*.*?\*/", "", code, flags=re.S)
    code = code.replace("r->", "r.").replace("std::sqrt", "math.sqrt").replace("const double ", "")
    code = re.sub(r"\bdouble ", "", code)
    code = re.sub(r"(?<![\w.])sqrt\(", "math.sqrt(", code)
    code = re.sub(r"for \(int i = 0; i < (\d+); \+\+i\) (.*?);", r"\nfor i in range(\1): \2\n", code)
    r = _Method()
    exec("\n".join(line.strip() for line in code.splitlines() if line.strip()), {"math": math, "r": r})
    return r


def _kernel_tables():
    text = open(os.path.join(ROOT, "geos-chem_gb300", "csrc", "ros_methods.h")).read()
    text = text[text.index("inline bool method_coefficients"):]
    return {int(m.group(1)): _run(m.group(2))
            for m in re.finditer(r"case (\d+): \{[^\n]*\n(.*?)return true;", text, re.S)}


def _oracle_tables():
    text = open(os.path.join(ROOT, "oracle", "kpp_oracle.c")).read()
    text = text[text.index("static int method_init"):]
    text = text[:text.index("\n}\n")]
    out = {}
    for m in re.finditer(r"if \(id == (\d+)((?: \|\| id == \d+)*)\) \{ /\* \w+ \*/\n(.*?)\n  \}", text, re.S):
        r = _run(m.group(3))
        for i in [int(m.group(1))] + [int(x) for x in re.findall(r"\d+", m.group(2))]:
            out[i] = r
    return out


def _standard_form(r):
    """(gamma, alpha, gamma_ij off the diagonal, b, b of the embedded method,
    the full gamma matrix) of a method in KPP's transformed form."""
    S, g = r.S, r.Gamma[0]
    A, C = np.zeros((S, S)), np.zeros((S, S))
    for i in range(S):
        for j in range(i):
            A[i, j] = r.A[i * (i - 1) // 2 + j]
            C[i, j] = r.C[i * (i - 1) // 2 + j]
    G = np.linalg.inv(np.diag(np.full(S, 1.0 / g)) - C)
    M, E = np.array(r.M[:S]), np.array(r.E[:S])
    return g, A @ G, G - np.diag(np.diag(G)), M @ G, (M - E) @ G, G


def _residuals(g, alpha, gam, b, p):
    beta = alpha + gam
    a, bp = alpha.sum(1), beta.sum(1)
    res = [b.sum() - 1.0]
    if p >= 2:
        res.append(b @ bp - (0.5 - g))
    if p >= 3:
        res += [b @ a ** 2 - 1.0 / 3.0, b @ (beta @ bp) - (1.0 / 6.0 - g + g * g)]
    if p >= 4:
        res += [b @ a ** 3 - 0.25, b @ (a * (alpha @ bp)) - (1.0 / 8.0 - g / 3.0),
                b @ (beta @ a ** 2) - (1.0 / 12.0 - g / 3.0),
                b @ (beta @ (beta @ bp)) - (1.0 / 24.0 - g / 2.0 + 1.5 * g * g - g ** 3)]
    return np.abs(np.array(res))


@pytest.fixture(scope="module")
def tables():
    return _kernel_tables(), _oracle_tables()


def test_kernel_and_oracle_tables_are_the_same_numbers(tables):
    k, o = tables
    assert sorted(k) == [1, 2, 3, 4, 5, 6] and set(k) <= set(o)
    for i in k:
        for f in FIELDS:
            assert getattr(k[i], f) == getattr(o[i], f), (i, f)
    assert o[0] is o[4]  # method 0 (the default) is Rodas3


@pytest.mark.parametrize("mid", [1, 2, 3, 4, 5, 6])
def test_order_conditions(tables, mid):
    r = tables[0][mid]
    g, alpha, gam, b, bh, G = _standard_form(r)
    p = ORDER[mid]
    assert _residuals(g, alpha, gam, b, p).max() < 1e-13
    assert _residuals(g, alpha, gam, bh, int(r.ELO) - 1).max() < 1e-13  # embedded estimator
    assert np.abs(np.array(r.Alpha[:r.S]) - alpha.sum(1)).max() < 1e-13
    assert np.abs(np.array(r.Gamma[:r.S]) - G.sum(1)).max() < 1e-13
    if p < 4:  # the method is of exactly its order: some condition of order p + 1 fails
        assert _residuals(g, alpha, gam, b, p + 1)[len(_residuals(g, alpha, gam, b, p)):].max() > 1e-3


def test_a_wrong_coefficient_breaks_the_conditions(tables):
    r = _kernel_tables()[4]  # a fresh copy of Rodas3
    r.C[5] *= 1.0 + 1e-6
    g, alpha, gam, b, bh, G = _standard_form(r)
    assert _residuals(g, alpha, gam, b, 3).max() > 1e-8
