"""A second KPP mechanism on the same engine: GEOS-Chem's Hg mechanism
(KPP/Hg, 43 species, 94 reactions, LU_NONZERO 161), extracted by the same
extractor into mechanism/Hg.json and built into libgckpp_gb300_Hg.so with the
same (table-driven) kernels."""
import ctypes
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))


@pytest.fixture(scope="module")
def hg():
    import gcchem.mechanism as mechanism

    return mechanism.load_ir("Hg")


def test_hg_oracle_matches_ir(hg):
    """The oracle's Fun_SPLIT and Jac_SP for Hg equal a statement-by-statement
    evaluation of the extracted IR, bit for bit."""
    import ir_eval
    import oracle

    rng = np.random.default_rng(3)
    d = hg["dims"]
    for _ in range(3):
        v = rng.lognormal(10, 4, d["nvar"])
        f = rng.lognormal(10, 4, d["nfix"])
        rct = rng.lognormal(-15, 4, d["nreact"])
        assert np.array_equal(oracle.fun_split(v, f, rct, mech="Hg"), np.array(ir_eval.fun_split(hg, v, f, rct)))
        assert np.array_equal(oracle.jac_sp(v, f, rct, mech="Hg"), np.array(ir_eval.jac_sp(hg, v, f, rct)))


def test_hg_library_dims():
    import gcchem.build as build
    import gcchem.capi as capi

    if not os.path.exists(build.lib_path("Hg")):
        pytest.skip("library not built")
    assert capi.dims("Hg") == {"nspec": 43, "nvar": 32, "nfix": 11, "nreact": 94, "lu_nonzero": 161}
    assert capi.dims("fullchem")["nspec"] == 356


@pytest.mark.gpu
@pytest.mark.parametrize("arith", ["strict", "fast"])
def test_hg_gpu_matches_oracle(hg, arith):
    import gcchem.capi as capi
    import gcchem.inputs as inputs
    import oracle

    n = 256
    cells = inputs.box_cells(n, seed=4, ir=hg)
    atol, rtol = inputs.tolerances(hg)
    icntrl, rcntrl = inputs.default_controls()
    s = capi.Solver(0, arith=arith, schedule="queue", mech="Hg")
    r = np.zeros((hg["dims"]["nreact"], n))
    s.update_rconst(cells["met"], cells["photol"], cells["c"], r)
    r_ref = oracle.update_rconst(cells["met"], cells["photol"], cells["c"], mech="Hg")
    assert np.allclose(r, r_ref, rtol=1e-13, atol=0)
    c = cells["c"].copy()
    ist = np.zeros((20, n), np.int32)
    ierr = np.zeros(n, np.int32)
    s.integrate(c, r_ref, atol, rtol, 0.0, 3600.0, icntrl, rcntrl, istatus=ist, ierr=ierr)
    c_ref, ist_ref, _, ierr_ref = oracle.integrate(cells["c"], r_ref, atol, rtol, 0.0, 3600.0, icntrl, rcntrl,
                                                   mech="Hg")
    nvar = hg["dims"]["nvar"]
    assert np.array_equal(ierr, ierr_ref) and np.all(ierr == 1)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    big = np.abs(c_ref[:nvar]) > 1e4
    rel = np.abs(c[:nvar] - c_ref[:nvar]) / np.maximum(np.abs(c_ref[:nvar]), 1e-300)
    # the fullchem parity bar: 1e-9 relative on species > 1e4 molec/cm3 on every
    # cell whose step sequence matches; strict cells all take the oracle's steps
    # (the step-size factor's Err**(1/3) comes from CUDA's pow, not glibc's, so
    # the values agree to rounding rather than bit for bit)
    assert same.mean() >= 0.99 and np.max(np.where(big, rel, 0.0)[:, same]) < 1e-9
    assert np.array_equal(c[nvar:], c_ref[nvar:])
    if arith == "strict":
        assert same.all()
