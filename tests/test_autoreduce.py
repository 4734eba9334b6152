"""Auto-reduction, the CPU restatement: ros_yIntegrator of
KPP/fullchem/gckpp_Integrator.F90:789-1237 with cKppDecomp (:2624-2661),
the DO_SLV-guarded KppSolve and AutoReduce_1stOrder (:1702-1712), selected by
ICNTRL(12) = 1 as INTEGRATE does (:388-394, :478-520).  The GPU solver does
not run it yet (ICNTRL(12) = 1 is refused with GC_KPP_EUNSUPPORTED)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def case():
    import gcchem.inputs as inputs
    import oracle

    n = 48
    cells = inputs.box_cells(n, seed=31)
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    r = oracle.update_rconst(cells["met"], cells["photol"], cells["c"])
    full = oracle.integrate(cells["c"], r, atol, rtol, 0.0, 600.0, ic, rc)
    return dict(cells=cells, atol=atol, rtol=rtol, ic=ic, rc=rc, r=r, full=full)


def _ar(case, thr=None, target=0, ratio=0.0, append=False):
    import oracle

    ic = case["ic"].copy()
    rc = case["rc"].copy()
    ic[11] = 1
    if append:
        ic[12] = 1
    if thr is not None:
        rc[11] = thr
    if target:
        ic[13] = target
        rc[13] = ratio
    return oracle.integrate(case["cells"]["c"], case["r"], case["atol"], case["rtol"], 0.0, 600.0, ic, rc)


def test_nothing_removed_is_the_full_integrator(case):
    """With a threshold below every production and loss rate no species is
    frozen, and ros_yIntegrator performs ros_Integrator's arithmetic."""
    c, ist, rst, ierr = _ar(case, thr=1e-300)
    c0, ist0, rst0, ierr0 = case["full"]
    assert np.all(ierr == 1)
    assert np.array_equal(c, c0) and np.array_equal(ist[:8], ist0[:8]) and np.array_equal(rst[:3], rst0[:3])


def test_reduced_integration_stays_close(case):
    """The default threshold (100 molec/cm3/s) freezes the slow species; the
    integration succeeds on every cell, takes no more steps than the full one
    on average, and the bulk of the species stays within the reduction's
    approximation."""
    c, ist, _, ierr = _ar(case)
    c0, ist0, _, _ = case["full"]
    assert np.all(ierr == 1)
    assert ist[2].mean() <= ist0[2].mean()
    big = np.abs(c0[:353]) > 1e4
    rel = np.abs(c[:353] - c0[:353]) / np.maximum(np.abs(c0[:353]), 1e-300)
    assert np.median(rel[big]) < 1e-3
    assert not np.array_equal(c, c0)  # something was frozen


def test_target_species_threshold_is_reported(case):
    """ICNTRL(14) = OH: the threshold is RCNTRL(14) x max(P, L*y) of OH at the
    first step, reported in RSTATUS(NARthr = 4)."""
    import oracle
    from gcchem.mechanism import load_ir

    ir = load_ir()
    oh = ir["species"].index("OH")
    c, ist, rst, ierr = _ar(case, target=oh + 1, ratio=1e-3)
    assert np.all(ierr == 1)
    cells = case["cells"]
    # P and L*y of OH at the initial state (Fun_SPLITF's P_VAR and D_VAR*y)
    nvar, nfix = ir["dims"]["nvar"], ir["dims"]["nfix"]
    for k in range(cells["c"].shape[1]):
        v = cells["c"][:nvar, k].copy()
        f = cells["c"][nvar:nvar + nfix, k].copy()
        p, d = oracle.fun_pd(v, f, case["r"][:, k])
        assert rst[3, k] == 1e-3 * max(d[oh] * v[oh], p[oh])
        vdot = oracle.fun_split(v, f, case["r"][:, k])
        assert np.array_equal(vdot, p - d * v)  # Fun_SPLITF and Fun_SPLIT agree


def test_append_form_is_not_restated(case):
    c, ist, rst, ierr = _ar(case, append=True)
    assert np.all(ierr == -100)


@pytest.mark.parametrize("thr", [1e2, 1e5])
def test_masked_full_decomposition_equals_the_compressed_one(case, thr):
    """The design of the GPU form: zeroing every Jac0 entry in a frozen row
    or column and factoring the full Ghimj = -Jac0 + ghinv I (ICNTRL(20) = 7
    selects it in the oracle) gives the compressed cKppDecomp path's
    integration bit for bit -- frozen entries only ever contribute exact
    zeros."""
    import oracle

    ic = case["ic"].copy()
    rc = case["rc"].copy()
    ic[11] = 1
    rc[11] = thr
    a = oracle.integrate(case["cells"]["c"], case["r"], case["atol"], case["rtol"], 0.0, 600.0, ic, rc)
    ic[19] = 7
    b = oracle.integrate(case["cells"]["c"], case["r"], case["atol"], case["rtol"], 0.0, 600.0, ic, rc)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
