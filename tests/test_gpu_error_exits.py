"""GPU tests of the integrator's error exits and of non-finite inputs, all
made on the host, against the CPU oracle: IERR, ISTATUS, RSTATUS and the
concentrations of every cell.

* -7, step size too small (KPP/fullchem/gckpp_Integrator.F90:659-662): a
  maximum step RCNTRL(2) below Roundoff (the first step runs with DeltaMin,
  :638, the next is clamped to Hmax), and a start time so large that
  T + 0.1*H == T before the first step.
* Singular decompositions (ros_PrepareMatrix, :1977-1995): rates that make
  one diagonal of Ghimj = 1/(H*gamma) - Jac0 exactly zero at the first H
  (one singular decomposition, H halved, then the integration goes on), and
  a step of infinite length over zero rates, where 1/(H*gamma) = 0 at every
  halving: the sixth consecutive singular matrix ends the cell with -8.
* NaN and Inf rate constants under the MIN/MAX policy of both sides (fmin /
  fmax: the non-NaN operand wins): ros_ErrorNorm's floor MAX(Err, 1e-10)
  turns a NaN norm into 1e-10, so the steps are accepted and the NaN
  propagates to the result with IERR = 1.
* The caller's retry (GeosCore/fullchem_mod.F90:1138-1162) of -7 cells.
"""
import numpy as np
import pytest

import gcchem.capi as capi
import gcchem.inputs as inputs
import gcchem.mechanism as mechanism

pytestmark = pytest.mark.gpu
NVAR = 353


@pytest.fixture(scope="module")
def case(orc):
    n = 96
    cells = inputs.box_cells(n, seed=41)
    r = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    return dict(n=n, cells=cells, r=r, atol=atol, rtol=rtol, ic=ic, rc=rc)


def _gpu(solver, c, r, case, tin, tout, arith, ic=None, rc=None, hstart=None):
    solver.set(arith=arith, schedule="plain", block=0)
    n = c.shape[1]
    c = c.copy()
    ist = np.zeros((20, n), np.int32)
    rst = np.zeros((20, n))
    ierr = np.zeros(n, np.int32)
    solver.integrate(c, r, case["atol"], case["rtol"], tin, tout, case["ic"] if ic is None else ic,
                     case["rc"] if rc is None else rc, hstart=hstart, istatus=ist, rstatus=rst, ierr=ierr)
    return c, ist, rst, ierr


def _same(got, ref, bar=1e-9, strict_seq=True):
    c, ist, rst, ierr = got
    c_ref, ist_ref, rst_ref, ierr_ref = ref
    assert np.array_equal(ierr, ierr_ref)
    if strict_seq:
        assert np.array_equal(ist[:8], ist_ref[:8])
        # Texit, Hexit, Hnew: the step-size factors come from pow (CUDA's and
        # glibc's differ in the last bit), so to the concentrations' bar
        assert np.allclose(rst[:3], rst_ref[:3], rtol=bar, atol=0)
    a, b = c[:NVAR], c_ref[:NVAR]
    assert np.array_equal(np.isnan(a), np.isnan(b))
    fin = np.isfinite(b) & (np.abs(b) > 1e4)
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    assert np.all(np.where(fin, rel, 0.0) < bar)


@pytest.mark.parametrize("arith", ["strict", "fast"])
@pytest.mark.parametrize("how", ["hmax", "tstart"])
def test_step_too_small_gives_minus7(solver, orc, case, arith, how):
    rc = case["rc"].copy()
    tin, tout = 0.0, 600.0
    if how == "hmax":
        rc[1] = 1.0e-20  # RCNTRL(2): every step after the first is below Roundoff
    else:
        tin, tout = 1.0e17, 1.0e17 + 600.0  # ulp(T) = 16 s: T + 0.1*H == T
    c0 = case["cells"]["c"]
    ref = orc.integrate(c0, case["r"], case["atol"], case["rtol"], tin, tout, case["ic"], rc)
    got = _gpu(solver, c0, case["r"], case, tin, tout, arith, rc=rc)
    assert np.all(ref[3] == -7)
    _same(got, ref, strict_seq=(arith == "strict" or how == "tstart"))
    if how == "tstart":
        assert np.all(got[1][:8] == 0)
        assert np.array_equal(got[0], c0)


def _ghinv_zero_rates(orc, ir, n):
    """Rates with only NO2 photolysis (R884 in the IR, PHOTOL(11)) set to -4:
    Jac0(NO2, NO2) = 4 = 1/(H*gamma1) at H = 0.5 for Rodas3 (gamma1 = 0.5)."""
    r = np.zeros((ir["dims"]["nreact"], n))
    k = next(i for i, a in enumerate(ir["fun"]["A"]) if a == ["R%d" % i, "V%d" % ir["species"].index("NO2")]
             and ir["rconst"][i].startswith("(PHOTOL"))
    r[k] = -4.0
    return r, k


@pytest.mark.parametrize("arith", ["strict", "fast"])
def test_one_singular_decomposition_halves_h(solver, orc, case, arith):
    ir = mechanism.load_ir()
    n = case["n"]
    r, k = _ghinv_zero_rates(orc, ir, n)
    c0 = case["cells"]["c"]
    ino2 = ir["species"].index("NO2")
    jac = orc.jac_sp(c0[:NVAR, 0], c0[NVAR:, 0], r[:, 0])
    assert jac[ir["lu"]["diag"][ino2]] == 4.0
    hs = np.full(n, 0.5)
    ref = orc.integrate(c0, r, case["atol"], case["rtol"], 0.0, 1.0, case["ic"], case["rc"], hstart=hs)
    got = _gpu(solver, c0, r, case, 0.0, 1.0, arith, hstart=hs)
    assert np.all(ref[1][7] >= 1)  # ISTATUS(Nsng): the first decomposition was singular
    assert np.all(ref[3] == 1)
    _same(got, ref, strict_seq=(arith == "strict"))
    assert np.all(got[1][7] >= 1)


@pytest.mark.parametrize("arith", ["strict", "fast"])
def test_six_singular_decompositions_give_minus8(solver, orc, case, arith):
    n = case["n"]
    r = np.zeros_like(case["r"])
    hs = np.full(n, np.inf)
    c0 = case["cells"]["c"]
    ref = orc.integrate(c0, r, case["atol"], case["rtol"], 0.0, np.inf, case["ic"], case["rc"], hstart=hs)
    got = _gpu(solver, c0, r, case, 0.0, np.inf, arith, hstart=hs)
    assert np.all(ref[3] == -8)
    assert np.all(ref[1][5] == 6) and np.all(ref[1][7] == 6)  # Ndec, Nsng
    _same(got, ref)
    assert np.array_equal(got[0], c0)


@pytest.mark.parametrize("arith", ["strict", "fast"])
def test_nonfinite_rates_follow_the_min_max_policy(solver, orc, case, arith):
    n = case["n"]
    r = case["r"].copy()
    r[:, 0] = np.nan  # every rate of cell 0
    r[884, 1] = np.nan  # one photolysis rate
    r[100, 2] = np.inf
    r[:, 3] = np.inf
    r[884, 4] = -np.inf
    c0 = case["cells"]["c"]
    ref = orc.integrate(c0, r, case["atol"], case["rtol"], 0.0, 600.0, case["ic"], case["rc"])
    got = _gpu(solver, c0, r, case, 0.0, 600.0, arith)
    bad = slice(0, 5)
    # the non-finite cells: same exit, counters and non-finite pattern
    assert np.array_equal(got[3][bad], ref[3][bad])
    if arith == "strict":
        assert np.array_equal(got[1][:8, bad], ref[1][:8, bad])
    assert np.array_equal(np.isnan(got[0][:NVAR, bad]), np.isnan(ref[0][:NVAR, bad]))
    assert np.array_equal(np.isinf(got[0][:NVAR, bad]), np.isinf(ref[0][:NVAR, bad]))
    # the cells beside them are unaffected (parity bar)
    _same(tuple(x[..., 5:] for x in got), tuple(x[..., 5:] for x in ref), strict_seq=(arith == "strict"))


def test_retry_of_minus7_cells(solver, orc, case):
    """Every cell fails with -7 (a maximum step below Roundoff), is
    integrated once more from C_before with Hstart = 0
    (fullchem_mod.F90:1138-1162), fails again and keeps IERR = -7; ISTATUS
    and RSTATUS are the second integration's, the concentrations are clamped
    at zero."""
    ir = mechanism.load_ir()
    n = case["n"]
    cells = case["cells"]
    rc = case["rc"].copy()
    rc[1] = 1.0e-20
    ic = case["ic"]
    # the reference loop body: zero families, rates, integrate, retry, clamp
    c = cells["c"].copy()
    for fam in ir["families"]:
        c[ir["species"].index(fam)] = 0.0
    r = orc.update_rconst(cells["met"], cells["photol"], c)
    hs = np.full(n, 7.0)  # KPPHvalue of the first attempt
    c1, ist, rst, ierr = orc.integrate(c, r, case["atol"], case["rtol"], 0.0, 600.0, ic, rc, hstart=hs)
    assert np.all(ierr == -7)
    c1, ist, rst, ierr = orc.integrate(c, r, case["atol"], case["rtol"], 0.0, 600.0, ic, rc)
    assert np.all(ierr == -7)
    c_ref = np.maximum(c1, 0.0)
    solver.set(arith="strict", schedule="plain", block=0)
    cg = cells["c"].copy()
    istg = np.zeros((20, n), np.int32)
    rstg = np.zeros((20, n))
    ierrg = np.zeros(n, np.int32)
    hsg = hs.copy()
    nretry = solver.fullchem_step(600.0, cells["met"], cells["photol"], cg, case["atol"], case["rtol"], ic, rc, hsg,
                                  istg, rstg, ierrg)
    assert nretry == n
    assert np.array_equal(ierrg, ierr)
    assert np.array_equal(istg[:8], ist[:8])
    assert np.all(cg >= 0.0)
    big = np.abs(c_ref[:NVAR]) > 1e4
    rel = np.abs(cg[:NVAR] - c_ref[:NVAR]) / np.maximum(np.abs(c_ref[:NVAR]), 1e-300)
    assert np.max(np.where(big, rel, 0.0)) < 1e-9
    # KPPHvalue is RSTATE(Nhnew) of the last integration
    assert np.array_equal(hsg, rstg[2])
