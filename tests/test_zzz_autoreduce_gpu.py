"""Auto-reduction on the GPU (ICNTRL(12) = 1, ros_yIntegrator of
KPP/fullchem/gckpp_Integrator.F90:789-1237) through the C ABI, against the
oracle's restatement of the same integrator.

The thread-per-cell kernel runs it with the full sparsity pattern: the
Jacobian rows and columns of the frozen species are zeroed, so that
-Jac0 + ghinv I factors like the reference's compressed matrix (the oracle
shows the two bit for bit, tests/test_autoreduce.py), the frozen stage
vectors stay 0 and the frozen species take AutoReduce_1stOrder (:1702-1712)
at the end.  The append form (ros_yIntegratorA, :1242-1700) masks an
appended species' column in the rows that entered before it.

Collected last (file name), after the allocation-free entry point."""
import numpy as np
import pytest

import gcchem.capi as capi
import gcchem.inputs as inputs

pytestmark = pytest.mark.gpu

NVAR = 353


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


@pytest.fixture(scope="module")
def case(orc):
    n = 256
    cells = inputs.box_cells(n, seed=41)
    rconst = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    return dict(n=n, cells=cells, rconst=rconst, atol=atol, rtol=rtol, icntrl=icntrl, rcntrl=rcntrl)


def _controls(case, thr=None, target=0, ratio=0.0, append=False, on=True):
    ic = case["icntrl"].copy()
    rc = case["rcntrl"].copy()
    if on:
        ic[11] = 1
    if append:
        ic[12] = 1
    if thr is not None:
        rc[11] = thr
    if target:
        ic[13] = target
        rc[13] = ratio
    return ic, rc


def _gpu(solver, case, ic, rc, arith="strict", schedule="plain"):
    solver.set(arith=arith, schedule=schedule, block=0)
    n = case["n"]
    c = case["cells"]["c"].copy()
    ist = np.zeros((20, n), np.int32)
    rst = np.zeros((20, n))
    ierr = np.zeros(n, np.int32)
    solver.integrate(c, case["rconst"], case["atol"], case["rtol"], 0.0, 600.0, ic, rc, istatus=ist, rstatus=rst,
                     ierr=ierr)
    return c, ist, rst, ierr


def _oracle(orc, case, ic, rc, rconst=None, **kw):
    r = case["rconst"] if rconst is None else rconst
    return orc.integrate(case["cells"]["c"], r, case["atol"], case["rtol"], 0.0, 600.0, ic, rc, **kw)


def _check(orc, case, got, ref, ic, rc, scale=1e-15, c_in=None, rconst=None, clamp=False, **kw):
    """The parity bar of the full integrator: 1e-9 relative on species above
    1e4 molec/cm3, on every cell whose step sequence matches the oracle's
    (at least 99 % of them).  A cell whose reduction or append decision sits
    at its threshold amplifies rounding: there the bar is 10x the oracle's own
    spread when its rate constants move by `scale` relative (two draws), so
    that the GPU is held to the oracle's conditioning, not beyond it."""
    c, ist, _, ierr = got
    c_ref, ist_ref, _, ierr_ref = ref
    assert np.array_equal(ierr, ierr_ref)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.99, same.mean()
    big = np.abs(c_ref[:NVAR]) > 1e4
    c_in = case["cells"]["c"] if c_in is None else c_in
    rconst = case["rconst"] if rconst is None else rconst
    spread = np.zeros(case["n"])
    for seed in (1, 2):
        rng = np.random.default_rng(seed)
        rp = rconst * (1.0 + rng.uniform(-scale, scale, rconst.shape))
        x = orc.integrate(c_in, rp, case["atol"], case["rtol"], 0.0, 600.0, ic, rc, **kw)[0]
        if clamp:
            x = np.maximum(x, 0.0)
        spread = np.maximum(spread, np.max(np.where(big, _rel(x[:NVAR], c_ref[:NVAR]), 0.0), axis=0))
    bar = np.maximum(1e-9, 10.0 * spread)
    dev = np.max(np.where(big, _rel(c[:NVAR], c_ref[:NVAR]), 0.0), axis=0)
    bad = np.nonzero(same & (dev >= bar))[0]
    assert bad.size == 0, (bad[:5], dev[bad][:5], bar[bad][:5])
    assert np.mean(bar > 1e-9) <= 0.05  # the exception stays an exception
    return same


@pytest.mark.parametrize("append", [False, True])
@pytest.mark.parametrize("arith", ["strict", "fast"])
@pytest.mark.parametrize("thr", [1e2, 1e5])
def test_autoreduce_matches_oracle(solver, orc, case, arith, thr, append):
    """The parity bar of the full integrator: 1e-9 relative on species above
    1e4 molec/cm3, on every cell whose step sequence matches the oracle's;
    with append (ICNTRL(13) = 1, ros_yIntegratorA) too."""
    ic, rc = _controls(case, thr=thr, append=append)
    got = _gpu(solver, case, ic, rc, arith=arith)
    ref = _oracle(orc, case, ic, rc)
    assert np.all(ref[3] == 1)
    same = _check(orc, case, got, ref, ic, rc)
    if arith == "strict":
        assert same.all()
    # and the reduction changed the answer (something was frozen)
    c_full = _oracle(orc, case, *_controls(case, on=False))[0]
    assert not np.array_equal(ref[0], c_full)


def test_target_species_threshold(solver, orc, case, ir):
    """ICNTRL(14) = OH, RCNTRL(14) = 1e-3: the threshold from OH's P and
    L*y at Tstart, reported in RSTATUS(4)."""
    oh = ir["species"].index("OH")
    ic, rc = _controls(case, target=oh + 1, ratio=1e-3)
    got = _gpu(solver, case, ic, rc)
    ref = _oracle(orc, case, ic, rc)
    assert np.all(got[3] == 1) and np.all(ref[3] == 1)
    assert np.max(_rel(got[2][3], ref[2][3])) < 1e-12
    _check(orc, case, got, ref, ic, rc)


@pytest.mark.parametrize("append", [False, True])
@pytest.mark.parametrize("arith", ["strict", "fast"])
def test_nothing_frozen_is_the_full_integrator(solver, case, arith, append):
    """A threshold below every rate freezes nothing (and leaves nothing to
    append): the auto-reduce kernel then performs the regular kernel's
    arithmetic, bit for bit."""
    a = _gpu(solver, case, *_controls(case, thr=1e-300, append=append), arith=arith)
    b = _gpu(solver, case, *_controls(case, on=False), arith=arith)
    assert np.array_equal(a[0], b[0])
    assert np.array_equal(a[1][:8], b[1][:8])
    assert np.array_equal(a[2][:3], b[2][:3])
    assert np.array_equal(a[3], b[3])


def test_queue_schedule_bit_identical_to_plain(solver, case):
    ic, rc = _controls(case)
    a = _gpu(solver, case, ic, rc, arith="fast", schedule="plain")
    b = _gpu(solver, case, ic, rc, arith="fast", schedule="queue")
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_fullchem_step_with_autoreduce(solver, orc, case, ir):
    """Do_FullChem's cell loop with ICNTRL(12) = 1 (the retry on failure and
    the final clamp run the same way) against the oracle's loop."""
    ic, rc = _controls(case)
    cells = case["cells"]
    n = case["n"]
    solver.set(arith="strict", schedule="plain", block=0)
    c = cells["c"].copy()
    ist = np.zeros((20, n), np.int32)
    rst = np.zeros((20, n))
    ierr = np.zeros(n, np.int32)
    nretry = solver.fullchem_step(600.0, cells["met"], cells["photol"], c, case["atol"], case["rtol"], ic, rc, None,
                                  ist, rst, ierr)
    c0 = cells["c"].copy()
    for fam in ir["families"]:
        c0[ir["species"].index(fam)] = 0.0
    r = orc.update_rconst(cells["met"], cells["photol"], c0)
    c_ref, ist_ref, rst_ref, ierr_ref = orc.integrate(c0, r, case["atol"], case["rtol"], 0.0, 600.0, ic, rc)
    assert nretry == 0 and np.all(ierr_ref == 1) and np.all(ierr == 1)
    c_ref = np.maximum(c_ref, 0.0)
    # the GPU step computes its own rates (CUDA libm, within 1e-12 of the
    # oracle's): the conditioning bar at that scale
    _check(orc, case, (c, ist, rst, ierr), (c_ref, ist_ref, rst_ref, ierr_ref), ic, rc, scale=1e-12, c_in=c0,
           rconst=r, clamp=True)
    assert np.all(c >= 0.0)


def test_unsupported_forms_are_refused(solver, case):
    # a target species outside VAR
    with pytest.raises(capi.GcKppError) as e:
        _gpu(solver, case, *_controls(case, target=NVAR + 1, ratio=1e-3))
    assert e.value.code == capi.GC_KPP_EUNSUPPORTED
    # two cells per thread
    with pytest.raises(capi.GcKppError) as e:
        _gpu(solver, case, *_controls(case), arith="fast2")
    assert e.value.code == capi.GC_KPP_EUNSUPPORTED
    solver.set(arith="fast")


@pytest.mark.parametrize("arith", ["strict", "fast"])
def test_per_cell_controls_and_kept_halogens(solver, orc, case, ir, arith):
    """Do_FullChem's auto-reduce set-up: per-cell thresholds (pressure-scaled
    on half of the cells, OH/NO2 key species on the other half) and the
    halogens kept active, through gc_kpp_ctx_set_autoreduce, against the
    oracle with the same per-cell controls and keepSpcActive (the fast
    arithmetic with the append form)."""
    import gcchem.autoreduce as ar

    n = case["n"]
    rng = np.random.default_rng(8)
    thr, target, ratio = ar.integrator_options(ir, n, threshold=1e3, pmid=rng.uniform(100, 1000, n),
                                               pmid_sfc=np.full(n, 1000.0), is_prs_threshold=True)
    t2, g2, r2 = ar.integrator_options(ir, n, is_key_threshold=True, suncos_mid=rng.uniform(-1, 1, n),
                                       tuning_oh=1e-3, tuning_no2=5e-5)
    half = np.arange(n) % 2 == 1
    thr[half], target[half], ratio[half] = t2[half], g2[half], r2[half]
    keep = ar.keep_mask(ir)
    ic, rc = _controls(case, append=(arith == "fast"))
    kw = dict(ar_thr=thr, ar_target=target, ar_ratio=ratio)
    try:
        solver.set_autoreduce(thr=thr, target=target, ratio=ratio, keep=keep)
        got = _gpu(solver, case, ic, rc, arith=arith)
        orc.set_keep(keep)
        ref = _oracle(orc, case, ic, rc, **kw)
        assert np.all(ref[3] == 1)
        assert np.max(_rel(got[2][3], ref[2][3])) < 1e-12
        assert np.all(got[2][3, ~half] == 0.0)
        _check(orc, case, got, ref, ic, rc, **kw)
    finally:
        solver.set_autoreduce()
        orc.set_keep(None)


def test_per_cell_controls_need_the_same_cell_count(solver, case):
    ic, rc = _controls(case)
    try:
        solver.set_autoreduce(thr=np.full(case["n"] + 1, 100.0))
        with pytest.raises(capi.GcKppError) as e:
            _gpu(solver, case, ic, rc)
        assert e.value.code == capi.GC_KPP_EINVAL
        with pytest.raises(capi.GcKppError) as e:
            solver.set_autoreduce(target=np.full(case["n"], NVAR + 1, np.int32))
        assert e.value.code == capi.GC_KPP_EUNSUPPORTED
    finally:
        solver.set_autoreduce()
    # without ICNTRL(12) the controls are ignored
    solver.set_autoreduce(thr=np.full(case["n"] + 1, 100.0))
    try:
        _gpu(solver, case, *_controls(case, on=False))
    finally:
        solver.set_autoreduce()
