"""Auto-reduction, the CPU restatement: ros_yIntegrator of
KPP/fullchem/gckpp_Integrator.F90:789-1237 with cKppDecomp (:2624-2661),
the DO_SLV-guarded KppSolve and AutoReduce_1stOrder (:1702-1712), selected by
ICNTRL(12) = 1 as INTEGRATE does (:388-394, :478-520), and its append form
ros_yIntegratorA (:1242-1700, APPEND :2663-2700) with ICNTRL(13) = 1.  The
GPU form is tested against it in test_zzz_autoreduce_gpu.py."""
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


def test_append_form_without_appends_is_ros_yintegrator(case, ir):
    """ros_yIntegratorA (ICNTRL(13) = 1) with RCNTRL(12) above every rate can
    append nothing: it is ros_yIntegrator bit for bit (here with the OH
    target threshold, which does not involve RCNTRL(12))."""
    oh = ir["species"].index("OH") + 1
    a = _ar(case, thr=1e300, target=oh, ratio=1e-3)
    b = _ar(case, thr=1e300, target=oh, ratio=1e-3, append=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("thr", [1e2, 1e4])
def test_append_brings_species_back(case, thr):
    """Species whose production or loss grows past RCNTRL(12) during the
    integration re-enter the solve (APPEND): every cell succeeds and the
    result moves towards the full integration."""
    a = _ar(case, thr=thr)
    b = _ar(case, thr=thr, append=True)
    full = case["full"][0][:353]
    assert np.all(b[3] == 1)
    assert not np.array_equal(a[0], b[0])
    big = np.abs(full) > 1e4

    def err(x):
        return np.median((np.abs(x[:353] - full) / np.maximum(np.abs(full), 1e-300))[big])

    assert err(b[0]) < 0.2 * err(a[0])


@pytest.mark.parametrize("append", [False, True])
@pytest.mark.parametrize("thr", [1e2, 1e5])
def test_masked_full_decomposition_equals_the_compressed_one(case, thr, append):
    """The design of the GPU form: zeroing every Jac0 entry in a frozen row
    or column and factoring the full Ghimj = -Jac0 + ghinv I (ICNTRL(20) = 7
    selects it in the oracle) gives the compressed cKppDecomp path's
    integration bit for bit -- frozen entries only ever contribute exact
    zeros.  With APPEND the appended species' row keeps the columns that
    entered no later than it and its column is zeroed in earlier rows."""
    import oracle

    ic = case["ic"].copy()
    rc = case["rc"].copy()
    ic[11] = 1
    ic[12] = 1 if append else 0
    rc[11] = thr
    a = oracle.integrate(case["cells"]["c"], case["r"], case["atol"], case["rtol"], 0.0, 600.0, ic, rc)
    ic[19] = 7
    b = oracle.integrate(case["cells"]["c"], case["r"], case["atol"], case["rtol"], 0.0, 600.0, ic, rc)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.fixture
def keep_off():
    import oracle

    yield
    oracle.set_keep(None)


def test_keep_every_species_is_the_full_integrator(case, keep_off):
    """keepActive with every species in keepSpcActive freezes nothing."""
    import oracle

    oracle.set_keep(np.ones(353, np.uint8))
    c, ist, rst, ierr = _ar(case, thr=1e5)
    c0, ist0, rst0, ierr0 = case["full"]
    assert np.array_equal(c, c0) and np.array_equal(ist[:8], ist0[:8])


def test_halogens_kept_active(case, keep_off, ir):
    """fullchem_AR_KeepHalogensActive's 40 species stay in the solve: with a
    threshold that freezes some of them, keeping them changes their result
    and brings it back towards the full integration."""
    import gcchem.autoreduce as ar
    import oracle

    mask = ar.keep_mask(ir)
    assert mask.sum() == 40
    free = _ar(case, thr=1e5)[0]
    oracle.set_keep(mask)
    kept = _ar(case, thr=1e5)[0]
    full = case["full"][0]
    hal = np.nonzero(mask)[0]
    assert not np.array_equal(free[hal], kept[hal])
    err_free = np.abs(free[hal] - full[hal]).sum()
    err_kept = np.abs(kept[hal] - full[hal]).sum()
    assert err_kept < err_free


def test_per_cell_controls_equal_per_cell_calls(case, ir):
    """The batch entry with per-cell RCNTRL(12)/ICNTRL(14)/RCNTRL(14) gives
    each cell what a call with those scalars gives it."""
    import gcchem.autoreduce as ar
    import oracle

    n = case["cells"]["c"].shape[1]
    rng = np.random.default_rng(5)
    thr, target, ratio = ar.integrator_options(ir, n, threshold=1e3, pmid=rng.uniform(100, 1000, n),
                                               pmid_sfc=np.full(n, 1000.0), is_prs_threshold=True)
    # half of the cells in key-species mode
    t2, g2, r2 = ar.integrator_options(ir, n, is_key_threshold=True, suncos_mid=rng.uniform(-1, 1, n),
                                       tuning_oh=1e-3, tuning_no2=5e-5)
    half = np.arange(n) % 2 == 1
    thr[half], target[half], ratio[half] = t2[half], g2[half], r2[half]
    ic = case["ic"].copy()
    ic[11] = 1
    got = oracle.integrate(case["cells"]["c"], case["r"], case["atol"], case["rtol"], 0.0, 600.0, ic, case["rc"],
                           ar_thr=thr, ar_target=target, ar_ratio=ratio)
    for k in range(0, n, 7):
        ick, rck = ic.copy(), case["rc"].copy()
        rck[11], ick[13], rck[13] = thr[k], target[k], ratio[k]
        one = oracle.integrate(case["cells"]["c"][:, k:k + 1], case["r"][:, k:k + 1], case["atol"], case["rtol"],
                               0.0, 600.0, ick, rck)
        for x, y in zip(got, one):
            assert np.array_equal(x[..., k], y[..., 0])
    assert np.all(got[3] == 1)
    # key-species cells report their threshold
    assert np.all(got[2][3, half] > 0) and np.all(got[2][3, ~half] == 0)


def test_integrator_options_follow_the_driver(ir):
    import gcchem.autoreduce as ar

    oh = ir["species"].index("OH") + 1
    no2 = ir["species"].index("NO2") + 1
    thr, target, ratio = ar.integrator_options(ir, 3, threshold=50.0)
    assert np.all(thr == 50.0) and np.all(target == 0) and np.all(ratio == 0)
    thr, _, _ = ar.integrator_options(ir, 2, threshold=50.0, pmid=np.array([500.0, 1000.0]),
                                      pmid_sfc=np.array([1000.0, 1000.0]), is_prs_threshold=True)
    assert np.array_equal(thr, [25.0, 50.0])
    sc = np.array([0.5, -0.1391731, -0.2, -0.1])
    thr, target, ratio = ar.integrator_options(ir, 4, is_key_threshold=True, suncos_mid=sc, tuning_oh=1e-3,
                                               tuning_no2=5e-5)
    assert list(target) == [oh, no2, no2, oh]
    assert list(ratio) == [1e-3, 5e-5, 5e-5, 1e-3]
