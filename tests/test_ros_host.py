"""The GPU thread-per-cell integrator's own source (ros_driver of
csrc/kpp_rosenbrock.cuh, plain and work-queue schedules), built for the host
with g++ (tests/host/ros_host.cpp) in the strict and the fast arithmetic (FMA
through std::fma), against the oracle: the kernel's integration logic --
step control, and auto-reduction with its Jacobian mask, APPEND, per-cell
controls, keepActive and the first-order update -- checked without a GPU.
Same 1e-9 bar as the GPU parity tests (the LU runs row-wise here and in
KppDecomp's order in the oracle, so the two agree to rounding)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "geos-chem_gb300", "csrc")
NVAR = 353


def _build(tmp_path_factory, mech):
    import gcchem.tables as tables
    from gcchem.mechanism import load_ir

    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    tmp = tmp_path_factory.mktemp("ros_host_" + mech)
    gen = tmp / "gen"
    tables.write_generated(str(gen), load_ir(mech))
    (tmp / "fake").mkdir()
    (tmp / "fake" / "cuda_runtime.h").write_text(
        "#pragma once\ntypedef int cudaError_t;\ntypedef void* cudaStream_t;\n"
        "struct uint2 { unsigned x, y; };\nstruct uint4 { unsigned x, y, z, w; };\n")
    exe = str(tmp / "ros")
    subprocess.check_call([gxx, "-O1", "-std=c++17", "-ffp-contract=off", "-Wno-unknown-pragmas", "-I",
                           str(tmp / "fake"), "-I", CSRC, "-I", str(gen),
                           os.path.join(ROOT, "tests", "host", "ros_host.cpp"), "-o", exe])
    return tmp, exe


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    return _build(tmp_path_factory, "fullchem")


@pytest.fixture(scope="module")
def case(orc):
    import gcchem.inputs as inputs

    n = 64
    cells = inputs.box_cells(n, seed=51)
    r = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    return dict(n=n, c=cells["c"], r=r, atol=atol, rtol=rtol, ic=ic, rc=rc)


def _host(harness, case, ar=0, append=0, thr=0.0, target=0, ratio=0.0, percell=None, keep=None, strict=True,
          queue=False, tout=600.0):
    tmp, exe = harness
    n = case["n"]
    for name, arr, dt in (("c", case["c"], np.float64), ("r", case["r"], np.float64),
                          ("atol", case["atol"], np.float64), ("rtol", case["rtol"], np.float64)):
        np.ascontiguousarray(arr, dt).tofile(str(tmp / (name + ".bin")))
    if percell is not None:
        np.ascontiguousarray(percell[0], np.float64).tofile(str(tmp / "pthr.bin"))
        np.ascontiguousarray(percell[1], np.int32).tofile(str(tmp / "ptgt.bin"))
        np.ascontiguousarray(percell[2], np.float64).tofile(str(tmp / "pratio.bin"))
    if keep is not None:
        np.ascontiguousarray(keep, np.uint8).tofile(str(tmp / "keep.bin"))
    subprocess.check_call([exe, str(n), repr(tout), str(ar), str(append), repr(thr), str(target), repr(ratio),
                           "1" if percell is not None else "0", "1" if keep is not None else "0",
                           "1" if strict else "0", "1" if queue else "0"], cwd=str(tmp))
    c = np.fromfile(str(tmp / "c_out.bin")).reshape(-1, n)
    ist = np.fromfile(str(tmp / "ist.bin"), np.int32).reshape(20, n)
    rst = np.fromfile(str(tmp / "rst.bin")).reshape(20, n)
    ierr = np.fromfile(str(tmp / "ierr.bin"), np.int32)
    return c, ist, rst, ierr


def _oracle(orc, case, ar=0, append=0, thr=0.0, target=0, ratio=0.0, percell=None, keep=None):
    ic = case["ic"].copy()
    rc = case["rc"].copy()
    ic[11], ic[12], ic[13] = ar, append, target
    rc[11], rc[13] = thr, ratio
    kw = {}
    if percell is not None:
        kw = dict(ar_thr=percell[0], ar_target=percell[1], ar_ratio=percell[2])
    orc.set_keep(keep)
    try:
        return orc.integrate(case["c"], case["r"], case["atol"], case["rtol"], 0.0, 600.0, ic, rc, **kw)
    finally:
        orc.set_keep(None)


def _agree(got, ref, nvar=NVAR):
    c, ist, rst, ierr = got
    c_ref, ist_ref, rst_ref, ierr_ref = ref
    assert np.all(ierr_ref == 1) and np.array_equal(ierr, ierr_ref)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.95, same.mean()
    big = np.abs(c_ref[:nvar]) > 1e4
    rel = np.abs(c[:nvar] - c_ref[:nvar]) / np.maximum(np.abs(c_ref[:nvar]), 1e-300)
    assert np.max(np.where(big, rel, 0.0)[:, same]) < 1e-9
    assert np.max(np.abs(rst[3] - rst_ref[3]) / np.maximum(np.abs(rst_ref[3]), 1e-300)) < 1e-12


@pytest.mark.parametrize("strict", [True, False])
def test_full_integrator(harness, orc, case, strict):
    _agree(_host(harness, case, strict=strict), _oracle(orc, case))


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("append", [0, 1])
@pytest.mark.parametrize("thr", [1e2, 1e5])
def test_autoreduce(harness, orc, case, thr, append, strict):
    _agree(_host(harness, case, ar=1, append=append, thr=thr, strict=strict),
           _oracle(orc, case, ar=1, append=append, thr=thr))


def test_target_species(harness, orc, case, ir):
    oh = ir["species"].index("OH") + 1
    got = _host(harness, case, ar=1, target=oh, ratio=1e-3)
    _agree(got, _oracle(orc, case, ar=1, target=oh, ratio=1e-3))
    assert np.all(got[2][3] > 0)


@pytest.mark.parametrize("append", [0, 1])
def test_per_cell_controls_and_keep(harness, orc, case, ir, append):
    import gcchem.autoreduce as ar

    strict = append == 0  # the append form in the fast arithmetic
    n = case["n"]
    rng = np.random.default_rng(4)
    thr, tgt, ratio = ar.integrator_options(ir, n, threshold=1e3, pmid=rng.uniform(100, 1000, n),
                                            pmid_sfc=np.full(n, 1000.0), is_prs_threshold=True)
    t2, g2, r2 = ar.integrator_options(ir, n, is_key_threshold=True, suncos_mid=rng.uniform(-1, 1, n),
                                       tuning_oh=1e-3, tuning_no2=5e-5)
    half = np.arange(n) % 2 == 1
    thr[half], tgt[half], ratio[half] = t2[half], g2[half], r2[half]
    pc = (thr, tgt, ratio)
    keep = ar.keep_mask(ir)
    got = _host(harness, case, ar=1, append=append, percell=pc, keep=keep, strict=strict)
    _agree(got, _oracle(orc, case, ar=1, append=append, percell=pc, keep=keep))
    assert np.all(got[2][3, ~half] == 0.0) and np.all(got[2][3, half] > 0.0)


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("append", [0, 1])
def test_nothing_frozen_is_the_full_integrator(harness, case, append, strict):
    a = _host(harness, case, ar=1, append=append, thr=1e-300, strict=strict)
    b = _host(harness, case, strict=strict)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("ar", [0, 1])
def test_queue_schedule_equals_plain(harness, case, ar):
    """The work queue over a permuted cell order, one workspace slot reused
    for every cell (the frozen set of one cell must not leak into the next):
    the same results as the plain schedule, bit for bit."""
    a = _host(harness, case, ar=ar, append=ar, thr=1e2, strict=False, queue=True)
    b = _host(harness, case, ar=ar, append=ar, thr=1e2, strict=False)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("ar", [0, 1])
@pytest.mark.parametrize("strict", [True, False])
def test_hg_mechanism(tmp_path_factory, orc, strict, ar):
    """The same source on the Hg mechanism's tables (KPP/Hg) against the
    oracle's Hg build, 1 h, with and without auto-reduction."""
    import gcchem.inputs as inputs
    from gcchem.mechanism import load_ir

    hg = load_ir("Hg")
    h = _build(tmp_path_factory, "Hg")
    n = 64
    cells = inputs.box_cells(n, seed=4, ir=hg)
    atol, rtol = inputs.tolerances(hg)
    ic, rc = inputs.default_controls()
    r = orc.update_rconst(cells["met"], cells["photol"], cells["c"], mech="Hg")
    case = dict(n=n, c=cells["c"], r=r, atol=atol, rtol=rtol)
    got = _host(h, case, ar=ar, thr=1e2, strict=strict, tout=3600.0)
    ic[11] = ar
    ref = orc.integrate(cells["c"], r, atol, rtol, 0.0, 3600.0, ic, rc, mech="Hg")
    _agree(got, ref, nvar=hg["dims"]["nvar"])
