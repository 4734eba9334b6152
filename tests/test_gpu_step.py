"""GPU tests of the chemistry-step boundary (gc_kpp_fullchem_step) and of the
reference's error behaviour, against the CPU oracle."""
import numpy as np
import pytest

import os
import sys

import gcchem.capi as capi
import gcchem.inputs as inputs
import gcchem.mechanism as mechanism

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from parity_bars import check_other_sequences  # noqa: E402

pytestmark = pytest.mark.gpu
NVAR = 353


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


def _oracle_step(orc, ir, cells, dt, icntrl, rcntrl, atol, rtol, hstart=None):
    """Do_FullChem loop body on the CPU: zero families, rates, integrate,
    retry once from C_before with Hstart=0, clamp (fullchem_mod.F90:943-1350)."""
    c = cells["c"].copy()
    for fam in ir["families"]:
        c[ir["species"].index(fam)] = 0.0
    r = orc.update_rconst(cells["met"], cells["photol"], c)
    c1, ist, rst, ierr = orc.integrate(c, r, atol, rtol, 0.0, dt, icntrl, rcntrl, hstart=hstart)
    bad = ierr < 0
    if bad.any():
        c2, ist2, rst2, ierr2 = orc.integrate(c[:, bad], r[:, bad], atol, rtol, 0.0, dt, icntrl, rcntrl)
        c1[:, bad], ist[:, bad], rst[:, bad], ierr[bad] = c2, ist2, rst2, ierr2
    return np.maximum(c1, 0.0), ist, rst, ierr, int(bad.sum())


@pytest.fixture(scope="module")
def step_case():
    n = 192
    cells = inputs.box_cells(n, seed=21)
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    return dict(n=n, cells=cells, atol=atol, rtol=rtol, icntrl=icntrl, rcntrl=rcntrl)


@pytest.fixture(scope="module")
def step_tight(orc, step_case):
    """The loop body of the step case integrated at RTOL 1e-8 (the accuracy
    reference for cells whose step sequence differs from the oracle's)."""
    k = step_case
    return _oracle_step(orc, mechanism.load_ir(), k["cells"], 600.0, k["icntrl"], k["rcntrl"], k["atol"],
                        np.full_like(k["rtol"], 1e-8))[0]


def _gpu_step(solver, case, icntrl=None, hstart=None, dt=600.0, arith="strict"):
    solver.set(arith=arith, schedule="plain", block=0)
    n = case["n"]
    c = case["cells"]["c"].copy()
    ist = np.zeros((20, n), np.int32)
    rst = np.zeros((20, n))
    ierr = np.zeros(n, np.int32)
    hs = None if hstart is None else hstart.copy()
    nretry = solver.fullchem_step(dt, case["cells"]["met"], case["cells"]["photol"], c, case["atol"], case["rtol"],
                                  case["icntrl"] if icntrl is None else icntrl, case["rcntrl"], hs, ist, rst, ierr)
    return c, ist, rst, ierr, nretry, hs


def test_fullchem_step_matches_oracle(solver, orc, step_case, step_tight):
    ir = mechanism.load_ir()
    c, ist, rst, ierr, nretry, _ = _gpu_step(solver, step_case)
    c_ref, ist_ref, rst_ref, ierr_ref, nretry_ref = _oracle_step(orc, ir, step_case["cells"], 600.0,
                                                                 step_case["icntrl"], step_case["rcntrl"],
                                                                 step_case["atol"], step_case["rtol"])
    assert nretry == nretry_ref == 0
    assert np.array_equal(ierr, ierr_ref)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.99
    big = np.abs(c_ref) > 1e4
    assert np.max(np.where(big, _rel(c, c_ref), 0.0)[:, same]) < 1e-9
    check_other_sequences(c, c_ref, step_tight, same, step_case["atol"], step_case["rtol"])
    assert np.all(c >= 0.0)
    for fam in ir["families"]:
        # dummies were zeroed before the integration, then produced again
        assert np.all(np.isfinite(c[ir["species"].index(fam)]))


def test_retry_policy_and_hnew_chain(solver, orc, step_case, step_tight):
    """Cells that fail (step cap, IERR=-6) are integrated once more from the
    saved concentrations with Hstart = 0; KPPHvalue = RSTATE(Nhnew)."""
    ir = mechanism.load_ir()
    ic = step_case["icntrl"].copy()
    ic[3] = 20  # Max_no_steps: most random cells fail at 600 s
    hs = np.full(step_case["n"], 1.0)
    c, ist, rst, ierr, nretry, hs_out = _gpu_step(solver, step_case, icntrl=ic, hstart=hs)
    c_ref, ist_ref, rst_ref, ierr_ref, nretry_ref = _oracle_step(orc, ir, step_case["cells"], 600.0, ic,
                                                                 step_case["rcntrl"], step_case["atol"],
                                                                 step_case["rtol"], hstart=hs)
    assert nretry == nretry_ref and nretry > 0
    assert np.array_equal(ierr, ierr_ref)
    assert set(np.unique(ierr)) <= {1, -6}
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.98
    assert np.allclose(hs_out, rst[2])
    big = np.abs(c_ref) > 1e4
    assert np.max(np.where(big, _rel(c, c_ref), 0.0)[:, same]) < 1e-9
    # cells that end the step successfully with another step sequence: bounded
    # against the uncapped RTOL 1e-8 loop body
    check_other_sequences(c, c_ref, step_tight, same, step_case["atol"], step_case["rtol"], sel=ierr == 1)


@pytest.mark.parametrize("field,value,code", [("rtol", 1.0, -5), ("atol", 0.0, -5), ("method", 9, -2),
                                              ("maxsteps", -1, -1)])
def test_option_errors_give_reference_ierr(solver, step_case, field, value, code):
    n = step_case["n"]
    at, rt = step_case["atol"].copy(), step_case["rtol"].copy()
    ic = step_case["icntrl"].copy()
    if field == "rtol":
        rt[5] = value
    elif field == "atol":
        at[7] = value
    elif field == "method":
        ic[2] = value
    else:
        ic[3] = value
    c = step_case["cells"]["c"].copy()
    r = np.ones((1058, n)) * 1e-12
    ist = np.full((20, n), 7, np.int32)
    ierr = np.zeros(n, np.int32)
    solver.integrate(c, r, at, rt, 0.0, 60.0, ic, step_case["rcntrl"], istatus=ist, ierr=ierr)
    assert np.all(ierr == code)
    assert np.all(ist == 0)
    assert np.array_equal(c, step_case["cells"]["c"])


@pytest.mark.parametrize("which", ["rate_updates", "autoreduce_2cells", "autoreduce_target"])
def test_unsupported_options_are_rejected(solver, step_case, which):
    """Forms outside the implemented path fail the call with
    GC_KPP_EUNSUPPORTED: rate updates inside the integrator, auto-reduction
    with 2 cells per thread (it runs 1 cell per thread only) and a target
    species outside 1..NVAR."""
    n = step_case["n"]
    ic = step_case["icntrl"].copy()
    if which == "rate_updates":
        ic[14] = 0  # INTEGRATE then defaults ICNTRL(15) to 5: updates inside the integrator
    elif which == "autoreduce_2cells":
        ic[11] = 1
        solver.set(arith="fast2")
    else:
        ic[11] = 1
        ic[13] = 354  # ICNTRL(14) beyond NVAR
    c = step_case["cells"]["c"].copy()
    r = np.ones((1058, n)) * 1e-12
    ierr = np.zeros(n, np.int32)
    try:
        with pytest.raises(capi.GcKppError) as e:
            solver.integrate(c, r, step_case["atol"], step_case["rtol"], 0.0, 60.0, ic, step_case["rcntrl"],
                             ierr=ierr)
    finally:
        solver.set(arith="fast")
    assert e.value.code == capi.GC_KPP_EUNSUPPORTED


def test_host_and_device_paths_agree(solver, orc, step_case):
    import torch

    n = step_case["n"]
    cells = step_case["cells"]
    r = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
    solver.set(arith="fast", schedule="queue", block=64)
    c_h = cells["c"].copy()
    ist_h = np.zeros((20, n), np.int32)
    ierr_h = np.zeros(n, np.int32)
    solver.integrate(c_h, r, step_case["atol"], step_case["rtol"], 0.0, 300.0, step_case["icntrl"],
                     step_case["rcntrl"], istatus=ist_h, ierr=ierr_h)
    dev = torch.device("cuda", 0)
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    c_d = T(cells["c"])
    ist_d = torch.zeros((20, n), dtype=torch.int32, device=dev)
    ierr_d = torch.zeros(n, dtype=torch.int32, device=dev)
    solver.integrate(c_d, T(r), T(step_case["atol"]), T(step_case["rtol"]), 0.0, 300.0, step_case["icntrl"],
                     step_case["rcntrl"], istatus=ist_d, ierr=ierr_d)
    torch.cuda.synchronize()
    assert np.array_equal(c_h, c_d.cpu().numpy())
    assert np.array_equal(ist_h, ist_d.cpu().numpy())
    assert np.array_equal(ierr_h, ierr_d.cpu().numpy())


@pytest.mark.parametrize("schedule", ["queue", "plain"])
def test_queue_order_changes_nothing_but_packing(solver, step_case, schedule):
    """gc_kpp_fullchem_step_ordered: any permutation gives bit-identical
    results to the unordered step, on host and device memory."""
    import torch

    n = step_case["n"]
    cells = step_case["cells"]
    ic = step_case["icntrl"]

    def run(order, device=False):
        solver.set(arith="fast", schedule=schedule, block=64)
        if device:
            dev = torch.device("cuda", 0)
            T = lambda a: torch.tensor(a, device=dev).contiguous()
            c = T(cells["c"])
            hs = torch.full((n,), 30.0, dtype=torch.float64, device=dev)
            ist = torch.zeros((20, n), dtype=torch.int32, device=dev)
            rst = torch.zeros((20, n), dtype=torch.float64, device=dev)
            ierr = torch.zeros(n, dtype=torch.int32, device=dev)
            solver.fullchem_step(600.0, T(cells["met"]), T(cells["photol"]), c, T(step_case["atol"]),
                                 T(step_case["rtol"]), ic, step_case["rcntrl"], hs, ist, rst, ierr,
                                 order=None if order is None else torch.tensor(order, dtype=torch.int32, device=dev))
            torch.cuda.synchronize()
            return [x.cpu().numpy() for x in (c, hs, ist, rst, ierr)]
        c = cells["c"].copy()
        hs = np.full(n, 30.0)
        ist = np.zeros((20, n), np.int32)
        rst = np.zeros((20, n))
        ierr = np.zeros(n, np.int32)
        solver.fullchem_step(600.0, cells["met"], cells["photol"], c, step_case["atol"], step_case["rtol"], ic,
                             step_case["rcntrl"], hs, ist, rst, ierr, order=order)
        return [c, hs, ist, rst, ierr]

    base = run(None)
    perm = np.random.default_rng(5).permutation(n).astype(np.int32)
    heavy_first = np.argsort(-base[2][2], kind="stable").astype(np.int32)
    for got in (run(perm), run(heavy_first), run(perm, device=True)):
        for a, b in zip(got, base):
            assert np.array_equal(a, b)


def test_host_order_must_be_a_permutation(solver, step_case):
    n = step_case["n"]
    cells = step_case["cells"]
    bad = np.arange(n, dtype=np.int32)
    bad[3] = 5
    c = cells["c"].copy()
    ierr = np.zeros(n, np.int32)
    with pytest.raises(capi.GcKppError) as e:
        solver.fullchem_step(600.0, cells["met"], cells["photol"], c, step_case["atol"], step_case["rtol"],
                             step_case["icntrl"], step_case["rcntrl"], ierr=ierr, order=bad)
    assert e.value.code == capi.GC_KPP_EINVAL


@pytest.mark.parametrize("arith,cell_block", [("fast", 256), ("fast", 32), ("strict", 128)])
def test_block_per_cell_matches_thread_per_cell(solver, step_case, arith, cell_block):
    """gc_kpp_fullchem_step_binned: cells routed to the block-per-cell kernel
    in its level form (shared-memory Jacobian/LU, level-scheduled
    factorization, GC_KPP_OPT_BLOCK_SPLIT 0) get bit for bit the results of
    the thread-per-cell kernel."""
    n = step_case["n"]
    cells = step_case["cells"]

    def run(order=None, nblock=0):
        solver.set(arith=arith, schedule="queue", block=64, cell_block=cell_block, block_split=False)
        c = cells["c"].copy()
        hs = np.full(n, 20.0)
        ist = np.zeros((20, n), np.int32)
        rst = np.zeros((20, n))
        ierr = np.zeros(n, np.int32)
        solver.fullchem_step(600.0, cells["met"], cells["photol"], c, step_case["atol"], step_case["rtol"],
                             step_case["icntrl"], step_case["rcntrl"], hs, ist, rst, ierr, order=order,
                             nblock=nblock)
        return [c, hs, ist, rst, ierr]

    base = run()
    perm = np.random.default_rng(11).permutation(n).astype(np.int32)
    for nblock in (1, 24, n):
        got = run(perm, nblock)
        for a, b in zip(got, base):
            assert np.array_equal(a, b), nblock
    solver.set(cell_block=0, block_split=True)


@pytest.mark.parametrize("evict_after", [0, 2])
def test_split_block_per_cell_agrees_with_thread_per_cell(solver, step_case, evict_after):
    """The split block-per-cell form (GC_KPP_OPT_BLOCK_SPLIT 1, the default):
    sums regrouped across warp lanes, so cells routed to it (binned, or handed
    over after k steps) agree with the thread-per-cell kernel to rounding: the
    parity bar of the fast arithmetic against the oracle (same step sequence
    on nearly every cell, 1e-9 relative on species > 1e4 molec/cm3 there)."""
    n = step_case["n"]
    cells = step_case["cells"]

    def run(order=None, nblock=0, evict=0):
        solver.set(arith="fast", schedule="queue", block=64, block_split=True, evict_after=evict)
        c = cells["c"].copy()
        hs = np.full(n, 20.0)
        ist = np.zeros((20, n), np.int32)
        rst = np.zeros((20, n))
        ierr = np.zeros(n, np.int32)
        solver.fullchem_step(600.0, cells["met"], cells["photol"], c, step_case["atol"], step_case["rtol"],
                             step_case["icntrl"], step_case["rcntrl"], hs, ist, rst, ierr, order=order,
                             nblock=nblock)
        return c, hs, ist, rst, ierr

    base = run()
    perm = np.random.default_rng(12).permutation(n).astype(np.int32)
    for nblock in ((24, n) if evict_after == 0 else (0, 16)):
        c, hs, ist, rst, ierr = run(perm, nblock, evict_after)
        assert np.array_equal(ierr, base[4]) and np.all(ierr == 1)
        same = np.all(ist[:8] == base[2][:8], axis=0)
        assert same.mean() >= 0.97, same.mean()
        big = np.abs(base[0][:NVAR]) > 1e4
        assert np.max(np.where(big, _rel(c[:NVAR], base[0][:NVAR]), 0.0)[:, same]) < 1e-9
        assert np.all(_rel(hs, base[1])[same] < 1e-6)
    # deterministic: the same call twice gives the same bits
    a, b = run(perm, 24, evict_after), run(perm, 24, evict_after)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    solver.set(evict_after=0)


def test_block_per_cell_strict_matches_oracle(solver, orc, step_case):
    """Every cell block-per-cell, strict arithmetic, against the oracle."""
    ir = mechanism.load_ir()
    n = step_case["n"]
    cells = step_case["cells"]
    solver.set(arith="strict", schedule="queue", block=0, cell_block=256)
    c = cells["c"].copy()
    ist = np.zeros((20, n), np.int32)
    rst = np.zeros((20, n))
    ierr = np.zeros(n, np.int32)
    solver.fullchem_step(600.0, cells["met"], cells["photol"], c, step_case["atol"], step_case["rtol"],
                         step_case["icntrl"], step_case["rcntrl"], None, ist, rst, ierr,
                         order=np.arange(n, dtype=np.int32), nblock=n)
    c_ref, ist_ref, rst_ref, ierr_ref, _ = _oracle_step(orc, ir, cells, 600.0, step_case["icntrl"],
                                                        step_case["rcntrl"], step_case["atol"], step_case["rtol"])
    # the same bar as the thread-per-cell step (rates differ from the
    # oracle's libm in the last bits)
    assert np.array_equal(ierr, ierr_ref)
    same = np.all(ist[:8] == ist_ref[:8], axis=0)
    assert same.mean() >= 0.99
    big = np.abs(c_ref) > 1e4
    assert np.max(np.where(big, _rel(c, c_ref), 0.0)[:, same]) < 1e-9


def test_async_steps_capture_in_a_cuda_graph(step_case):
    """GC_KPP_OPT_ASYNC: three chemistry steps (with the KPPHvalue chain and
    the device-side retry) captured in one CUDA graph and replayed give the
    results of three synchronous steps."""
    import torch

    n = step_case["n"]
    cells = step_case["cells"]
    dev = torch.device("cuda", 0)
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    met, ph, c0, at, rt = (T(cells["met"]), T(cells["photol"]), T(cells["c"]), T(step_case["atol"]),
                           T(step_case["rtol"]))
    ic, rc = step_case["icntrl"], step_case["rcntrl"]
    solver = capi.Solver(0, arith="fast", schedule="queue", block=64)
    z = lambda *s, dt=torch.float64: torch.zeros(s, dtype=dt, device=dev)

    def steps(c, hs, ist, rst, ierr, stream=None):
        for _ in range(3):
            solver.fullchem_step(600.0, met, ph, c, at, rt, ic, rc, hs, ist, rst, ierr, stream=stream)

    c, hs, ist, rst, ierr = c0.clone(), z(n), z(20, n, dt=torch.int32), z(20, n), z(n, dt=torch.int32)
    steps(c, hs, ist, rst, ierr)  # synchronous: checks the tolerances, sizes the buffers
    torch.cuda.synchronize()
    ref = [x.cpu().numpy() for x in (c, hs, ist, rst, ierr)]
    solver.set(async_steps=True)
    c, hs = c0.clone(), z(n)
    ist, rst, ierr = z(20, n, dt=torch.int32), z(20, n), z(n, dt=torch.int32)
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        steps(c, hs, ist, rst, ierr, stream=torch.cuda.current_stream().cuda_stream)
    for _ in range(2):  # replay twice from the same start
        c.copy_(c0)
        hs.zero_()
        g.replay()
        torch.cuda.synchronize()
        for a, b in zip([x.cpu().numpy() for x in (c, hs, ist, rst, ierr)], ref):
            assert np.array_equal(a, b)
    solver.set(async_steps=False)


@pytest.mark.parametrize("arith,evict_after,drained", [("fast", 1, 0), ("fast", 3, 0), ("strict", 2, 0),
                                                       ("fast", 2, 1)])
def test_handover_to_block_per_cell_changes_nothing(solver, step_case, arith, evict_after, drained):
    """GC_KPP_OPT_EVICT_AFTER: cells still running after k steps finish in the
    block-per-cell kernel from their saved state, with the results of an
    uninterrupted integration (also combined with binned cells)."""
    n = step_case["n"]
    cells = step_case["cells"]

    def run(evict, order=None, nblock=0):
        solver.set(arith=arith, schedule="queue", block=64, cell_block=128, evict_after=evict,
                   evict_drained=drained, block_split=False)
        c = cells["c"].copy()
        hs = np.full(n, 20.0)
        ist = np.zeros((20, n), np.int32)
        rst = np.zeros((20, n))
        ierr = np.zeros(n, np.int32)
        solver.fullchem_step(600.0, cells["met"], cells["photol"], c, step_case["atol"], step_case["rtol"],
                             step_case["icntrl"], step_case["rcntrl"], hs, ist, rst, ierr, order=order,
                             nblock=nblock)
        return [c, hs, ist, rst, ierr]

    base = run(0)
    assert base[2][2].max() > evict_after  # some cells are handed over
    perm = np.random.default_rng(4).permutation(n).astype(np.int32)
    for got in (run(evict_after), run(evict_after, perm, 16)):
        for a, b in zip(got, base):
            assert np.array_equal(a, b)
    solver.set(evict_after=0, evict_drained=0, cell_block=0, block_split=True)


@pytest.mark.parametrize("arith", ["fast", "strict"])
def test_queue_chunk_changes_nothing(solver, step_case, arith):
    """GC_KPP_OPT_QUEUE_CHUNK: lanes that take 2, 5 or 64 queue positions per
    claim integrate the same cells with the same arithmetic, so the results
    equal those of one-position claims bit for bit (also with a queue order
    and the hand-over)."""
    n = step_case["n"]
    cells = step_case["cells"]

    def run(chunk, evict, order):
        solver.set(arith=arith, schedule="queue", block=64, queue_chunk=chunk, evict_after=evict, cell_block=128,
                   block_split=False)
        c = cells["c"].copy()
        hs = np.full(n, 20.0)
        ist = np.zeros((20, n), np.int32)
        rst = np.zeros((20, n))
        ierr = np.zeros(n, np.int32)
        solver.fullchem_step(600.0, cells["met"], cells["photol"], c, step_case["atol"], step_case["rtol"],
                             step_case["icntrl"], step_case["rcntrl"], hs, ist, rst, ierr, order=order)
        return [c, hs, ist, rst, ierr]

    perm = np.random.default_rng(9).permutation(n).astype(np.int32)
    for evict, order in ((0, None), (2, perm)):
        base = run(1, evict, order)
        for chunk in (2, 5, 64):
            for a, b in zip(run(chunk, evict, order), base):
                assert np.array_equal(a, b)
    with pytest.raises(capi.GcKppError):
        solver.set(queue_chunk=65)
    solver.set(queue_chunk=0, evict_after=0, cell_block=0, block_split=True)
