"""Ragged batch sizes: a chemistry step over any number of cells (0, 1, and
sizes that are not multiples of a warp or a block) gives every cell the
result it gets in a larger batch -- the cells are independent, as in the
reference's cell loop -- for the plain step (strict and fast arithmetic, both
schedules) and the learned step (host and device memory)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    import gcchem.inputs as inputs

    n = 300
    cells = inputs.grid_cells(20, 5, 3, seed=5)
    cells = {k: np.ascontiguousarray(v[:, :n]) for k, v in cells.items() if k in ("met", "photol", "c")}
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    return dict(n=n, cells=cells, atol=atol, rtol=rtol, ic=ic, rc=rc)


def _step(solver, case, m, learned=None):
    cells = case["cells"]
    c = np.array(cells["c"][:, :m], order="C")  # a copy: the step writes c in place
    ist = np.zeros((20, m), np.int32)
    rst = np.zeros((20, m))
    ierr = np.zeros(m, np.int32)
    hs = np.zeros(m)
    args = (600.0, np.ascontiguousarray(cells["met"][:, :m]), np.ascontiguousarray(cells["photol"][:, :m]), c,
            case["atol"], case["rtol"], case["ic"], case["rc"], hs, ist, rst, ierr)
    if learned is None:
        solver.fullchem_step(*args)
    else:
        solver.fullchem_step_learned(learned, *args)
    return c, ist, rst, ierr, hs


@pytest.mark.parametrize("arith,schedule", [("strict", "queue"), ("strict", "plain"), ("fast", "queue")])
def test_plain_step_any_batch_size(case, arith, schedule):
    import gcchem.capi as capi

    s = capi.Solver(0, arith=arith, schedule=schedule)
    full = _step(s, case, case["n"])
    for m in (1, 33, 129, 257):
        part = _step(s, case, m)
        for a, b in zip(part, full):
            assert np.array_equal(a, b[..., :m]), (m, arith, schedule)
    empty = _step(s, case, 0)
    assert all(x.size == 0 for x in empty)
    s.close()


def test_learned_step_any_batch_size(case):
    import gcchem.capi as capi
    import gcchem.learned as learned

    prop = learned.Proposer(0)
    prop.load_state(dict(np.load(learned.WEIGHTS)))
    cp = learned.CProposer(prop)
    # the level block form: results identical whichever kernel takes a cell
    s = capi.Solver(0, arith="fast", schedule="queue")
    s.set(block_split=False, evict_after=4)
    full = _step(s, case, case["n"], cp.handle)
    for m in (1, 33, 129):
        part = _step(s, case, m, cp.handle)
        for a, b in zip(part, full):
            assert np.array_equal(a, b[..., :m]), m
    s.close()
    cp.close()
