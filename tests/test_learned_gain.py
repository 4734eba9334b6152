"""What the trained proposer gains over the method without it, on a grid seed
it was not trained on (counts, not timings: the timed comparison is
bench.py's learned vs plain arms).

* Cold start (no KPPHvalue, RCNTRL(3) = 0): seeding Hstart with the
  network's H0 (capped at learned.H0_CAP) cuts the Rosenbrock steps, at an
  error against an RTOL = 1e-8 integration no worse than the plain step's:
  the largest, the 99.9th-percentile and the median relative error over
  species above 1e4 molec/cm3 each within 5 % of the plain step's.
* The top stiffness bin finds the cells that need tens of steps, which the
  binned step then runs block-per-cell.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def held_out():
    import torch
    import gcchem.capi as capi
    import gcchem.inputs as inputs
    import gcchem.learned as learned

    prop = learned.Proposer(0)
    prop.load_state(dict(np.load(learned.WEIGHTS)))
    solver = capi.Solver(0, arith="fast", schedule="queue")
    cells = inputs.grid_cells(36, 23, 72, seed=1000)
    dev = prop.dev
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    n = cells["c"].shape[1]
    d = {"met": T(cells["met"]), "ph": T(cells["photol"]), "c": T(cells["c"])}
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    at, rt = T(atol), T(rtol)
    z = lambda *s, dt=torch.float64: torch.zeros(s, dtype=dt, device=dev)
    hs = z(n)
    ist, rst, ierr = z(20, n, dt=torch.int32), z(20, n), z(n, dt=torch.int32)
    solver.fullchem_step(86400.0, d["met"], d["ph"], d["c"], at, rt, ic, rc, hs, ist, rst, ierr)
    torch.cuda.synchronize()
    return dict(prop=prop, solver=solver, d=d, n=n, at=at, rt=rt, ic=ic, rc=rc, z=z, hs_chain=hs.clone())


def _step(h, hstart, order=None, nblock=0, rtol=None, solver=None):
    import torch

    d, z, n = h["d"], h["z"], h["n"]
    c = d["c"].clone()
    ist, rst, ierr = z(20, n, dt=torch.int32), z(20, n), z(n, dt=torch.int32)
    (solver or h["solver"]).fullchem_step(1200.0, d["met"], d["ph"], c, h["at"], h["rt"] if rtol is None else rtol,
                                          h["ic"], h["rc"], hstart, ist, rst, ierr, order=order, nblock=nblock)
    return c, ist.cpu().numpy(), ierr.cpu().numpy()


def test_h0_proposals_cut_steps_at_equal_error(held_out):
    import torch
    import gcchem.capi as capi
    import gcchem.learned as learned

    h = held_out
    n = h["n"]
    c_plain, ist_plain, ierr_plain = _step(h, h["z"](n))
    hs = h["z"](n)
    _, _, order = learned.plan(h["prop"], h["d"]["met"], h["d"]["ph"], h["d"]["c"], hstart=hs, hmax=1200.0)
    nb = int(h["prop"].last_counts[3].item())
    c_learned, ist_learned, ierr_learned = _step(h, hs, order=order, nblock=nb)
    assert np.all(ierr_plain == 1) and np.all(ierr_learned == 1)
    steps_plain, steps_learned = ist_plain[2].sum(), ist_learned[2].sum()
    assert steps_learned < 0.5 * steps_plain, (steps_learned, steps_plain)
    # error against a tight integration of the same cells (every 16th cell)
    tight = capi.Solver(0, arith="strict", schedule="queue")
    idx = torch.arange(0, n, 16, device=h["prop"].dev)
    sub = dict(h, d={k: v.index_select(1, idx).contiguous() for k, v in h["d"].items()}, n=idx.numel())
    c_ref, _, _ = _step(sub, h["hs_chain"].index_select(0, idx).contiguous(), rtol=torch.full_like(h["rt"], 1e-8),
                        solver=tight)

    def err(c):
        got = c.index_select(1, idx)[:353]
        ref = c_ref[:353]
        m = ref > 1e4
        e = ((got - ref).abs() / ref)[m]
        q = torch.quantile(e.float(), torch.tensor([0.5, 0.999], device=e.device)).tolist()
        return {"max": float(e.max().item()), "p99.9": q[1], "median": q[0]}

    e_plain, e_learned = err(c_plain), err(c_learned)
    print("error vs RTOL 1e-8: plain %s learned %s; steps plain %d learned %d"
          % (e_plain, e_learned, steps_plain, steps_learned))
    for key in ("max", "p99.9", "median"):
        assert e_learned[key] <= 1.05 * e_plain[key], (key, e_learned[key], e_plain[key])


def test_top_bin_finds_the_stiff_cells(held_out):
    import gcchem.learned as learned

    h = held_out
    _, ist, _ = _step(h, h["hs_chain"].clone())
    x = h["prop"].features(h["d"]["met"], h["d"]["ph"], h["d"]["c"])
    _, bins = h["prop"].propose(x)
    b = bins.cpu().numpy()
    stiff = ist[2] >= learned.BIN_EDGES[-1]
    assert stiff.sum() > 0
    recall = (b[stiff] == 3).mean()
    false_pos = (b == 3).sum() - (b[stiff] == 3).sum()
    assert recall >= 0.8, recall
    # the block-per-cell set stays small: few light cells are sent there
    assert false_pos <= 0.5 * stiff.sum() + 50, (false_pos, stiff.sum())
