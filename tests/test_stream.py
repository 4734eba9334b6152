"""Chunked streaming of chemistry steps (stream.py): chunk planning on the
CPU; on the GPU, a streamed step equals one step over the whole grid, cell
for cell, for the plain and the learned forms."""
import numpy as np
import pytest


def test_plan_chunks_cover_the_grid():
    import gcchem.stream as stream

    for n, free in ((13_996_800, 250 << 30), (1000, 1 << 30), (5_000_000, 40 << 30)):
        ch = stream.plan_chunks(n, free)
        assert ch[0][0] == 0 and ch[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(ch, ch[1:]))
        per = ch[0][1] - ch[0][0]
        assert per * stream._BYTES_PER_CELL <= max(free - stream.RESERVE, stream._BYTES_PER_CELL * 1024)
        assert per <= stream.MAX_CHUNK
    assert len(stream.plan_chunks(100_000, 1 << 40, max_chunk=30_000)) == 4


@pytest.mark.gpu
@pytest.mark.parametrize("learned_form", [False, True])
def test_streamed_step_equals_one_step(learned_form):
    import torch
    import gcchem.capi as capi
    import gcchem.inputs as inputs
    import gcchem.learned as learned
    import gcchem.stream as stream

    cells = inputs.grid_cells(20, 10, 16, seed=12)
    n = cells["c"].shape[1]
    dev = torch.device("cuda", 0)
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    at, rt = T(atol), T(rtol)
    solver = capi.Solver(0, arith="fast", schedule="queue")
    solver.set(evict_after=2 if learned_form else 0)
    met, ph, c = T(cells["met"]), T(cells["photol"]), T(cells["c"])
    z = lambda *s, dt=torch.float64: torch.zeros(s, dtype=dt, device=dev)
    hs, ist, rst, ierr = z(n), z(20, n, dt=torch.int32), z(20, n), z(n, dt=torch.int32)
    solver.fullchem_step(43200.0, met, ph, c, at, rt, ic, rc, hs, ist, rst, ierr)  # spin-up
    c_spun, hs0 = c.clone(), torch.zeros_like(hs)
    cp = None
    if learned_form:
        prop = learned.Proposer(0)
        prop.load_state(dict(np.load(learned.WEIGHTS)))
        cp = learned.CProposer(prop)
    # one step over all cells
    c1, h1 = c_spun.clone(), hs0.clone()
    if cp:
        solver.fullchem_step_learned(cp.handle, 1200.0, met, ph, c1, at, rt, ic, rc, h1, ist, rst, ierr)
    else:
        solver.fullchem_step(1200.0, met, ph, c1, at, rt, ic, rc, h1, ist, rst, ierr)
    ref_steps = ist[2].cpu().numpy()
    # streamed in chunks of 700 cells
    chunks = stream.host_chunks(cells["met"], cells["photol"], c_spun.cpu().numpy(), hs0.cpu().numpy(), 700)
    st = stream.Streamer(solver, n, 700, proposer=cp)
    st.step(chunks, 1200.0, at, rt, ic, rc)
    assert np.array_equal(stream.gather(chunks, "c"), c1.cpu().numpy())
    assert np.array_equal(stream.gather(chunks, "hs"), h1.cpu().numpy())
    assert np.array_equal(stream.gather(chunks, "steps"), ref_steps)
    solver.set(evict_after=0)
