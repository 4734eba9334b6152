"""Multi-rank path on the CPU: two gloo ranks integrate disjoint cell ranges
of one grid (the oracle stands in for the GPU solver), gather, and reproduce
the single-process result exactly -- with an even split and with the split
bench.py uses on N GPUs, balanced by per-cell work from stiffness bins."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_ranges_cover_cells():
    sys.path.insert(0, ROOT)
    import __graft_entry__

    __graft_entry__.load_package()
    from gcchem.shard import shard_range

    for n, w in ((10, 3), (1, 4), (238464, 8), (0, 2)):
        ranges = [shard_range(n, r, w) for r in range(w)]
        assert ranges[0][0] == 0 and ranges[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
    work = np.r_[np.ones(50), 10 * np.ones(50)]
    r0, r1 = shard_range(100, 0, 2, work), shard_range(100, 1, 2, work)
    # 50 cells of work 1 then 50 of work 10: half the work (275) ends at cell 72-73
    assert r0[1] == r1[0] and 72 <= r0[1] <= 74


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _bins(n):
    # stiffness bins as the proposer would give them (seeded stand-in)
    return np.random.default_rng(3).integers(0, 4, n)


def _worker(rank, world, port, out_path, weighted=False):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import __graft_entry__

    __graft_entry__.load_package()
    import gcchem.inputs as inputs
    from gcchem.shard import gather_cells, shard_range, work_from_bins

    orc = __graft_entry__.load_oracle()
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    n = 24
    cells = inputs.box_cells(n, seed=9)
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    work = work_from_bins(_bins(n)) if weighted else None
    a, b = shard_range(n, rank, world, work)
    r = orc.update_rconst(cells["met"][:, a:b], cells["photol"][:, a:b], cells["c"][:, a:b])
    c, ist, _, ierr = orc.integrate(cells["c"][:, a:b], r, atol, rtol, 0.0, 120.0, icntrl, rcntrl, nthreads=1)
    full = gather_cells(c, n, world, work=work)
    steps = gather_cells(ist[2:3].astype(np.float64), n, world, work=work)
    if rank == 0:
        np.savez(out_path, c=full, steps=steps)
    dist.destroy_process_group()


@pytest.mark.parametrize("weighted", [False, True])
def test_two_gloo_ranks_match_single_process(tmp_path, orc, weighted):
    sys.path.insert(0, ROOT)
    import gcchem.inputs as inputs

    out = str(tmp_path / "gathered.npz")
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out, weighted)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = np.load(out)
    n = 24
    cells = inputs.box_cells(n, seed=9)
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    r = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
    c, ist, _, _ = orc.integrate(cells["c"], r, atol, rtol, 0.0, 120.0, icntrl, rcntrl, nthreads=1)
    assert np.array_equal(got["c"], c)
    assert np.array_equal(got["steps"][0], ist[2].astype(np.float64))
