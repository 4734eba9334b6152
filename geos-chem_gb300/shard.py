"""Cell sharding across ranks (one process per GPU).

Grid cells are independent within a chemistry step, so ranks take disjoint
cell ranges and no collective touches the data path; only scalar timings and
diagnostics are reduced.  ``shard_range`` splits contiguous ranges (weighted
by an optional per-cell work estimate, e.g. the previous step's ISTATUS(3) or
the proposer's bin), ``gather_cells`` reassembles per-rank results for
diagnostics on the host.
"""
import numpy as np


def shard_range(ncell, rank, world, work=None):
    """[start, stop) of the cells of ``rank`` out of ``world``.

    Without ``work`` the split is even; with a per-cell work estimate the
    boundaries equalise the cumulative work."""
    if world <= 1:
        return 0, ncell
    if work is None:
        base, extra = divmod(ncell, world)
        start = rank * base + min(rank, extra)
        return start, start + base + (1 if rank < extra else 0)
    w = np.asarray(work, dtype=np.float64)
    assert w.shape == (ncell,)
    cum = np.concatenate([[0.0], np.cumsum(np.maximum(w, 0.0))])
    total = cum[-1]
    bounds = [0] + [int(np.searchsorted(cum, total * r / world, side="left")) for r in range(1, world)] + [ncell]
    bounds = np.maximum.accumulate(np.clip(bounds, 0, ncell))
    return int(bounds[rank]), int(bounds[rank + 1])


# expected Rosenbrock steps per chemistry step of a cell in each stiffness
# bin of the learned proposer (1 | 2-3 | 4-15 | >= 16 steps): the work
# estimate that balances the shards when no step counts are known yet
BIN_WORK = (1.0, 2.5, 8.0, 40.0)


def work_from_bins(bins, bin_work=BIN_WORK):
    """Per-cell work estimate from the proposer's stiffness bins."""
    return np.asarray(bin_work, dtype=np.float64)[np.asarray(bins, dtype=np.int64)]


def gather_cells(local, ncell, world, group=None, work=None):
    """All-gather per-rank [K, n_r] arrays (cell-interleaved) into [K, ncell]
    with torch.distributed (host tensors, e.g. the gloo backend); ``work`` is
    the estimate the ranges were split by (None: even split)."""
    import torch
    import torch.distributed as dist

    local = torch.as_tensor(np.ascontiguousarray(local))
    sizes = [shard_range(ncell, r, world, work) for r in range(world)]
    width = max(b - a for a, b in sizes)
    padded = torch.zeros((local.shape[0], width), dtype=local.dtype)
    padded[:, : local.shape[1]] = local
    parts = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(parts, padded, group=group)
    return torch.cat([p[:, : b - a] for p, (a, b) in zip(parts, sizes)], dim=1).numpy()
