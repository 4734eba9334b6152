"""Chemistry steps over grids larger than the GPU holds: chunked streaming.

The cells live in host memory (pinned, cell-interleaved `[k][ncell]` rows);
a step walks them in chunks sized from the device's free memory.  While the
solver integrates chunk i on the compute stream, a copy stream stages chunk
i+1's inputs (met, J-values, C, KPPHvalue) into the other half of a double
buffer and brings chunk i-1's results (C, KPPHvalue, ISTATUS(3), IERR) back.
Every chunk is an ordinary chemistry step of the C ABI, so the results are
those of one step over the whole grid, cell for cell.

Used for the C180 cube-sphere configuration (6 x 180 x 180 x 72 = 13,996,800
cells), whose per-cell inputs and workspace do not fit at once.
"""
import numpy as np


NMET, NPHOTOL = 18, 200
# device bytes per cell of a chunk: inputs and outputs (two buffers each),
# the solver's per-call scratch (RCONST, C_before, retry list, order) and the
# learned plan's activations (56 + 2*128 + 5 floats, bins, order)
_IN_ROWS = NMET + NPHOTOL  # read-only rows
_BYTES_PER_CELL = (2 * (8 * (_IN_ROWS + 356 + 1 + 20) + 4 * (20 + 1)) + 8 * (1058 + 356) + 4 * 4
                   + 4 * (56 + 2 * 128 + 5) + 4 * 3)
# the solver's fixed device memory: the queue workspace (one 153 KB slot per
# resident thread, 152 SMs x 1024) and the block-per-cell slots, with margin
RESERVE = 32 << 30
MAX_CHUNK = 4_000_000  # more chunks than needed keep copies and solves overlapping


def plan_chunks(ncell, free_bytes, reserve_bytes=RESERVE, max_chunk=MAX_CHUNK):
    """Chunk boundaries [(i0, i1), ...] so that a chunk's buffers fit in
    free_bytes - reserve_bytes (the reserve keeps the solver's queue
    workspace and the MLP activations)."""
    room = max(free_bytes - reserve_bytes, _BYTES_PER_CELL * 1024)
    per = max(1024, int(room // _BYTES_PER_CELL))
    if max_chunk:
        per = min(per, int(max_chunk))
    return [(i, min(ncell, i + per)) for i in range(0, ncell, per)]


class Streamer:
    """Double-buffered chunk streaming of chemistry steps (one CUDA device)."""

    def __init__(self, solver, ncell, chunk, proposer=None):
        import torch

        self.torch = torch
        self.solver = solver
        self.dev = torch.device("cuda", 0)
        self.chunk = chunk
        self.proposer = proposer  # learned.CProposer or None (plain step)
        self.copy = torch.cuda.Stream(self.dev)
        self.comp = torch.cuda.Stream(self.dev)
        # flat buffers: a chunk of m cells uses the first rows*m entries as a
        # contiguous [rows, m] array, so host<->device copies are plain copies
        self.rows = {"met": NMET, "ph": NPHOTOL, "c": 356, "hs": 1, "ist": 20, "rst": 20, "ierr": 1}
        dts = {"ist": torch.int32, "ierr": torch.int32}
        self.buf = [{k: torch.empty(r * chunk, dtype=dts.get(k, torch.float64), device=self.dev)
                     for k, r in self.rows.items()} for _ in range(2)]
        self.staged = [torch.cuda.Event() for _ in range(2)]
        self.solved = [torch.cuda.Event() for _ in range(2)]
        self.freed = [torch.cuda.Event() for _ in range(2)]

    def _view(self, b, key, m):
        r = self.rows[key]
        flat = b[key][: r * m]
        return flat if key in ("hs", "ierr") else flat.view(r, m)

    def step(self, chunks, dt, atol, rtol, icntrl, rcntrl):
        """One chemistry step over host chunks: a list of dicts of pinned,
        contiguous torch CPU tensors met [18, m], ph [200, m], c [356, m]
        (in/out), hs [m] (in/out, the KPPHvalue chain), steps [m] and ierr
        [m] (out: ISTATUS(3), IERR), m <= the chunk size.  Returns the number
        of cells retried (the reference's second Integrate)."""
        torch = self.torch
        retried = [0]

        def stage(k):
            h, b = chunks[k], self.buf[k % 2]
            m = h["c"].shape[1]
            with torch.cuda.stream(self.copy):
                self.copy.wait_event(self.freed[k % 2])
                for key in ("met", "ph", "c", "hs"):
                    self._view(b, key, m).copy_(h[key], non_blocking=True)
                self.staged[k % 2].record(self.copy)

        def retrieve(k):
            h, b = chunks[k], self.buf[k % 2]
            m = h["c"].shape[1]
            with torch.cuda.stream(self.copy):
                self.copy.wait_event(self.solved[k % 2])
                h["c"].copy_(self._view(b, "c", m), non_blocking=True)
                h["hs"].copy_(self._view(b, "hs", m), non_blocking=True)
                h["steps"].copy_(self._view(b, "ist", m)[2], non_blocking=True)
                h["ierr"].copy_(self._view(b, "ierr", m), non_blocking=True)
                self.freed[k % 2].record(self.copy)

        for e in self.freed:
            e.record(self.copy)
        stage(0)
        for k in range(len(chunks)):
            if k + 1 < len(chunks):
                stage(k + 1)  # overlaps the solve of chunk k
            m = chunks[k]["c"].shape[1]
            b = self.buf[k % 2]
            self.comp.wait_event(self.staged[k % 2])
            v = {key: self._view(b, key, m) for key in self.rows}
            sp = self.comp.cuda_stream
            if self.proposer is not None:
                nr, _ = self.solver.fullchem_step_learned(self.proposer.handle, dt, v["met"], v["ph"], v["c"], atol,
                                                          rtol, icntrl, rcntrl, v["hs"], v["ist"], v["rst"],
                                                          v["ierr"], stream=sp)
            else:
                nr = self.solver.fullchem_step(dt, v["met"], v["ph"], v["c"], atol, rtol, icntrl, rcntrl, v["hs"],
                                               v["ist"], v["rst"], v["ierr"], stream=sp)
            retried[0] += max(nr, 0)
            self.solved[k % 2].record(self.comp)
            retrieve(k)  # overlaps the solve of chunk k + 1
        self.copy.synchronize()
        return retried[0]


def host_chunks(met, ph, c, hs, chunk):
    """Split cell-interleaved host arrays (numpy) into pinned contiguous
    chunks for Streamer.step."""
    import torch

    n = c.shape[1]
    out = []
    for i0 in range(0, n, chunk):
        i1 = min(n, i0 + chunk)
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        out.append({"met": pin(met[:, i0:i1]), "ph": pin(ph[:, i0:i1]), "c": pin(c[:, i0:i1]),
                    "hs": pin(hs[i0:i1]), "steps": torch.zeros(i1 - i0, dtype=torch.int32).pin_memory(),
                    "ierr": torch.zeros(i1 - i0, dtype=torch.int32).pin_memory()})
    return out


def gather(chunks, key):
    """Concatenate one array of the chunks back into a cell-interleaved numpy array."""
    arrs = [ch[key].numpy() for ch in chunks]
    return np.concatenate(arrs, axis=arrs[0].ndim - 1)
