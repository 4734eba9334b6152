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

from . import capi


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


def photol_runs(ir=None):
    """Contiguous runs [(r0, r1), ...] of the PHOTOL rows that the
    mechanism's Update_RCONST reads (168 of the 200 for fullchem, in 8 runs):
    the only J-value rows a step needs on the device."""
    import re

    from . import mechanism

    ir = ir or mechanism.load_ir()
    rows = sorted({int(k) for e in ir["rconst"] for k in re.findall(r"PHOTOL\[(\d+)\]", e)})
    runs = []
    for r in rows:
        if runs and runs[-1][1] == r:
            runs[-1][1] = r + 1
        else:
            runs.append([r, r + 1])
    return [tuple(x) for x in runs]


class Streamer:
    """Double-buffered chunk streaming of chemistry steps (one CUDA device).

    With several solver contexts (``solvers``), consecutive chunks run on
    different contexts and compute streams, so that one chunk's block-per-cell
    tail overlaps the next chunk's queue kernel; each context keeps its own
    scratch, so the chunks stay independent.  Host-to-device copies run on one
    copy stream, device-to-host copies on another.  With ``photol_rows`` (the
    runs of ``photol_runs``) only the J-value rows the mechanism reads are
    copied; the device buffer's other rows stay zero."""

    def __init__(self, solver, ncell, chunk, proposer=None, solvers=None, photol_rows=None):
        import torch

        self.torch = torch
        self.solvers = list(solvers) if solvers else [solver]
        self.solver = self.solvers[0]
        self.dev = torch.device("cuda", 0)
        self.chunk = chunk
        self.proposer = proposer  # learned.CProposer or None (plain step)
        self.photol_rows = photol_rows
        self.h2d = torch.cuda.Stream(self.dev)
        self.d2h = torch.cuda.Stream(self.dev)
        self.comp = [torch.cuda.Stream(self.dev) for _ in self.solvers]
        nbuf = max(2, len(self.solvers))
        self.nbuf = nbuf
        # flat buffers: a chunk of m cells uses the first rows*m entries as a
        # contiguous [rows, m] array, so host<->device copies are plain copies
        self.rows = {"met": NMET, "ph": NPHOTOL, "c": 356, "hs": 1, "ist": 20, "rst": 20, "ierr": 1}
        dts = {"ist": torch.int32, "ierr": torch.int32}
        self.buf = [{k: torch.zeros(r * chunk, dtype=dts.get(k, torch.float64), device=self.dev)
                     for k, r in self.rows.items()} for _ in range(nbuf)]
        self.staged = [torch.cuda.Event() for _ in range(nbuf)]
        self.solved = [torch.cuda.Event() for _ in range(nbuf)]
        self.freed = [torch.cuda.Event() for _ in range(nbuf)]

    def _view(self, b, key, m):
        r = self.rows[key]
        flat = b[key][: r * m]
        return flat if key in ("hs", "ierr") else flat.view(r, m)

    def bytes_per_cell(self):
        """(host-to-device, device-to-host) bytes per cell of one step."""
        nph = NPHOTOL if self.photol_rows is None else sum(b - a for a, b in self.photol_rows)
        return 8 * (NMET + nph + 356 + 1), 8 * (356 + 1) + 4 + 4

    def step(self, chunks, dt, atol, rtol, icntrl, rcntrl):
        """One chemistry step over host chunks: a list of dicts of pinned,
        contiguous torch CPU tensors met [18, m], ph [200, m], c [356, m],
        hs [m] (the KPPHvalue chain), steps [m] and ierr [m] (out: ISTATUS(3),
        IERR), m <= the chunk size.  Results go to c_out / hs_out when a chunk
        has them, else back into c / hs.  Returns the number of cells retried
        (the reference's second Integrate)."""
        torch = self.torch
        retried = [0]
        nb = self.nbuf

        # the copies run on the SMs (gc_kpp_copy_rows reads and writes the
        # page-locked host chunks directly), stream-ordered on the copy streams
        cp = lambda dst, src, st: capi.copy_rows(dst, src, stream=st.cuda_stream, lib=self.solver.lib)

        def stage(k):
            h, b = chunks[k], self.buf[k % nb]
            m = h["c"].shape[1]
            with torch.cuda.stream(self.h2d):
                self.h2d.wait_event(self.freed[k % nb])
                for key in ("met", "c", "hs"):
                    cp(self._view(b, key, m), h[key], self.h2d)
                ph = self._view(b, "ph", m)
                if self.photol_rows is None:
                    cp(ph, h["ph"], self.h2d)
                else:
                    for r0, r1 in self.photol_rows:
                        cp(ph[r0:r1], h["ph"][r0:r1], self.h2d)
                self.staged[k % nb].record(self.h2d)

        def retrieve(k):
            h, b = chunks[k], self.buf[k % nb]
            m = h["c"].shape[1]
            with torch.cuda.stream(self.d2h):
                self.d2h.wait_event(self.solved[k % nb])
                cp(h.get("c_out", h["c"]), self._view(b, "c", m), self.d2h)
                cp(h.get("hs_out", h["hs"]), self._view(b, "hs", m), self.d2h)
                cp(h["steps"], self._view(b, "ist", m)[2], self.d2h)
                cp(h["ierr"], self._view(b, "ierr", m), self.d2h)
                self.freed[k % nb].record(self.d2h)

        for e in self.freed:
            e.record(self.d2h)
        stage(0)
        for k in range(len(chunks)):
            if k + 1 < len(chunks):
                stage(k + 1)  # overlaps the solve of chunk k
            m = chunks[k]["c"].shape[1]
            b = self.buf[k % nb]
            solver = self.solvers[k % len(self.solvers)]
            comp = self.comp[k % len(self.solvers)]
            comp.wait_event(self.staged[k % nb])
            v = {key: self._view(b, key, m) for key in self.rows}
            sp = comp.cuda_stream
            if self.proposer is not None:
                nr, _ = solver.fullchem_step_learned(self.proposer.handle, dt, v["met"], v["ph"], v["c"], atol,
                                                     rtol, icntrl, rcntrl, v["hs"], v["ist"], v["rst"], v["ierr"],
                                                     stream=sp)
            else:
                nr = solver.fullchem_step(dt, v["met"], v["ph"], v["c"], atol, rtol, icntrl, rcntrl, v["hs"],
                                          v["ist"], v["rst"], v["ierr"], stream=sp)
            retried[0] += max(nr, 0)
            self.solved[k % nb].record(comp)
            retrieve(k)  # overlaps the solve of chunk k + 1
        self.d2h.synchronize()
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
