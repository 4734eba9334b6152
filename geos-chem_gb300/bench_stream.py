"""Large-grid streaming: one chemistry step over more cells than fit on the GPU.

    python geos-chem_gb300/bench_stream.py [--cells 13996800] [--chunk 0]

The C180 cube-sphere grid has 6 x 180 x 180 x 72 = 13,996,800 cells.  Its
cells are drawn (with a fixed stride permutation) from a pool of spun-up cells
of the 4x5x72 grid -- 24 h on the GPU from the seeded generator -- so that the
states are consistent without a 14M-cell spin-up.  The host arrays (met, J,
C, KPPHvalue; ~4.6 KB per cell) are pinned chunks; `stream.Streamer` stages
chunk i+1 while chunk i integrates.  The chunk size comes from the device's
free memory (`stream.plan_chunks`) unless --chunk is given.  One step of
--dt seconds from Hstart = 0, plain and learned, on the same chunks.  Prints
one JSON line.
"""
import argparse
import json
import os
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--cells", type=int, default=6 * 180 * 180 * 72)
    ap.add_argument("--chunk", type=int, default=0, help="cells per chunk (0: from free device memory)")
    ap.add_argument("--dt", type=float, default=600.0)
    ap.add_argument("--pool-grid", default="72x46x72")
    args = ap.parse_args(argv)
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    import __graft_entry__

    __graft_entry__.load_package()
    import numpy as np
    import torch

    import gcchem.capi as capi
    import gcchem.inputs as inputs
    import gcchem.learned as learned
    import gcchem.stream as stream

    dev = torch.device("cuda", 0)
    nlon, nlat, nlev = (int(v) for v in args.pool_grid.split("x"))
    pool = inputs.grid_cells(nlon, nlat, nlev, seed=7)
    npool = pool["c"].shape[1]
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    at, rt = T(atol), T(rtol)
    solver = capi.Solver(0, arith="fast", schedule="queue")
    met, ph, c = T(pool["met"]), T(pool["photol"]), T(pool["c"])
    z = lambda *s, dt=torch.float64: torch.zeros(s, dtype=dt, device=dev)
    hs, ist, rst, ierr = z(npool), z(20, npool, dt=torch.int32), z(20, npool), z(npool, dt=torch.int32)
    solver.fullchem_step(86400.0, met, ph, c, at, rt, ic, rc, hs, ist, rst, ierr)
    pool_c = c.cpu().numpy()
    del met, ph, c, hs, ist, rst, ierr
    torch.cuda.empty_cache()
    free, total = torch.cuda.mem_get_info(dev)
    chunk = args.chunk or (stream.plan_chunks(args.cells, free)[0][1])
    n = args.cells
    # cell i of the large grid takes pool cell (i * stride) mod npool
    stride = 7919
    t0 = time.perf_counter()
    chunks = []
    for i0 in range(0, n, chunk):
        i1 = min(n, i0 + chunk)
        idx = (np.arange(i0, i1, dtype=np.int64) * stride) % npool
        rows = lambda a: torch.from_numpy(np.ascontiguousarray(a[:, idx])).pin_memory()
        chunks.append({"met": rows(pool["met"]), "ph": rows(pool["photol"]), "c": rows(pool_c),
                       "hs": torch.zeros(i1 - i0, dtype=torch.float64).pin_memory(),
                       "steps": torch.zeros(i1 - i0, dtype=torch.int32).pin_memory(),
                       "ierr": torch.zeros(i1 - i0, dtype=torch.int32).pin_memory()})
    build_s = time.perf_counter() - t0
    c0 = [ch["c"].clone() for ch in chunks]
    prop = learned.Proposer(0)
    prop.load_state(dict(np.load(learned.WEIGHTS)))
    cp = learned.CProposer(prop)
    res = {}
    # hand-over after 4 steps from the cold start (H0 proposals capped at learned.H0_CAP)
    for name, proposer, evict in (("plain", None, 0), ("learned", cp, 4)):
        for ch, c0k in zip(chunks, c0):
            ch["c"].copy_(c0k)
            ch["hs"].zero_()
        solver.set(evict_after=evict)
        st = stream.Streamer(solver, n, chunk, proposer=proposer, photol_rows=stream.photol_runs())
        torch.cuda.synchronize()
        t = time.perf_counter()
        retried = st.step(chunks, args.dt, at, rt, ic, rc)
        torch.cuda.synchronize()
        s = time.perf_counter() - t
        steps = np.concatenate([ch["steps"].numpy() for ch in chunks])
        ok = np.concatenate([ch["ierr"].numpy() for ch in chunks]) == 1
        res[name] = {"seconds": s, "value": n / s, "steps_per_cell": float(steps.mean()),
                     "ierr_ok_fraction": float(ok.mean()), "retried_cells": int(retried)}
        del st
        torch.cuda.empty_cache()
    line = {"metric": "fullchem cells/s, one %.0f s step over a grid streamed through the GPU in chunks" % args.dt,
            "value": res["learned"]["value"], "unit": "cells/s", "n_gpus": 1, "dtype": "f64",
            "config": {"workload": "%d cells (C180 cube-sphere 6x180x180x72 when 13,996,800), states drawn from a "
                                   "24 h spun-up 4x5x72 pool, Hstart = 0" % n,
                       "chunk_cells": chunk, "chunks": len(chunks), "device_free_gb": free / 2**30,
                       "host_pinned_gb": sum(sum(v.numel() * v.element_size() for v in ch.values())
                                             for ch in chunks) / 2**30, "host_build_s": build_s},
            "plain": res["plain"], "learned": res["learned"],
            "learned_over_plain": res["learned"]["value"] / res["plain"]["value"]}
    print(json.dumps(line), flush=True)
    cp.close()


if __name__ == "__main__":
    main()
