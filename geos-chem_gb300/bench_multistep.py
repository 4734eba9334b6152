"""Multi-step chemistry on the 2x2.5 degree grid, one CUDA graph per run.

    python geos-chem_gb300/bench_multistep.py [--grid 144x91x72] [--steps 6] [--dt 600]

The 144 x 91 x 72 = 943,488-cell grid with NOx seeded log-uniform
1e8-1e12 molecules/cm3 in the lowest 10 levels, spun up 24 h, then runs of
`--steps` consecutive chemistry steps of `--dt` seconds (the first from
Hstart = 0, the rest on the KPPHvalue chain, as a model run does):

* plain   - gc_kpp_fullchem_step per step, synchronous;
* learned - gc_kpp_fullchem_step_learned per step (H0 proposals, stiffness
            bins, top bin block-per-cell, hand-over after 4 steps on the cold
            first step and 1 on the chain), the whole
            run captured once in a CUDA graph (GC_KPP_OPT_ASYNC) and replayed.

Each run starts from the same spun-up state; the time is CUDA-event time on
the launching stream around the run.  Prints one JSON line.
"""
import argparse
import json
import os
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--grid", default="144x91x72")
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--dt", type=float, default=600.0)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--seed", type=int, default=0)
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

    nlon, nlat, nlev = (int(v) for v in args.grid.split("x"))
    t0 = time.perf_counter()
    cells = inputs.grid_cells(nlon, nlat, nlev, seed=args.seed, nox_boundary_layer=True)
    gen_s = time.perf_counter() - t0
    dev = torch.device("cuda", 0)
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    n = cells["c"].shape[1]
    met, ph, c0 = T(cells["met"]), T(cells["photol"]), T(cells["c"])
    del cells
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    at, rt = T(atol), T(rtol)
    z = lambda *s, dt=torch.float64: torch.zeros(s, dtype=dt, device=dev)
    ist, rst, ierr = z(20, n, dt=torch.int32), z(20, n), z(n, dt=torch.int32)
    solver = capi.Solver(0, arith="fast", schedule="queue")
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    hs = z(n)
    t0 = time.perf_counter()
    solver.fullchem_step(86400.0, met, ph, c0, at, rt, ic, rc, hs, ist, rst, ierr, stream=sp)
    torch.cuda.synchronize()
    spin_s = time.perf_counter() - t0
    c = c0.clone()
    hs.zero_()
    steps_sum = []

    def plain_run():
        for _ in range(args.steps):
            solver.fullchem_step(args.dt, met, ph, c, at, rt, ic, rc, hs, ist, rst, ierr, stream=sp)
            steps_sum.append(int(ist[2].sum().item()))

    prop = learned.Proposer(0)
    prop.load_state(dict(np.load(learned.WEIGHTS)))
    cp = learned.CProposer(prop)

    def learned_run(stream_ptr=sp):
        for k in range(args.steps):
            # hand-over after 4 steps from the cold start (H0 proposals are
            # capped at learned.H0_CAP), after 1 on the KPPHvalue chain
            solver.set(evict_after=4 if k == 0 else 1)
            solver.fullchem_step_learned(cp.handle, args.dt, met, ph, c, at, rt, ic, rc, hs, ist, rst, ierr,
                                         stream=stream_ptr)

    def timed(fn):
        best = None
        for _ in range(args.reps):
            c.copy_(c0)
            hs.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return best

    solver.set(evict_after=0)
    plain_ms = timed(plain_run)
    plain_steps = steps_sum[-args.steps:]
    # learned: one synchronous run sizes the buffers, then one graph per run
    solver.set(cell_block=256)
    c.copy_(c0)
    hs.zero_()
    learned_run()
    torch.cuda.synchronize()
    learned_sync_ms = timed(learned_run)
    solver.set(async_steps=True)
    g = torch.cuda.CUDAGraph()
    c.copy_(c0)
    hs.zero_()
    torch.cuda.synchronize()
    with torch.cuda.graph(g):
        learned_run(torch.cuda.current_stream().cuda_stream)
    graph_ms = timed(g.replay)
    solver.set(async_steps=False)
    line = {
        "metric": "fullchem cells/s over %d consecutive %.0f s steps, learned-binned (one CUDA graph) vs plain GPU"
                  % (args.steps, args.dt),
        "value": args.steps * n / (graph_ms * 1e-3), "unit": "cells/s", "n_gpus": 1, "dtype": "f64",
        "config": {"workload": "fullchem %s grid (%d cells), NOx seeded in the lowest 10 levels, %d x %.0f s steps, "
                               "Rodas3, RTOL 5e-3 / ATOL 1e-2" % (args.grid, n, args.steps, args.dt),
                   "spinup_wall_s": spin_s, "generate_s": gen_s},
        "plain": {"ms_per_run": plain_ms, "value": args.steps * n / (plain_ms * 1e-3),
                  "rosenbrock_steps_per_chemistry_step": plain_steps},
        "learned_sync": {"ms_per_run": learned_sync_ms, "value": args.steps * n / (learned_sync_ms * 1e-3)},
        "learned_graph": {"ms_per_run": graph_ms},
        "learned_over_plain": plain_ms / graph_ms,
    }
    print(json.dumps(line), flush=True)
    cp.close()


if __name__ == "__main__":
    main()
