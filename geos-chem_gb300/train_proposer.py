"""Train the learned step-size / stiffness proposer on plain GPU runs.

    python geos-chem_gb300/train_proposer.py --out weights.npz

Training rows come from plain GPU chemistry steps (``learned.collect``) on
seeded global grids -- the standard-atmosphere grid and the same grid with
NOx seeded log-uniform 1e8-1e12 molecules/cm3 in the lowest 10 levels -- and
the network is trained on the GPU by the package's own MLP kernels.  A grid
from a seed outside the training set is held out and scored.  Needs a CUDA
device.
"""
import argparse
import json
import os
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", required=True, help="weights file (.npz) to write")
    ap.add_argument("--grid", default="72x46x72", help="NLONxNLATxNLEV of the training grids")
    ap.add_argument("--train-seeds", default="11,12,13", help="grid seeds used for training")
    ap.add_argument("--test-seed", type=int, default=14, help="held-out grid seed")
    ap.add_argument("--extra-grid", default=None, help="a second grid (e.g. 144x91x72, NOx-seeded) for more rows")
    ap.add_argument("--extra-seeds", default="", help="seeds of the second grid")
    ap.add_argument("--nsteps", type=int, default=2, help="1200 s steps recorded per grid after spin-up")
    ap.add_argument("--spinup", type=float, default=86400.0)
    ap.add_argument("--epochs", type=int, default=6)
    ap.add_argument("--report", default=None, help="optional JSON report path")
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
    solver = capi.Solver(0, arith="fast", schedule="queue")
    prop = learned.Proposer(0, seed=0)
    log = lambda msg: print(msg, flush=True)
    t0 = time.time()
    parts = []
    for s in (int(v) for v in args.train_seeds.split(",")):
        for nox in (False, True):
            cells = inputs.grid_cells(nlon, nlat, nlev, seed=s, nox_boundary_layer=nox)
            parts.append(learned.collect(solver, prop, cells, nsteps=args.nsteps, spinup=args.spinup, log=log))
            log("seed %d nox %s collected (%.0f s)" % (s, nox, time.time() - t0))
    if args.extra_grid:
        elon, elat, elev = (int(v) for v in args.extra_grid.split("x"))
        for s in (int(v) for v in args.extra_seeds.split(",") if v):
            cells = inputs.grid_cells(elon, elat, elev, seed=s, nox_boundary_layer=True)
            parts.append(learned.collect(solver, prop, cells, nsteps=args.nsteps, spinup=args.spinup, log=log))
            del cells
            log("extra grid seed %d collected (%.0f s)" % (s, time.time() - t0))
    data = {k: torch.cat([p[k] for p in parts]) for k in parts[0]}
    log("training rows: %d" % data["x"].shape[0])
    hist = learned.fit(prop, data, epochs=args.epochs, log=log)
    held = learned.collect(solver, prop, inputs.grid_cells(nlon, nlat, nlev, seed=args.test_seed,
                                                           nox_boundary_layer=True),
                           nsteps=1, spinup=args.spinup)
    score = learned.evaluate(prop, held)
    log("held-out: %s" % json.dumps(score))
    np.savez(args.out, **prop.state())
    if args.report:
        with open(args.report, "w") as f:
            json.dump({"loss_history": hist, "held_out": score, "rows": int(data["x"].shape[0]),
                       "train_seeds": args.train_seeds, "test_seed": args.test_seed, "grid": args.grid,
                       "extra_grid": args.extra_grid, "extra_seeds": args.extra_seeds,
                       "seconds": time.time() - t0}, f, indent=1)


if __name__ == "__main__":
    main()
