"""Autotuner of the chemistry step's launch configuration.

For a representative cell set (device arrays), it times one chemistry step for
each candidate of

* threads per block of the thread-per-cell queue kernel (32, 64, 128, 256),
* cells per thread (the layout: 1 or 2 cells per thread share a table walk),
* the queue chunk: queue positions a lane takes per claim (1, 2, 4, 8; the
  reference's cell loop is SCHEDULE(DYNAMIC, 24)),
* the block-per-cell form: split sums (256 threads), or the level form with
  32 (one warp per cell), 128 or 256 threads per block,
* the hand-over point k (steps after which a cell moves to the block kernel),

one axis at a time from the defaults (coordinate descent, two sweeps), and
returns the fastest settings.  Candidates without the split form give
bit-identical results (the schedule never changes a cell's arithmetic); the
split form regroups sums, so its candidates must agree to rounding (same IERR,
1e-8 relative on species above 1e4 molec/cm3 for 99 % of the cells); `tune`
checks both.

    python geos-chem_gb300/autotune.py --grid 72x46x72 --out tuned.json
"""
import argparse
import json
import os
import sys
import time

AXES = {
    "block": [32, 64, 128, 256],
    "arith": ["fast", "fast2"],
    "queue_chunk": [1, 2, 4, 8],
    "cell_block": [32, 128, 256],
    "block_split": [True, False],
    "evict_after": [0, 2, 4, 8, 16],
}
DEFAULTS = {"block": 128, "arith": "fast", "queue_chunk": 1, "cell_block": 256, "block_split": True,
            "evict_after": 0}
SETTINGS = ("arith", "block", "queue_chunk", "cell_block", "block_split", "evict_after")


def canonical(cfg):
    """The split form always runs 256 threads per block, so its candidates
    differ in nothing when only cell_block differs."""
    cfg = dict(cfg)
    if cfg.get("block_split", True):
        cfg["cell_block"] = 256
    return cfg


def time_step(solver, cfg, case, hs0, order=None, nblock=0):
    """Wall time of one chemistry step (synchronised) and its outputs."""
    import torch

    solver.set(arith=cfg["arith"], schedule="queue", block=cfg["block"], cell_block=cfg["cell_block"],
               evict_after=cfg["evict_after"], block_split=cfg.get("block_split", True),
               queue_chunk=cfg.get("queue_chunk", 1))
    c = case["c"].clone()
    hs = hs0.clone()
    torch.cuda.synchronize()
    t = time.perf_counter()
    solver.fullchem_step(case["dt"], case["met"], case["ph"], c, case["at"], case["rt"], case["ic"], case["rc"],
                         hs, case["ist"], case["rst"], case["ierr"], order=order, nblock=nblock)
    torch.cuda.synchronize()
    return time.perf_counter() - t, (c, case["ierr"].clone())


def _agrees(cfg, got, ref, nvar):
    """Bit for bit, or (split block-per-cell form) to rounding."""
    import torch

    if torch.equal(got[0], ref[0]) and torch.equal(got[1], ref[1]):
        return True
    if not cfg.get("block_split", True) or not torch.equal(got[1], ref[1]):
        return False
    a, b = got[0][:nvar], ref[0][:nvar]
    rel = torch.where(b.abs() > 1e4, (a - b).abs() / b.abs().clamp_min(1e-300), torch.zeros_like(b))
    return (rel.max(dim=0).values <= 1e-8).double().mean().item() >= 0.99


def tune(solver, case, hs0, order=None, nblock=0, sweeps=2, reps=2, axes=None, log=None):
    """Coordinate descent over the axes; returns (best config, seconds, table)."""
    import torch

    import gcchem.capi as capi

    axes = axes or AXES
    best = canonical({k: (DEFAULTS[k] if k not in axes or DEFAULTS[k] in axes[k] else axes[k][0]) for k in DEFAULTS})
    nvar = capi.dims(getattr(solver, "mech", "fullchem"))["nvar"]
    _, ref = time_step(solver, best, case, hs0, order, nblock)
    seen = {}

    def measure(cfg):
        cfg = canonical(cfg)
        key = json.dumps(cfg, sort_keys=True)
        if key not in seen:
            ts = []
            for _ in range(reps):
                t, c = time_step(solver, cfg, case, hs0, order, nblock)
                if not _agrees(cfg, c, ref, nvar):
                    raise RuntimeError("configuration %s changed the results" % key)
                ts.append(t)
            seen[key] = min(ts)
            if log:
                log("%s: %.1f ms" % (key, seen[key] * 1e3))
        return seen[key]

    best_t = measure(best)
    for _ in range(sweeps):
        for axis, values in axes.items():
            for v in values:
                cand = canonical(dict(best, **{axis: v}))
                t = measure(cand)
                if t < best_t:
                    best, best_t = cand, t
    solver.set(**{k: best[k] for k in SETTINGS})
    table = [dict(json.loads(k), ms=v * 1e3) for k, v in sorted(seen.items(), key=lambda kv: kv[1])]
    return best, best_t, table


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--grid", default="72x46x72")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--chained", action="store_true", help="start from the spin-up's KPPHvalue chain")
    ap.add_argument("--out", default=None, help="write the result as JSON")
    args = ap.parse_args(argv)
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    import __graft_entry__

    __graft_entry__.load_package()
    import torch

    import gcchem.capi as capi
    import gcchem.inputs as inputs

    nlon, nlat, nlev = (int(v) for v in args.grid.split("x"))
    cells = inputs.grid_cells(nlon, nlat, nlev, seed=args.seed)
    dev = torch.device("cuda", 0)
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    n = cells["c"].shape[1]
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    case = {"met": T(cells["met"]), "ph": T(cells["photol"]), "c": T(cells["c"]), "at": T(atol), "rt": T(rtol),
            "ic": ic, "rc": rc, "dt": 1200.0, "ist": torch.zeros((20, n), dtype=torch.int32, device=dev),
            "rst": torch.zeros((20, n), dtype=torch.float64, device=dev),
            "ierr": torch.zeros(n, dtype=torch.int32, device=dev)}
    solver = capi.Solver(0, arith="fast", schedule="queue")
    hs = torch.zeros(n, dtype=torch.float64, device=dev)
    solver.fullchem_step(86400.0, case["met"], case["ph"], case["c"], case["at"], case["rt"], ic, rc, hs,
                         case["ist"], case["rst"], case["ierr"])
    hs0 = hs if args.chained else torch.zeros_like(hs)
    best, t, table = tune(solver, case, hs0, log=lambda m: print(m, flush=True))
    print("best %s: %.1f ms" % (json.dumps(best), t * 1e3))
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"best": best, "ms": t * 1e3, "grid": args.grid, "chained": args.chained, "table": table},
                      f, indent=1)


if __name__ == "__main__":
    main()
