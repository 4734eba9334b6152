"""Benchmark: fullchem cells/s for one 1200 s chemistry step on a 4x5x72 grid.

Workload: 72 x 46 x 72 = 238,464 cells (the 4 deg x 5 deg global grid with 72
levels), one chemistry step of DT = 1200 s through the Do_FullChem cell-loop
replacement (rates, Rodas3 integration with RTOL 5e-3 / ATOL 1e-2 from the
species database, retry, clamp), FP64 throughout.  Cell states come from the
seeded synthetic generator (standard atmosphere, solar zenith angle day/night
split, random initial concentrations) spun up 24 h on the GPU before timing.

A "step" is one pass of the chemistry step over the whole grid; before each
step the concentrations are reset to the spun-up state.  The per-step inputs
(C 0.68 GB, RCONST 2.0 GB, the 40 GB workspace) are larger than the 129 MB L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the CPU restatement of the reference cell loop
(the oracle's OpenMP build, all host cores) on bounded samples of the same
workload.  Prints one JSON line on rank 0.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402

METRIC = "fullchem cells/s per 1200 s step, learned-binned vs plain GPU, at RTOL 5e-3"
GRID = (72, 46, 72)
DT = 1200.0
SPINUP_S = 86400.0
# hand-over point of the learned arms.  From a cold start the proposals are
# capped at learned.H0_CAP (16.8 s, a step of the plain method's ramp from
# DeltaMin), so a cell needs about 4 Rosenbrock steps; the best k of a sweep
# with that cap on this grid was 4 (k = 5, 6 slower).  On the KPPHvalue chain
# k = 1 (1.15M cells/s; k = 2 964k, k = 3 855k).
EVICT_LEARNED = 4
EVICT_LEARNED_CHAINED = 1
# DRAM bytes (read + write) per Rosenbrock step attempt of the learned
# step's three Rosenbrock launches, measured with ncu (dram__bytes_read.sum
# + dram__bytes_write.sum) on this workload: 1,090.3 GB for 998,044 attempts
# (profiles/learned_step_grid72x46x72_launch_list.md).  roofline.traffic is
# this figure times the attempts (ISTATUS(6), decompositions) of the timed step.
DRAM_BYTES_PER_ATTEMPT = 1.0924e6
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "geos-chem_gb300", "weights", "proposer_fullchem.npz")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--schedule", default="queue", choices=["plain", "queue"])
    ap.add_argument("--grid", default="%dx%dx%d" % GRID)
    ap.add_argument("--spinup", type=float, default=SPINUP_S, help="spin-up seconds before timing")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU-baseline sample duration")
    ap.add_argument("--weights", default=WEIGHTS, help="trained proposer weights (.npz)")
    ap.add_argument("--error-cells", type=int, default=2048, help="cells integrated at RTOL 1e-8 for the error")
    ap.add_argument("--e2e-chunks", type=int, default=0,
                    help="> 0: the end-to-end step streams this many chunks through gcchem.stream.Streamer "
                         "(0: one host-memory call of the C ABI)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_flops(tables, istatus, method_S=4):
    """FP64 operations of the reference algorithm implied by the ISTATUS
    counters: Nfun*Fun + Njac*Jac + Ndec*(LU + Ghimj diagonal) + Nsol*Solve +
    Nstp*(Rodas3 stage/update/error-norm vector work)."""
    f = tables.flops()
    nvar = tables.nvar
    # Rodas3 per attempt: K2 (1 axpy), Ynew3 (1), K3 (2), Ynew4 (2), K4 (3),
    # Ynew (3), Yerr (1) axpys of 2 flops, error norm 5 flops per species.
    vec = (1 + 1 + 2 + 2 + 3 + 3 + 1) * 2 * nvar + 5 * nvar
    tot = (istatus[0].sum() * f["fun"] + istatus[1].sum() * f["jac"] + istatus[5].sum() * (f["decomp"] + 1)
           + istatus[6].sum() * f["solve"] + istatus[2].sum() * vec)
    return float(tot)


def cpu_baseline_sample(orc, cells_host, rconst_host, atol, rtol, icntrl, rcntrl, target_s, threads, hstart=None):
    """Time the oracle's OpenMP cell loop on evenly spaced cells of the grid."""
    ncell = cells_host["c"].shape[1]

    def run(m):
        idx = np.linspace(0, ncell - 1, m).astype(np.int64)
        c = cells_host["c"][:, idx]
        r = rconst_host[:, idx]
        hs = None if hstart is None else np.ascontiguousarray(hstart[idx])
        t0 = time.perf_counter()
        orc.integrate(c, r, atol, rtol, 0.0, DT, icntrl, rcntrl, hstart=hs, variant="fast", nthreads=threads)
        return time.perf_counter() - t0

    m = 4 * threads
    dt = run(m)
    m2 = int(min(ncell, max(m, m * target_s / max(dt, 1e-3))))
    dt2 = run(m2)
    return m2, dt2


def run_reference(args):
    """CPU reference arm: the oracle's OpenMP loop on bounded samples."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    gcchem = __graft_entry__.load_package()  # noqa: F841
    import gcchem.inputs as inputs

    orc = __graft_entry__.load_oracle()
    threads = os.cpu_count() or 1
    nlon, nlat, nlev = (int(x) for x in args.grid.split("x"))
    cells = inputs.grid_cells(nlon, nlat, nlev, seed=args.seed)
    ncell = cells["c"].shape[1]
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    # sample cells evenly over the grid; spin them up on the CPU
    m = min(ncell, 256 * threads)
    idx = np.linspace(0, ncell - 1, m).astype(np.int64)
    met = cells["met"][:, idx]
    ph = cells["photol"][:, idx]
    c = cells["c"][:, idx].copy()
    r = orc.update_rconst(met, ph, c, variant="fast")
    if args.spinup > 0:
        c, _, _, _ = orc.integrate(c, r, atol, rtol, 0.0, args.spinup, icntrl, rcntrl, variant="fast",
                                   nthreads=threads)
        c = np.maximum(c, 0.0)
    times = []
    sel = None
    for it in range(args.warmup + args.steps):
        if sel is None:
            t0 = time.perf_counter()
            orc.integrate(c[:, : 2 * threads], r[:, : 2 * threads], atol, rtol, 0.0, DT, icntrl, rcntrl,
                          variant="fast", nthreads=threads)
            dt0 = time.perf_counter() - t0
            per = int(min(m, max(threads, 2 * threads * 8.0 / max(dt0, 1e-3))))
            # the timed cells: evenly spaced over the sample, so over the whole grid
            sel = np.unique(np.linspace(0, m - 1, per).astype(np.int64))
            met_s, ph_s, c_s = (np.ascontiguousarray(x[:, sel]) for x in (met, ph, c))
        t0 = time.perf_counter()
        rr = orc.update_rconst(met_s, ph_s, c_s, variant="fast")
        orc.integrate(c_s, rr, atol, rtol, 0.0, DT, icntrl, rcntrl, variant="fast", nthreads=threads)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    per = len(sel)
    value = per / float(np.mean(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(times)) * 1e3,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded standard-atmosphere grid, 24 h CPU spin-up of the sampled cells)",
        "config": {"workload": "fullchem 4x5x72 grid (238,464 cells), one 1200 s step, Rodas3, RTOL 5e-3",
                   "cells": ncell, "dt_s": DT, "sample_cells_per_step": per},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
                         "sample": "%d evenly spaced cells of the grid per step (rates + integrate from "
                                   "Hstart = 0, from the CPU-spun state)" % per},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    __graft_entry__.load_package()
    import gcchem.capi as capi
    import gcchem.inputs as inputs
    import gcchem.learned as learned
    import gcchem.tables as tables_mod
    from gcchem import build as gbuild

    nlon, nlat, nlev = (int(x) for x in args.grid.split("x"))
    # every rank builds the same grid; with N > 1 ranks each times its own
    # shard of it (gcchem.shard, balanced by the proposer's stiffness bins)
    cells = inputs.grid_cells(nlon, nlat, nlev, seed=args.seed)
    ncell = cells["c"].shape[1]
    ncell_total = ncell
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    solver = capi.Solver(local, arith="fast", schedule=args.schedule)
    lib = solver.lib
    lib.gc_kpp_last_kernel_ms.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_int)]
    lib.gc_kpp_last_launch_count.argtypes = [ctypes.c_void_p]

    def T(x, dt=torch.float64):
        return torch.tensor(x, dtype=dt, device=dev).contiguous()

    met, ph, c0 = T(cells["met"]), T(cells["photol"]), T(cells["c"])
    at, rt = T(atol), T(rtol)
    ist = torch.zeros((20, ncell), dtype=torch.int32, device=dev)
    rst = torch.zeros((20, ncell), dtype=torch.float64, device=dev)
    ierr = torch.zeros(ncell, dtype=torch.int32, device=dev)
    dev_t = {"met": met, "ph": ph, "ist": ist, "rst": rst, "ierr": ierr, "at": at, "rt": rt}
    last = {"nretry": 0}

    def step(c, hs, order=None, nblock=0, dt=DT, tt=dev_t, solver_=solver, rtol_=None):
        last["nretry"] = solver_.fullchem_step(dt, tt["met"], tt["ph"], c, tt["at"],
                                               tt["rt"] if rtol_ is None else rtol_, icntrl, rcntrl, hs,
                                               tt["ist"], tt["rst"], tt["ierr"], order=order, nblock=nblock,
                                               stream=sp)

    # spin-up (untimed): 24 h from the random initial state; hs_spun receives
    # the KPPHvalue chain (RSTATE(Nhnew)) that the timed steps start from
    t0 = time.perf_counter()
    c_spun = c0.clone()
    hs_spun = torch.zeros(ncell, dtype=torch.float64, device=dev)
    if args.spinup > 0:
        step(c_spun, hs_spun, dt=args.spinup)
    torch.cuda.synchronize()
    spin_s = time.perf_counter() - t0
    spin_steps = float(ist[2].double().mean().item())

    prop = learned.Proposer(local)
    prop.load_state(dict(np.load(args.weights)))

    shard = (0, ncell)
    if world > 1:
        # one grid split N ways with no collective on the data path: every
        # rank spun up the whole grid (the same bits on every GPU), weighs
        # each cell by its predicted stiffness bin and keeps its range
        import gcchem.shard as shard_mod

        x = prop.features(met, ph, c_spun, stream=sp)
        _, bins = prop.propose(x, stream=sp, hmax=DT)
        shard = shard_mod.shard_range(ncell, rank, world, shard_mod.work_from_bins(bins.cpu().numpy()))
        a, b = shard
        met, ph = met[:, a:b].contiguous(), ph[:, a:b].contiguous()
        c_spun, hs_spun = c_spun[:, a:b].contiguous(), hs_spun[a:b].contiguous()
        ncell = b - a
        ist = torch.zeros((20, ncell), dtype=torch.int32, device=dev)
        rst = torch.zeros((20, ncell), dtype=torch.float64, device=dev)
        ierr = torch.zeros(ncell, dtype=torch.int32, device=dev)
        dev_t.update(met=met, ph=ph, ist=ist, rst=rst, ierr=ierr)

    def plain_arm(w, hs):
        solver.set(evict_after=0)
        step(w, hs)

    def handover_arm(k):
        # no learning: grid order, cells still running after k steps finish
        # block-per-cell
        def arm(w, hs):
            solver.set(evict_after=k)
            step(w, hs)
        return arm

    def learned_arm(w, hs, met_=met, ph_=ph, tt=dev_t, evict=EVICT_LEARNED):
        # H0 proposals seed RCNTRL(3) where the cell has no KPPHvalue yet;
        # stiffness bins order the queue and the top bin goes block-per-cell;
        # cells the network missed are handed over after `evict` steps
        solver.set(evict_after=evict)
        _, _, order = learned.plan(prop, met_, ph_, w, stream=sp, hstart=hs, hmax=DT)
        nheavy = int(prop.last_counts[learned.NBIN - 1].item())
        last["nblock"] = nheavy
        step(w, hs, order=order, nblock=nheavy, tt=tt)

    # cold: every cell starts from RCNTRL(3) = 0 (DeltaMin) unless the network
    # proposes H0; chained: every cell starts from its KPPHvalue.  The
    # hand-over-only arms use the best k of a sweep over 2, 4, 8, 16 steps.
    cold0 = torch.zeros_like(hs_spun)
    arms = {"plain": (plain_arm, 0, cold0), "handover": (handover_arm(16), 0, cold0),
            "learned": (learned_arm, learned.PLAN_LAUNCHES, cold0),
            "plain_chained": (plain_arm, 0, hs_spun), "handover_chained": (handover_arm(2), 0, hs_spun),
            "learned_chained": (lambda w, hs: learned_arm(w, hs, evict=EVICT_LEARNED_CHAINED),
                                learned.PLAN_LAUNCHES, hs_spun)}

    def time_arm(name):
        fn, extra, hs0 = arms[name]
        work = c_spun.clone()
        hs = hs0.clone()
        for _ in range(args.warmup):
            work.copy_(c_spun)
            hs.copy_(hs0)
            fn(work, hs)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        lib.gc_kpp_ctx_set_option(solver.ctx, 6, 1)  # GC_KPP_OPT_TIMING
        sampler = ClockSampler(local)
        sampler.start()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        kernel_ms, launches = [], 0
        ev0.record(stream)
        for _ in range(args.steps):
            work.copy_(c_spun)  # reset to the spun-up state (and its KPPHvalue chain)
            hs.copy_(hs0)
            fn(work, hs)
            ms = ctypes.c_double(0.0)
            nl = ctypes.c_int(0)
            lib.gc_kpp_last_kernel_ms(solver.ctx, ctypes.byref(ms), ctypes.byref(nl))
            kernel_ms.append(ms.value)
            launches += lib.gc_kpp_last_launch_count(solver.ctx) + extra
        ev1.record(stream)
        torch.cuda.synchronize()
        clocks = sampler.stop()
        lib.gc_kpp_ctx_set_option(solver.ctx, 6, 0)
        ms_step = ev0.elapsed_time(ev1) / args.steps
        if world > 1:
            t = torch.tensor([ms_step], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms_step = float(t.item())
        return {"ms_per_step": ms_step, "value": ncell_total / (ms_step * 1e-3),
                "kernel_ms": float(np.mean(kernel_ms)), "gpu_launches": int(launches), "clocks": clocks,
                "ist": ist.cpu().numpy(), "ierr": ierr.cpu().numpy(), "retried_cells": int(last["nretry"]),
                "block_per_cell_cells": int(last.get("nblock", 0)) if name.startswith("learned") else 0,
                "c": work.clone()}

    res = {name: time_arm(name) for name in arms}
    head = res["learned"]
    tabs = tables_mod.Tables(__import__("gcchem.mechanism", fromlist=["x"]).load_ir())
    flops = algorithmic_flops(tabs, head["ist"])
    achieved_tf = flops / (head["kernel_ms"] * 1e-3) / 1e12
    flops_plain = algorithmic_flops(tabs, res["plain"]["ist"])
    achieved_plain_tf = flops_plain / (res["plain"]["kernel_ms"] * 1e-3) / 1e12
    flops_ho = algorithmic_flops(tabs, res["handover"]["ist"])
    achieved_ho_tf = flops_ho / (res["handover"]["kernel_ms"] * 1e-3) / 1e12

    # FP64 peak measured on this GPU (roofline denominator)
    peak_gf = None
    try:
        probe = ctypes.CDLL(gbuild.probe_path())
        probe.gc_probe_fp64_gflops.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        g = ctypes.c_double(0.0)
        if probe.gc_probe_fp64_gflops(local, ctypes.byref(g)) == 0:
            peak_gf = g.value
    except OSError:
        pass

    # error of both forms against an RTOL = 1e-8 FP64 integration (strict
    # arithmetic) of evenly spaced cells, from the same state and chain
    idx = torch.linspace(0, ncell - 1, min(ncell, args.error_cells), device=dev).long()
    sub = {k: v.index_select(1, idx).contiguous() for k, v in (("met", met), ("ph", ph))}
    m = idx.numel()
    sub.update(ist=torch.zeros((20, m), dtype=torch.int32, device=dev),
               rst=torch.zeros((20, m), dtype=torch.float64, device=dev),
               ierr=torch.zeros(m, dtype=torch.int32, device=dev), at=at, rt=rt)
    tight = capi.Solver(local, arith="strict", schedule="queue")
    c_ref = c_spun.index_select(1, idx).contiguous()
    step(c_ref, hs_spun.index_select(0, idx).contiguous(), tt=sub, solver_=tight,
         rtol_=torch.full_like(rt, 1e-8))
    torch.cuda.synchronize()
    tight_steps = float(sub["ist"][2].double().mean().item())
    tight.close()
    nvar = 353

    def rel_err(c):
        got = c.index_select(1, idx)[:nvar]
        ref = c_ref[:nvar]
        mask = ref > 1e4
        e = ((got - ref).abs() / ref.clamp_min(1e-300))[mask]
        q = torch.quantile(e.float(), torch.tensor([0.5, 0.99, 0.999], device=e.device)).tolist()
        return {"max": float(e.max().item()), "p99.9": q[2], "p99": q[1], "median": float(e.median().item())}

    errors = {name: rel_err(res[name]["c"]) for name in arms}

    # end to end through the reference-facing call: the grid's arrays in
    # page-locked host memory and one gc_kpp_fullchem_step_learned with
    # GC_KPP_MEM_HOST, which stages met, the J-value rows that the rates and
    # the features read, C and KPPHvalue in, and C, KPPHvalue, ISTATUS and
    # IERR out (SM copies through the host memory's device alias), all inside
    # the timed region.  --e2e-chunks N > 0 streams N chunks through
    # gcchem.stream.Streamer instead.
    e2e = None
    if rank == 0 or world > 1:
        cp = learned.CProposer(prop, local)
        solver.set(evict_after=EVICT_LEARNED, async_steps=False)
        pin = lambda x: x.contiguous().cpu().pin_memory()
        if args.e2e_chunks <= 0:
            h = {"met": pin(met), "ph": pin(ph), "c0": pin(c_spun), "at": at.cpu().numpy(), "rt": rt.cpu().numpy()}
            h["c"] = torch.empty_like(h["c0"]).pin_memory()
            h["hs"] = torch.zeros(ncell, dtype=torch.float64).pin_memory()
            h["ist"] = torch.zeros((20, ncell), dtype=torch.int32).pin_memory()
            h["ierr"] = torch.zeros(ncell, dtype=torch.int32).pin_memory()
            tms = []
            for it in range(1 + min(args.steps, 3)):
                h["c"].copy_(h["c0"])  # the step's input state (host memcpy, outside the timed region)
                h["hs"].zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                solver.fullchem_step_learned(cp.handle, DT, h["met"], h["ph"], h["c"], h["at"], h["rt"], icntrl,
                                             rcntrl, h["hs"], h["ist"], None, h["ierr"])
                torch.cuda.synchronize()
                if it > 0:
                    tms.append(time.perf_counter() - t0)
            steps_e2e = h["ist"][2].numpy()
            nph = int((capi.photol_rows(solver.lib) | np.isin(np.arange(200), learned.feature_rows()[0])).sum())
            h2d = 8 * (18 + nph + c_spun.shape[0] + 1)
            d2h = 8 * (c_spun.shape[0] + 1) + 4 * (20 + 1)
            path = ("gc_kpp_fullchem_step_learned with GC_KPP_MEM_HOST on page-locked host arrays (SM staging "
                    "copies, %d of 200 PHOTOL rows)" % nph)
            nch = 1
        else:
            import gcchem.stream as stream

            nch = args.e2e_chunks
            chunk = -(-ncell // nch)
            host_in = {"met": met.cpu(), "ph": ph.cpu(), "c": c_spun.cpu(), "hs": cold0.cpu()}
            chunks = []
            for i0 in range(0, ncell, chunk):
                i1 = min(ncell, i0 + chunk)
                ch = {k: v[..., i0:i1].contiguous().pin_memory() for k, v in host_in.items()}
                ch.update(c_out=torch.empty_like(ch["c"]).pin_memory(), hs_out=torch.empty_like(ch["hs"]).pin_memory(),
                          steps=torch.zeros(i1 - i0, dtype=torch.int32).pin_memory(),
                          ierr=torch.zeros(i1 - i0, dtype=torch.int32).pin_memory())
                chunks.append(ch)
            solvers = [solver]
            if len(chunks) > 1:
                solvers.append(capi.Solver(local, arith="fast", schedule=args.schedule))
            for sv in solvers:
                sv.set(evict_after=EVICT_LEARNED)
            st = stream.Streamer(solver, ncell, chunk, proposer=cp, solvers=solvers, photol_rows=stream.photol_runs())
            st.step(chunks, DT, at, rt, icntrl, rcntrl)  # synchronous: sizes each context's buffers
            for sv in solvers:
                sv.set(async_steps=True)
            tms = []
            for it in range(1 + min(args.steps, 3)):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                st.step(chunks, DT, at, rt, icntrl, rcntrl)
                torch.cuda.synchronize()
                if it > 0:
                    tms.append(time.perf_counter() - t0)
            for sv in solvers:
                sv.set(async_steps=False)
            steps_e2e = np.concatenate([ch["steps"].numpy() for ch in chunks])
            h2d, d2h = st.bytes_per_cell()
            path = ("gcchem.stream.Streamer over gc_kpp_fullchem_step_learned, pinned host chunks, %d chunk(s) on "
                    "%d solver context(s)" % (len(chunks), len(solvers)))
            for sv in solvers[1:]:
                sv.close()
        tmax = float(np.mean(tms))
        if world > 1:
            t = torch.tensor([tmax], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            tmax = float(t.item())
        e2e = {"value": ncell_total / tmax, "unit": "cells/s", "h2d_bytes_per_step": int(h2d * ncell_total),
               "d2h_bytes_per_step": int(d2h * ncell_total), "chunks": nch,
               "steps_match_learned_arm": bool(np.array_equal(steps_e2e, head["ist"][2])), "path": path}
        cp.close()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        orc = __graft_entry__.load_oracle()
        r_dev = torch.zeros((1058, ncell), dtype=torch.float64, device=dev)
        solver.update_rconst(met, ph, c_spun, r_dev)
        threads = os.cpu_count() or 1
        host = {"c": c_spun.cpu().numpy()}
        m_cpu, dt = cpu_baseline_sample(orc, host, r_dev.cpu().numpy(), atol, rtol, icntrl, rcntrl,
                                        args.cpu_seconds, threads)
        cpu = {"value": m_cpu / dt, "unit": "cells/s", "cores": threads, "kind": "port",
               "sample": "%d evenly spaced spun-up cells of the grid, one 1200 s Integrate each from "
                         "Hstart = 0, oracle -O3 OpenMP DYNAMIC,24 (%.1f s)" % (m_cpu, dt)}

    if rank == 0:
        summary = lambda r, name: {"value": r["value"], "ms_per_step": r["ms_per_step"], "kernel_ms": r["kernel_ms"],
                             "steps_per_cell": float(r["ist"][2].mean()),
                             "max_steps_per_cell": int(r["ist"][2].max()),
                             "ierr_ok_fraction": float((r["ierr"] == 1).mean()),
                             "retried_cells": r["retried_cells"], "error_vs_rtol_1e-8": errors[name],
                             "block_per_cell_cells": r["block_per_cell_cells"]}
        arms_out = {name: summary(res[name], name) for name in arms}
        line = {
            "metric": METRIC, "value": head["value"], "unit": "cells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded standard-atmosphere 4x5x72 grid, 24 h GPU spin-up)",
            "config": {"workload": "fullchem 4x5x72 grid (238,464 cells), one 1200 s chemistry step, Rodas3, "
                                   "RTOL 5e-3 / ATOL 1e-2, FP64, Hstart = 0 (DeltaMin) unless the network "
                                   "proposes H0",
                       "cells_per_gpu": ncell, "dt_s": DT,
                       "shard": [int(shard[0]), int(shard[1])] if world > 1 else None,
                       "solver": "%s schedule, fast arithmetic, 1 cell per thread" % args.schedule,
                       "value_is": "learned-binned arm: MLP H0 proposals (at most %.3g s) seed Hstart, "
                                   "stiffness bins order the persistent queue and send the top bin "
                                   "block-per-cell, cells still running after %d steps finish block-per-cell"
                                   % (prop.h0_cap, EVICT_LEARNED),
                       "l2": "inputs larger than L2 (C 0.68 GB, RCONST 2.0 GB per step)",
                       "weights": os.path.basename(args.weights),
                       "spinup_s": args.spinup, "spinup_wall_s": spin_s, "spinup_steps_per_cell": spin_steps,
                       "error_cells": int(m), "rtol_1e-8_steps_per_cell": tight_steps},
            "plain": arms_out["plain"],
            "learned": arms_out["learned"],
            "learned_over_plain": head["value"] / res["plain"]["value"],
            "handover_only": dict(arms_out["handover"], evict_after=16,
                                  note="no network: grid order, cells past 16 steps finish block-per-cell"),
            "learned_over_handover_only": head["value"] / res["handover"]["value"],
            "chained": {"note": "every cell starts from its KPPHvalue (RSTATE(Nhnew) of the spin-up), "
                                "as Do_FullChem does after its first step",
                        "plain": arms_out["plain_chained"], "learned": arms_out["learned_chained"],
                        "handover_only": dict(arms_out["handover_chained"], evict_after=2),
                        "learned_over_plain": res["learned_chained"]["value"] / res["plain_chained"]["value"]},
            "e2e": e2e,
            "gpu_launches": head["gpu_launches"],
            "roofline": {"bound": "fp64", "achieved": achieved_tf,
                         "peak": (peak_gf / 1e3) if peak_gf else None, "unit": "TFLOP/s",
                         "frac": (achieved_tf / (peak_gf / 1e3)) if peak_gf else None,
                         "traffic": float(DRAM_BYTES_PER_ATTEMPT * head["ist"][5].sum(dtype=np.int64)),
                         "traffic_note": "bytes per launch: ncu DRAM read + write per step attempt of this "
                                         "workload (1.09 MB) x the step attempts of the timed step; the "
                                         "algorithmic minimum is the cells' inputs and outputs (~3 KB a cell)",
                         "kernel": "gckpp::ros_kernel (thread per cell) + gckpp::ros_block_kernel (block per "
                                   "cell), learned arm, one step's Rosenbrock launches",
                         "kernel_ms": head["kernel_ms"], "flops_per_launch": flops,
                         "peak_source": "measured FP64 FMA probe on this GPU (of measured)",
                         "plain_kernel": {"kernel": "gckpp::ros_kernel, plain arm", "achieved": achieved_plain_tf,
                                          "frac": (achieved_plain_tf / (peak_gf / 1e3)) if peak_gf else None,
                                          "kernel_ms": res["plain"]["kernel_ms"], "flops_per_launch": flops_plain},
                         "handover_only_kernel": {
                             "kernel": "gckpp::ros_kernel + block-per-cell hand-over after 16 steps, no network",
                             "achieved": achieved_ho_tf,
                             "frac": (achieved_ho_tf / (peak_gf / 1e3)) if peak_gf else None,
                             "kernel_ms": res["handover"]["kernel_ms"], "flops_per_launch": flops_ho}},
            "cpu_baseline": cpu,
            "clocks": head["clocks"],
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
