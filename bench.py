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


def cpu_baseline_sample(orc, cells_host, rconst_host, atol, rtol, icntrl, rcntrl, target_s, threads):
    """Time the oracle's OpenMP cell loop on evenly spaced cells of the grid."""
    ncell = cells_host["c"].shape[1]

    def run(m):
        idx = np.linspace(0, ncell - 1, m).astype(np.int64)
        c = cells_host["c"][:, idx]
        r = rconst_host[:, idx]
        t0 = time.perf_counter()
        orc.integrate(c, r, atol, rtol, 0.0, DT, icntrl, rcntrl, variant="fast", nthreads=threads)
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
    m = min(ncell, 64 * threads)
    idx = np.linspace(0, ncell - 1, m).astype(np.int64)
    met = cells["met"][:, idx]
    ph = cells["photol"][:, idx]
    c = cells["c"][:, idx].copy()
    r = orc.update_rconst(met, ph, c, variant="fast")
    if args.spinup > 0:
        c, _, _, _ = orc.integrate(c, r, atol, rtol, 0.0, args.spinup, icntrl, rcntrl, variant="fast",
                                   nthreads=threads)
        c = np.maximum(c, 0.0)
    sample = {"c": c}
    times = []
    per = None
    for it in range(args.warmup + args.steps):
        if per is None:
            t0 = time.perf_counter()
            orc.integrate(c[:, : 2 * threads], r[:, : 2 * threads], atol, rtol, 0.0, DT, icntrl, rcntrl,
                          variant="fast", nthreads=threads)
            dt0 = time.perf_counter() - t0
            per = int(min(m, max(threads, 2 * threads * 8.0 / max(dt0, 1e-3))))
        t0 = time.perf_counter()
        rr = orc.update_rconst(met[:, :per], ph[:, :per], c[:, :per], variant="fast")
        orc.integrate(sample["c"][:, :per], rr, atol, rtol, 0.0, DT, icntrl, rcntrl, variant="fast",
                      nthreads=threads)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    value = per / float(np.mean(times))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(times)) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded standard-atmosphere grid, 24 h CPU spin-up of the sampled cells)",
        "config": {"workload": "fullchem 4x5x72 grid (238,464 cells), one 1200 s step, Rodas3, RTOL 5e-3",
                   "cells": ncell, "dt_s": DT, "sample_cells_per_step": per},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
                         "sample": "%d evenly spaced cells of the grid per step (rates + integrate)" % per},
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
    import gcchem.tables as tables_mod
    from gcchem import build as gbuild

    nlon, nlat, nlev = (int(x) for x in args.grid.split("x"))
    cells = inputs.grid_cells(nlon, nlat, nlev, seed=args.seed + rank)
    ncell = cells["c"].shape[1]
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    solver = capi.Solver(local, arith="fast", schedule=args.schedule)
    lib = solver.lib
    lib.gc_kpp_fullchem_step.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double] + \
        [ctypes.c_void_p, ctypes.c_longlong] * 3 + [ctypes.c_void_p] * 5 + \
        [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
         ctypes.c_int, ctypes.c_void_p]
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
    icn = np.ascontiguousarray(icntrl, np.int32)
    rcn = np.ascontiguousarray(rcntrl, np.float64)
    nretry = ctypes.c_int(0)

    def step(c, hstart=None, dt=DT, mem=capi.MEM_DEVICE, stream_ptr=sp, tensors=None):
        tt = tensors or {"met": met, "ph": ph, "c": c, "ist": ist, "rst": rst, "ierr": ierr, "at": at, "rt": rt}
        rc = lib.gc_kpp_fullchem_step(
            solver.ctx, ncell, float(dt), capi._ptr(tt["met"]), ncell, capi._ptr(tt["ph"]), ncell,
            capi._ptr(tt["c"]), ncell, capi._ptr(tt["at"]), capi._ptr(tt["rt"]),
            icn.ctypes.data_as(ctypes.c_void_p), rcn.ctypes.data_as(ctypes.c_void_p),
            capi._ptr(hstart), capi._ptr(tt["ist"]), capi._ptr(tt["rst"]), ncell, capi._ptr(tt["ierr"]),
            ctypes.byref(nretry), mem, ctypes.c_void_p(stream_ptr))
        if rc != 0:
            raise capi.GcKppError(rc, lib.gc_kpp_last_error().decode())

    # spin-up (untimed): 24 h from the random initial state
    t0 = time.perf_counter()
    c_spun = c0.clone()
    if args.spinup > 0:
        step(c_spun, dt=args.spinup)
    torch.cuda.synchronize()
    spin_s = time.perf_counter() - t0
    spin_steps = float(ist[2].double().mean().item())

    # rate constants of the spun-up state (for the roofline / CPU baseline)
    work = c_spun.clone()
    for _ in range(args.warmup):
        work.copy_(c_spun)
        step(work)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    solver.set_timing = None
    lib.gc_kpp_ctx_set_option(solver.ctx, 6, 1)  # GC_KPP_OPT_TIMING
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    kernel_ms = []
    launches = 0
    ev0.record(stream)
    for _ in range(args.steps):
        work.copy_(c_spun)
        step(work)
        ms = ctypes.c_double(0.0)
        nl = ctypes.c_int(0)
        lib.gc_kpp_last_kernel_ms(solver.ctx, ctypes.byref(ms), ctypes.byref(nl))
        kernel_ms.append(ms.value / max(nl.value, 1))
        launches += lib.gc_kpp_last_launch_count(solver.ctx)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    lib.gc_kpp_ctx_set_option(solver.ctx, 6, 0)
    ms_step = ev0.elapsed_time(ev1) / args.steps
    if world > 1:
        t = torch.tensor([ms_step], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step = float(t.item())
    value = world * ncell / (ms_step * 1e-3)

    ist_h = ist.cpu().numpy()
    ierr_h = ierr.cpu().numpy()
    tabs = tables_mod.Tables(__import__("gcchem.mechanism", fromlist=["x"]).load_ir())
    flops = algorithmic_flops(tabs, ist_h)
    kms = float(np.mean(kernel_ms))
    achieved_tf = flops / (kms * 1e-3) / 1e12

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

    # end-to-end: the same chemistry step through the C ABI with host buffers
    e2e = None
    if rank == 0 or world > 1:
        pin = {
            "met": torch.tensor(cells["met"]).pin_memory(), "ph": torch.tensor(cells["photol"]).pin_memory(),
            "c": c_spun.cpu().pin_memory(), "ist": torch.zeros((20, ncell), dtype=torch.int32).pin_memory(),
            "rst": torch.zeros((20, ncell), dtype=torch.float64).pin_memory(),
            "ierr": torch.zeros(ncell, dtype=torch.int32).pin_memory(),
            "at": torch.tensor(atol).contiguous(), "rt": torch.tensor(rtol).contiguous(),
        }
        c_host0 = pin["c"].clone()
        tms = []
        for it in range(1 + min(args.steps, 2)):
            pin["c"].copy_(c_host0)
            t0 = time.perf_counter()
            step(None, mem=capi.MEM_HOST, stream_ptr=sp, tensors=pin)
            dt = time.perf_counter() - t0
            if it > 0:
                tms.append(dt)
        h2d = ncell * 8 * (18 + 200 + 356) + 2 * 353 * 8
        d2h = ncell * (8 * 356 + 4 + 20 * 4 + 20 * 8)
        e2e = {"value": world * ncell / float(np.mean(tms)), "unit": "cells/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        orc = __graft_entry__.load_oracle()
        r_dev = torch.zeros((1058, ncell), dtype=torch.float64, device=dev)
        solver.update_rconst(met, ph, c_spun, r_dev)
        threads = os.cpu_count() or 1
        host = {"c": c_spun.cpu().numpy()}
        m, dt = cpu_baseline_sample(orc, host, r_dev.cpu().numpy(), atol, rtol, icntrl, rcntrl, args.cpu_seconds,
                                    threads)
        cpu = {"value": m / dt, "unit": "cells/s", "cores": threads, "kind": "port",
               "sample": "%d evenly spaced spun-up cells of the grid, one 1200 s Integrate each, oracle -O3 "
                         "OpenMP DYNAMIC,24 (%.1f s)" % (m, dt)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded standard-atmosphere 4x5x72 grid, 24 h GPU spin-up)",
            "config": {"workload": "fullchem 4x5x72 grid (238,464 cells), one 1200 s chemistry step, Rodas3, "
                                   "RTOL 5e-3 / ATOL 1e-2, FP64",
                       "cells_per_gpu": ncell, "dt_s": DT, "solver": "%s schedule, fast arithmetic" % args.schedule,
                       "l2": "inputs larger than L2 (C 0.68 GB, RCONST 2.0 GB per step)",
                       "steps_per_cell": float(ist_h[2].mean()), "max_steps_per_cell": int(ist_h[2].max()),
                       "ierr_ok_fraction": float((ierr_h == 1).mean()), "retried_cells": int(nretry.value),
                       "spinup_s": args.spinup, "spinup_wall_s": spin_s, "spinup_steps_per_cell": spin_steps},
            "e2e": e2e,
            "gpu_launches": int(launches),
            "roofline": {"bound": "fp64", "achieved": achieved_tf,
                         "peak": (peak_gf / 1e3) if peak_gf else None, "unit": "TFLOP/s",
                         "frac": (achieved_tf / (peak_gf / 1e3)) if peak_gf else None, "traffic": None,
                         "kernel": "gckpp::ros_kernel (Rosenbrock, thread per cell)",
                         "kernel_ms": kms, "flops_per_launch": flops,
                         "peak_source": "measured FP64 FMA probe on this GPU"},
            "cpu_baseline": cpu,
            "clocks": clocks,
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
