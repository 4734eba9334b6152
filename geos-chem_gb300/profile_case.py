"""A small, self-contained chemistry case for profiling the kernels.

    python geos-chem_gb300/profile_case.py --cells 4096 --tout 60 --arith fast [--probe]
    python geos-chem_gb300/profile_case.py --grid 72x46x8 --binned 64 [--phase-cycles]
    python geos-chem_gb300/profile_case.py --grid 72x46x24 --learned
    python geos-chem_gb300/profile_case.py --grid 72x46x24 --autoreduce 100 [--append]
    python geos-chem_gb300/profile_case.py --routines 4096

Box cells (``inputs.box_cells``) are integrated once from 0 to TOUT with
``Solver.integrate``; ``--grid`` instead spins up a grid and runs one 1200 s
chemistry step (``--binned N``: the N cells with the most steps go
block-per-cell; ``--learned``: the learned form from a cold start;
``--autoreduce THR``: the timed step with auto-reduction).  It prints the
time of the timed call (one cold run), the ISTATUS sums and the algorithmic
FP64 operations of the reference routines for them; ``--probe`` also runs
the FP64 throughput probe.  Meant to run under ncu on one GPU with few
launches.
"""
import argparse
import ctypes
import os
import sys


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--cells", type=int, default=4096)
    ap.add_argument("--tout", type=float, default=60.0)
    ap.add_argument("--arith", default="fast", choices=["fast", "strict", "fast2", "fast4"])
    ap.add_argument("--schedule", default="queue", choices=["plain", "queue"])
    ap.add_argument("--block", type=int, default=128)
    ap.add_argument("--max-slots", type=int, default=0, help="cap on cells in flight (0: all resident threads)")
    ap.add_argument("--queue-chunk", type=int, default=1, help="queue positions a lane takes per claim")
    ap.add_argument("--phase-cycles", action="store_true",
                    help="with --grid: build and use the profiling library whose split block-per-cell kernel "
                         "counts clock64 cycles per phase, and print them per step attempt of the timed step")
    ap.add_argument("--grid", default=None, help="NLONxNLATxNLEV: grid step instead of box cells")
    ap.add_argument("--binned", type=int, default=0, help="grid step: cells sent block-per-cell")
    ap.add_argument("--cold", action="store_true",
                    help="grid step without --learned: Hstart = 0 (DeltaMin) instead of the spin-up's KPPHvalue")
    ap.add_argument("--learned", action="store_true",
                    help="grid step: the learned form (cold start, capped H0 proposals, bins, hand-over)")
    ap.add_argument("--evict", type=int, default=4, help="with --learned: hand-over after this many steps")
    ap.add_argument("--block-form", default="split", choices=["split", "level"],
                    help="block-per-cell kernel form (GC_KPP_OPT_BLOCK_SPLIT 1 or 0)")
    ap.add_argument("--repeat", type=int, default=1,
                    help="grid step: run the timed step this many times from the same state (the last is reported)")
    ap.add_argument("--producers", action="store_true",
                    help="grid step: after it, time the per-cell producers (sulfur, SET_SO2, HetState, HetDropChem)")
    ap.add_argument("--copies", action="store_true",
                    help="grid step: after it, time 1 GB host<->device copies of page-locked buffers by the copy "
                         "engine and by gc_kpp_copy_rows (SM copies), each right after a step")
    ap.add_argument("--probe", action="store_true")
    ap.add_argument("--routines", type=int, default=0,
                    help="> 0: only launch each mechanism routine once over this many cells (decomp, solve, "
                         "fun, bprod, jac; libgckpp_routines.so), to count instructions per routine")
    ap.add_argument("--autoreduce", type=float, default=0.0,
                    help="> 0: the timed step or integration with auto-reduction (ICNTRL(12)=1) at this "
                         "RCNTRL(12) threshold (thread-per-cell kernel; not with --learned/--binned)")
    ap.add_argument("--append", action="store_true", help="with --autoreduce: the append form (ICNTRL(13)=1)")
    args = ap.parse_args(argv)

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    import __graft_entry__

    __graft_entry__.load_package()
    import numpy as np
    import torch

    import gcchem.build as build

    if args.routines:
        rb = ctypes.CDLL(build.routines_path())
        rb.gc_routine_bench.argtypes = [ctypes.c_int, ctypes.c_int]
        rcode = rb.gc_routine_bench(0, args.routines)
        print("routines over %d cells: rc %d" % (args.routines, rcode))
        if rcode != 0:
            raise SystemExit(1)
        return
    import gcchem.capi as capi
    import gcchem.inputs as inputs
    from gcchem.mechanism import load_ir
    from gcchem.tables import Tables

    dev = torch.device("cuda", 0)
    T = lambda x: torch.tensor(x, device=dev).contiguous()
    phase_lib = build.build_phase_cycles()[1] if args.phase_cycles else None
    s = capi.Solver(0, arith=args.arith, schedule=args.schedule, block=args.block, max_slots=args.max_slots,
                    lib_path=phase_lib)
    phase_buf = (ctypes.c_ulonglong * 16)()
    if phase_lib:
        s.lib.gc_kpp_phase_cycles.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]
    s.set(block_split=args.block_form == "split", queue_chunk=args.queue_chunk)
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    ic_t, rc_t = ic.copy(), rc.copy()  # controls of the timed step
    if args.autoreduce > 0:
        ic_t[11] = 1
        ic_t[12] = 1 if args.append else 0
        rc_t[11] = args.autoreduce
    at, rt = T(atol), T(rtol)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if args.grid:
        nlon, nlat, nlev = (int(v) for v in args.grid.split("x"))
        cells = inputs.grid_cells(nlon, nlat, nlev, seed=0)
    else:
        cells = inputs.box_cells(args.cells, seed=1)
    n = cells["c"].shape[1]
    met, ph, c = T(cells["met"]), T(cells["photol"]), T(cells["c"])
    ist = torch.zeros((20, n), dtype=torch.int32, device=dev)
    rst = torch.zeros((20, n), dtype=torch.float64, device=dev)
    ierr = torch.zeros(n, dtype=torch.int32, device=dev)
    if args.grid:
        hs = torch.zeros(n, dtype=torch.float64, device=dev)
        s.fullchem_step(86400.0, met, ph, c, at, rt, ic, rc, hs, ist, rst, ierr)
        if args.cold:
            hs.zero_()
        order, nb = None, 0
        if args.learned:
            import gcchem.learned as learned

            prop = learned.Proposer(0)
            prop.load_state(dict(np.load(learned.WEIGHTS)))
            hs.zero_()
            _, _, order = learned.plan(prop, met, ph, c, hstart=hs, hmax=1200.0)
            nb = int(prop.last_counts[learned.NBIN - 1].item())
            s.set(evict_after=args.evict)
        elif args.binned:
            s.fullchem_step(1200.0, met, ph, c.clone(), at, rt, ic, rc, hs.clone(), ist, rst, ierr)
            order = torch.argsort(ist[2], descending=True, stable=True).int()
            nb = args.binned
        c0, hs0 = c.clone(), hs.clone()
        for rep in range(args.repeat - 1):  # earlier runs of the same step, each from the same state
            torch.cuda.synchronize()
            t0.record()
            s.fullchem_step(1200.0, met, ph, c, at, rt, ic_t, rc_t, hs, ist, rst, ierr, order=order, nblock=nb)
            t1.record()
            torch.cuda.synchronize()
            print("run %d: %.3f ms" % (rep, t0.elapsed_time(t1)))
            c.copy_(c0)
            hs.copy_(hs0)
        if phase_lib:
            s.lib.gc_kpp_phase_cycles(phase_buf, 1)
        torch.cuda.synchronize()
        t0.record()
        s.fullchem_step(1200.0, met, ph, c, at, rt, ic_t, rc_t, hs, ist, rst, ierr, order=order, nblock=nb)
        t1.record()
    else:
        r = torch.zeros((1058, n), dtype=torch.float64, device=dev)
        s.update_rconst(met, ph, c, r)
        torch.cuda.synchronize()
        t0.record()
        s.integrate(c, r, at, rt, 0.0, args.tout, ic_t, rc_t, istatus=ist, ierr=ierr)
        t1.record()
    torch.cuda.synchronize()
    print("timed call %.3f ms (%s, default stream)" % (t0.elapsed_time(t1), "one cold run" if args.repeat <= 1 else
                                                         "after %d runs of the same step" % (args.repeat - 1)))
    ih = ist.cpu().numpy().astype(np.int64)
    t = Tables(load_ir())
    f = t.flops()
    vec = 15 * 2 * t.nvar + 5 * t.nvar
    flops = (ih[0].sum() * f["fun"] + ih[1].sum() * f["jac"] + ih[5].sum() * (f["decomp"] + 1)
             + ih[6].sum() * f["solve"] + ih[2].sum() * vec)
    print("cells %d steps/cell %.3f max %d" % (n, ih[2].mean(), ih[2].max()))
    print("ISTATUS sums fun jac stp acc rej dec sol sng", ih[:8].sum(axis=1).tolist())
    if args.grid and nb > 0:
        sel = order[:nb].long().cpu().numpy()
        print("block-per-cell cells %d: ISTATUS sums %s" % (nb, ih[:8, sel].sum(axis=1).tolist()))
        if phase_lib:
            # cycles of the block-per-cell launches of the timed step, summed
            # over blocks, per step attempt (ISTATUS(6), decompositions) of
            # the block-per-cell cells
            rc_ = s.lib.gc_kpp_phase_cycles(phase_buf, 0)
            att = max(int(ih[5, sel].sum()), 1)
            names = ["LU", "forward subst.", "backward subst.", "Fun_SPLIT", "Jac_SP", "", "", "whole kernel"]
            print("phase cycles (rc %d), per step attempt of a block:" % rc_)
            for k in (0, 1, 2, 3, 4, 7):
                if phase_buf[8 + k]:
                    print("  %-16s %10.0f  (%d calls)" % (names[k], phase_buf[k] / att, phase_buf[8 + k]))
    print("algorithmic FP64 flops %.4e" % flops)
    if args.producers and args.grid:
        # Do_FullChem's per-cell producers on this grid (synthetic grid-box
        # fields): SulfurAqChem, SET_SO2, SetStateHet, HetDropChem, timed
        # together with CUDA events (device arrays)
        import gcchem.hetstate as hetstate

        hin = T(hetstate.hetin_cells(n, seed=2))
        het = torch.zeros((168, n), dtype=torch.float64, device=dev)
        sres = torch.zeros(n, dtype=torch.int32, device=dev)
        metp = met.clone()

        def producers():
            s.sulfur_aq_rates(hin, c, metp)
            s.sulfur_cld_rates(hin, c, metp, 1, sres)
            s.set_state_het(hin, c, het)
            s.het_drop_chem(1200.0, hin, c, het, sres, metp)

        producers()
        for rep in range(2):
            torch.cuda.synchronize()
            t0.record()
            producers()
            t1.record()
            torch.cuda.synchronize()
            print("producers (SulfurAqChem, SET_SO2, SetStateHet, HetDropChem) over %d cells: %.3f ms"
                  % (n, t0.elapsed_time(t1)))
    if args.copies and args.grid:
        # first pass over a page-locked buffer right after a chemistry step:
        # copy engine against SM copies, each direction
        nb_ = 1 << 27
        bufs = [torch.ones(nb_, dtype=torch.float64).pin_memory() for _ in range(2)]
        dbuf = torch.empty(nb_, dtype=torch.float64, device=dev)

        def ev_time(fn):
            torch.cuda.synchronize()
            t0.record()
            fn()
            t1.record()
            torch.cuda.synchronize()
            return t0.elapsed_time(t1)

        def again():
            c.copy_(c0)
            hs.copy_(hs0)
            s.fullchem_step(1200.0, met, ph, c, at, rt, ic_t, rc_t, hs, ist, rst, ierr, order=order, nblock=nb)
            torch.cuda.synchronize()

        for rep in range(2):
            again()
            ce = ev_time(lambda: dbuf.copy_(bufs[0], non_blocking=True))
            smc = ev_time(lambda: capi.copy_rows(dbuf, bufs[1], lib=s.lib))
            again()
            ce2 = ev_time(lambda: bufs[0].copy_(dbuf, non_blocking=True))
            smc2 = ev_time(lambda: capi.copy_rows(bufs[1], dbuf, lib=s.lib))
            print("1 GB after a step: host->device copy engine %.1f ms, SM copy %.1f ms; device->host copy engine "
                  "%.1f ms, SM copy %.1f ms" % (ce, smc, ce2, smc2))
    if args.probe:
        probe = ctypes.CDLL(build.probe_path())
        probe.gc_probe_fp64_gflops.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        g = ctypes.c_double()
        rcode = probe.gc_probe_fp64_gflops(0, ctypes.byref(g))
        print("FP64 probe rc %d: %.1f GFLOP/s" % (rcode, g.value))


if __name__ == "__main__":
    main()
