"""Host-side binding of the C ABI (include/gckpp_gb300.h) via ctypes.

This mirrors, for Python callers, what a Fortran caller binds with
ISO_C_BINDING: ``Solver.integrate`` is the batched INTEGRATE
(KPP/fullchem/gckpp_Integrator.F90:80-162) over cells held in
cell-interleaved arrays ``X[k, cell]``; ``Solver.update_rconst`` is the
batched Update_RCONST (KPP/fullchem/gckpp_Rates.F90:408-1503).

Arrays may be numpy arrays (host memory: the library stages them through the
device) or CUDA torch tensors (device memory: no copies).  The library must be
built (``gcchem.build.build()``); if it is missing, loading fails loudly --
there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import build as _build

GC_KPP_OK = 0
GC_KPP_EINVAL = -101
GC_KPP_ECUDA = -102
GC_KPP_ENOMEM = -103
GC_KPP_EUNSUPPORTED = -104
MEM_HOST = 0
MEM_DEVICE = 1
OPT_ARITH = 1
OPT_SCHEDULE = 2
OPT_BLOCK = 3
OPT_BLOCKS_PER_SM = 4
OPT_MAX_SLOTS = 5
OPT_TIMING = 6
OPT_LU = 7
OPT_CELL_BLOCK = 8
OPT_ASYNC = 9
OPT_EVICT_AFTER = 10
OPT_EVICT_DRAINED = 11
OPT_BLOCK_SPLIT = 12
OPT_RATES_DIRECT = 13
OPT_QUEUE_CHUNK = 14

EXPORTED = [
    "gc_kpp_mechanism_dims",
    "gc_kpp_ctx_create",
    "gc_kpp_ctx_destroy",
    "gc_kpp_ctx_set_option",
    "gc_kpp_last_error",
    "gc_kpp_integrate_batch",
    "gc_kpp_update_rconst_batch",
    "gc_kpp_update_rconst_het_batch",
    "gc_kpp_set_state_het_batch",
    "gc_kpp_sulfur_aq_rates_batch",
    "gc_kpp_sulfur_cld_rates_batch",
    "gc_kpp_het_drop_chem_batch",
    "gc_kpp_ctx_set_hetstate",
    "gc_kpp_ctx_set_autoreduce",
    "gc_kpp_fullchem_step",
    "gc_kpp_fullchem_step_ordered",
    "gc_kpp_fullchem_step_binned",
    "gc_kpp_fullchem_step_learned",
    "gc_kpp_proposer_create",
    "gc_kpp_proposer_destroy",
    "gc_kpp_proposer_set_h0_cap",
    "gc_kpp_integrate_batch_noalloc",
    "gc_kpp_last_launch_count",
    "gc_kpp_last_kernel_ms",
    "gc_kpp_copy_rows",
    "gc_kpp_photol_rows",
]

_libs = {}


class GcKppError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gc_kpp error %d: %s" % (code, msg))
        self.code = code


def load_library(path=None, mech="fullchem"):
    """Load the library of a mechanism, libgckpp_gb300.so for fullchem
    (raises OSError if it has not been built)."""
    if path is None and mech in _libs:
        return _libs[mech]
    path = path or _build.lib_path(mech)
    if not os.path.exists(path):
        raise OSError("CUDA library %s is not built; run gcchem.build.build()" % path)
    lib = ctypes.CDLL(path)
    vp, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
    lib.gc_kpp_mechanism_dims.argtypes = [ctypes.POINTER(i32)] * 5
    lib.gc_kpp_ctx_create.argtypes = [ctypes.POINTER(vp), i32]
    lib.gc_kpp_ctx_destroy.argtypes = [vp]
    lib.gc_kpp_ctx_set_option.argtypes = [vp, i32, i64]
    lib.gc_kpp_last_error.restype = ctypes.c_char_p
    lib.gc_kpp_integrate_batch.argtypes = [vp, i32, f64, f64, vp, i64, vp, i64, vp, vp, vp, vp, vp, vp, vp, i64,
                                           vp, i32, vp]
    lib.gc_kpp_update_rconst_batch.argtypes = [vp, i32, vp, i64, vp, i64, vp, i64, vp, i64, i32, vp]
    lib.gc_kpp_update_rconst_het_batch.argtypes = [vp, i32, vp, i64, vp, i64, vp, i64, vp, i64, vp, i64, i32, vp]
    lib.gc_kpp_ctx_set_hetstate.argtypes = [vp, i32, vp, i64, i32]
    lib.gc_kpp_ctx_set_autoreduce.argtypes = [vp, i32, vp, vp, vp, vp, i32]
    lib.gc_kpp_set_state_het_batch.argtypes = [vp, i32, vp, i64, vp, i64, f64, i32, i32, vp, i64, i32, vp]
    lib.gc_kpp_sulfur_aq_rates_batch.argtypes = [vp, i32, vp, i64, vp, i64, vp, i64, i32, vp]
    lib.gc_kpp_sulfur_cld_rates_batch.argtypes = [vp, i32, vp, i64, vp, i64, vp, i64, i32, vp, i32, vp]
    lib.gc_kpp_het_drop_chem_batch.argtypes = [vp, i32, f64, vp, i64, vp, i64, vp, i64, vp, vp, i64, i32, vp]
    lib.gc_kpp_copy_rows.argtypes = [vp, i64, vp, i64, i64, i64, vp]
    lib.gc_kpp_photol_rows.argtypes = [vp]
    if path == _build.lib_path(mech):
        _libs[mech] = lib
    return lib


def dims(mech="fullchem"):
    lib = load_library(mech=mech)
    out = [ctypes.c_int() for _ in range(5)]
    lib.gc_kpp_mechanism_dims(*[ctypes.byref(o) for o in out])
    return dict(zip(["nspec", "nvar", "nfix", "nreact", "lu_nonzero"], [o.value for o in out]))


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _ptr(x):
    if x is None:
        return None
    if _is_torch(x):
        return ctypes.c_void_p(x.data_ptr())
    if isinstance(x, np.ndarray):
        return x.ctypes.data_as(ctypes.c_void_p)
    raise TypeError("unsupported array type %r" % type(x))


def _ld(x, ncell):
    if _is_torch(x):
        return x.stride(0) if x.dim() == 2 else ncell
    return x.strides[0] // x.itemsize if x.ndim == 2 else ncell


class Solver:
    """A solver context on one CUDA device (gc_kpp_ctx)."""

    def __init__(self, device=0, arith="fast", schedule="plain", block=0, blocks_per_sm=0, max_slots=0,
                 mech="fullchem", lib_path=None):
        # lib_path: another build of the mechanism's library (a profiling copy)
        self.lib = load_library(lib_path, mech=mech)
        self.mech = mech
        self.ctx = ctypes.c_void_p()
        self._check(self.lib.gc_kpp_ctx_create(ctypes.byref(self.ctx), device))
        self.set(arith=arith, schedule=schedule, block=block, blocks_per_sm=blocks_per_sm, max_slots=max_slots)

    def _check(self, rc):
        if rc != GC_KPP_OK:
            raise GcKppError(rc, self.lib.gc_kpp_last_error().decode())

    def set(self, arith=None, schedule=None, block=None, blocks_per_sm=None, max_slots=None, cell_block=None,
            async_steps=None, evict_after=None, evict_drained=None, block_split=None, rates_direct=None,
            queue_chunk=None):
        if arith is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_ARITH, {"fast": 0, "strict": 1, "fast2": 2, "fast4": 3}[arith]))
        if schedule is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_SCHEDULE, {"plain": 0, "queue": 1}[schedule]))
        if block is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_BLOCK, int(block)))
        if blocks_per_sm is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_BLOCKS_PER_SM, int(blocks_per_sm)))
        if max_slots is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_MAX_SLOTS, int(max_slots)))
        if cell_block is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_CELL_BLOCK, int(cell_block)))
        if evict_after is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_EVICT_AFTER, int(evict_after)))
        if evict_drained is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_EVICT_DRAINED, 1 if evict_drained else 0))
        if async_steps is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_ASYNC, 1 if async_steps else 0))
        if block_split is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_BLOCK_SPLIT, 1 if block_split else 0))
        if rates_direct is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_RATES_DIRECT, 1 if rates_direct else 0))
        if queue_chunk is not None:
            self._check(self.lib.gc_kpp_ctx_set_option(self.ctx, OPT_QUEUE_CHUNK, int(queue_chunk)))

    def close(self):
        if self.ctx:
            self.lib.gc_kpp_ctx_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def integrate(self, c, rconst, atol, rtol, tin, tout, icntrl=None, rcntrl=None, hstart=None,
                  istatus=None, rstatus=None, ierr=None, stream=None):
        """Batched INTEGRATE.  c: [NSPEC, ncell] (in/out); rconst: [NREACT, ncell];
        istatus/rstatus: [20, ncell] outputs; ierr: [ncell] output."""
        dev = _is_torch(c) and c.is_cuda
        ncell = c.shape[1]
        if icntrl is not None:
            icntrl = np.ascontiguousarray(icntrl, dtype=np.int32)
        if rcntrl is not None:
            rcntrl = np.ascontiguousarray(rcntrl, dtype=np.float64)
        if dev:
            import torch  # noqa: F401
            mem = MEM_DEVICE
        else:
            mem = MEM_HOST
        args_ok = [a for a in (c, rconst, atol, rtol, ierr) if a is not None]
        if len(args_ok) != 5:
            raise ValueError("c, rconst, atol, rtol and ierr are required")
        ldo = _ld(istatus, ncell) if istatus is not None else (_ld(rstatus, ncell) if rstatus is not None else ncell)
        s = ctypes.c_void_p(stream) if stream else None
        rc = self.lib.gc_kpp_integrate_batch(
            self.ctx, ncell, float(tin), float(tout), _ptr(c), _ld(c, ncell), _ptr(rconst), _ld(rconst, ncell),
            _ptr(atol), _ptr(rtol),
            icntrl.ctypes.data_as(ctypes.c_void_p) if icntrl is not None else None,
            rcntrl.ctypes.data_as(ctypes.c_void_p) if rcntrl is not None else None,
            _ptr(hstart), _ptr(istatus), _ptr(rstatus), ldo, _ptr(ierr), mem, s)
        self._check(rc)

    def fullchem_step(self, dt, met, photol, c, atol, rtol, icntrl=None, rcntrl=None, hstart=None, istatus=None,
                      rstatus=None, ierr=None, order=None, nblock=0, stream=None):
        """One Do_FullChem chemistry step over all cells (gc_kpp_fullchem_step;
        gc_kpp_fullchem_step_ordered when a queue ``order`` is given;
        gc_kpp_fullchem_step_binned when the first ``nblock`` cells of the
        order run block-per-cell).  Returns the number of cells integrated a
        second time (retry)."""
        lib = self.lib
        if not getattr(lib, "_step_typed", False):
            vp, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
            head = [vp, i32, f64, vp, i64, vp, i64, vp, i64, vp, vp, vp, vp, vp, vp, vp, i64, vp, vp]
            lib.gc_kpp_fullchem_step.argtypes = head + [i32, vp]
            lib.gc_kpp_fullchem_step_ordered.argtypes = head + [vp, i32, vp]
            lib.gc_kpp_fullchem_step_binned.argtypes = head + [vp, i32, i32, vp]
            lib._step_typed = True
        dev = _is_torch(c) and c.is_cuda
        ncell = c.shape[1]
        icn = np.ascontiguousarray(icntrl if icntrl is not None else np.zeros(20), dtype=np.int32)
        rcn = np.ascontiguousarray(rcntrl if rcntrl is not None else np.zeros(20), dtype=np.float64)
        nretry = ctypes.c_int(0)
        ldo = _ld(istatus, ncell) if istatus is not None else ncell
        s = ctypes.c_void_p(stream) if stream else None
        args = [self.ctx, ncell, float(dt), _ptr(met), _ld(met, ncell), _ptr(photol), _ld(photol, ncell), _ptr(c),
                _ld(c, ncell), _ptr(atol), _ptr(rtol), icn.ctypes.data_as(ctypes.c_void_p),
                rcn.ctypes.data_as(ctypes.c_void_p), _ptr(hstart), _ptr(istatus), _ptr(rstatus), ldo, _ptr(ierr),
                ctypes.byref(nretry)]
        mem = MEM_DEVICE if dev else MEM_HOST
        if order is None:
            rc = lib.gc_kpp_fullchem_step(*args, mem, s)
        else:
            if not _is_torch(order):
                order = np.ascontiguousarray(order, dtype=np.int32)
            if nblock:
                rc = lib.gc_kpp_fullchem_step_binned(*args, _ptr(order), int(nblock), mem, s)
            else:
                rc = lib.gc_kpp_fullchem_step_ordered(*args, _ptr(order), mem, s)
        self._check(rc)
        return nretry.value

    def fullchem_step_learned(self, proposer, dt, met, photol, c, atol, rtol, icntrl=None, rcntrl=None,
                              hstart=None, istatus=None, rstatus=None, ierr=None, stream=None):
        """gc_kpp_fullchem_step_learned with a gc_kpp_proposer handle
        (``learned.CProposer``).  Returns (cells retried, cells block-per-cell)."""
        lib = self.lib
        if not getattr(lib, "_learned_typed", False):
            vp, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
            lib.gc_kpp_fullchem_step_learned.argtypes = [vp, vp, i32, f64, vp, i64, vp, i64, vp, i64, vp, vp, vp,
                                                         vp, vp, vp, vp, i64, vp, vp, vp, i32, vp]
            lib._learned_typed = True
        dev = _is_torch(c) and c.is_cuda
        ncell = c.shape[1]
        icn = np.ascontiguousarray(icntrl if icntrl is not None else np.zeros(20), dtype=np.int32)
        rcn = np.ascontiguousarray(rcntrl if rcntrl is not None else np.zeros(20), dtype=np.float64)
        nretry, nblock = ctypes.c_int(0), ctypes.c_int(0)
        ldo = _ld(istatus, ncell) if istatus is not None else ncell
        s = ctypes.c_void_p(stream) if stream else None
        rc = lib.gc_kpp_fullchem_step_learned(
            self.ctx, proposer, ncell, float(dt), _ptr(met), _ld(met, ncell), _ptr(photol), _ld(photol, ncell),
            _ptr(c), _ld(c, ncell), _ptr(atol), _ptr(rtol), icn.ctypes.data_as(ctypes.c_void_p),
            rcn.ctypes.data_as(ctypes.c_void_p), _ptr(hstart), _ptr(istatus), _ptr(rstatus), ldo, _ptr(ierr),
            ctypes.byref(nretry), ctypes.byref(nblock), MEM_DEVICE if dev else MEM_HOST, s)
        self._check(rc)
        return nretry.value, nblock.value

    def set_autoreduce(self, thr=None, target=None, ratio=None, keep=None):
        """Auto-reduce controls of the following integrations with
        ICNTRL(12) = 1: per-cell RCNTRL(12) / ICNTRL(14) / RCNTRL(14) arrays
        [ncell] (numpy or torch CUDA; copied) and the keepSpcActive mask
        [NVAR] (host).  Each call replaces every earlier setting; no
        arguments clear them (see gcchem.autoreduce for the arrays Do_FullChem
        would pass)."""
        cells = [a for a in (thr, target, ratio) if a is not None]
        n = int(cells[0].shape[0]) if cells else 0
        if any(int(a.shape[0]) != n for a in cells):
            raise ValueError("per-cell arrays of different lengths")
        dev = bool(cells) and _is_torch(cells[0]) and cells[0].is_cuda
        if any((_is_torch(a) and a.is_cuda) != dev for a in cells):
            raise ValueError("per-cell arrays must all be host or all be device arrays")

        def conv(a, dt):
            if a is None:
                return a
            if dev:
                if not a.is_contiguous() or a.element_size() != np.dtype(dt).itemsize or a.dtype.is_floating_point \
                        != (np.dtype(dt).kind == "f"):
                    raise ValueError("device arrays must be contiguous float64 (thr, ratio) / int32 (target)")
                return a
            return np.ascontiguousarray(a, dtype=dt)

        thr, target, ratio = conv(thr, np.float64), conv(target, np.int32), conv(ratio, np.float64)
        k = None if keep is None else np.ascontiguousarray(np.asarray(keep) != 0, dtype=np.uint8)
        self._ar_keep = (thr, target, ratio, k)
        self._check(self.lib.gc_kpp_ctx_set_autoreduce(self.ctx, n, _ptr(thr), _ptr(target), _ptr(ratio), _ptr(k),
                                                       MEM_DEVICE if dev else MEM_HOST))

    def set_hetstate(self, het):
        """HetState rows [168, ncell] (numpy: copied; torch CUDA: kept by
        pointer) used by the following chemistry steps; None clears it."""
        if het is None:
            self._check(self.lib.gc_kpp_ctx_set_hetstate(self.ctx, 0, None, 0, MEM_HOST))
            self._het = None
            return
        dev = _is_torch(het) and het.is_cuda
        if not dev:
            het = np.ascontiguousarray(het, dtype=np.float64)
        n = het.shape[1]
        self._check(self.lib.gc_kpp_ctx_set_hetstate(self.ctx, n, _ptr(het), _ld(het, n),
                                                     MEM_DEVICE if dev else MEM_HOST))
        self._het = het if dev else None

    def set_state_het(self, hetin, c, het, gamma_ho2=0.2, lpscchem=1, turn_off_het_rates=0, stream=None):
        """Batched fullchem_SetStateHet (gc_kpp_set_state_het_batch).
        hetin: [NHETIN, ncell] grid-box fields (gcchem.hetstate.HETIN_FIELDS);
        c: [NSPEC, ncell]; het: [168, ncell] output HetState rows.  numpy
        arrays (host) or CUDA torch tensors (device), all of one kind."""
        dev = _is_torch(het) and het.is_cuda
        ncell = het.shape[1]
        if not dev:
            hetin = np.ascontiguousarray(hetin, dtype=np.float64)
            c = np.ascontiguousarray(c, dtype=np.float64)
        s = ctypes.c_void_p(stream) if stream else None
        rc = self.lib.gc_kpp_set_state_het_batch(self.ctx, ncell, _ptr(hetin), _ld(hetin, ncell), _ptr(c),
                                                 _ld(c, ncell), float(gamma_ho2), int(lpscchem),
                                                 int(turn_off_het_rates), _ptr(het), _ld(het, ncell),
                                                 MEM_DEVICE if dev else MEM_HOST, s)
        self._check(rc)

    def sulfur_cld_rates(self, hetin, c, met, lmetalcatso2=1, size_res=None, stream=None):
        """Batched SET_SO2 (gc_kpp_sulfur_cld_rates_batch): K_CLD rows of met
        [NMET, ncell] (the other rows untouched), the HSO3_aq, SO3_aq, pHCloud
        (and fupdateHOBr/HOCl = 1) rows of hetin [NHETIN, ncell] rewritten in
        place, size_res [ncell] int32 (optional) out.  All numpy (host) or all
        CUDA torch tensors (device)."""
        dev = _is_torch(met) and met.is_cuda
        ncell = met.shape[1]
        if not dev:
            for a in (hetin, met):
                if not (isinstance(a, np.ndarray) and a.flags.c_contiguous and a.dtype == np.float64):
                    raise ValueError("host arrays written in place must be C-contiguous float64 numpy arrays")
            c = np.ascontiguousarray(c, dtype=np.float64)
        s = ctypes.c_void_p(stream) if stream else None
        rc = self.lib.gc_kpp_sulfur_cld_rates_batch(self.ctx, ncell, _ptr(hetin), _ld(hetin, ncell), _ptr(c),
                                                    _ld(c, ncell), _ptr(met), _ld(met, ncell), int(lmetalcatso2),
                                                    _ptr(size_res), MEM_DEVICE if dev else MEM_HOST, s)
        self._check(rc)

    def het_drop_chem(self, dt, hetin, c, het, size_res, met, stream=None):
        """Batched fullchem_HetDropChem (gc_kpp_het_drop_chem_batch): the
        SRHOCl and SRHOBr rows of met [NMET, ncell] (in/out) from the grid-box
        rows after SET_SO2, c, the HetState het [168, ncell] and size_res
        [ncell] int32.  All numpy (host) or all CUDA torch tensors (device)."""
        dev = _is_torch(met) and met.is_cuda
        ncell = met.shape[1]
        if not dev:
            if not (isinstance(met, np.ndarray) and met.flags.c_contiguous and met.dtype == np.float64):
                raise ValueError("met is written in place: a C-contiguous float64 numpy array")
            hetin = np.ascontiguousarray(hetin, dtype=np.float64)
            c = np.ascontiguousarray(c, dtype=np.float64)
            het = np.ascontiguousarray(het, dtype=np.float64)
            size_res = np.ascontiguousarray(size_res, dtype=np.int32)
        s = ctypes.c_void_p(stream) if stream else None
        rc = self.lib.gc_kpp_het_drop_chem_batch(self.ctx, ncell, float(dt), _ptr(hetin), _ld(hetin, ncell), _ptr(c),
                                                 _ld(c, ncell), _ptr(het), _ld(het, ncell), _ptr(size_res),
                                                 _ptr(met), _ld(met, ncell), MEM_DEVICE if dev else MEM_HOST, s)
        self._check(rc)

    def sulfur_aq_rates(self, hetin, c, met, stream=None):
        """Batched fullchem_SulfurAqChem (gc_kpp_sulfur_aq_rates_batch): the
        K_MT rows of met [NMET, ncell] (in/out; TEMP and NUMDEN read) from
        hetin [NHETIN, ncell] and c [NSPEC, ncell]."""
        dev = _is_torch(met) and met.is_cuda
        ncell = met.shape[1]
        if not dev:
            hetin = np.ascontiguousarray(hetin, dtype=np.float64)
            c = np.ascontiguousarray(c, dtype=np.float64)
        s = ctypes.c_void_p(stream) if stream else None
        rc = self.lib.gc_kpp_sulfur_aq_rates_batch(self.ctx, ncell, _ptr(hetin), _ld(hetin, ncell), _ptr(c),
                                                   _ld(c, ncell), _ptr(met), _ld(met, ncell),
                                                   MEM_DEVICE if dev else MEM_HOST, s)
        self._check(rc)

    def update_rconst(self, met, photol, c, rconst, stream=None, het=None):
        """Batched Update_RCONST.  met: [NMET, ncell]; photol: [200, ncell];
        c: [NSPEC, ncell]; rconst: [NREACT, ncell] output; het: the cells'
        HetState rows [168, ncell] (gcchem.hetstate) or None (heterogeneous
        rates 0)."""
        dev = _is_torch(rconst) and rconst.is_cuda
        ncell = rconst.shape[1]
        s = ctypes.c_void_p(stream) if stream else None
        mem = MEM_DEVICE if dev else MEM_HOST
        if het is None:
            rc = self.lib.gc_kpp_update_rconst_batch(
                self.ctx, ncell, _ptr(met), _ld(met, ncell), _ptr(photol), _ld(photol, ncell), _ptr(c),
                _ld(c, ncell), _ptr(rconst), _ld(rconst, ncell), mem, s)
        else:
            if not _is_torch(het):
                het = np.ascontiguousarray(het, dtype=np.float64)
            rc = self.lib.gc_kpp_update_rconst_het_batch(
                self.ctx, ncell, _ptr(met), _ld(met, ncell), _ptr(photol), _ld(photol, ncell), _ptr(c),
                _ld(c, ncell), _ptr(het), _ld(het, ncell), _ptr(rconst), _ld(rconst, ncell), mem, s)
        self._check(rc)


def copy_rows(dst, src, stream=None, lib=None):
    """dst.copy_(src) for two 1-D or 2-D torch tensors of the same shape and
    dtype, host or CUDA.  Rows of contiguous elements (any row stride) go
    through gc_kpp_copy_rows: page-locked host memory is read and written by
    the SMs, which after a chemistry step is an order of magnitude faster
    than a copy engine.  Other layouts use torch's copy.  Stream-ordered on
    `stream` (a CUDA stream handle, default the current torch stream)."""
    import torch

    lib = lib or load_library()
    if dst.shape != src.shape or dst.dtype != src.dtype:
        raise ValueError("copy_rows: shapes or dtypes differ")
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    rowwise = lambda t: t.dim() == 1 and t.stride(0) == 1 or t.dim() == 2 and t.stride(1) == 1
    if not (rowwise(dst) and rowwise(src)):
        # a layout that is not rows of contiguous elements (column-major host
        # arrays, say): torch's own copy, on the same stream
        with torch.cuda.stream(torch.cuda.ExternalStream(stream)):
            dst.copy_(src, non_blocking=True)
        return
    d2 = dst if dst.dim() == 2 else dst.reshape(1, -1)
    s2 = src if src.dim() == 2 else src.reshape(1, -1)
    es = dst.element_size()
    rc = lib.gc_kpp_copy_rows(ctypes.c_void_p(d2.data_ptr()), d2.stride(0) * es, ctypes.c_void_p(s2.data_ptr()),
                              s2.stride(0) * es, d2.shape[1] * es, d2.shape[0], ctypes.c_void_p(stream))
    if rc != GC_KPP_OK:
        raise GcKppError(rc, lib.gc_kpp_last_error().decode())


def photol_rows(lib=None):
    """Boolean mask of the PHOTOL rows the mechanism's rates read."""
    lib = lib or load_library()
    mask = np.zeros(200, dtype=np.uint8)
    rc = lib.gc_kpp_photol_rows(mask.ctypes.data_as(ctypes.c_void_p))
    if rc != GC_KPP_OK:
        raise GcKppError(rc, lib.gc_kpp_last_error().decode())
    return mask.astype(bool)
