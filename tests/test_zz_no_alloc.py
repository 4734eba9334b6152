"""The allocation-free integrate entry point, for callers that cannot call
cudaMalloc (a host application that owns all device memory, or code that runs
while its allocator must not be touched), gives the same results as the
regular entry point, through the C ABI, on two calls in a row.

Collected near the end (file name), so a run that stops at its first failure
has run the parity tests of the regular entry points before this one."""
import ctypes

import numpy as np
import pytest

import gcchem.capi as capi
import gcchem.inputs as inputs

pytestmark = pytest.mark.gpu

NVAR = 353


def _noalloc(lib):
    f = lib.gc_kpp_integrate_batch_noalloc
    vp, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
    f.argtypes = [i32, f64, f64, vp, i64, vp, i64, vp, vp, vp, vp, vp, vp, vp, i64, vp, vp]
    return f


def test_noalloc_matches_regular_entry_point_twice(orc):
    import torch

    lib = capi.load_library()
    f = _noalloc(lib)
    dev = torch.device("cuda", 0)
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    icn = np.ascontiguousarray(icntrl, np.int32)
    rcn = np.ascontiguousarray(rcntrl, np.float64)
    solver = capi.Solver(0, arith="fast", schedule="plain")
    for seed, n in ((31, 300), (32, 1024)):
        cells = inputs.box_cells(n, seed=seed)
        rconst = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
        T = lambda a, dt=torch.float64: torch.tensor(a, dtype=dt, device=dev).contiguous()
        r_d, at_d, rt_d = T(rconst), T(atol), T(rtol)
        # regular entry point (allocating context)
        c_ref = T(cells["c"])
        ist_ref = torch.zeros((20, n), dtype=torch.int32, device=dev)
        rst_ref = torch.zeros((20, n), dtype=torch.float64, device=dev)
        ierr_ref = torch.zeros(n, dtype=torch.int32, device=dev)
        solver.integrate(c_ref, r_d, at_d, rt_d, 0.0, 600.0, icntrl, rcntrl, istatus=ist_ref, rstatus=rst_ref,
                         ierr=ierr_ref)
        # allocation-free entry point
        c = T(cells["c"])
        ist = torch.zeros((20, n), dtype=torch.int32, device=dev)
        rst = torch.zeros((20, n), dtype=torch.float64, device=dev)
        ierr = torch.zeros(n, dtype=torch.int32, device=dev)
        rc = f(n, 0.0, 600.0, capi._ptr(c), n, capi._ptr(r_d), n, capi._ptr(at_d), capi._ptr(rt_d),
               icn.ctypes.data_as(ctypes.c_void_p), rcn.ctypes.data_as(ctypes.c_void_p), None, capi._ptr(ist),
               capi._ptr(rst), n, capi._ptr(ierr), None)
        assert rc == 0, lib.gc_kpp_last_error()
        torch.cuda.synchronize()
        assert torch.equal(ierr, ierr_ref)
        assert torch.equal(ist[:8], ist_ref[:8])
        assert torch.equal(rst[:3], rst_ref[:3])
        a, b = c[:NVAR].cpu().numpy(), c_ref[:NVAR].cpu().numpy()
        big = np.abs(b) > 1e4
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
        # same kernel and arithmetic: the tolerance of the parity tests holds
        assert np.max(rel[big]) < 1e-9
    solver.close()


def test_noalloc_padded_rows_hstart_and_errors(orc):
    """Leading dimensions above ncell, a per-cell Hstart, vector tolerances;
    an invalid RTOL gives IERR = -5 in every cell with ISTATUS/RSTATUS
    zeroed; auto-reduction is refused."""
    import torch

    lib = capi.load_library()
    f = _noalloc(lib)
    dev = torch.device("cuda", 0)
    n, ld = 200, 256
    cells = inputs.box_cells(n, seed=33)
    atol, rtol = inputs.tolerances()
    icntrl, rcntrl = inputs.default_controls()
    icn = np.ascontiguousarray(icntrl, np.int32)
    rcn = np.ascontiguousarray(rcntrl, np.float64)
    rconst = orc.update_rconst(cells["met"], cells["photol"], cells["c"])
    hs = np.geomspace(1e-3, 10.0, n)

    def padded(a, dt=torch.float64):
        out = torch.full((a.shape[0], ld), -7.0, dtype=dt, device=dev)
        out[:, :n] = torch.tensor(a, dtype=dt, device=dev)
        return out

    at_d = torch.tensor(atol, device=dev)
    rt_d = torch.tensor(rtol, device=dev)
    hs_d = torch.tensor(hs, device=dev)
    r_d = padded(rconst)
    c = padded(cells["c"])
    ist = torch.zeros((20, ld), dtype=torch.int32, device=dev)
    rst = torch.zeros((20, ld), dtype=torch.float64, device=dev)
    ierr = torch.zeros(n, dtype=torch.int32, device=dev)
    rc = f(n, 0.0, 600.0, capi._ptr(c), ld, capi._ptr(r_d), ld, capi._ptr(at_d), capi._ptr(rt_d),
           icn.ctypes.data_as(ctypes.c_void_p), rcn.ctypes.data_as(ctypes.c_void_p), capi._ptr(hs_d),
           capi._ptr(ist), capi._ptr(rst), ld, capi._ptr(ierr), None)
    assert rc == 0, lib.gc_kpp_last_error()
    torch.cuda.synchronize()
    # the padding columns are untouched
    assert torch.all(c[:, n:] == -7.0)
    assert torch.all(ist[:, n:] == 0)
    solver = capi.Solver(0, arith="fast", schedule="plain")
    c_ref = torch.tensor(cells["c"], device=dev)
    ist_ref = torch.zeros((20, n), dtype=torch.int32, device=dev)
    rst_ref = torch.zeros((20, n), dtype=torch.float64, device=dev)
    ierr_ref = torch.zeros(n, dtype=torch.int32, device=dev)
    solver.integrate(c_ref, torch.tensor(rconst, device=dev), at_d, rt_d, 0.0, 600.0, icntrl, rcntrl,
                     hstart=hs_d, istatus=ist_ref, rstatus=rst_ref, ierr=ierr_ref)
    torch.cuda.synchronize()
    assert torch.equal(ierr, ierr_ref)
    assert torch.equal(ist[:8, :n], ist_ref[:8])
    assert torch.equal(rst[:3, :n], rst_ref[:3])
    a, b = c[:NVAR, :n].cpu().numpy(), c_ref[:NVAR].cpu().numpy()
    big = np.abs(b) > 1e4
    assert np.max((np.abs(a - b) / np.maximum(np.abs(b), 1e-300))[big]) < 1e-9
    solver.close()

    # RTOL >= 1 in one species: Rosenbrock's -5 for every cell
    rt_bad = rt_d.clone()
    rt_bad[11] = 1.0
    ist.fill_(5)
    rst.fill_(5.0)
    c_before = c.clone()
    rc = f(n, 0.0, 600.0, capi._ptr(c), ld, capi._ptr(r_d), ld, capi._ptr(at_d), capi._ptr(rt_bad),
           icn.ctypes.data_as(ctypes.c_void_p), rcn.ctypes.data_as(ctypes.c_void_p), None,
           capi._ptr(ist), capi._ptr(rst), ld, capi._ptr(ierr), None)
    assert rc == 0, lib.gc_kpp_last_error()
    torch.cuda.synchronize()
    assert torch.all(ierr == -5)
    assert torch.all(ist[:, :n] == 0) and torch.all(rst[:, :n] == 0.0)
    assert torch.all(ist[:, n:] == 5)
    assert torch.equal(c, c_before)

    # auto-reduction is not run here: refused, nothing written
    ic_ar = icn.copy()
    ic_ar[11] = 1
    ierr.fill_(3)
    rc = f(n, 0.0, 600.0, capi._ptr(c), ld, capi._ptr(r_d), ld, capi._ptr(at_d), capi._ptr(rt_d),
           ic_ar.ctypes.data_as(ctypes.c_void_p), rcn.ctypes.data_as(ctypes.c_void_p), None,
           capi._ptr(ist), capi._ptr(rst), ld, capi._ptr(ierr), None)
    assert rc == capi.GC_KPP_EUNSUPPORTED
    torch.cuda.synchronize()
    assert torch.all(ierr == 3)


def test_noalloc_rejects_oversized_batch():
    lib = capi.load_library()
    f = _noalloc(lib)
    rc = f(1025, 0.0, 1.0, None, 1025, None, 1025, None, None, None, None, None, None, None, 1025, None, None)
    assert rc == capi.GC_KPP_EINVAL
    assert b"1024" in lib.gc_kpp_last_error()
