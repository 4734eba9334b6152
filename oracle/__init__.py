"""CPU oracle of the KPP fullchem solve -- TEST INFRASTRUCTURE.

ctypes binding of the C restatement in this directory (kpp_oracle.c and the
generated mechanism/rate code).  Imported only by the tests, by the smoke
check and by the CPU-baseline leg of bench.py, always to check or time
against, never as the thing measured or shipped.

Two builds of the same sources:
  "strict"  -O2 -ffp-contract=off  (reference arithmetic, parity oracle)
  "fast"    -O3                    (timed CPU baseline)
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NHET = 168  # rows of the HetState array (the batch interface's field list)
_libs = {}


def _builder():
    import importlib.util

    spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(HERE, "build_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def build(verbose=False):
    return _builder().build(verbose=verbose)


def load(variant="strict", mech="fullchem"):
    """The oracle library of one mechanism (KPP/<mech>) and arithmetic variant."""
    key = (mech, variant)
    if key in _libs:
        return _libs[key]
    b = _builder()
    path = b.lib_path(variant, mech)
    if not os.path.exists(path):
        b.build(mechs=(mech,))
    lib = ctypes.CDLL(path)
    vp, i32, i64, f64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_double
    lib.oracle_integrate_batch.argtypes = [i32, f64, f64, vp, i64, vp, i64, vp, vp, vp, vp, vp, vp, vp, i64, vp, i32]
    lib.oracle_integrate_batch_ar.argtypes = [i32, f64, f64, vp, i64, vp, i64, vp, vp, vp, vp, vp, vp, vp, i64, vp,
                                              i32, vp, vp, vp]
    lib.oracle_set_keep.argtypes = [vp]
    lib.oracle_update_rconst_batch.argtypes = [i32, vp, i64, vp, i64, vp, i64, vp, i64]
    lib.oracle_update_rconst_het_batch.argtypes = [i32, vp, i64, vp, i64, vp, i64, vp, i64, vp, i64]
    lib.oracle_fun_split.argtypes = [vp, vp, vp, vp]
    lib.oracle_fun_pd.argtypes = [vp, vp, vp, vp, vp]
    lib.oracle_jac_sp.argtypes = [vp, vp, vp, vp]
    lib.oracle_kpp_solve.argtypes = [vp, vp]
    lib.oracle_kpp_decomp.argtypes = [vp]
    lib.oracle_kpp_decomp.restype = i32
    lib.oracle_max_threads.restype = i32
    lib.oracle_set_state_het_batch.argtypes = [i32, vp, i64, vp, i64, f64, i32, i32, vp, i64]
    lib.oracle_sulfur_aq_rates_batch.argtypes = [i32, vp, i64, vp, i64, vp, vp, vp, i64]
    lib.oracle_sulfur_cld_rates_batch.argtypes = [i32, vp, i64, vp, i64, i32, vp, i64, vp, vp]
    lib.oracle_het_drop_chem_batch.argtypes = [i32, f64, vp, i64, vp, i64, vp, i64, vp, vp, i64]
    lib.oracle_sulfite_uptakes.argtypes = [vp, vp, vp, i64, vp]
    _libs[key] = lib
    return lib


def _dims(mech):
    import json

    with open(os.path.join(HERE, "..", "geos-chem_gb300", "mechanism", mech + ".json")) as fh:
        return json.load(fh)["dims"]


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def integrate(c, rconst, atol, rtol, tin, tout, icntrl=None, rcntrl=None, hstart=None, variant="strict",
              nthreads=0, mech="fullchem", ar_thr=None, ar_target=None, ar_ratio=None):
    """Batched INTEGRATE on the CPU.  c [NSPEC, n] (copied), rconst [NREACT, n].
    ar_thr/ar_target/ar_ratio [n]: per-cell RCNTRL(12), ICNTRL(14),
    RCNTRL(14) of auto-reduction (optional).
    Returns (c_out, istatus [20, n], rstatus [20, n], ierr [n])."""
    lib = load(variant, mech)
    c = np.array(c, dtype=np.float64, order="C", copy=True)
    rconst = _c(rconst, np.float64)
    n = c.shape[1]
    ist = np.zeros((20, n), np.int32)
    rst = np.zeros((20, n), np.float64)
    ierr = np.zeros(n, np.int32)
    ic = _c(icntrl, np.int32) if icntrl is not None else None
    rc = _c(rcntrl, np.float64) if rcntrl is not None else None
    hs = _c(hstart, np.float64) if hstart is not None else None
    at = _c(ar_thr, np.float64) if ar_thr is not None else None
    ag = _c(ar_target, np.int32) if ar_target is not None else None
    ar = _c(ar_ratio, np.float64) if ar_ratio is not None else None
    lib.oracle_integrate_batch_ar(n, float(tin), float(tout), _p(c), n, _p(rconst), n, _p(_c(atol, np.float64)),
                                  _p(_c(rtol, np.float64)), _p(ic), _p(rc), _p(hs), _p(ist), _p(rst), n, _p(ierr),
                                  int(nthreads), _p(at), _p(ag), _p(ar))
    return c, ist, rst, ierr


def set_keep(keep, variant="strict", mech="fullchem"):
    """keepSpcActive of auto-reduction: a [NVAR] boolean mask of species that
    are never frozen (keepActive on), or None (keepActive off)."""
    lib = load(variant, mech)
    k = None if keep is None else _c(np.asarray(keep) != 0, np.uint8)
    lib.oracle_set_keep(_p(k))


def update_rconst(met, photol, c, variant="strict", mech="fullchem", het=None):
    """Batched Update_RCONST; het [168, n] HetState rows or None (zeroed)."""
    lib = load(variant, mech)
    met = _c(met, np.float64)
    photol = _c(photol, np.float64)
    c = _c(c, np.float64)
    n = met.shape[1]
    nreact = _dims(mech)["nreact"]
    out = np.zeros((nreact, n), np.float64)
    if het is None:
        lib.oracle_update_rconst_batch(n, _p(met), n, _p(photol), n, _p(c), n, _p(out), n)
    else:
        het = _c(het, np.float64)
        lib.oracle_update_rconst_het_batch(n, _p(met), n, _p(photol), n, _p(c), n, _p(het), n, _p(out), n)
    return out


def set_state_het(hetin, c, gamma_ho2=0.2, lpscchem=1, turn_off_het_rates=0, mech="fullchem"):
    """Batched fullchem_SetStateHet: hetin [NHETIN, n] grid-box fields and
    c [NSPEC, n] -> HetState rows [168, n]."""
    lib = load("strict", mech)
    hetin = _c(hetin, np.float64)
    c = _c(c, np.float64)
    n = hetin.shape[1]
    out = np.zeros((NHET, n), np.float64)
    lib.oracle_set_state_het_batch(n, _p(hetin), n, _p(c), n, float(gamma_ho2), int(lpscchem),
                                   int(turn_off_het_rates), _p(out), n)
    return out


def sulfur_aq_rates(hetin, c, temp, numden, mech="fullchem"):
    """Batched fullchem_SulfurAqChem: K_MT(1:6) [6, n] from the grid-box
    fields hetin [NHETIN, n], c [NSPEC, n], TEMP [n] and NUMDEN [n]."""
    lib = load("strict", mech)
    hetin, c = _c(hetin, np.float64), _c(c, np.float64)
    temp, numden = _c(temp, np.float64), _c(numden, np.float64)
    n = hetin.shape[1]
    out = np.zeros((6, n), np.float64)
    lib.oracle_sulfur_aq_rates_batch(n, _p(hetin), n, _p(c), n, _p(temp), _p(numden), _p(out), n)
    return out


def sulfur_cld_rates(hetin, c, lmetalcatso2=1, mech="fullchem"):
    """Batched SET_SO2 (fullchem_SulfurCldChem) with Set_Sulfur_Chem_Rates'
    fupdateHOBr/HOCl = 1: returns (hetin with HSO3_aq, SO3_aq, pHCloud,
    fupdateHOBr, fupdateHOCl rewritten, K_CLD [6, n], size_res [n],
    GET_HPLUS iterations [n])."""
    lib = load("strict", mech)
    hetin = _c(hetin, np.float64).copy()
    c = _c(c, np.float64)
    n = hetin.shape[1]
    kcld = np.zeros((6, n), np.float64)
    sr = np.zeros(n, np.int32)
    it = np.zeros(n, np.int32)
    lib.oracle_sulfur_cld_rates_batch(n, _p(hetin), n, _p(c), n, int(lmetalcatso2), _p(kcld), n, _p(sr), _p(it))
    return hetin, kcld, sr, it


def sulfite_uptakes(met, c, het, mech="fullchem"):
    """HOClUptkByHSO3m, HOClUptkBySO3mm, HOBrUptkByHSO3m, HOBrUptkBySO3mm of
    every cell [4, n] (met [18, n], c [NSPEC, n], HetState het [168, n])."""
    lib = load("strict", mech)
    met, c, het = _c(met, np.float64), _c(c, np.float64), _c(het, np.float64)
    n = met.shape[1]
    out = np.zeros((4, n))
    for j in range(n):
        m = np.ascontiguousarray(met[:, j])
        cc = np.ascontiguousarray(c[:, j])
        o = np.zeros(4)
        lib.oracle_sulfite_uptakes(_p(m), _p(cc), _p(het[:, j:]), n, _p(o))
        out[:, j] = o
    return out


def het_drop_chem(dt, hetin, c, het, size_res, met, mech="fullchem"):
    """Batched fullchem_HetDropChem under Do_FullChem's call conditions:
    returns met [18, n] with the SRHOCl and SRHOBr rows rewritten (0 where
    it is not called)."""
    lib = load("strict", mech)
    hetin, c, het = _c(hetin, np.float64), _c(c, np.float64), _c(het, np.float64)
    sr = _c(size_res, np.int32)
    met = _c(met, np.float64).copy()
    n = met.shape[1]
    lib.oracle_het_drop_chem_batch(n, float(dt), _p(hetin), n, _p(c), n, _p(het), n, _p(sr), _p(met), n)
    return met


def fun_split(v, f, rct, mech="fullchem"):
    lib = load("strict", mech)
    v, f, rct = _c(v, np.float64), _c(f, np.float64), _c(rct, np.float64)
    out = np.zeros_like(v)
    lib.oracle_fun_split(_p(v), _p(f), _p(rct), _p(out))
    return out


def fun_pd(v, f, rct, mech="fullchem"):
    """Fun_SPLITF: production P_VAR and destruction D_VAR (Vdot = P - D*V)."""
    lib = load("strict", mech)
    v, f, rct = _c(v, np.float64), _c(f, np.float64), _c(rct, np.float64)
    p = np.zeros_like(v)
    d = np.zeros_like(v)
    lib.oracle_fun_pd(_p(v), _p(f), _p(rct), _p(p), _p(d))
    return p, d


def jac_sp(v, f, rct, lu_nonzero=None, mech="fullchem"):
    lib = load("strict", mech)
    lu_nonzero = lu_nonzero or _dims(mech)["lu_nonzero"]
    v, f, rct = _c(v, np.float64), _c(f, np.float64), _c(rct, np.float64)
    out = np.zeros(lu_nonzero, np.float64)
    lib.oracle_jac_sp(_p(v), _p(f), _p(rct), _p(out))
    return out


def decomp(jvs, mech="fullchem"):
    lib = load("strict", mech)
    jvs = np.array(jvs, dtype=np.float64, copy=True)
    ier = lib.oracle_kpp_decomp(_p(jvs))
    return jvs, ier


def solve(jvs, x, mech="fullchem"):
    lib = load("strict", mech)
    jvs = _c(jvs, np.float64)
    x = np.array(x, dtype=np.float64, copy=True)
    lib.oracle_kpp_solve(_p(jvs), _p(x))
    return x


def max_threads(variant="fast"):
    return load(variant).oracle_max_threads()
