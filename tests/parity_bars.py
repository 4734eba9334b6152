"""The parity bar for cells whose ISTATUS step sequence differs from the
oracle's (a rounding difference flipped an accept/reject decision).  Such a
cell is a different RTOL 5e-3 integration of the same problem, so it is held
to the accuracy the method promises instead of to the oracle's bits: its
weighted RMS deviation from an RTOL 1e-8 integration, in the integrator's own
norm (ros_ErrorNorm, KPP/fullchem/gckpp_Integrator.F90:1715-1745), must be no
larger than twice the oracle's own deviation for that cell, or than the
oracle's largest deviation over the cells compared, whichever is larger."""
import numpy as np

NVAR = 353


def wrms(a, b, atol, rtol):
    """Weighted RMS of a - b per cell (scale ATOL + RTOL * max(|a|, |b|))."""
    a, b = a[:NVAR], b[:NVAR]
    sc = atol[:NVAR, None] + rtol[:NVAR, None] * np.maximum(np.abs(a), np.abs(b))
    return np.sqrt(np.mean(((a - b) / sc) ** 2, axis=0))


def check_other_sequences(c, c_ref, tight, same, atol, rtol, sel=None):
    """Asserts the bar on the cells (of `sel`, default all) whose step
    sequence differs from the oracle's; returns how many there are."""
    pool = np.ones(c.shape[1], bool) if sel is None else np.asarray(sel, bool)
    e_orc = wrms(c_ref, tight, atol, rtol)
    e_gpu = wrms(c, tight, atol, rtol)
    bound = np.maximum(2.0 * e_orc, e_orc[pool].max() if pool.any() else 0.0)
    diff = ~same & pool
    assert np.all(e_gpu[diff] <= bound[diff]), (np.flatnonzero(diff), e_gpu[diff], bound[diff])
    return int(diff.sum())
