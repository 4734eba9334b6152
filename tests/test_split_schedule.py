"""The pass schedules of the split block-per-cell kernel (tables.py
_split_schedules), replayed on the CPU the way the kernel runs them: within a
dependency level (the passes up to one with the barrier bit) every lane reads
the values the previous levels left, sums its chunk, the lanes of a segment
add their partial sums, and the segment's first lane stores the item.  The
replay must give the sequential evaluation of the same sums (LU factors,
substitutions, Fun_SPLIT, Jac_SP) to rounding, for both mechanisms."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))


@pytest.fixture(scope="module", params=["fullchem", "Hg"])
def tab(request):
    import gcchem.mechanism as mechanism
    import gcchem.tables as tables

    return tables.Tables(mechanism.load_ir(request.param))


def _levels(task, info, nt):
    """Yield the lanes (item, seglog, n, y, z, lane) of each level."""
    task = task.reshape(-1, 4)
    lanes = []
    for p, w in enumerate(info):
        for lane in range(nt):
            x, y, z, _ = (int(v) for v in task[p * nt + lane])
            item = x & 0xFFFF
            if item != 0xFFFF:
                lanes.append((item, (x >> 16) & 7, (x >> 19) & 31, y, z, lane))
        if int(w) & 8:
            yield lanes
            lanes = []
    assert not lanes


def _replay(tab, ph, base, term, finish):
    import gcchem.tables as tables

    task, info = tab.split[ph]
    nt = tables.SPLIT_PHASE_NT[ph]
    assert nt in (32, tables.SPLIT_NT)
    for lanes in _levels(task, info, nt):
        sums = {}
        for item, slog, n, y, z, lane in lanes:
            seg = 1 << slog
            assert (lane - lane % seg) // 32 == (lane - lane % seg + seg - 1) // 32  # inside one warp
            acc = base(item, z) if lane % seg == 0 else 0.0
            for k in range(n):
                acc = term(item, y + k, acc)
            key = (item, lane // seg)
            sums.setdefault(key, [z, 0.0])
            sums[key][1] += acc
        seen = set()
        for (item, _), (z, v) in sums.items():
            assert item not in seen  # one segment per item
            seen.add(item)
        for (item, _), (z, v) in sums.items():
            finish(item, z, v)


def test_split_chunks_fit_the_kernel(tab):
    import gcchem.tables as tables

    for ph, (task, info) in tab.split.items():
        x = task.reshape(-1, 4)[:, 0]
        assert ((x >> 19) & 31).max() <= tables.SPLIT_MAXCH
        assert len(task) == 4 * len(info) * tables.SPLIT_PHASE_NT[ph]
        assert np.all(info & 7 <= 5)
        # the fourth word: the bounds of each warp of a pass, the same on its 32 lanes
        tw = task.reshape(-1, 32, 4).astype(np.int64)
        busy = (tw[:, :, 0] & 0xFFFF) != 0xFFFF
        n = np.where(busy, (tw[:, :, 0] >> 19) & 31, 0)
        slog = np.where(busy, (tw[:, :, 0] >> 16) & 7, 0)
        want = np.where(busy.any(axis=1), 1 | n.max(axis=1) << 1 | slog.max(axis=1) << 5, 0)
        assert np.array_equal(tw[:, :, 3], np.repeat(want[:, None], 32, axis=1))


def test_split_lu_and_solves_match_sequential(tab):
    rng = np.random.default_rng(11)
    t = tab
    nz, nvar = t.lu_nonzero, t.nvar
    irow = np.repeat(np.arange(nvar), np.diff(t.crow))
    J0 = rng.standard_normal(nz)
    ghinv = 3.0 * nvar
    # sequential dot-product LU with the fast form's conventions
    ref = np.zeros(nz)
    for k in range(nvar):
        for e in range(t.crow[k], t.crow[k + 1]):
            acc = J0[e] + (ghinv if e == t.diag[k] else 0.0)
            for u in t.dot_term[t.dot_start[e]:t.dot_start[e + 1]].view(np.uint32):
                acc -= ref[int(u) >> 16] * ref[int(u) & 0xFFFF]
            if e < t.diag[k]:
                acc *= ref[t.diag[t.icol[e]]]
            elif e == t.diag[k]:
                acc = 1.0 / acc
            ref[e] = acc
    G = np.full(nz, np.nan)
    dot = t.dot_term.view(np.uint32)

    def lu_finish(e, z, v):
        if z == 0xFFFFFFFF:
            assert e == t.diag[irow[e]]
            v = 1.0 / v
        elif z != 0xFFFFFFFE:
            assert e < t.diag[irow[e]] and z == t.diag[t.icol[e]]
            v = v * G[z]
        G[e] = v

    _replay(t, "lu", lambda e, z: J0[e] + (ghinv if z == 0xFFFFFFFF else 0.0),
            lambda e, k, acc: acc - G[int(dot[k]) >> 16] * G[int(dot[k]) & 0xFFFF], lu_finish)
    assert np.allclose(G, ref, rtol=1e-11, atol=0)
    # substitutions with those factors
    b = rng.standard_normal(nvar)
    x = b.copy()
    for i in range(nvar):
        for kk in range(t.crow[i], t.diag[i]):
            x[i] -= ref[kk] * x[t.icol[kk]]
    for i in range(nvar - 1, -1, -1):
        for kk in range(t.diag[i] + 1, t.crow[i + 1]):
            x[i] -= ref[kk] * x[t.icol[kk]]
        x[i] *= ref[t.diag[i]]
    X = b.copy()

    def sfinish(back):
        def f(i, z, v):
            if back:
                assert z == t.diag[i]
                v = v * G[z]
            X[i] = v
        return f

    for ph, back in (("fs", False), ("bs", True)):
        _replay(t, ph, lambda i, z: X[i], lambda i, kk, acc: acc - G[kk] * X[t.icol[kk]], sfinish(back))
    assert np.allclose(X, x, rtol=1e-9, atol=1e-12 * np.abs(x).max())


def test_split_fun_and_jac_match_sequential(tab):
    rng = np.random.default_rng(12)
    t = tab
    nvar = t.nvar
    A = rng.standard_normal(t.nreact)
    B = rng.standard_normal(t.nb)
    V = rng.standard_normal(nvar)
    slit = np.array(t.slit)
    ps, ds, js = t.p_sterm, t.d_sterm, t.j_sterm

    def csum(terms, s, e, X):
        return sum(slit[int(u) >> 20] * X[int(u) & 0xFFFFF] for u in terms[s:e])

    ref = np.array([csum(ps, t.p_start[i], t.p_start[i + 1], A) -
                    csum(ds, t.d_start[i], t.d_start[i + 1], B) * V[i] for i in range(nvar)])
    P = np.full(nvar, np.nan)
    D = np.full(nvar, np.nan)

    def fterm(item, k, acc):
        if item < nvar:
            return acc + slit[int(ps[k]) >> 20] * A[int(ps[k]) & 0xFFFFF]
        return acc + slit[int(ds[k]) >> 20] * B[int(ds[k]) & 0xFFFFF]

    def ffinish(item, z, v):
        if item < nvar:
            P[item] = v
        else:
            D[item - nvar] = v

    _replay(t, "fun", lambda i, z: 0.0, fterm, ffinish)
    assert np.allclose(P - D * V, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    jref = np.array([-csum(js, t.j_start[e], t.j_start[e + 1], B) for e in range(t.lu_nonzero)])
    J = np.full(t.lu_nonzero, np.nan)

    def jfinish(e, z, v):
        J[e] = v

    _replay(t, "jac", lambda e, z: 0.0,
            lambda e, k, acc: acc - slit[int(js[k]) >> 20] * B[int(js[k]) & 0xFFFFF], jfinish)
    assert np.allclose(J, jref, rtol=1e-12, atol=1e-12 * np.abs(jref).max())


def test_solve_records_carry_the_substitution_schedule(tab):
    """The 32-byte lane records that the kernel stages for the substitution
    passes hold each lane's task word, the level-end bit on every lane of a
    level's last pass (all lanes of the warp then meet at the warp barrier),
    the warp's chunk and butterfly bounds, the first term and finish word,
    and the columns of the lane's terms, so the records replay the schedule
    above."""
    import gcchem.tables as tables

    t = tab
    for ph in ("fs", "bs"):
        task, info = t.split[ph]
        npass = len(info)
        rec = t.split_rec[ph].reshape(npass, 32, 8).astype(np.int64)
        tk = task.reshape(npass, 32, 4).astype(np.int64)
        assert np.array_equal(rec[:, :, 0] & 0xFFFFFF, tk[:, :, 0])
        assert np.array_equal((rec[:, :, 0] >> 24) & 1, np.repeat(((info.astype(np.int64) >> 3) & 1)[:, None], 32, 1))
        assert np.array_equal((rec[:, :, 0] >> 25) & 15, (tk[:, :, 3] >> 1) & 15)
        assert np.array_equal(rec[:, :, 0] >> 29, (tk[:, :, 3] >> 5) & 7)
        assert np.array_equal(rec[:, :, 1] & 0xFFFF, tk[:, :, 1])
        assert np.array_equal(rec[:, :, 1] >> 16, tk[:, :, 2])
        for p in range(npass):
            for lane in range(32):
                n = (int(rec[p, lane, 0]) >> 19) & 31
                y = int(rec[p, lane, 1]) & 0xFFFF
                cols = [(int(rec[p, lane, 2 + k // 2]) >> (16 * (k & 1))) & 0xFFFF for k in range(tables.SPLIT_MAXCH)]
                assert cols[:n] == [int(c) for c in t.icol[y:y + n]] and not any(cols[n:])
