"""Device tables for the table-driven mechanism engine.

The mechanism IR (``mechanism/fullchem.json``) is lowered here to flat integer
tables that the CUDA engine (``csrc/kpp_mech.cuh``) walks with warp-uniform
loops: every lane of a warp runs the same table entry for its own cell, so the
table reads are broadcasts and the per-cell data reads are coalesced.

Operand codes (int32) used by products:

    [0, NVAR)                       V(i)    variable species (current point)
    [NVAR, NVAR+NFIX)               F(i)    fixed species
    [NVAR+NFIX, NVAR+NFIX+NREACT)   RCT(r)  rate constants
    [LIT0, ...)                     literal constant LIT[code-LIT0]

Products: ``prod_start``/``prod_fac``; products [0,NREACT) are the reaction
rates A(r) of Fun_SPLIT (KPP/fullchem/gckpp_Function.F90:2172-2230ff), products
[NREACT, NREACT+NB) are the Jacobian partials B(b) of Jac_SP
(KPP/fullchem/gckpp_Jacobian.F90:48ff).  Every D_VAR term of Fun_SPLIT is the
same product as one B(b); the tables record which.

Signed coefficient terms (P_VAR over A, JVS over B, D_VAR over B products)
are packed as ``sign<<31 | coef<<20 | index`` with ``coef == 0x7ff`` meaning
no coefficient (a bare reference).

The LU program follows KppDecomp (KPP/fullchem/gckpp_LinearAlgebra.F90:46-83):
for each row k, for each L entry (k,j) in column order, a = W(j)/pivot(j) and
W(c) -= a*U(j,c) for the U part of row j.  W is row k of the matrix itself
(KPP's dense work vector only ever holds row k's pattern).  ``lop`` lists the
L entries (position of (k,j), position of diag j, start of its U ops);
``uop`` packs (position of (k,c)) << 16 | (position of (j,c)).
"""
import os
import struct

import numpy as np

from . import mechanism

NOCOEF = 0x7FF
# threads of the split block-per-cell kernel, the lanes each phase's passes
# use (the substitutions run on the first warp alone, with warp barriers), and
# per phase the largest number of terms a lane sums before a segment combines
# its partial sums
SPLIT_NT = 256
SPLIT_PHASE_NT = {"lu": 256, "fs": 32, "bs": 32, "fun": 256, "jac": 256}
SPLIT_CHUNK = {"lu": 8, "fs": 8, "bs": 8, "fun": 8, "jac": 8}
SPLIT_MAXCH = 12  # register slots of a lane's chunk in the kernel


def _hexfloat(x):
    return float(x).hex()


class Tables:
    def __init__(self, ir):
        d = ir["dims"]
        self.nvar, self.nfix, self.nreact = d["nvar"], d["nfix"], d["nreact"]
        self.nspec = d["nspec"]
        self.lu_nonzero = d["lu_nonzero"]
        self.nb = len(ir["jac"]["B"])
        self.lit0 = self.nvar + self.nfix + self.nreact
        self.literals = []
        self._lit_index = {}

        def lit(tok):
            v = float(tok.replace("d", "e").replace("D", "e"))
            key = struct.pack("<d", v)
            if key not in self._lit_index:
                self._lit_index[key] = len(self.literals)
                self.literals.append(v)
            return self._lit_index[key]

        def fac(tok):
            kind, rest = tok[0], tok[1:]
            if kind == "V":
                return int(rest)
            if kind == "F":
                return self.nvar + int(rest)
            if kind == "R":
                return self.nvar + self.nfix + int(rest)
            return self.lit0 + lit(tok)

        prods = list(ir["fun"]["A"]) + [b if b is not None else [] for b in ir["jac"]["B"]]
        self.prod_start = np.zeros(len(prods) + 1, np.int32)
        facs = []
        for i, p in enumerate(prods):
            facs += [fac(t) for t in p]
            self.prod_start[i + 1] = len(facs)
        self.prod_fac = np.array(facs, np.int32)

        # Packed products for the engine: every product of the mechanism has
        # the shape  pre [* 2] * s1 * s2 * s3  with pre a rate constant (or
        # one of the two constant-rate literals, kept as extra rate slots),
        # an optional literal 2 right after it, and up to three species
        # factors (variable or fixed species, indices into [V | F]).
        #   x = pre | times2 << 12 | nspecies << 13 | s1 << 16
        #   y = s2 | s3 << 16
        self.pre_literals = []
        packed = []
        for p in prods:
            if not p:
                packed.append((0, 0))
                continue
            head = p[0]
            if head[0] == "R":
                pre = int(head[1:])
            else:
                v = float(head)
                if v not in self.pre_literals:
                    self.pre_literals.append(v)
                pre = self.nreact + self.pre_literals.index(v)
            rest = p[1:]
            two = 0
            if rest and not rest[0][0].isalpha():
                assert float(rest[0]) == 2.0, p
                two = 1
                rest = rest[1:]
            sp = []
            for t in rest:
                assert t[0] in "VF", p
                sp.append(int(t[1:]) if t[0] == "V" else self.nvar + int(t[1:]))
            assert len(sp) <= 3 and pre < 4096
            s = sp + [0] * (3 - len(sp))
            packed.append((pre | (two << 12) | (len(sp) << 13) | (s[0] << 16), s[1] | (s[2] << 16)))
        self.prod_packed = np.array(packed, np.uint32)
        self.naux = self.nreact + len(self.pre_literals)
        # the A products (reactions) and the B products, each listed by class
        # c = 2 * nspecies + times2 (stable within a class): a loop over one
        # class multiplies a fixed number of times, with no per-product test
        x = self.prod_packed[:, 0].astype(np.int64)
        cls = ((x >> 13) & 3) * 2 + ((x >> 12) & 1)
        self.prod_ids_a, self.a_cls_start = _by_class(cls[: self.nreact])
        self.prod_ids_b, self.b_cls_start = _by_class(cls[self.nreact:])

        def coef_terms(lists):
            start = np.zeros(len(lists) + 1, np.int32)
            out = []
            for i, terms in enumerate(lists):
                for sign, coef, idx in terms:
                    c = NOCOEF if coef is None else lit(coef)
                    assert (coef is None or c < NOCOEF) and idx < (1 << 20)
                    out.append(((1 if sign == "-" else 0) << 31) | (c << 20) | idx)
                start[i + 1] = len(out)
            return start, np.array(out, np.uint32).view(np.int32)

        self.p_start, self.p_term = coef_terms(ir["fun"]["P"])
        self.j_start, self.j_term = coef_terms(ir["jac"]["JVS"])

        bmap = {tuple(b): i for i, b in enumerate(ir["jac"]["B"]) if b is not None}
        dl = []
        for terms in ir["fun"]["D"]:
            dl.append([[s, None, bmap[tuple(f)]] for s, f in terms])
        self.d_start, self.d_term = coef_terms(dl)

        # Device form of the same terms: the sign folded into a signed
        # coefficient table (a bare reference becomes +/-1.0, which multiplies
        # exactly), so every term is  acc += slit[c] * X[idx]  with no branch.
        #   sterm = c << 20 | idx
        self.slit = []
        slit_index = {}

        def sterms(packed):
            out = []
            for u in packed.view(np.uint32):
                u = int(u)
                c = (u >> 20) & 0x7FF
                v = 1.0 if c == NOCOEF else self.literals[c]
                if u >> 31:
                    v = -v
                key = struct.pack("<d", v)
                if key not in slit_index:
                    slit_index[key] = len(self.slit)
                    self.slit.append(v)
                out.append((slit_index[key] << 20) | (u & 0xFFFFF))
            return np.array(out, np.uint32)

        self.p_sterm = sterms(self.p_term)
        self.j_sterm = sterms(self.j_term)
        self.d_sterm = sterms(self.d_term)
        assert len(self.slit) < 4096

        lu = ir["lu"]
        crow, diag, icol = lu["crow"], lu["diag"], lu["icol"]
        self.crow = np.array(crow, np.int32)
        self.diag = np.array(diag, np.int32)
        self.icol = np.array(icol, np.int32)
        self.irow = np.array(lu["irow"], np.int32)
        lrow_start = [0]
        lop = []
        uop = []
        for k in range(self.nvar):
            pos = {icol[kk]: kk for kk in range(crow[k], crow[k + 1])}
            for kk in range(crow[k], diag[k]):
                j = icol[kk]
                lop.append((kk, diag[j], len(uop)))
                for jj in range(diag[j] + 1, crow[j + 1]):
                    uop.append((pos[icol[jj]] << 16) | jj)
            lrow_start.append(len(lop))
        self.lrow_start = np.array(lrow_start, np.int32)
        self.lop_kk = np.array([x[0] for x in lop], np.int32)
        self.lop_dj = np.array([x[1] for x in lop], np.int32)
        self.lop_u = np.array([x[2] for x in lop] + [len(uop)], np.int32)
        self.uop = np.array(uop, np.uint32).view(np.int32)
        # The same updates regrouped per target entry (row-wise "dot product"
        # form): entry e = (k,c) receives W(c) -= L(k,j)*U(j,c) for the L
        # entries j of row k in ascending order, exactly the sequence of
        # updates KppDecomp applies to W(c).  ``dot_start[e]`` indexes
        # ``dot_term`` = (position of (k,j)) << 16 | (position of (j,c)).
        upos = [{icol[jj]: jj for jj in range(diag[j] + 1, crow[j + 1])} for j in range(self.nvar)]
        self.dot_start = np.zeros(self.lu_nonzero + 1, np.int32)
        dot = []
        for k in range(self.nvar):
            for e in range(crow[k], crow[k + 1]):
                c = icol[e]
                for kk in range(crow[k], diag[k]):
                    j = icol[kk]
                    if j >= c:
                        break
                    jj = upos[j].get(c)
                    if jj is not None:
                        dot.append((kk << 16) | jj)
                self.dot_start[e + 1] = len(dot)
        self.dot_term = np.array(dot, np.uint32).view(np.int32)
        assert len(self.dot_term) == len(self.uop)
        assert self.lu_nonzero < (1 << 16)
        self._level_schedules(crow, diag, icol)
        self.lit = np.array(self.literals, np.float64)
        self.family_species = np.array([ir["species"].index(f) for f in ir.get("families", [])], np.int32)

    def _level_schedules(self, crow, diag, icol):
        """Dependency levels for the block-per-cell kernel, where the threads
        of a block share one cell.  Each LU entry (k,c) is still one
        sequential dot product (the same operation order as the thread-per-cell
        form); an entry's level is one more than the highest level among the
        entries it reads (L(k,j), U(j,c), and the pivot (c,c) for c < k).  The
        substitutions get row levels the same way.  Within a level, the
        longest items come first so that round-robin assignment starts them
        early.  Fun_SPLIT rows and Jac_SP entries are independent and are
        listed longest first."""
        nvar, nz = self.nvar, self.lu_nonzero
        lvl = np.zeros(nz, np.int64)
        cost = np.zeros(nz, np.int64)
        terms = self.dot_term.view(np.uint32)
        for k in range(nvar):
            for e in range(crow[k], crow[k + 1]):
                t0, t1 = self.dot_start[e], self.dot_start[e + 1]
                m = 0
                for t in terms[t0:t1]:
                    m = max(m, lvl[int(t) >> 16], lvl[int(t) & 0xFFFF])
                if icol[e] < k:
                    m = max(m, lvl[diag[icol[e]]])
                lvl[e] = m + 1
                cost[e] = t1 - t0
        order = sorted(range(nz), key=lambda e: (lvl[e], -cost[e], e))
        self.lu_lvl_entry = np.array(order, np.int32)
        nl = int(lvl.max())
        self.lu_lvl_start = np.searchsorted(lvl[order], np.arange(1, nl + 2)).astype(np.int32)

        def row_levels(rows, deps):
            lv = np.zeros(nvar, np.int64)
            ln = np.zeros(nvar, np.int64)
            for i in rows:
                d = deps(i)
                lv[i] = 1 + max((lv[j] for j in d), default=0)
                ln[i] = len(d)
            o = sorted(range(nvar), key=lambda i: (lv[i], -ln[i], i))
            n = int(lv.max())
            return np.array(o, np.int32), np.searchsorted(lv[o], np.arange(1, n + 2)).astype(np.int32)

        self.fs_lvl_row, self.fs_lvl_start = row_levels(
            range(nvar), lambda i: [icol[kk] for kk in range(crow[i], diag[i])])
        self.bs_lvl_row, self.bs_lvl_start = row_levels(
            range(nvar - 1, -1, -1), lambda i: [icol[kk] for kk in range(diag[i] + 1, crow[i + 1])])
        flen = np.diff(self.p_start) + np.diff(self.d_start)
        self.fun_rows_by_len = np.array(sorted(range(nvar), key=lambda i: (-flen[i], i)), np.int32)
        jlen = np.diff(self.j_start)
        self.jac_by_len = np.array(sorted(range(nz), key=lambda e: (-jlen[e], e)), np.int32)
        self._split_schedules(crow, diag)

    def _split_schedules(self, crow, diag):
        """Pass schedules of the split block-per-cell kernel.

        Every sum of the block phases (an LU entry's dot product, a
        substitution row, a Fun_SPLIT P or D row, a Jac_SP entry) is one item;
        an item of L terms gets a segment of s lanes (s a power of two, the
        smallest with ceil(L/s) <= SPLIT_CHUNK[phase], at most 32), each lane sums a
        contiguous chunk of the terms and the segment adds its partial sums
        with a butterfly of warp shuffles.  Within a dependency level the
        segments are placed largest first, so each starts at a multiple of its
        size and none crosses a warp; the level is cut into passes of
        SPLIT_PHASE_NT[phase] lanes and only its last pass ends with a barrier.

        task (four uint32 per lane): x = item | seglog << 16 | nterms << 19,
        y = index of the lane's first term in the phase's term array, z =
        the phase's finish word (LU: position of the pivot of an L entry,
        0xFFFFFFFF for a diagonal entry, 0xFFFFFFFE for a U entry; backward
        substitution: position of the row's diagonal), and w, the same for
        the 32 lanes of a warp: 1 if one of them has an item | their largest
        nterms << 1 | their largest seglog << 5 (so a warp learns its chunk
        loop and butterfly bounds without a warp reduction); item 0xFFFF is
        an idle lane.  pass word: max seglog of the pass | barrier << 3."""
        nvar, nz = self.nvar, self.lu_nonzero

        def passes(levels, ph):
            NT, CH = SPLIT_PHASE_NT[ph], SPLIT_CHUNK[ph]
            task, info = [], []
            for items in levels:
                segs = []
                for it, t0, n, z in items:
                    s = 1
                    while s < 32 and -(-n // s) > CH:
                        s *= 2
                    segs.append((s, n, it, t0, z))
                if not segs:
                    continue
                segs.sort(key=lambda x: (-x[0], -x[1], x[2]))
                lanes = []
                for s, n, it, t0, z in segs:
                    ch = -(-n // s)
                    assert ch <= SPLIT_MAXCH and it < 0xFFFF
                    for j in range(s):
                        a, b = min(n, j * ch), min(n, (j + 1) * ch)
                        lanes.append((it | (s.bit_length() - 1) << 16 | (b - a) << 19, t0 + a, z))
                npass = -(-len(lanes) // NT)
                lanes += [(0xFFFF, 0, 0)] * (npass * NT - len(lanes))
                for p in range(npass):
                    blk = lanes[p * NT:(p + 1) * NT]
                    maxlog = max((x >> 16) & 7 for x, _, _ in blk)
                    info.append(maxlog | (8 if p == npass - 1 else 0))
                    for w0 in range(0, NT, 32):
                        warp = blk[w0:w0 + 32]
                        busy = [x for x, _, _ in warp if (x & 0xFFFF) != 0xFFFF]
                        wd = (1 | max((x >> 19) & 31 for x in busy) << 1 | max((x >> 16) & 7 for x in busy) << 5
                              if busy else 0)
                        for x, y, z in warp:
                            task += [x, y, z, wd]
            return np.array(task, np.uint32), np.array(info, np.uint32)

        def levels_of(order, start, item):
            return [[item(int(i)) for i in order[start[l]:start[l + 1]]] for l in range(len(start) - 1)]

        irow = np.repeat(np.arange(nvar), np.diff(crow))

        def lu_z(e):
            k = int(irow[e])
            if e == diag[k]:
                return 0xFFFFFFFF
            return int(diag[self.icol[e]]) if e < diag[k] else 0xFFFFFFFE

        self.split = {}
        self.split["lu"] = passes(levels_of(
            self.lu_lvl_entry, self.lu_lvl_start,
            lambda e: (e, int(self.dot_start[e]), int(self.dot_start[e + 1] - self.dot_start[e]), lu_z(e))),
            "lu")
        # substitution terms are positions kk of the LU pattern (G[kk] times
        # X[icol[kk]]); forward rows without terms are left out
        fs = levels_of(self.fs_lvl_row, self.fs_lvl_start,
                       lambda i: (i, int(crow[i]), int(diag[i] - crow[i]), 0))
        self.split["fs"] = passes([[x for x in lv if x[2] > 0] for lv in fs], "fs")
        self.split["bs"] = passes(levels_of(self.bs_lvl_row, self.bs_lvl_start,
                                            lambda i: (i, int(diag[i]) + 1, int(crow[i + 1] - diag[i] - 1),
                                                       int(diag[i]))),
                                  "bs")
        # Fun_SPLIT: items [0, NVAR) are P rows (p_sterm), [NVAR, 2 NVAR) D rows (d_sterm)
        self.split["fun"] = passes([
            [(i, int(self.p_start[i]), int(self.p_start[i + 1] - self.p_start[i]), 0) for i in range(nvar)] +
            [(nvar + i, int(self.d_start[i]), int(self.d_start[i + 1] - self.d_start[i]), 0) for i in range(nvar)]],
            "fun")
        self.split["jac"] = passes([[(e, int(self.j_start[e]), int(self.j_start[e + 1] - self.j_start[e]), 0)
                                     for e in range(nz)]], "jac")
        self.split_rec = {ph: self._solve_records(ph) for ph in ("fs", "bs")}

    def _solve_records(self, ph):
        """Lane records of the substitution passes, which the kernel copies
        into shared memory a few passes ahead: eight uint32 per lane per pass,
        x | level end << 24 | the warp's largest nterms << 25 | its largest
        seglog << 29 (the last three the same on every lane of the pass),
        first term | finish word << 16, then the columns icol[first + k] of
        the lane's terms, two 16-bit columns per word (SPLIT_MAXCH of them)."""
        task, info = self.split[ph]
        nt = SPLIT_PHASE_NT[ph]
        assert nt == 32 and 2 + (SPLIT_MAXCH + 1) // 2 <= 8
        task = task.reshape(-1, 4)
        rec = np.zeros((len(info) * nt, 8), np.uint32)
        for p, w in enumerate(info):
            end = (int(w) >> 3) & 1
            for lane in range(nt):
                x, y, z, wd = (int(v) for v in task[p * nt + lane])
                n = (x >> 19) & 31
                nmax, lmax = (wd >> 1) & 15, (wd >> 5) & 7
                assert x < (1 << 24) and y < 0x10000 and z < 0x10000 and n <= SPLIT_MAXCH <= 15 and lmax <= 5
                words = [x | end << 24 | nmax << 25 | lmax << 29, y | z << 16] + [0] * 6
                for k in range(n):
                    col = int(self.icol[y + k])
                    assert col < 0x10000
                    words[2 + k // 2] |= col << (16 * (k & 1))
                rec[p * nt + lane] = words
        return rec.reshape(-1)

    # flop bookkeeping used by the roofline accounting (FP64 operations per
    # call, counting a multiply-add as 2, a division as 1, in STRICT form)
    def flops(self):
        nfac_a = int(self.prod_start[self.nreact])
        mul_a = nfac_a - self.nreact
        mul_b = int(self.prod_start[-1] - self.prod_start[self.nreact]) - sum(
            1 for i in range(self.nreact, len(self.prod_start) - 1) if self.prod_start[i + 1] > self.prod_start[i])
        pt = self.p_term.view(np.uint32)
        jt = self.j_term.view(np.uint32)
        coefp = int(np.sum(((pt >> 20) & 0x7FF) != NOCOEF))
        coefj = int(np.sum(((jt >> 20) & 0x7FF) != NOCOEF))
        addp = len(pt) - np.count_nonzero(np.diff(self.p_start) > 0)
        addj = len(jt) - np.count_nonzero(np.diff(self.j_start) > 0)
        dfac = 0
        for t in self.d_term.view(np.uint32):
            b = int(t & 0xFFFFF) + self.nreact
            dfac += int(self.prod_start[b + 1] - self.prod_start[b]) - 1
        addd = len(self.d_term) - np.count_nonzero(np.diff(self.d_start) > 0)
        fun = mul_a + coefp + int(addp) + dfac + int(addd) + 2 * self.nvar
        jac = mul_b + coefj + int(addj)
        lu_fma = len(self.uop)
        decomp = 2 * lu_fma + len(self.lop_kk) + self.nvar  # FMA + L divisions + diag shift
        solve = 2 * int(sum((self.crow[i + 1] - self.crow[i] - 1) for i in range(self.nvar))) + self.nvar
        return {"fun": int(fun), "jac": int(jac), "decomp": int(decomp), "solve": int(solve)}

    def emit_c(self):
        """C source defining the tables (included by the CUDA library)."""
        out = ["// Generated by gcchem.tables from mechanism/fullchem.json. Do not edit.",
               "#pragma once",
               "namespace gcmech_tables {",
               "constexpr int NVAR = %d, NFIX = %d, NSPEC = %d, NREACT = %d, LU_NONZERO = %d, NB = %d, LIT0 = %d;"
               % (self.nvar, self.nfix, self.nspec, self.nreact, self.lu_nonzero, self.nb, self.lit0),
               "constexpr unsigned NOCOEF = 0x%x;" % NOCOEF]

        def arr(name, a, ctype="int"):
            vals = ",".join(str(int(v)) for v in a)
            out.append("static const %s %s[%d] = {%s};" % (ctype, name, len(a), vals))

        arr("prod_start", self.prod_start)
        arr("prod_fac", self.prod_fac)
        arr("prod_packed", self.prod_packed.reshape(-1), "unsigned")
        arr("prod_ids_a", self.prod_ids_a)
        arr("prod_ids_b", self.prod_ids_b)
        arr("a_cls_start", self.a_cls_start)
        arr("b_cls_start", self.b_cls_start)
        arr("p_sterm", self.p_sterm, "unsigned")
        arr("d_sterm", self.d_sterm, "unsigned")
        arr("j_sterm", self.j_sterm, "unsigned")
        out.append("static const double slit[%d] = {%s};" % (len(self.slit), ",".join(_hexfloat(v) for v in self.slit)))
        out.append("constexpr int NAUX = %d;" % self.naux)
        out.append("static const double pre_literals[%d] = {%s};" % (
            max(1, len(self.pre_literals)), ",".join(_hexfloat(v) for v in self.pre_literals) or "0.0"))
        arr("p_start", self.p_start)
        arr("p_term", self.p_term.view(np.uint32), "unsigned")
        arr("d_start", self.d_start)
        arr("d_term", self.d_term.view(np.uint32), "unsigned")
        arr("j_start", self.j_start)
        arr("j_term", self.j_term.view(np.uint32), "unsigned")
        arr("lu_crow", self.crow)
        arr("lu_diag", self.diag)
        arr("lu_icol", self.icol)
        arr("lrow_start", self.lrow_start)
        arr("lop_kk", self.lop_kk)
        arr("lop_dj", self.lop_dj)
        arr("lop_u", self.lop_u)
        arr("uop", self.uop.view(np.uint32), "unsigned")
        arr("family_species", self.family_species)
        arr("dot_start", self.dot_start)
        arr("dot_term", self.dot_term.view(np.uint32), "unsigned")
        arr("lu_irow", np.repeat(np.arange(self.nvar), np.diff(self.crow)))
        arr("lu_lvl_start", self.lu_lvl_start)
        arr("lu_lvl_entry", self.lu_lvl_entry)
        arr("fs_lvl_start", self.fs_lvl_start)
        arr("fs_lvl_row", self.fs_lvl_row)
        arr("bs_lvl_start", self.bs_lvl_start)
        arr("bs_lvl_row", self.bs_lvl_row)
        arr("fun_rows_by_len", self.fun_rows_by_len)
        arr("jac_by_len", self.jac_by_len)
        out.append("constexpr int LU_NLVL = %d, FS_NLVL = %d, BS_NLVL = %d;" % (
            len(self.lu_lvl_start) - 1, len(self.fs_lvl_start) - 1, len(self.bs_lvl_start) - 1))
        out.append("constexpr int SPLIT_NT = %d;" % SPLIT_NT)
        for ph in ("lu", "fs", "bs", "fun", "jac"):
            task, info = self.split[ph]
            out.append("constexpr int SPLIT_%s_NT = %d, SPLIT_%s_NPASS = %d;" % (
                ph.upper(), SPLIT_PHASE_NT[ph], ph.upper(), len(info)))
            arr("split_%s_task" % ph, task if len(task) else np.zeros(4, np.uint32), "unsigned")
            arr("split_%s_pass" % ph, info if len(info) else np.zeros(1, np.uint32), "unsigned")
            if ph in self.split_rec:
                rec = self.split_rec[ph]
                arr("split_%s_rec" % ph, rec if len(rec) else np.zeros(8, np.uint32), "unsigned")
        out.append("static const double lit[%d] = {%s};" % (
            len(self.literals), ",".join(_hexfloat(v) for v in self.literals)))
        out.append("}  // namespace gcmech_tables")
        return "\n".join(out) + "\n"


def _by_class(cls, nclass=8):
    """Indices sorted by class (stable) and the start of each class, [nclass + 1]."""
    order = np.argsort(cls, kind="stable").astype(np.int32)
    start = np.searchsorted(cls[order], np.arange(nclass + 1)).astype(np.int32)
    return order, start


def build_tables(ir=None):
    return Tables(ir or mechanism.load_ir())


def write_generated(outdir, ir=None):
    t = build_tables(ir)
    os.makedirs(outdir, exist_ok=True)
    path = os.path.join(outdir, "mech_tables.inc")
    text = t.emit_c()
    old = open(path).read() if os.path.exists(path) else None
    if old != text:
        with open(path, "w") as fh:
            fh.write(text)
    return path
