// Table-driven per-cell mechanism engine: Fun_SPLIT, Jac_SP, KppDecomp
// (fused with ros_PrepareMatrix) and KppSolve, for NC cells per thread.
//
// Every lane of a warp executes the same table entry for its own cells, so
// table reads are warp-uniform broadcasts and the per-cell reads/writes are
// coalesced.  A warp's workspace tile interleaves 32*NC cells: entry e of the
// thread's cell q sits at p[e * 32 * NC + q * 32] from the thread's base
// pointer.  With NC > 1 every table entry drives NC independent loads and
// FP64 operations, which is what hides memory and FP64-pipe latency.
//
// STRICT=true reproduces the KPP-generated Fortran statement by statement in
// the same evaluation order (the translation unit is compiled -fmad=false):
//   Fun_SPLIT       KPP/fullchem/gckpp_Function.F90:2172-5059
//   Jac_SP          KPP/fullchem/gckpp_Jacobian.F90:48-20887
//   PrepareMatrix   KPP/fullchem/gckpp_Integrator.F90:1969-1974
//   KppDecomp       KPP/fullchem/gckpp_LinearAlgebra.F90:46-83
//   KppSolve        KPP/fullchem/gckpp_LinearAlgebra.F90:644-2309
// STRICT=false is the production arithmetic: fused multiply-adds, the
// Jacobian stored negated, and reciprocal pivots stored on the LU diagonal so
// that L factors and back substitution multiply instead of divide.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gckpp {

constexpr int TS = 32;  // lanes per warp

struct MechDev {
  int nvar, nfix, nreact, nspec, lu_nonzero, nb, lit0;
  const uint2* prod_packed;  // pre | times2<<12 | nspecies<<13 | s1<<16, s2 | s3<<16
  const double* pre_lit;     // constant-rate literals, appended to RCT in aux
  int naux;
  // the A products (reaction r) and B products (b) listed by class
  // c = 2 * nspecies + times2; class c is [x_cls[c], x_cls[c + 1]) of the list
  const int* prod_ids_a;
  const int* prod_ids_b;
  int a_cls[9], b_cls[9];
  const int* p_start;
  const unsigned* p_sterm;
  const int* d_start;
  const unsigned* d_sterm;
  const int* j_start;
  const unsigned* j_sterm;
  const double* slit;  // signed term coefficients
  const int* lu_crow;
  const int* lu_diag;
  const int* lu_icol;
  const int* lrow_start;
  const int* lop_kk;
  const int* lop_dj;
  const int* lop_u;
  const unsigned* uop;
  const int* dot_start;
  const unsigned* dot_term;
  const double* lit;
  // level schedules of the block-per-cell kernel (tables.py _level_schedules)
  const int* lu_irow;
  const int* lu_lvl_start;
  const int* lu_lvl_entry;
  const int* fs_lvl_start;
  const int* fs_lvl_row;
  const int* bs_lvl_start;
  const int* bs_lvl_row;
  const int* fun_rows_by_len;
  const int* jac_by_len;
  int lu_nlvl, fs_nlvl, bs_nlvl;
  // pass schedules of the split block-per-cell kernel (tables.py
  // _split_schedules), indexed by SplitPhase
  const uint4* sp_task[5];  // x, y, z, 0 per lane per pass
  const unsigned* sp_pass[5];
  int sp_npass[5];
  int sp_nt[5];
  // the substitution passes (SP_FS, SP_BS) as 32-byte lane records
  // (tables.py _solve_records), two uint4 per lane per pass
  const uint4* sp_rec[2];
};

enum SplitPhase : int { SP_LU = 0, SP_FS = 1, SP_BS = 2, SP_FUN = 3, SP_JAC = 4 };

__device__ __forceinline__ int ldi(const int* p) { return __ldg(p); }
__device__ __forceinline__ unsigned ldu(const unsigned* p) { return __ldg(p); }

// Per-cell workspace read.  With GCKPP_LDCG the read bypasses L1 (the tables
// then keep L1 to themselves); otherwise it is an ordinary cached load.
__device__ __forceinline__ double ldw(const double* p) {
#if defined(GCKPP_LDCG) && GCKPP_LDCG
  return __ldcg(p);
#else
  return *p;
#endif
}

// |x| < TINY(1.0_dp), on the bit pattern
__device__ __forceinline__ bool tiny_abs(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffULL) <
         0x0010000000000000ULL;
}

// The products of one class (NS species factors, TIMES2) at list positions
// [s, e): out[id] = pre [* 2] * s1 * s2 * s3, in the Fortran's left-to-right
// order, for id = ids[i], product index base + id.  aux holds RCT (and the
// constant-rate literals), Y the species [V | F].  The factor count is fixed
// at compile time, so a warp executes only the multiplications the products
// have, and all loads are issued before the multiplications.
template <int NS, bool TIMES2, int NC>
__device__ __forceinline__ void product_class(const MechDev& m, const int* __restrict__ ids, int s, int e, int base,
                                              const double* Y, const double* aux, double* out) {
  constexpr int TSN = TS * NC;
#pragma unroll 2
  for (int i = s; i < e; ++i) {
    const int id = ldi(ids + i);
    const uint2 t = __ldg(m.prod_packed + base + id);
    const int ia = (t.x & 0xfffu) * TSN, i1 = (t.x >> 16) * TSN, i2 = (t.y & 0xffffu) * TSN,
              i3 = (t.y >> 16) * TSN;
    double a[NC], v1[NC], v2[NC], v3[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      a[q] = ldw(aux + ia + q * TS);
      if (NS >= 1) v1[q] = ldw(Y + i1 + q * TS);
      if (NS >= 2) v2[q] = ldw(Y + i2 + q * TS);
      if (NS >= 3) v3[q] = ldw(Y + i3 + q * TS);
    }
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      double r = a[q];
      if (TIMES2) r = r * 2.0;
      if (NS >= 1) r = r * v1[q];
      if (NS >= 2) r = r * v2[q];
      if (NS >= 3) r = r * v3[q];
      out[id * TSN + q * TS] = r;
    }
  }
}

// Every product of a list (A: base 0, ids prod_ids_a, cls a_cls; B: base
// nreact, ids prod_ids_b, cls b_cls), class by class.
template <int NC>
__device__ __forceinline__ void products_by_class(const MechDev& m, const int* ids, const int* cls, int base,
                                                  const double* Y, const double* aux, double* out) {
  product_class<0, false, NC>(m, ids, cls[0], cls[1], base, Y, aux, out);
  product_class<0, true, NC>(m, ids, cls[1], cls[2], base, Y, aux, out);
  product_class<1, false, NC>(m, ids, cls[2], cls[3], base, Y, aux, out);
  product_class<1, true, NC>(m, ids, cls[3], cls[4], base, Y, aux, out);
  product_class<2, false, NC>(m, ids, cls[4], cls[5], base, Y, aux, out);
  product_class<2, true, NC>(m, ids, cls[5], cls[6], base, Y, aux, out);
  product_class<3, false, NC>(m, ids, cls[6], cls[7], base, Y, aux, out);
  product_class<3, true, NC>(m, ids, cls[7], cls[8], base, Y, aux, out);
}

// Sum of signed terms  slit[c] * X[idx]  (sterm = c << 20 | idx) in the
// reference's left-to-right order.  The sign is folded into the coefficient
// (a bare X(idx) is +/-1.0 * X(idx), exact), so the loop has no branch and
// consecutive terms' loads overlap.  FLIP negates the sum (exact).
template <bool STRICT, bool FLIP, int NC>
__device__ __forceinline__ void term_sum(const MechDev& m, const unsigned* __restrict__ terms, int s, int e,
                                         const double* __restrict__ X, double* acc) {
  constexpr int TSN = TS * NC;
#pragma unroll
  for (int q = 0; q < NC; ++q) acc[q] = 0.0;
#pragma unroll 4
  for (int i = s; i < e; ++i) {
    const unsigned t = ldu(terms + i);
    const double cf = __ldg(m.slit + (t >> 20));
    const double* xp = X + (t & 0xfffffu) * TSN;
    double x[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) x[q] = ldw(xp + q * TS);
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      if (STRICT) {
        const double v = cf * x[q];
        acc[q] = (i == s) ? (FLIP ? -v : v) : (FLIP ? acc[q] - v : acc[q] + v);
      } else {
        acc[q] = fma(FLIP ? -cf : cf, x[q], acc[q]);
      }
    }
  }
}

// term_sum in the reference's arithmetic, whatever the translation unit's
// contraction setting: every product and sum rounds on its own, as the
// oracle's -ffp-contract=off build and the Fortran do.  The auto-reduction
// decisions and AutoReduce_1stOrder read P_VAR/D_VAR through this form, so
// the fast kernel freezes exactly the species the reference freezes.
template <int NC>
__device__ __forceinline__ void term_sum_exact(const MechDev& m, const unsigned* __restrict__ terms, int s, int e,
                                               const double* __restrict__ X, double* acc) {
  constexpr int TSN = TS * NC;
#pragma unroll
  for (int q = 0; q < NC; ++q) acc[q] = 0.0;
  for (int i = s; i < e; ++i) {
    const unsigned t = ldu(terms + i);
    const double cf = __ldg(m.slit + (t >> 20));
    const double* xp = X + (t & 0xfffffu) * TSN;
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      const double v = __dmul_rn(cf, ldw(xp + q * TS));
      acc[q] = (i == s) ? v : __dadd_rn(acc[q], v);
    }
  }
}

// B(b): the partial-derivative products of Jac_SP, which are also the
// D_VAR products of Fun_SPLIT (same factor lists, same order).
template <int NC>
__device__ __forceinline__ void b_products(const MechDev& m, const double* __restrict__ Y,
                                           const double* __restrict__ aux, double* __restrict__ B) {
  products_by_class<NC>(m, m.prod_ids_b, m.b_cls, m.nreact, Y, aux, B);
}

// Fun_SPLIT: Vdot = P_VAR - D_VAR*V at point Y = [V | F] (aux = RCT).
// B must hold the B products at Y (b_products).  With PD, P_VAR and D_VAR
// are stored too (Fun_SPLITF, gckpp_Function.F90:5081-7260: the same
// statements), always in the reference's arithmetic (term_sum_exact); Vdot
// keeps the variant's own arithmetic, so that it equals the Vdot of a call
// without PD bit for bit.
template <bool STRICT, int NC, bool PD = false>
__device__ void fun_split(const MechDev& m, const double* __restrict__ V, const double* __restrict__ aux,
                          double* __restrict__ A, const double* __restrict__ B, double* __restrict__ Vdot,
                          double* __restrict__ P = nullptr, double* __restrict__ D = nullptr) {
  constexpr int TSN = TS * NC;
  products_by_class<NC>(m, m.prod_ids_a, m.a_cls, 0, V, aux, A);
  for (int i = 0; i < m.nvar; ++i) {
    double p[NC], d[NC];
    term_sum<STRICT, false, NC>(m, m.p_sterm, ldi(m.p_start + i), ldi(m.p_start + i + 1), A, p);
    term_sum<STRICT, false, NC>(m, m.d_sterm, ldi(m.d_start + i), ldi(m.d_start + i + 1), B, d);
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      const double v = V[i * TSN + q * TS];
      Vdot[i * TSN + q * TS] = STRICT ? p[q] - d[q] * v : fma(-d[q], v, p[q]);
      if (PD && STRICT) {
        P[i * TSN + q * TS] = p[q];
        D[i * TSN + q * TS] = d[q];
      }
    }
    if (PD && !STRICT) {
      term_sum_exact<NC>(m, m.p_sterm, ldi(m.p_start + i), ldi(m.p_start + i + 1), A, p);
      term_sum_exact<NC>(m, m.d_sterm, ldi(m.d_start + i), ldi(m.d_start + i + 1), B, d);
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        P[i * TSN + q * TS] = p[q];
        D[i * TSN + q * TS] = d[q];
      }
    }
  }
}

// Jac_SP: JVS in LU order from the B products.  STRICT stores JVS; the fast
// form stores -JVS (what ros_PrepareMatrix needs).
template <bool STRICT, int NC>
__device__ void jac_sp(const MechDev& m, const double* __restrict__ B, double* __restrict__ J) {
  constexpr int TSN = TS * NC;
  for (int k = 0; k < m.lu_nonzero; ++k) {
    double v[NC];
    term_sum<STRICT, !STRICT, NC>(m, m.j_sterm, ldi(m.j_start + k), ldi(m.j_start + k + 1), B, v);
#pragma unroll
    for (int q = 0; q < NC; ++q) J[k * TSN + q * TS] = v[q];
  }
}

// Singular check of KppDecomp (gckpp_LinearAlgebra.F90:61-66): each row's
// diagonal is tested at the start of that row, and rows are only modified in
// their own iteration, so the test runs up front on Ghimj's diagonal.
// ier[q] = 0 or the 1-based first row whose diagonal is below TINY.
template <bool STRICT, int NC>
__device__ __forceinline__ void singular_rows(const MechDev& m, const double* __restrict__ J0, const double* ghinv,
                                              int* ier) {
  constexpr int TSN = TS * NC;
#pragma unroll
  for (int q = 0; q < NC; ++q) ier[q] = 0;
  for (int i = 0; i < m.nvar; ++i) {
    const int d = ldi(m.lu_diag + i);
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      const double j = ldw(J0 + d * TSN + q * TS);
      const double g = (STRICT ? -j : j) + ghinv[q];
      if (ier[q] == 0 && tiny_abs(g)) ier[q] = i + 1;
    }
  }
}

// Ghimj = -Jac0 + diag(ghinv), then KppDecomp in place, in KppDecomp's own
// right-looking order (W(c) updated in memory for each L entry of a row).
template <bool STRICT, int NC>
__device__ void decomp(const MechDev& m, const double* __restrict__ J0, const double* ghinv, double* __restrict__ G,
                       int* ier) {
  constexpr int TSN = TS * NC;
  singular_rows<STRICT, NC>(m, J0, ghinv, ier);
  for (int e = 0; e < m.lu_nonzero; ++e)
#pragma unroll
    for (int q = 0; q < NC; ++q) G[e * TSN + q * TS] = STRICT ? -J0[e * TSN + q * TS] : J0[e * TSN + q * TS];
  for (int i = 0; i < m.nvar; ++i) {
    const int d = ldi(m.lu_diag + i);
#pragma unroll
    for (int q = 0; q < NC; ++q) G[d * TSN + q * TS] = G[d * TSN + q * TS] + ghinv[q];
  }
  for (int k = 0; k < m.nvar; ++k) {
    const int l0 = ldi(m.lrow_start + k), l1 = ldi(m.lrow_start + k + 1);
    for (int l = l0; l < l1; ++l) {
      const int kk = ldi(m.lop_kk + l), dj = ldi(m.lop_dj + l);
      const int u0 = ldi(m.lop_u + l), u1 = ldi(m.lop_u + l + 1);
      double a[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        if (STRICT) {
          a[q] = -G[kk * TSN + q * TS] / G[dj * TSN + q * TS];
          G[kk * TSN + q * TS] = -a[q];
        } else {
          const double v = G[kk * TSN + q * TS] * G[dj * TSN + q * TS];  // diag j holds 1/pivot
          G[kk * TSN + q * TS] = v;
          a[q] = -v;
        }
      }
      for (int u = u0; u < u1; ++u) {
        const unsigned op = ldu(m.uop + u);
        const int t = static_cast<int>(op >> 16) * TSN, s = static_cast<int>(op & 0xffffu) * TSN;
#pragma unroll
        for (int q = 0; q < NC; ++q) {
          if (STRICT) G[t + q * TS] = G[t + q * TS] + a[q] * G[s + q * TS];
          else G[t + q * TS] = fma(a[q], G[s + q * TS], G[t + q * TS]);
        }
      }
    }
    if (!STRICT) {
      const int d = ldi(m.lu_diag + k);
#pragma unroll
      for (int q = 0; q < NC; ++q) G[d * TSN + q * TS] = 1.0 / G[d * TSN + q * TS];
    }
  }
}

// acc -= sum of L(k,j)*U(j,c) over the dot-product terms of LU entry e, in
// the table's order.
template <bool STRICT, int NC>
__device__ __forceinline__ void dot_terms(const MechDev& m, const double* __restrict__ G, int e, double* acc) {
  constexpr int TSN = TS * NC;
  const int t0 = ldi(m.dot_start + e), t1 = ldi(m.dot_start + e + 1);
#pragma unroll 4
  for (int t = t0; t < t1; ++t) {
    const unsigned op = ldu(m.dot_term + t);
    const double* lp = G + (op >> 16) * TSN;
    const double* up = G + (op & 0xffffu) * TSN;
    double l[NC], u[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      l[q] = ldw(lp + q * TS);
      u[q] = ldw(up + q * TS);
    }
#pragma unroll
    for (int q = 0; q < NC; ++q) acc[q] = STRICT ? acc[q] - l[q] * u[q] : fma(-l[q], u[q], acc[q]);
  }
}

// The same factorization, with every entry (k,c) of row k computed as one
// accumulation in a register:  W(c) = Ghimj(k,c) - sum_j L(k,j)*U(j,c) over
// the L entries j < c of row k in ascending order -- the updates KppDecomp
// applies to W(c), in the same order, so STRICT stays bit-for-bit.  Each
// entry is loaded from Jac0 and stored once, and Ghimj is never stored.  A
// row runs as three loops -- its L entries (divided by, or in the fast form
// multiplied by the reciprocal of, their pivot), its diagonal (+ 1/(H gamma);
// the fast form stores the reciprocal) and its U entries -- so that no entry
// executes another part's arithmetic under a predicate.
template <bool STRICT, int NC>
__device__ void decomp_rows(const MechDev& m, const double* __restrict__ J0, const double* ghinv,
                            double* __restrict__ G, int* ier) {
  constexpr int TSN = TS * NC;
  singular_rows<STRICT, NC>(m, J0, ghinv, ier);
  for (int k = 0; k < m.nvar; ++k) {
    const int e0 = ldi(m.lu_crow + k), e1 = ldi(m.lu_crow + k + 1), dk = ldi(m.lu_diag + k);
    for (int e = e0; e < dk; ++e) {
      double acc[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        const double j = ldw(J0 + e * TSN + q * TS);
        acc[q] = STRICT ? -j : j;
      }
      dot_terms<STRICT, NC>(m, G, e, acc);
      const double* pv = G + ldi(m.lu_diag + ldi(m.lu_icol + e)) * TSN;
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        const double piv = ldw(pv + q * TS);
        G[e * TSN + q * TS] = STRICT ? acc[q] / piv : acc[q] * piv;  // fast: diag holds 1/pivot
      }
    }
    {
      double acc[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        const double j = ldw(J0 + dk * TSN + q * TS);
        acc[q] = (STRICT ? -j : j) + ghinv[q];
      }
      dot_terms<STRICT, NC>(m, G, dk, acc);
#pragma unroll
      for (int q = 0; q < NC; ++q) G[dk * TSN + q * TS] = STRICT ? acc[q] : 1.0 / acc[q];
    }
    for (int e = dk + 1; e < e1; ++e) {
      double acc[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        const double j = ldw(J0 + e * TSN + q * TS);
        acc[q] = STRICT ? -j : j;
      }
      dot_terms<STRICT, NC>(m, G, e, acc);
#pragma unroll
      for (int q = 0; q < NC; ++q) G[e * TSN + q * TS] = acc[q];
    }
  }
}

// KppSolve: forward (L, unit diagonal) then backward (U) substitution.
template <bool STRICT, int NC>
__device__ void solve(const MechDev& m, const double* __restrict__ G, double* __restrict__ X) {
  constexpr int TSN = TS * NC;
  for (int i = 0; i < m.nvar; ++i) {
    const int s = ldi(m.lu_crow + i), d = ldi(m.lu_diag + i);
    if (s < d) {
      double x[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q) x[q] = X[i * TSN + q * TS];
#pragma unroll 4
      for (int kk = s; kk < d; ++kk) {
        const double* gp = G + kk * TSN;
        const double* yp = X + ldi(m.lu_icol + kk) * TSN;
        double g[NC], y[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) {
          g[q] = ldw(gp + q * TS);
          y[q] = ldw(yp + q * TS);
        }
#pragma unroll
        for (int q = 0; q < NC; ++q) x[q] = STRICT ? x[q] - g[q] * y[q] : fma(-g[q], y[q], x[q]);
      }
#pragma unroll
      for (int q = 0; q < NC; ++q) X[i * TSN + q * TS] = x[q];
    }
  }
  for (int i = m.nvar - 1; i >= 0; --i) {
    const int d = ldi(m.lu_diag + i), e = ldi(m.lu_crow + i + 1);
    double x[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) x[q] = X[i * TSN + q * TS];
#pragma unroll 4
    for (int kk = d + 1; kk < e; ++kk) {
      const double* gp = G + kk * TSN;
      const double* yp = X + ldi(m.lu_icol + kk) * TSN;
      double g[NC], y[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        g[q] = ldw(gp + q * TS);
        y[q] = ldw(yp + q * TS);
      }
#pragma unroll
      for (int q = 0; q < NC; ++q) x[q] = STRICT ? x[q] - g[q] * y[q] : fma(-g[q], y[q], x[q]);
    }
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      const double piv = ldw(G + d * TSN + q * TS);
      X[i * TSN + q * TS] = STRICT ? x[q] / piv : x[q] * piv;
    }
  }
}

}  // namespace gckpp
