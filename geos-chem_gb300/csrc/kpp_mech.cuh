// Table-driven per-cell mechanism engine: Fun_SPLIT, Jac_SP, KppDecomp
// (fused with ros_PrepareMatrix) and KppSolve for one cell per thread.
//
// Every lane of a warp executes the same table entry for its own cell, so
// table reads are warp-uniform broadcasts and the per-cell reads/writes are
// coalesced: a lane's entry e lives at p[e * TS] in its warp's tile.
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

constexpr int TS = 32;  // lanes per tile

struct MechDev {
  int nvar, nfix, nreact, nspec, lu_nonzero, nb, lit0;
  const uint2* prod_packed;  // pre | times2<<12 | nspecies<<13 | s1<<16, s2 | s3<<16
  const double* pre_lit;     // constant-rate literals, appended to RCT in aux
  int naux;
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
};


__device__ __forceinline__ int ldi(const int* p) { return __ldg(p); }

// Per-cell workspace read.  With GCKPP_LDCG the read bypasses L1 (the tables
// then keep L1 to themselves); otherwise it is an ordinary cached load.
__device__ __forceinline__ double ldw(const double* p) {
#if defined(GCKPP_LDCG) && GCKPP_LDCG
  return __ldcg(p);
#else
  return *p;
#endif
}
__device__ __forceinline__ unsigned ldu(const unsigned* p) { return __ldg(p); }

// |x| < TINY(1.0_dp), on the bit pattern
__device__ __forceinline__ bool tiny_abs(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffULL) <
         0x0010000000000000ULL;
}

// One product of the mechanism, pre [* 2] * s1 * s2 * s3, in the Fortran's
// left-to-right order.  aux holds RCT (and the constant-rate literals), Y the
// species [V | F].  The species loads are issued unconditionally so that the
// loads of consecutive products overlap.
__device__ __forceinline__ double product(const MechDev& m, int p, const double* Y, const double* aux) {
  const uint2 t = __ldg(m.prod_packed + p);
  double a = ldw(aux + (t.x & 0xfffu) * TS);
  const unsigned ns = (t.x >> 13) & 3u;
  const double v1 = ldw(Y + (t.x >> 16) * TS), v2 = ldw(Y + (t.y & 0xffffu) * TS), v3 = ldw(Y + (t.y >> 16) * TS);
  if (t.x & 0x1000u) a = a * 2.0;
  if (ns >= 1u) a = a * v1;
  if (ns >= 2u) a = a * v2;
  if (ns >= 3u) a = a * v3;
  return a;
}

// Sum of signed terms  slit[c] * X[idx]  (sterm = c << 20 | idx) in the
// reference's left-to-right order.  The sign is folded into the coefficient
// (a bare X(idx) is +/-1.0 * X(idx), exact), so the loop has no branch and
// consecutive terms' loads overlap.  FLIP negates the sum (exact).
template <bool STRICT, bool FLIP>
__device__ __forceinline__ double term_sum(const MechDev& m, const unsigned* __restrict__ terms, int s, int e,
                                           const double* __restrict__ X) {
  double acc = 0.0;
#pragma unroll 4
  for (int i = s; i < e; ++i) {
    const unsigned t = ldu(terms + i);
    const double cf = __ldg(m.slit + (t >> 20));
    const double x = ldw(X + (t & 0xfffffu) * TS);
    if (STRICT) {
      const double v = cf * x;
      acc = (i == s) ? (FLIP ? -v : v) : (FLIP ? acc - v : acc + v);
    } else {
      acc = fma(FLIP ? -cf : cf, x, acc);
    }
  }
  return acc;
}

// B(b): the partial-derivative products of Jac_SP, which are also the
// D_VAR products of Fun_SPLIT (same factor lists, same order).
__device__ __forceinline__ void b_products(const MechDev& m, const double* __restrict__ Y,
                                           const double* __restrict__ aux, double* __restrict__ B) {
#pragma unroll 4
  for (int b = 0; b < m.nb; ++b) B[b * TS] = product(m, m.nreact + b, Y, aux);
}

// Fun_SPLIT: Vdot = P_VAR - D_VAR*V at point Y = [V | F] (aux = RCT).
// B must hold the B products at Y (b_products).
template <bool STRICT>
__device__ void fun_split(const MechDev& m, const double* __restrict__ V, const double* __restrict__ aux,
                          double* __restrict__ A, const double* __restrict__ B, double* __restrict__ Vdot) {
#pragma unroll 4
  for (int r = 0; r < m.nreact; ++r) A[r * TS] = product(m, r, V, aux);
  for (int i = 0; i < m.nvar; ++i) {
    const double p = term_sum<STRICT, false>(m, m.p_sterm, ldi(m.p_start + i), ldi(m.p_start + i + 1), A);
    const double d = term_sum<STRICT, false>(m, m.d_sterm, ldi(m.d_start + i), ldi(m.d_start + i + 1), B);
    const double v = V[i * TS];
    Vdot[i * TS] = STRICT ? p - d * v : fma(-d, v, p);
  }
}

// Jac_SP: JVS in LU order from the B products.  STRICT stores JVS; the fast
// form stores -JVS (what ros_PrepareMatrix needs).
template <bool STRICT>
__device__ void jac_sp(const MechDev& m, const double* __restrict__ B, double* __restrict__ J) {
  for (int k = 0; k < m.lu_nonzero; ++k)
    J[k * TS] = term_sum<STRICT, !STRICT>(m, m.j_sterm, ldi(m.j_start + k), ldi(m.j_start + k + 1), B);
}

// Ghimj = -Jac0 + diag(ghinv), then KppDecomp in place.  Returns 0 or the
// 1-based row whose diagonal was below TINY before elimination (KppDecomp
// checks each row's diagonal at the start of that row, and rows are only
// modified in their own iteration, so the check can run up front).
template <bool STRICT>
__device__ int decomp(const MechDev& m, const double* __restrict__ J0, double ghinv, double* __restrict__ G) {
#pragma unroll 8
  for (int e = 0; e < m.lu_nonzero; ++e) G[e * TS] = STRICT ? -J0[e * TS] : J0[e * TS];
  int ier = 0;
  for (int i = 0; i < m.nvar; ++i) {
    const int d = ldi(m.lu_diag + i);
    const double g = G[d * TS] + ghinv;
    G[d * TS] = g;
    if (ier == 0 && tiny_abs(g)) ier = i + 1;
  }
  if (ier) return ier;
  for (int k = 0; k < m.nvar; ++k) {
    const int l0 = ldi(m.lrow_start + k), l1 = ldi(m.lrow_start + k + 1);
    for (int l = l0; l < l1; ++l) {
      const int kk = ldi(m.lop_kk + l), dj = ldi(m.lop_dj + l);
      const int u0 = ldi(m.lop_u + l), u1 = ldi(m.lop_u + l + 1);
      double a;
      if (STRICT) {
        a = -G[kk * TS] / G[dj * TS];
        G[kk * TS] = -a;
      } else {
        a = G[kk * TS] * G[dj * TS];  // diag j holds 1/pivot
        G[kk * TS] = a;
        a = -a;
      }
#pragma unroll 4
      for (int u = u0; u < u1; ++u) {
        const unsigned op = ldu(m.uop + u);
        const int t = static_cast<int>(op >> 16), s = static_cast<int>(op & 0xffffu);
        if (STRICT) G[t * TS] = G[t * TS] + a * G[s * TS];
        else G[t * TS] = fma(a, G[s * TS], G[t * TS]);
      }
    }
    if (!STRICT) {
      const int d = ldi(m.lu_diag + k);
      G[d * TS] = 1.0 / G[d * TS];
    }
  }
  return 0;
}

// The same factorization, with every entry (k,c) of row k computed as one
// accumulation in a register:  W(c) = Ghimj(k,c) - sum_j L(k,j)*U(j,c) over
// the L entries j < c of row k in ascending order -- the updates KppDecomp
// applies to W(c), in the same order, so STRICT stays bit-for-bit.  Each
// entry is loaded from Jac0 and stored once (no read-modify-write of the
// row in memory), and Ghimj is never materialised.
template <bool STRICT>
__device__ int decomp_rows(const MechDev& m, const double* __restrict__ J0, double ghinv, double* __restrict__ G) {
  for (int i = 0; i < m.nvar; ++i) {
    const int d = ldi(m.lu_diag + i);
    const double g = (STRICT ? -J0[d * TS] : J0[d * TS]) + ghinv;
    if (tiny_abs(g)) return i + 1;
  }
  for (int k = 0; k < m.nvar; ++k) {
    const int e0 = ldi(m.lu_crow + k), e1 = ldi(m.lu_crow + k + 1), dk = ldi(m.lu_diag + k);
    for (int e = e0; e < e1; ++e) {
      double acc = STRICT ? -ldw(J0 + e * TS) : ldw(J0 + e * TS);
      if (e == dk) acc = acc + ghinv;
      const int t0 = ldi(m.dot_start + e), t1 = ldi(m.dot_start + e + 1);
#pragma unroll 4
      for (int t = t0; t < t1; ++t) {
        const unsigned op = ldu(m.dot_term + t);
        const double l = ldw(G + (op >> 16) * TS), u = ldw(G + (op & 0xffffu) * TS);
        acc = STRICT ? acc - l * u : fma(-l, u, acc);
      }
      if (e < dk) {
        const int dc = ldi(m.lu_diag + ldi(m.lu_icol + e));
        acc = STRICT ? acc / ldw(G + dc * TS) : acc * ldw(G + dc * TS);  // fast: diag holds 1/pivot
      } else if (e == dk && !STRICT) {
        acc = 1.0 / acc;
      }
      G[e * TS] = acc;
    }
  }
  return 0;
}

// KppSolve: forward (L, unit diagonal) then backward (U) substitution.
template <bool STRICT>
__device__ void solve(const MechDev& m, const double* __restrict__ G, double* __restrict__ X) {
  for (int i = 0; i < m.nvar; ++i) {
    const int s = ldi(m.lu_crow + i), d = ldi(m.lu_diag + i);
    if (s < d) {
      double x = X[i * TS];
#pragma unroll 4
      for (int kk = s; kk < d; ++kk) {
        const double g = ldw(G + kk * TS), y = ldw(X + ldi(m.lu_icol + kk) * TS);
        x = STRICT ? x - g * y : fma(-g, y, x);
      }
      X[i * TS] = x;
    }
  }
  for (int i = m.nvar - 1; i >= 0; --i) {
    const int d = ldi(m.lu_diag + i), e = ldi(m.lu_crow + i + 1);
    double x = X[i * TS];
#pragma unroll 4
    for (int kk = d + 1; kk < e; ++kk) {
      const double g = ldw(G + kk * TS), y = ldw(X + ldi(m.lu_icol + kk) * TS);
      x = STRICT ? x - g * y : fma(-g, y, x);
    }
    X[i * TS] = STRICT ? x / G[d * TS] : x * G[d * TS];
  }
}

}  // namespace gckpp
