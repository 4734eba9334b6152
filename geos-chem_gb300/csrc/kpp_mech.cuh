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
  const int* prod_start;
  const int* prod_fac;
  const int* p_start;
  const unsigned* p_term;
  const int* d_start;
  const unsigned* d_term;
  const int* j_start;
  const unsigned* j_term;
  const int* lu_crow;
  const int* lu_diag;
  const int* lu_icol;
  const int* lrow_start;
  const int* lop_kk;
  const int* lop_dj;
  const int* lop_u;
  const unsigned* uop;
  const double* lit;
};

constexpr unsigned NOCOEF = 0x7ffu;

__device__ __forceinline__ int ldi(const int* p) { return __ldg(p); }
__device__ __forceinline__ unsigned ldu(const unsigned* p) { return __ldg(p); }

// |x| < TINY(1.0_dp), on the bit pattern
__device__ __forceinline__ bool tiny_abs(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffULL) <
         0x0010000000000000ULL;
}

__device__ __forceinline__ double operand(const MechDev& m, int code, const double* V, const double* aux) {
  if (code < m.nvar) return V[code * TS];
  if (code < m.lit0) return aux[(code - m.nvar) * TS];
  return __ldg(m.lit + (code - m.lit0));
}

// Left-to-right product of a factor list (Fortran evaluation order).
__device__ __forceinline__ double product(const MechDev& m, int p, const double* V, const double* aux) {
  const int s = ldi(m.prod_start + p), e = ldi(m.prod_start + p + 1);
  double acc = operand(m, ldi(m.prod_fac + s), V, aux);
  for (int i = s + 1; i < e; ++i) acc = acc * operand(m, ldi(m.prod_fac + i), V, aux);
  return acc;
}

// Signed sum of [coef*]X(idx) terms; FLIP negates every term (exact).
template <bool STRICT, bool FLIP>
__device__ __forceinline__ double coef_sum(const MechDev& m, const unsigned* terms, int s, int e, const double* X) {
  if (s == e) return 0.0;
  double acc;
  {
    const unsigned t = ldu(terms + s);
    const unsigned c = (t >> 20) & 0x7ffu;
    const double x = X[(t & 0xfffffu) * TS];
    const double v = (c == NOCOEF) ? x : __ldg(m.lit + c) * x;
    const bool neg = ((t >> 31) != 0) != FLIP;
    acc = neg ? -v : v;
  }
  for (int i = s + 1; i < e; ++i) {
    const unsigned t = ldu(terms + i);
    const unsigned c = (t >> 20) & 0x7ffu;
    const double x = X[(t & 0xfffffu) * TS];
    const bool neg = ((t >> 31) != 0) != FLIP;
    if (STRICT) {
      const double v = (c == NOCOEF) ? x : __ldg(m.lit + c) * x;
      acc = neg ? acc - v : acc + v;
    } else {
      if (c == NOCOEF) {
        acc = neg ? acc - x : acc + x;
      } else {
        const double cf = __ldg(m.lit + c);
        acc = fma(neg ? -cf : cf, x, acc);
      }
    }
  }
  return acc;
}

// Sum of signed B products (D_VAR of Fun_SPLIT).  With Bv the products are
// read from an earlier Jacobian evaluation at the same point.
template <bool STRICT>
__device__ __forceinline__ double dsum(const MechDev& m, int s, int e, const double* V, const double* aux,
                                       const double* Bv) {
  if (s == e) return 0.0;
  double acc = 0.0;
  for (int i = s; i < e; ++i) {
    const unsigned t = ldu(m.d_term + i);
    const int b = static_cast<int>(t & 0xfffffu);
    const double v = Bv ? Bv[b * TS] : product(m, m.nreact + b, V, aux);
    const bool neg = (t >> 31) != 0;
    if (i == s) acc = neg ? -v : v;
    else acc = neg ? acc - v : acc + v;
  }
  return acc;
}

// Fun_SPLIT: Vdot = P_VAR - D_VAR*V at point V (aux = [F, RCT]).
template <bool STRICT>
__device__ void fun_split(const MechDev& m, const double* __restrict__ V, const double* __restrict__ aux,
                          double* __restrict__ A, const double* __restrict__ Bv, double* __restrict__ Vdot) {
#pragma unroll 2
  for (int r = 0; r < m.nreact; ++r) A[r * TS] = product(m, r, V, aux);
  for (int i = 0; i < m.nvar; ++i) {
    const double p = coef_sum<STRICT, false>(m, m.p_term, ldi(m.p_start + i), ldi(m.p_start + i + 1), A);
    const double d = dsum<STRICT>(m, ldi(m.d_start + i), ldi(m.d_start + i + 1), V, aux, Bv);
    const double v = V[i * TS];
    Vdot[i * TS] = STRICT ? p - d * v : fma(-d, v, p);
  }
}

// Jac_SP: B partials then JVS in LU order.  STRICT stores JVS; the fast form
// stores -JVS (what ros_PrepareMatrix needs).
template <bool STRICT>
__device__ void jac_sp(const MechDev& m, const double* __restrict__ V, const double* __restrict__ aux,
                       double* __restrict__ B, double* __restrict__ J) {
  for (int b = 0; b < m.nb; ++b) {
    const int p = m.nreact + b;
    if (ldi(m.prod_start + p + 1) > ldi(m.prod_start + p)) B[b * TS] = product(m, p, V, aux);
  }
  for (int k = 0; k < m.lu_nonzero; ++k)
    J[k * TS] = coef_sum<STRICT, !STRICT>(m, m.j_term, ldi(m.j_start + k), ldi(m.j_start + k + 1), B);
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

// KppSolve: forward (L, unit diagonal) then backward (U) substitution.
template <bool STRICT>
__device__ void solve(const MechDev& m, const double* __restrict__ G, double* __restrict__ X) {
  for (int i = 0; i < m.nvar; ++i) {
    const int s = ldi(m.lu_crow + i), d = ldi(m.lu_diag + i);
    if (s < d) {
      double x = X[i * TS];
#pragma unroll 4
      for (int kk = s; kk < d; ++kk) {
        const double g = G[kk * TS], y = X[ldi(m.lu_icol + kk) * TS];
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
      const double g = G[kk * TS], y = X[ldi(m.lu_icol + kk) * TS];
      x = STRICT ? x - g * y : fma(-g, y, x);
    }
    X[i * TS] = STRICT ? x / G[d * TS] : x * G[d * TS];
  }
}

}  // namespace gckpp
