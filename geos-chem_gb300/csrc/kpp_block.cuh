// Block-per-cell Rosenbrock: all threads of one block integrate one cell,
// whose working set (rates, Y, stage vectors, A/B products and the LU
// factors, about 71 KB for Rodas3) sits in shared memory; Jac0, the rate
// constants and the A/B products, which are read in parallel loops off the
// critical path, stay in a per-block global slot (L2-resident).  Three cells
// fit on an SM.
//
// This is the latency form of the solver, for the few stiff cells that need
// tens of steps while most cells need one or two: a thread-per-cell warp
// would run such a cell alone at the end of the launch, with every table
// walk a chain of dependent global loads.  Here the independent items of
// each phase run in parallel (products, Fun_SPLIT rows, Jac_SP entries, the
// stage vectors), and the LU factorization and the two substitutions run in
// dependency levels (tables.py _level_schedules) with a barrier between
// levels.  In this level form every item is evaluated by one thread with
// exactly the operations and order of the thread-per-cell engine
// (kpp_mech.cuh), and the error norm is summed by one thread in species
// order, so both engines give the same numbers for a cell.  A block of 32
// threads is the warp-per-cell layout.  The split form (SPLIT = true, fast
// arithmetic, 256 threads; below) cuts each sum across the lanes of a warp
// segment instead and agrees with the thread-per-cell engine to rounding.
#pragma once
#include <climits>

#include "kpp_rosenbrock.cuh"

namespace gckpp {

// Shared-memory layout of one cell (offsets in doubles) for a method with
// `stages` stages; dFdT only for non-autonomous problems.
struct BlockLayout {
  int y0, y1, fcn0, fcn, dfdt, k, g, e, total;  // shared memory
  int j0, aux, a, b, slot;                      // global slot of the block
};

__host__ __device__ inline BlockLayout block_layout(int naux, int nspec, int nvar, int nreact, int nb, int lunz,
                                                    int stages, int autonomous) {
  BlockLayout l{};
  int o = 0;
  l.y0 = o; o += nspec;
  l.y1 = o; o += nspec;
  l.fcn0 = o; o += nvar;
  l.fcn = o; o += nvar;
  l.dfdt = o; o += autonomous ? 0 : nvar;
  l.k = o; o += stages * nvar;
  l.g = o; o += lunz;
  l.e = o; o += nvar;
  l.total = o;
  o = 0;
  l.j0 = o; o += lunz;
  l.aux = o; o += naux;
  l.a = o; o += nreact;
  l.b = o; o += nb;
  l.slot = o;
  return l;
}

// Sum of signed terms slit[c] * X[idx] (the operations of term_sum<.,.,1>).
template <bool STRICT, bool FLIP>
__device__ __forceinline__ double bk_term_sum(const MechDev& m, const unsigned* __restrict__ terms, int s, int e,
                                              const double* X) {
  double acc = 0.0;
#pragma unroll 4
  for (int i = s; i < e; ++i) {
    const unsigned t = __ldg(terms + i);
    const double cf = __ldg(m.slit + (t >> 20));
    const double x = X[t & 0xfffffu];
    if (STRICT) {
      const double v = cf * x;
      acc = (i == s) ? (FLIP ? -v : v) : (FLIP ? acc - v : acc + v);
    } else {
      acc = fma(FLIP ? -cf : cf, x, acc);
    }
  }
  return acc;
}

// The products of one class (NS species factors, TIMES2) at list positions
// [s, e), spread over the block's threads: out[id] = pre [* 2] * s1 * s2 *
// s3 in the Fortran's left-to-right order (the operations of product_class
// in kpp_mech.cuh) for id = ids[i], product index base + id.
template <int NS, bool TIMES2>
__device__ __forceinline__ void bk_product_class(const MechDev& m, const int* ids, int s, int e, int base,
                                                 const double* Y, const double* aux, double* out) {
  for (int i = s + threadIdx.x; i < e; i += blockDim.x) {
    const int id = __ldg(ids + i);
    const uint2 t = __ldg(m.prod_packed + base + id);
    double r = aux[t.x & 0xfffu];
    if (TIMES2) r = r * 2.0;
    if (NS >= 1) r = r * Y[t.x >> 16];
    if (NS >= 2) r = r * Y[t.y & 0xffffu];
    if (NS >= 3) r = r * Y[t.y >> 16];
    out[id] = r;
  }
}

__device__ __forceinline__ void bk_products_by_class(const MechDev& m, const int* ids, const int* cls, int base,
                                                     const double* Y, const double* aux, double* out) {
  bk_product_class<0, false>(m, ids, cls[0], cls[1], base, Y, aux, out);
  bk_product_class<0, true>(m, ids, cls[1], cls[2], base, Y, aux, out);
  bk_product_class<1, false>(m, ids, cls[2], cls[3], base, Y, aux, out);
  bk_product_class<1, true>(m, ids, cls[3], cls[4], base, Y, aux, out);
  bk_product_class<2, false>(m, ids, cls[4], cls[5], base, Y, aux, out);
  bk_product_class<2, true>(m, ids, cls[5], cls[6], base, Y, aux, out);
  bk_product_class<3, false>(m, ids, cls[6], cls[7], base, Y, aux, out);
  bk_product_class<3, true>(m, ids, cls[7], cls[8], base, Y, aux, out);
}

// B products at Y (Jac_SP partials, also Fun's D_VAR products).
__device__ __forceinline__ void bk_b_products(const MechDev& m, const double* Y, const double* aux, double* B) {
  bk_products_by_class(m, m.prod_ids_b, m.b_cls, m.nreact, Y, aux, B);
}

// Fun_SPLIT at V; B must hold the B products at V and be visible to the
// block.  Ends with a barrier.
template <bool STRICT>
__device__ void bk_fun(const MechDev& m, const double* V, const double* aux, double* A, const double* B,
                       double* Vdot) {
  bk_products_by_class(m, m.prod_ids_a, m.a_cls, 0, V, aux, A);
  __syncthreads();
  for (int n = threadIdx.x; n < m.nvar; n += blockDim.x) {
    const int i = __ldg(m.fun_rows_by_len + n);
    const double p = bk_term_sum<STRICT, false>(m, m.p_sterm, __ldg(m.p_start + i), __ldg(m.p_start + i + 1), A);
    const double d = bk_term_sum<STRICT, false>(m, m.d_sterm, __ldg(m.d_start + i), __ldg(m.d_start + i + 1), B);
    Vdot[i] = STRICT ? p - d * V[i] : fma(-d, V[i], p);
  }
  __syncthreads();
}

// Jac_SP (STRICT stores JVS, the fast form -JVS).  No barrier.
template <bool STRICT>
__device__ void bk_jac(const MechDev& m, const double* B, double* J) {
  for (int n = threadIdx.x; n < m.lu_nonzero; n += blockDim.x) {
    const int e = __ldg(m.jac_by_len + n);
    J[e] = bk_term_sum<STRICT, !STRICT>(m, m.j_sterm, __ldg(m.j_start + e), __ldg(m.j_start + e + 1), B);
  }
}

// Ghimj = -Jac0 + diag(ghinv) and its LU factors (the operations of
// decomp_rows), level by level.  *ier receives the 1-based first row whose
// diagonal is below TINY (0 if none), as singular_rows finds it.  Ends with
// a barrier.
template <bool STRICT>
__device__ void bk_decomp(const MechDev& m, const double* J0, double ghinv, double* G, int* ier) {
  if (threadIdx.x == 0) *ier = INT_MAX;
  __syncthreads();
  for (int i = threadIdx.x; i < m.nvar; i += blockDim.x) {
    const double j = J0[__ldg(m.lu_diag + i)];
    const double g = (STRICT ? -j : j) + ghinv;
    if (tiny_abs(g)) atomicMin(ier, i + 1);
  }
  for (int l = 0; l < m.lu_nlvl; ++l) {
    const int n1 = __ldg(m.lu_lvl_start + l + 1);
    for (int n = __ldg(m.lu_lvl_start + l) + threadIdx.x; n < n1; n += blockDim.x) {
      const int e = __ldg(m.lu_lvl_entry + n);
      const int k = __ldg(m.lu_irow + e);
      const int dk = __ldg(m.lu_diag + k);
      const double j = J0[e];
      double acc = STRICT ? -j : j;
      if (e == dk) acc = acc + ghinv;
      const int t1 = __ldg(m.dot_start + e + 1);
#pragma unroll 4
      for (int t = __ldg(m.dot_start + e); t < t1; ++t) {
        const unsigned op = __ldg(m.dot_term + t);
        const double lv = G[op >> 16];
        const double uv = G[op & 0xffffu];
        acc = STRICT ? acc - lv * uv : fma(-lv, uv, acc);
      }
      if (e < dk) {
        const double piv = G[__ldg(m.lu_diag + __ldg(m.lu_icol + e))];
        acc = STRICT ? acc / piv : acc * piv;  // fast: diag holds 1/pivot
      } else if (e == dk && !STRICT) {
        acc = 1.0 / acc;
      }
      G[e] = acc;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && *ier == INT_MAX) *ier = 0;
  __syncthreads();
}

// KppSolve (the operations of solve), forward then backward, row levels.
// Ends with a barrier.
template <bool STRICT>
__device__ void bk_solve(const MechDev& m, const double* G, double* X) {
  for (int l = 0; l < m.fs_nlvl; ++l) {
    const int n1 = __ldg(m.fs_lvl_start + l + 1);
    for (int n = __ldg(m.fs_lvl_start + l) + threadIdx.x; n < n1; n += blockDim.x) {
      const int i = __ldg(m.fs_lvl_row + n);
      const int s = __ldg(m.lu_crow + i), d = __ldg(m.lu_diag + i);
      if (s < d) {
        double x = X[i];
#pragma unroll 4
        for (int kk = s; kk < d; ++kk) {
          const double g = G[kk];
          const double y = X[__ldg(m.lu_icol + kk)];
          x = STRICT ? x - g * y : fma(-g, y, x);
        }
        X[i] = x;
      }
    }
    __syncthreads();
  }
  for (int l = 0; l < m.bs_nlvl; ++l) {
    const int n1 = __ldg(m.bs_lvl_start + l + 1);
    for (int n = __ldg(m.bs_lvl_start + l) + threadIdx.x; n < n1; n += blockDim.x) {
      const int i = __ldg(m.bs_lvl_row + n);
      const int d = __ldg(m.lu_diag + i), e = __ldg(m.lu_crow + i + 1);
      double x = X[i];
#pragma unroll 4
      for (int kk = d + 1; kk < e; ++kk) {
        const double g = G[kk];
        const double y = X[__ldg(m.lu_icol + kk)];
        x = STRICT ? x - g * y : fma(-g, y, x);
      }
      const double piv = G[d];
      X[i] = STRICT ? x / piv : x * piv;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Split form (fast arithmetic only).  The level-by-level form above keeps
// each sum in one thread, so one long LU dot product or substitution row
// (up to ~260 terms) sets a level's time.  Here every sum is cut into chunks
// of at most SPLIT_MAXCH terms, summed by the lanes of an aligned segment of
// one warp and combined by a shuffle butterfly; the static pass schedule
// (tables.py _split_schedules) says which chunk each lane takes in each pass.
// The next pass's task word and term indices are loaded before the current
// pass computes, so the table reads overlap the arithmetic.  The sums are
// regrouped, so the split form agrees with the thread-per-cell form to
// rounding, not bit for bit.
constexpr int SPLIT_MAXCH = 12;

// Profiling build only (GCKPP_PHASE_CYCLES, build.build_phase_cycles): the
// first thread of each phase adds the phase's clock64 cycles to
// g_phase_cycles[phase] and its calls to g_phase_cycles[8 + phase]; entry 7
// is the whole kernel, per block.  Read by gc_kpp_phase_cycles.
#ifdef GCKPP_PHASE_CYCLES
__device__ unsigned long long g_phase_cycles[16];
#define GCKPP_PHASE_BEGIN() const long long phase_c0_ = clock64()
#define GCKPP_PHASE_END(ph, first)                                                          \
  if (first) {                                                                              \
    atomicAdd(&g_phase_cycles[(ph)], (unsigned long long)(clock64() - phase_c0_));          \
    atomicAdd(&g_phase_cycles[8 + (ph)], 1ull);                                             \
  }
#else
#define GCKPP_PHASE_BEGIN()
#define GCKPP_PHASE_END(ph, first)
#endif

// Each phase is a functor: terms(item) is the term array of the item,
// pre(item, z) a value loaded together with the task of the next pass (it
// may only depend on data that the phase does not change), base(item, z,
// pre) the starting value of the sum, term(...) one multiply-add, and
// finish(item, z, v) stores the item.  z is the task's third word.
//
// LU entry e of Ghimj = -Jac0 + diag(ghinv) (J0 holds -JVS), L entries times
// the reciprocal pivot (z = its position), the diagonal stored inverted
// (z = SPLIT_DIAG), U entries as they are (z = SPLIT_UPPER).
constexpr unsigned SPLIT_DIAG = 0xffffffffu, SPLIT_UPPER = 0xfffffffeu;

struct SplitLu {
  const MechDev& m;
  const double* J0;
  double ghinv;
  double* G;
  __device__ const unsigned* terms(int) const { return m.dot_term; }
  __device__ double pre(int e, unsigned) const { return J0[e]; }
  __device__ double base(int, unsigned z, double j) const { return z == SPLIT_DIAG ? j + ghinv : j; }
  __device__ double term(int, int, unsigned w, double acc) const { return fma(-G[w >> 16], G[w & 0xffffu], acc); }
  __device__ void finish(int e, unsigned z, double v) const {
    if (z == SPLIT_DIAG)
      v = 1.0 / v;
    else if (z != SPLIT_UPPER)
      v = v * G[z];
    G[e] = v;
  }
};

// Fun_SPLIT sums: items [0, NVAR) are P_VAR rows over A (into Vdot), items
// [NVAR, 2 NVAR) D_VAR rows over B (into D).
struct SplitFun {
  const MechDev& m;
  const double* A;
  const double* B;
  double* Vdot;
  double* D;
  __device__ const unsigned* terms(int item) const { return item < m.nvar ? m.p_sterm : m.d_sterm; }
  __device__ double pre(int, unsigned) const { return 0.0; }
  __device__ double base(int, unsigned, double) const { return 0.0; }
  __device__ double term(int item, int, unsigned w, double acc) const {
    const double* X = item < m.nvar ? A : B;
    return fma(__ldg(m.slit + (w >> 20)), X[w & 0xfffffu], acc);
  }
  __device__ void finish(int item, unsigned, double v) const {
    if (item < m.nvar)
      Vdot[item] = v;
    else
      D[item - m.nvar] = v;
  }
};

// Jac_SP entries, stored negated (-JVS) as the fast form keeps them.
struct SplitJac {
  const MechDev& m;
  const double* B;
  double* J;
  __device__ const unsigned* terms(int) const { return m.j_sterm; }
  __device__ double pre(int, unsigned) const { return 0.0; }
  __device__ double base(int, unsigned, double) const { return 0.0; }
  __device__ double term(int, int, unsigned w, double acc) const {
    return fma(-__ldg(m.slit + (w >> 20)), B[w & 0xfffffu], acc);
  }
  __device__ void finish(int e, unsigned, double v) const { J[e] = v; }
};

// Task of one lane in one pass: x = item | seglog << 16 | nterms << 19,
// y = first term, z = the phase's finish word, w = the warp's bounds (1 if
// any lane has an item | longest chunk << 1 | widest seglog << 5); item
// 0xFFFF is an idle lane.
// With it travel the lane's term words, the functor's pre value and the
// pass word.
struct SplitTask {
  uint4 t;
  double pre;
  unsigned info;
  unsigned w[SPLIT_MAXCH];
};

// Loads the term words and pre value of s.t (whose task word is known).
template <class PH>
__device__ __forceinline__ void split_terms(const PH& f, SplitTask& s) {
  const int item = s.t.x & 0xffff;
  const int n = (s.t.x >> 19) & 31;
  const unsigned* t = f.terms(item) + s.t.y;
#pragma unroll
  for (int k = 0; k < SPLIT_MAXCH; ++k) s.w[k] = k < n ? __ldg(t + k) : 0u;
  s.pre = item != 0xffff ? f.pre(item, s.t.z) : 0.0;
}

// Runs the passes of one phase on the first sp_nt[ph] threads (32 or the
// whole block; the host checks this).  A pass whose word has bit 3 set ends
// with a barrier over those threads.  The caller adds the block barrier when
// the phase used fewer threads than the block.  Loads run two passes ahead
// for the task word and one pass ahead for what it points to, so a pass
// waits on no chain of dependent loads.
template <class PH>
__device__ __forceinline__ void split_run(const MechDev& m, int ph, const PH& f) {
  const int nt = m.sp_nt[ph];
  const int np = m.sp_npass[ph];
  const int tid = threadIdx.x;
  if (tid >= nt || np == 0) return;
  GCKPP_PHASE_BEGIN();
  const uint4* task = m.sp_task[ph];
  const unsigned* pw = m.sp_pass[ph];
  const uint4 idle = make_uint4(0xffffu, 0u, 0u, 0u);
  SplitTask cur, nxt;
  cur.t = __ldg(task + tid);
  uint4 ahead = np > 1 ? __ldg(task + nt + tid) : idle;
  split_terms(f, cur);
  cur.info = __ldg(pw);
  for (int p = 0; p < np; ++p) {
    nxt.t = ahead;
    ahead = p + 2 < np ? __ldg(task + (p + 2) * nt + tid) : idle;
    split_terms(f, nxt);
    nxt.info = p + 1 < np ? __ldg(pw + p + 1) : 0u;
    const int item = cur.t.x & 0xffff;
    const bool busy = item != 0xffff;
    const int seglog = busy ? (cur.t.x >> 16) & 7 : 0;
    const int seg = 1 << seglog;
    const int n = (cur.t.x >> 19) & 31;
    // A warp runs as many multiply-adds as its longest chunk and as many
    // butterfly levels as its widest segment; a warp with no item in this
    // pass issues no arithmetic (predicated-off FP64 instructions still
    // take the SM's FP64 pipe).  The schedule stores these warp-uniform
    // bounds in the task's fourth word.
    if (cur.t.w & 1u) {
      const int nmax = (cur.t.w >> 1) & 15;
      const int lmax = (cur.t.w >> 5) & 7;
      const bool lead = busy && (tid & (seg - 1)) == 0;
      double acc = lead ? f.base(item, cur.t.z, cur.pre) : 0.0;
#pragma unroll
      for (int k = 0; k < SPLIT_MAXCH; ++k) {
        if (k >= nmax) break;
        if (k < n) acc = f.term(item, (int)cur.t.y + k, cur.w[k], acc);
      }
      for (int o = (1 << lmax) >> 1; o > 0; o >>= 1) {
        const double v = __shfl_xor_sync(0xffffffffu, acc, o);
        if (o < seg) acc += v;
      }
      if (lead) f.finish(item, cur.t.z, acc);
    }
    if (cur.info & 8u) {
      if (nt == 32)
        __syncwarp();
      else
        __syncthreads();
    }
    cur = nxt;
  }
  GCKPP_PHASE_END(ph, tid == 0)
}

// Fun_SPLIT at V in the split form; B must hold the B products at V.  D is a
// scratch vector of NVAR.  Ends with a barrier.
__device__ inline void bk_fun_split(const MechDev& m, const double* V, const double* aux, double* A, const double* B,
                             double* Vdot, double* D) {
  bk_products_by_class(m, m.prod_ids_a, m.a_cls, 0, V, aux, A);
  __syncthreads();
  split_run(m, SP_FUN, SplitFun{m, A, B, Vdot, D});
  if (m.sp_nt[SP_FUN] < (int)blockDim.x) __syncthreads();
  for (int i = threadIdx.x; i < m.nvar; i += blockDim.x) Vdot[i] = fma(-D[i], V[i], Vdot[i]);
  __syncthreads();
}

// Singular check and LU factors in the split form.  Ends with a barrier.
__device__ inline void bk_decomp_split(const MechDev& m, const double* J0, double ghinv, double* G, int* ier) {
  if (threadIdx.x == 0) *ier = INT_MAX;
  __syncthreads();
  for (int i = threadIdx.x; i < m.nvar; i += blockDim.x) {
    const double g = J0[__ldg(m.lu_diag + i)] + ghinv;
    if (tiny_abs(g)) atomicMin(ier, i + 1);
  }
  split_run(m, SP_LU, SplitLu{m, J0, ghinv, G});
  __syncthreads();
  if (threadIdx.x == 0 && *ier == INT_MAX) *ier = 0;
  __syncthreads();
}

// Substitution passes with staged lane records.  The forward and backward
// substitutions run on the first warp, one dependency level after another,
// and a pass is shorter than an L2 round trip, so table words loaded one pass
// ahead would still be in flight when the pass ends.  Here every lane copies
// its own 32-byte record of pass p + SPLIT_STAGE - 1 into a ring of
// SPLIT_STAGE slots in shared memory (cp.async) while pass p computes, and
// waits only for its own copies (cp.async.wait_group), so no barrier orders
// the copies and nothing waits on another thread.  Record (tables.py
// _solve_records): x | level end << 24 | the warp's longest chunk << 25 |
// its widest seglog << 29, first term | finish word << 16, the columns of the
// lane's terms as 16-bit words.  Row i's sum is X(i) - sum
// G(kk) X(icol(kk)) over the LU positions kk of its chunk; the backward
// substitution multiplies by the stored reciprocal pivot G(finish word).
constexpr int SPLIT_STAGE = 4;
constexpr int SPLIT_RING_BYTES = SPLIT_STAGE * 32 * 32;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <bool BACK>
__device__ __forceinline__ void split_solve_staged(const MechDev& m, int ph, const double* __restrict__ G,
                                                   double* X, uint4* ring) {
  const int np = m.sp_npass[ph];
  GCKPP_PHASE_BEGIN();
  const int lane = threadIdx.x;  // the first warp
  const uint4* rec = m.sp_rec[ph - SP_FS] + 2 * lane;
  uint4* mine = ring + 2 * lane;  // slot k of this lane: mine[64 k], mine[64 k + 1]
#pragma unroll
  for (int d = 0; d < SPLIT_STAGE - 1; ++d) {
    if (d < np) {
      cp_async16(mine + 64 * d, rec + 64 * d);
      cp_async16(mine + 64 * d + 1, rec + 64 * d + 1);
    }
    cp_async_commit();
  }
  for (int p = 0; p < np; ++p) {
    const int q = p + SPLIT_STAGE - 1;
    if (q < np) {
      const int sq = 64 * (q % SPLIT_STAGE);
      cp_async16(mine + sq, rec + 64 * q);
      cp_async16(mine + sq + 1, rec + 64 * q + 1);
    }
    cp_async_commit();
    cp_async_wait<SPLIT_STAGE - 1>();  // this pass's copies (committed SPLIT_STAGE - 1 groups ago) landed
    const int sp = 64 * (p % SPLIT_STAGE);
    const uint4 a = mine[sp], b = mine[sp + 1];
    const unsigned cw[6] = {a.z, a.w, b.x, b.y, b.z, b.w};
    const int item = a.x & 0xffff;
    const bool busy = item != 0xffff;
    const int seglog = (a.x >> 16) & 7;
    const int seg = 1 << seglog;
    const int n = (a.x >> 19) & 31;
    const int y = a.y & 0xffff;
    const int nmax = (a.x >> 25) & 15;  // the warp's longest chunk and widest segment
    const int lmax = a.x >> 29;
    const bool lead = busy && (lane & (seg - 1)) == 0;
    double acc = lead ? X[item] : 0.0;
#pragma unroll
    for (int k = 0; k < SPLIT_MAXCH; ++k) {
      if (k >= nmax) break;
      if (k < n) acc = fma(-G[y + k], X[(cw[k >> 1] >> (16 * (k & 1))) & 0xffffu], acc);
    }
    for (int o = (1 << lmax) >> 1; o > 0; o >>= 1) {
      const double v = __shfl_xor_sync(0xffffffffu, acc, o);
      if (o < seg) acc += v;
    }
    if (lead) X[item] = BACK ? acc * G[a.y >> 16] : acc;
    if ((a.x >> 24) & 1u) __syncwarp();
  }
  cp_async_wait<0>();
  GCKPP_PHASE_END(ph, lane == 0)
}

// Forward and backward substitution in the split form, on the first warp
// with staged records (the host checks that both phases use 32 lanes).
// Ends with a barrier.
__device__ inline void bk_solve_split(const MechDev& m, const double* G, double* X, uint4* ring) {
  if (threadIdx.x < 32) {
    split_solve_staged<false>(m, SP_FS, G, X, ring);
    __syncwarp();
    split_solve_staged<true>(m, SP_BS, G, X, ring);
  }
  __syncthreads();
}

// Shared scalars of the block's cell.
struct BlockShared {
  Lane L;
  int ier, flag, next, nconsec;
  double red[32];
};

// One block integrates cells order[0..ncell) (or 0..ncell) taken from a
// per-launch queue (p.queue_counter), one at a time.  Dynamic shared memory:
// block_layout(...).total doubles; p.ws holds block_layout(...).slot doubles
// per block of the grid.
template <bool STRICT, bool SPLIT = false>
__device__ void ros_block_driver(const MechDev& m, const RosMethod& r, const RosParams& p) {
  static_assert(!(STRICT && SPLIT), "the split form is fast arithmetic only");
  extern __shared__ double sm[];
  __shared__ BlockShared sh;
  const BlockLayout lay = block_layout(m.naux, m.nspec, m.nvar, m.nreact, m.nb, m.lu_nonzero, r.S, p.autonomous);
  double* slot = p.ws + (long long)blockIdx.x * lay.slot;
  double* aux = slot + lay.aux;
  double* Y = sm + lay.y0;
  double* Ynew = sm + lay.y1;
  double* F0 = sm + lay.fcn0;
  double* F = sm + lay.fcn;
  double* dfdt = sm + lay.dfdt;
  double* K = sm + lay.k;
  double* A = slot + lay.a;
  double* B = slot + lay.b;
  double* J0 = slot + lay.j0;
  double* G = sm + lay.g;
  double* E = sm + lay.e;
  // split form: the ring of staged substitution records after the cell's
  // arrays (16-byte aligned)
  uint4* ring = reinterpret_cast<uint4*>(sm + ((lay.total + 1) & ~1));
  const int nvar = m.nvar;
  const int tid = threadIdx.x, nt = blockDim.x;
  const double dir = (p.tend >= p.tstart) ? 1.0 : -1.0;
  Rosenbrock<STRICT, 1> ros(m, r, p);
  int qlo = 0, qhi = p.ncell;
  if (p.qrange) {
    qlo = p.qrange[0];
    qhi = p.qrange[1];
  }
  while (true) {
    if (tid == 0) sh.next = qlo + atomicAdd(p.queue_counter, 1);
    __syncthreads();
    const int idx = sh.next;
    if (idx >= qhi) break;
    const int cell = p.order ? p.order[idx] : idx;
    if ((unsigned)cell >= (unsigned)p.cell_limit) {
      __syncthreads();
      continue;
    }
    // load the cell (aux = [RCT | constant-rate literals], Y = [V | F])
    for (int k = tid; k < m.naux; k += nt)
      aux[k] = k < m.nreact ? p.rconst[(long long)k * p.ldr + cell] : __ldg(m.pre_lit + (k - m.nreact));
    for (int i = tid; i < m.nspec; i += nt) {
      const double v = p.c_in[(long long)i * p.ldc + cell];
      Y[i] = v;
      if (i >= nvar) Ynew[i] = v;
    }
    if (tid == 0) {
      if (p.resume)
        ros.load_lane(sh.L, cell);  // a cell handed over by the thread-per-cell kernel
      else
        ros.init_lane(sh.L, cell);
    }
    __syncthreads();
    while (true) {
      // TimeLoop head
      if (tid == 0 && sh.L.phase == PH_NEWSTEP) ros.step_checks(sh.L);
      __syncthreads();
      if (sh.L.phase == PH_DONE) break;
      // Fun0 and Jac0 (B products shared)
      bk_b_products(m, Y, aux, B);
      __syncthreads();
      if constexpr (SPLIT) {
        split_run(m, SP_JAC, SplitJac{m, B, J0});
        if (m.sp_nt[SP_JAC] < nt) __syncthreads();
        bk_fun_split(m, Y, aux, A, B, F0, E);
      } else {
        bk_jac<STRICT>(m, B, J0);
        bk_fun<STRICT>(m, Y, aux, A, B, F0);
      }
      if (!p.autonomous) {
        if constexpr (SPLIT)
          bk_fun_split(m, Y, aux, A, B, dfdt, E);
        else
          bk_fun<STRICT>(m, Y, aux, A, B, dfdt);
        const double delta = sqrt(p.roundoff) * fmax(1.0e-6, fabs(sh.L.T));
        const double rd = 1.0 / delta;
        for (int i = tid; i < nvar; i += nt) {
          double v = dfdt[i] + (-1.0) * F0[i];
          if (rd != 1.0) v = rd * v;
          dfdt[i] = v;
        }
        __syncthreads();
      }
      if (tid == 0) {
        sh.L.nfun += p.autonomous ? 1 : 2;
        sh.L.njac += 1;
        sh.L.phase = PH_ATTEMPT;
      }
      __syncthreads();
      while (sh.L.phase == PH_ATTEMPT) {
        // ros_PrepareMatrix with the singular-matrix retry
        if (tid == 0) sh.nconsec = 0;
        __syncthreads();
        while (true) {
          const double ghinv = 1.0 / (dir * sh.L.H * r.Gamma[0]);
          if constexpr (SPLIT)
            bk_decomp_split(m, J0, ghinv, G, &sh.ier);
          else
            bk_decomp<STRICT>(m, J0, ghinv, G, &sh.ier);
          if (tid == 0) sh.flag = ros.singular_retry(sh.L, sh.ier, sh.nconsec) ? 1 : 0;
          __syncthreads();
          if (!sh.flag) break;
        }
        if (sh.L.phase == PH_DONE) break;
        const double* fcn = F0;
        for (int s = 0; s < r.S; ++s) {
          if (s > 0 && r.NewF[s]) {
            for (int i = tid; i < nvar; i += nt) {
              double y = Y[i];
              for (int j = 0; j < s; ++j) {
                const int ia = (s * (s - 1)) / 2 + j;
                if (!((r.nzA >> ia) & 1u)) continue;  // WAXPY's alpha = 0 skip
                const double kj = K[j * nvar + i];
                y = STRICT ? y + r.A[ia] * kj : fma(r.A[ia], kj, y);
              }
              Ynew[i] = y;
            }
            __syncthreads();
            bk_b_products(m, Ynew, aux, B);
            __syncthreads();
            if constexpr (SPLIT)
              bk_fun_split(m, Ynew, aux, A, B, F, E);
            else
              bk_fun<STRICT>(m, Ynew, aux, A, B, F);
            if (tid == 0) sh.L.nfun += 1;
            fcn = F;
          }
          double hc[SMAX];
          unsigned hbits = 0u;  // bit j: hc(j) != 0 (WAXPY's alpha = 0 skip)
          for (int j = 0; j < s; ++j) {
            hc[j] = r.C[(s * (s - 1)) / 2 + j] / (dir * sh.L.H);
            if (hc[j] != 0.0) hbits |= 1u << j;
          }
          const double hg = dir * sh.L.H * r.Gamma[s];
          const bool use_dfdt = (!p.autonomous) && (r.Gamma[s] != 0.0);
          double* Ks = K + s * nvar;
          for (int i = tid; i < nvar; i += nt) {
            double k = fcn[i];
            for (int j = 0; j < s; ++j) {
              if (!((hbits >> j) & 1u)) continue;
              const double kj = K[j * nvar + i];
              k = STRICT ? k + hc[j] * kj : fma(hc[j], kj, k);
            }
            if (use_dfdt && hg != 0.0) {
              const double dd = dfdt[i];
              k = STRICT ? k + hg * dd : fma(hg, dd, k);
            }
            Ks[i] = k;
          }
          __syncthreads();
          if constexpr (SPLIT)
            bk_solve_split(m, G, Ks, ring);
          else
            bk_solve<STRICT>(m, G, Ks);
          if (tid == 0) sh.L.nsol += 1;
        }
        // new solution, error estimate, scaled errors
        for (int i = tid; i < nvar; i += nt) {
          const double at = p.vector_tol ? __ldg(p.atol + i) : __ldg(p.atol);
          const double rt = p.vector_tol ? __ldg(p.rtol + i) : __ldg(p.rtol);
          const double y0 = Y[i];
          double y = y0;
          double yerr = 0.0;
          for (int j = 0; j < r.S; ++j) {
            const double kj = K[j * nvar + i];
            if ((r.nzM >> j) & 1u) y = STRICT ? y + r.M[j] * kj : fma(r.M[j], kj, y);
            if ((r.nzE >> j) & 1u) yerr = STRICT ? yerr + r.E[j] * kj : fma(r.E[j], kj, yerr);
          }
          Ynew[i] = y;
          const double ymax = fmax(fabs(y0), fabs(y));
          const double scale = STRICT ? at + rt * ymax : fma(rt, ymax, at);
          E[i] = yerr / scale;
        }
        __syncthreads();
        // error norm (summed in species order, or in the split form by a
        // block reduction), then the step size control
        if constexpr (SPLIT) {
          double s = 0.0;
          for (int i = tid; i < nvar; i += nt) s = fma(E[i], E[i], s);
          for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
          if ((tid & 31) == 0) sh.red[tid >> 5] = s;
          __syncthreads();
          if (tid == 0) {
            double err = 0.0;
            for (int w = 0; w < (nt >> 5); ++w) err += sh.red[w];
            sh.flag = ros.control(sh.L, err, dir) ? 1 : 0;
          }
        } else if (tid == 0) {
          double err = 0.0;
          for (int i = 0; i < nvar; ++i) {
            const double e = E[i];
            err = STRICT ? err + e * e : fma(e, e, err);
          }
          sh.flag = ros.control(sh.L, err, dir) ? 1 : 0;
        }
        __syncthreads();
        if (sh.flag) {
          for (int i = tid; i < nvar; i += nt) {
            const double v = Ynew[i];
            Y[i] = p.clamp_negative ? fmax(v, 0.0) : v;
          }
          __syncthreads();
        }
      }
    }
    // store the cell
    for (int i = tid; i < nvar; i += nt) p.c_out[(long long)i * p.ldc + cell] = Y[i];
    if (p.c_out != p.c_in)
      for (int f = tid; f < m.nfix; f += nt)
        p.c_out[(long long)(nvar + f) * p.ldc + cell] = p.c_in[(long long)(nvar + f) * p.ldc + cell];
    if (tid == 0) {
      const Lane& L = sh.L;
      if (p.istatus) {
        const int v[8] = {L.nfun, L.njac, L.nstp, L.nacc, L.nrej, L.ndec, L.nsol, L.nsng};
        for (int k = 0; k < 20; ++k) p.istatus[(long long)k * p.ldo + cell] = k < 8 ? v[k] : 0;
      }
      if (p.rstatus) {
        for (int k = 0; k < 20; ++k) {
          double v = 0.0;
          if (k == 0) v = L.texit;
          if (k == 1) v = L.hexit;
          if (k == 2) v = L.hnew_out;
          p.rstatus[(long long)k * p.ldo + cell] = v;
        }
      }
      if (p.ierr) p.ierr[cell] = L.ierr;
    }
    __syncthreads();
  }
}

}  // namespace gckpp
