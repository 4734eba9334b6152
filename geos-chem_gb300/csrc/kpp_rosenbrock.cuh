// Rosenbrock integrator, NC cells per thread, written as a per-cell state
// machine so that a warp always executes the same phase code: every loop
// iteration is one step attempt for every active cell of the thread.
//
// The control flow restates ros_Integrator
// (KPP/fullchem/gckpp_Integrator.F90:578-786) with the method tables of
// Ros2/Ros3/Ros4/Rodas3/Rodas4/Rang3 (:2060-2480), ros_ErrorNorm (:1715-1745),
// ros_FunTimeDerivative (:1748-1769) and ros_PrepareMatrix's singular-matrix
// retry (:1921-1999).  ICNTRL/RCNTRL are resolved on the host exactly as
// Rosenbrock does (:333-477) and passed in RosParams.
//
// The NC cells of a thread share every table walk; each keeps its own step
// size, counters and accept/reject state.  When one cell needs a new
// Jacobian and another is retrying a rejected step, both are evaluated
// (re-evaluating Jac0/Fcn0 at an unchanged Y reproduces the same values) and
// only the cell that needed it counts it.
//
// Two schedules share the state machine:
//   plain  - each thread integrates NC fixed cells, one workspace slot each;
//   queue  - persistent threads; when a cell finishes, its slot claims the
//            next cell of a device work queue (warp-aggregated atomics).
#pragma once
#include "kpp_mech.cuh"

namespace gckpp {

constexpr int SMAX = 6;

struct RosMethod {
  int S;
  double A[15], C[15], M[SMAX], E[SMAX], Alpha[SMAX], Gamma[SMAX], ELO;
  int NewF[SMAX];
  unsigned nzA, nzC, nzM, nzE;  // nonzero-coefficient bits (method_masks)
  // the nonzero A(s, j), M(j), E(j) as lists (method_masks): stage s adds
  // a_n[s] terms j = a_j[s][t]; the new solution m_n terms m_j[t], the
  // error estimate e_n terms e_j[t] -- loops that run only the terms the
  // method has (WAXPY's alpha = 0 skip without a test per species)
  int a_n[SMAX], a_j[SMAX][SMAX], m_n, m_j[SMAX], e_n, e_j[SMAX];
};

struct WsLayout {
  int aux, y0, y1, fcn0, fcn, dfdt, k, a, b, j0, g;
  // auto-reduction only (else -1): the order of entry of each species into
  // the solve (-1 frozen, 0 from the start, t the t-th appended one), P_VAR
  // and D_VAR at Tstart, and P_VAR/D_VAR of the current step (append form)
  int slv, prod, loss, pcur, dcur;
  int total;
};

struct RosParams {
  // cells
  int ncell;
  const int* order;       // optional queue order (cell ids), length ncell
  int cell_limit;         // cell ids must lie in [0, cell_limit); others are skipped
  const int* qrange;      // optional device {begin, end}: queue positions [begin, end) of order
                          // instead of [0, ncell) (sizes known only on the device)
  int* queue_counter;     // queue schedule: next queue position
  int queue_chunk;        // queue schedule: positions a lane takes per claim (0 or 1: one)
  // boundary arrays, cell-interleaved: X[k*ld + cell]
  const double* c_in;
  double* c_out;
  long long ldc;
  const double* rconst;
  long long ldr;
  const double* hstart;   // optional per-cell RCNTRL(3)
  int* istatus;           // [20][ldo]
  double* rstatus;        // [20][ldo]
  long long ldo;
  int* ierr;              // [ncell]
  // tolerances
  const double* atol;
  const double* rtol;
  int vector_tol;
  // resolved integration parameters
  double tstart, tend;
  double hmin, hmax, hstart_default, facmin, facmax, facrej, facsafe, roundoff;
  int autonomous, max_steps, clamp_negative;
  int lu_form;  // 0 decomp_rows, 1 decomp (KppDecomp order)
  // auto-reduction (ros_yIntegrator, gckpp_Integrator.F90:789-1237): at the
  // first step, species with |P_VAR| and |D_VAR*y| below the threshold are
  // frozen -- their Jac0 rows and columns are zeroed, their stage vectors
  // kept 0 -- and take the first-order solution at the end.  The threshold
  // is ar_thr, or with ar_target > 0 (1-based species) ar_ratio * max(P, L*y)
  // of that species, reported in RSTATUS(4).  Kernels built with AR only.
  // Per-cell arrays, when set, replace the three scalars cell by cell
  // (fullchem_AutoReduceFuncs.F90:293-343 sets them per grid box; a
  // threshold <= 0 means the default 100, a ratio <= 0 means 0), and
  // ar_keep [nvar] marks species never frozen (keepActive/keepSpcActive).
  // ar_append selects the append form (ros_yIntegratorA, :1242-1700): at
  // every step a frozen species whose |P| or |L*y| exceeds the RCNTRL(12)
  // threshold re-enters the solve after the species already in it.
  int ar_target, ar_append;
  double ar_thr, ar_ratio;
  const double* ar_thr_cell;
  const int* ar_target_cell;
  const double* ar_ratio_cell;
  const unsigned char* ar_keep;
  // hand-over of long-running cells to the block-per-cell kernel: a cell
  // about to start step evict_after + 1 leaves its state (Y in c_out, T and H
  // in RSTATUS(4:5), counters in ISTATUS(1:8)) and its id at
  // evict_list[atomicAdd(evict_count, 1)]; the block kernel with resume = 1
  // continues it from there with the same arithmetic
  int evict_after;   // 0 = never
  int evict_drained; // 1: only once the queue has no unclaimed cell left
  int* evict_list;
  int* evict_count;
  int resume;
  // workspace: per warp a tile of 32*NC cells x lay.total entries
  double* ws;
  WsLayout lay;
  long long nslot;
};

enum : int { PH_DONE = 0, PH_NEWSTEP = 1, PH_ATTEMPT = 2, PH_EVICTED = 3 };

struct Lane {
  int cell;
  int phase;
  double T, H;
  int rej_last, rej_more;
  int nfun, njac, nstp, nacc, nrej, ndec, nsol, nsng;
  double texit, hexit, hnew_out;
  int ierr;
  int ar_built;   // auto-reduction: the frozen set is chosen
  int ar_report;  // auto-reduction: threshold from a target species (RSTATUS(4))
  int ar_napp;    // auto-reduction: species appended so far
  double ar_thr;  // auto-reduction: the threshold used
  double ar_thr_app;  // auto-reduction: the RCNTRL(12) threshold of APPEND
};

template <bool STRICT, int NC, bool AR = false>
struct Rosenbrock {
  static_assert(!AR || NC == 1, "auto-reduction runs one cell per thread");
  static constexpr int TSN = TS * NC;
  const MechDev& m;
  const RosMethod& r;
  const RosParams& p;

  __device__ Rosenbrock(const MechDev& m_, const RosMethod& r_, const RosParams& p_) : m(m_), r(r_), p(p_) {}

  // entry 0 of the workspace array at `off` for cell q of this thread
  __device__ __forceinline__ double* arr(double* w, int off, int q) const { return w + off * TSN + q * TS; }

  __device__ void load_cell(double* w, int q, Lane& L, int cell) {
    const int nvar = m.nvar;
    // aux = [RCT | constant-rate literals]; Y0 (current Y) and Y1 (Ynew) = [V | F]
    double* aux = arr(w, p.lay.aux, q);
    for (int k = 0; k < m.nreact; ++k) aux[k * TSN] = p.rconst[(long long)k * p.ldr + cell];
    for (int k = m.nreact; k < m.naux; ++k) aux[k * TSN] = __ldg(m.pre_lit + (k - m.nreact));
    double* y = arr(w, p.lay.y0, q);
    double* y1 = arr(w, p.lay.y1, q);
    for (int i = 0; i < nvar; ++i) y[i * TSN] = p.c_in[(long long)i * p.ldc + cell];
    for (int f = 0; f < m.nfix; ++f) {
      const double v = p.c_in[(long long)(nvar + f) * p.ldc + cell];
      y[(nvar + f) * TSN] = v;
      y1[(nvar + f) * TSN] = v;
    }
    init_lane(L, cell);
  }

  // Hand a cell at a step boundary over to the block-per-cell kernel.
  __device__ void evict_cell(double* w, int q, const Lane& L) {
    const int nvar = m.nvar;
    const double* y = arr(w, p.lay.y0, q);
    const int cell = L.cell;
    for (int i = 0; i < nvar; ++i) p.c_out[(long long)i * p.ldc + cell] = y[i * TSN];
    if (p.c_out != p.c_in)
      for (int f = 0; f < m.nfix; ++f)
        p.c_out[(long long)(nvar + f) * p.ldc + cell] = p.c_in[(long long)(nvar + f) * p.ldc + cell];
    save_lane(L);
    p.evict_list[atomicAdd(p.evict_count, 1)] = cell;
  }

  // The scalar state of a cell at a step boundary, kept in its own status
  // rows until the block kernel resumes it.
  __device__ void save_lane(const Lane& L) const {
    const int v[8] = {L.nfun, L.njac, L.nstp, L.nacc, L.nrej, L.ndec, L.nsol, L.nsng};
    for (int k = 0; k < 8; ++k) p.istatus[(long long)k * p.ldo + L.cell] = v[k];
    const double d[5] = {L.texit, L.hexit, L.hnew_out, L.T, L.H};
    for (int k = 0; k < 5; ++k) p.rstatus[(long long)k * p.ldo + L.cell] = d[k];
  }

  __device__ void load_lane(Lane& L, int cell) const {
    init_lane(L, cell);
    int* v[8] = {&L.nfun, &L.njac, &L.nstp, &L.nacc, &L.nrej, &L.ndec, &L.nsol, &L.nsng};
    for (int k = 0; k < 8; ++k) *v[k] = p.istatus[(long long)k * p.ldo + cell];
    L.texit = p.rstatus[cell];
    L.hexit = p.rstatus[p.ldo + cell];
    L.hnew_out = p.rstatus[2 * p.ldo + cell];
    L.T = p.rstatus[3 * p.ldo + cell];
    L.H = p.rstatus[4 * p.ldo + cell];
  }

  // Per-cell scalar state at the start of the integration.
  __device__ void init_lane(Lane& L, int cell) const {
    L.cell = cell;
    L.nfun = L.njac = L.nstp = L.nacc = L.nrej = L.ndec = L.nsol = L.nsng = 0;
    L.texit = 0.0;
    L.hexit = 0.0;
    L.hnew_out = 0.0;
    L.ierr = 0;
    L.ar_built = 0;
    L.ar_report = 0;
    L.ar_napp = 0;
    L.ar_thr = 0.0;
    L.ar_thr_app = 0.0;
    // Hstart (Rosenbrock :420-428; INTEGRATE keeps only RCNTRL > 0, :115-117)
    double hs = p.hstart_default;
    if (p.hstart) {
      const double u = p.hstart[cell];
      if (u > 0.0) hs = fmin(fabs(u), fabs(p.tend - p.tstart));
    }
    // ros_Integrator initial preparations (:629-647)
    L.T = p.tstart;
    double H = fmin(fmax(fabs(p.hmin), fabs(hs)), fabs(p.hmax));
    if (fabs(H) <= 10.0 * p.roundoff) H = 1.0e-5;
    const double dir = (p.tend >= p.tstart) ? 1.0 : -1.0;
    L.H = dir * H;
    L.rej_last = 0;
    L.rej_more = 0;
    L.phase = PH_NEWSTEP;
  }

  // After a decomposition with singularity flag ier (:1977-1995): true if
  // the cell retries with H halved, false if it proceeds; a sixth
  // consecutive singular matrix ends the cell with IERR = -8.
  __device__ bool singular_retry(Lane& c, int ier, int& nconsec) const {
    c.ndec += 1;
    if (ier == 0) return false;
    c.nsng += 1;
    nconsec += 1;
    if (nconsec <= 5) {
      c.H = c.H * 0.5;
      return true;
    }
    c.ierr = -8;
    c.phase = PH_DONE;
    return false;
  }

  // Step size control (:742-778) from the error norm's sum of squares.
  // Returns true if the step is accepted (the caller then copies Ynew).
  __device__ bool control(Lane& c, double err_sum, double dir) const {
    double e = sqrt(err_sum / (double)m.nvar);
    e = fmax(e, 1.0e-10);
    const double fac = fmin(p.facmax, fmax(p.facmin, p.facsafe / pow(e, 1.0 / r.ELO)));
    double hnew = c.H * fac;
    c.nstp += 1;
    if ((e <= 1.0) || (c.H <= p.hmin)) {
      c.nacc += 1;
      c.T = c.T + dir * c.H;
      hnew = fmax(p.hmin, fmin(hnew, p.hmax));
      if (c.rej_last) hnew = fmin(hnew, c.H);
      c.hexit = c.H;
      c.hnew_out = hnew;
      c.texit = c.T;
      c.rej_last = 0;
      c.rej_more = 0;
      c.H = hnew;
      c.phase = PH_NEWSTEP;
      return true;
    }
    if (c.rej_more) hnew = c.H * p.facrej;
    c.rej_more = c.rej_last;
    c.rej_last = 1;
    c.H = hnew;
    if (c.nacc >= 1) c.nrej += 1;
    return false;
  }

  __device__ void store_cell(double* w, int q, const Lane& L) {
    const int nvar = m.nvar;
    const double* y = arr(w, p.lay.y0, q);
    const int cell = L.cell;
    if constexpr (AR) {
      // AutoReduce_1stOrder (:1702-1712) for every frozen species, after a
      // successful integration (:1226-1232)
      if (L.ierr == 1 && L.ar_built) {
        double* yw = arr(w, p.lay.y0, q);
        const double* slv = arr(w, p.lay.slv, q);
        const double* pr = arr(w, p.lay.prod, q);
        const double* lo = arr(w, p.lay.loss, q);
        const double dt = p.tend - p.tstart;
        for (int i = 0; i < nvar; ++i) {
          if (slv[i * TSN] >= 0.0) continue;  // in the solve
          const double k = lo[i * TSN];
          const double yi = yw[i * TSN];
          if (k <= 1.0e-30 || yi <= 1.0e-30) continue;
          const double term = pr[i * TSN] / k;
          // each operation rounded on its own, as the reference: when
          // P/k >> y the sum cancels, and a fused multiply-add would round
          // the cancelling terms differently from the reference
          yw[i * TSN] = __dadd_rn(term, __dmul_rn(__dadd_rn(yi, -term), exp(__dmul_rn(-k, dt))));
        }
      }
    }
    for (int i = 0; i < nvar; ++i) p.c_out[(long long)i * p.ldc + cell] = y[i * TSN];
    if (p.c_out != p.c_in)
      for (int f = 0; f < m.nfix; ++f)
        p.c_out[(long long)(nvar + f) * p.ldc + cell] = p.c_in[(long long)(nvar + f) * p.ldc + cell];
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
        if (AR && k == 3 && L.ar_report) v = L.ar_thr;  // RSTATUS(NARthr)
        p.rstatus[(long long)k * p.ldo + cell] = v;
      }
    }
    if (p.ierr) p.ierr[cell] = L.ierr;
  }

  // TimeLoop head (ros_Integrator :652-665): leaves the cell in NEWSTEP if
  // it needs Fun0/Jac0, else DONE with its IERR.
  __device__ void step_checks(Lane& L) const {
    const double dir = (p.tend >= p.tstart) ? 1.0 : -1.0;
    const bool go = (dir > 0.0) ? ((L.T - p.tend) + p.roundoff <= 0.0) : ((p.tend - L.T) + p.roundoff <= 0.0);
    if (!go) {
      L.ierr = 1;
      L.phase = PH_DONE;
    } else if (L.nstp > p.max_steps) {
      L.ierr = -6;
      L.phase = PH_DONE;
    } else if (((L.T + 0.1 * L.H) == L.T) || (L.H <= p.roundoff)) {
      L.ierr = -7;
      L.phase = PH_DONE;
    } else {
      L.H = fmin(L.H, fabs(p.tend - L.T));
    }
  }

  // The frozen set of ros_yIntegrator (:917-958) from P_VAR/D_VAR at
  // Tstart: order of entry -1 for the frozen species, 0 for the others.
  __device__ void ar_build(Lane& L, const double* Y, const double* pr, const double* lo, double* slv) const {
    const int cell = L.cell;
    double thr = p.ar_thr, ratio = p.ar_ratio;
    int tgt = p.ar_target;
    if (p.ar_thr_cell) {
      const double v = p.ar_thr_cell[cell];
      thr = v > 0.0 ? v : 1.0e2;
    }
    L.ar_thr_app = thr;
    if (p.ar_target_cell) tgt = p.ar_target_cell[cell];
    if (p.ar_ratio_cell) {
      const double v = p.ar_ratio_cell[cell];
      ratio = v > 0.0 ? v : 0.0;
    }
    if (tgt > 0) {  // 1..nvar, checked on the host
      const int t = tgt - 1;
      thr = ratio * fmax(lo[t * TSN] * Y[t * TSN], pr[t * TSN]);
    }
    for (int i = 0; i < m.nvar; ++i) {
      const double lossy = lo[i * TSN] * Y[i * TSN];
      const bool keep = p.ar_keep && p.ar_keep[i];
      slv[i * TSN] = (!keep && fabs(lossy) < thr && fabs(pr[i * TSN]) < thr) ? -1.0 : 0.0;
    }
    L.ar_thr = thr;
    L.ar_report = tgt > 0;
    L.ar_built = 1;
  }

  // Fun0 and Jac0 at Y for all NC cells (ros_Integrator :667-677), and the
  // time derivative for non-autonomous problems (:1748-1769; rates are frozen
  // for the step, ICNTRL(15)=-1, so FunTemplate(T+Delta) evaluates the same
  // point).
  __device__ void fun0_jac0(double* w, Lane* L) {
    const double* aux = arr(w, p.lay.aux, 0);
    const double* Y = arr(w, p.lay.y0, 0);
    double* B = arr(w, p.lay.b, 0);
    // B products once for both Jac_SP and Fun0's D_VAR terms.
    b_products<NC>(m, Y, aux, B);
    if constexpr (AR) {
      double* J0 = arr(w, p.lay.j0, 0);
      double* slv = arr(w, p.lay.slv, 0);
      const bool first = !L[0].ar_built && L[0].T == p.tstart;
      if (first || p.ar_append) {
        // FunSplitF: P_VAR and D_VAR as well, at T = Tstart (kept for
        // AutoReduce_1stOrder) and, in the append form, at every step
        double* pr = arr(w, first ? p.lay.prod : p.lay.pcur, 0);
        double* lo = arr(w, first ? p.lay.loss : p.lay.dcur, 0);
        fun_split<STRICT, NC, true>(m, Y, aux, arr(w, p.lay.a, 0), B, arr(w, p.lay.fcn0, 0), pr, lo);
        if (first) ar_build(L[0], Y, pr, lo, slv);
        if (p.ar_append) {
          // APPEND (:1460-1474, :2663-2700), in species order, against the
          // RCNTRL(12) threshold
          const double ta = L[0].ar_thr_app;
          for (int i = 0; i < m.nvar; ++i)
            if (slv[i * TSN] < 0.0 && (fabs(lo[i * TSN] * Y[i * TSN]) > ta || fabs(pr[i * TSN]) > ta))
              slv[i * TSN] = (double)(++L[0].ar_napp);
        }
      } else {
        fun_split<STRICT, NC>(m, Y, aux, arr(w, p.lay.a, 0), B, arr(w, p.lay.fcn0, 0));
      }
      jac_sp<STRICT, NC>(m, B, J0);
      // frozen rows and columns of Jac0 to 0: Ghimj = -Jac0 + ghinv I then
      // factors like cKppDecomp's compressed matrix (the frozen species only
      // meet exact zeros).  An appended species' row keeps the columns that
      // entered no later than it, its column is zeroed in earlier rows: the
      // compressed pattern of APPEND, whose new row comes last.
      for (int e = 0; e < m.lu_nonzero; ++e) {
        const double orr = slv[ldi(m.lu_irow + e) * TSN], oc = slv[ldi(m.lu_icol + e) * TSN];
        if (orr < 0.0 || oc < 0.0 || oc > orr) J0[e * TSN] = 0.0;
      }
    } else {
      jac_sp<STRICT, NC>(m, B, arr(w, p.lay.j0, 0));
      fun_split<STRICT, NC>(m, Y, aux, arr(w, p.lay.a, 0), B, arr(w, p.lay.fcn0, 0));
    }
    if (!p.autonomous) {
      double* dfdt = arr(w, p.lay.dfdt, 0);
      const double* f0 = arr(w, p.lay.fcn0, 0);
      fun_split<STRICT, NC>(m, Y, aux, arr(w, p.lay.a, 0), B, dfdt);
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        const double delta = sqrt(p.roundoff) * fmax(1.0e-6, fabs(L[q].T));
        const double rd = 1.0 / delta;
        for (int i = 0; i < m.nvar; ++i) {
          double v = dfdt[i * TSN + q * TS] + (-1.0) * f0[i * TSN + q * TS];
          if (rd != 1.0) v = rd * v;
          dfdt[i * TSN + q * TS] = v;
        }
      }
    }
  }

  // One pass of UntilAccepted (:681-778) for the cells with act[q].  The
  // other cells are computed along (their results are never used).
  __device__ void attempt(double* w, Lane* L, const bool* act) {
    const double dir = (p.tend >= p.tstart) ? 1.0 : -1.0;
    const int nvar = m.nvar;
    double* G = arr(w, p.lay.g, 0);
    const double* J0 = arr(w, p.lay.j0, 0);
    bool live[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) live[q] = act[q];
    // ros_PrepareMatrix with singular retry (:1921-1999): a cell whose
    // matrix is singular halves H and decomposes again, up to 5 times.
    {
      int nconsec[NC];
      bool pending[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        nconsec[q] = 0;
        pending[q] = live[q];
      }
      while (true) {
        double ghinv[NC];
        int ier[NC];
#pragma unroll
        for (int q = 0; q < NC; ++q) ghinv[q] = 1.0 / (dir * L[q].H * r.Gamma[0]);
        if (p.lu_form) decomp<STRICT, NC>(m, J0, ghinv, G, ier);
        else decomp_rows<STRICT, NC>(m, J0, ghinv, G, ier);
        bool again = false;
#pragma unroll
        for (int q = 0; q < NC; ++q) {
          if (!pending[q]) continue;
          if (singular_retry(L[q], ier[q], nconsec[q])) {
            again = true;
          } else {
            pending[q] = false;
            if (L[q].phase == PH_DONE) live[q] = false;
          }
        }
        if (!again) break;
      }
    }
    bool any_live = false;
#pragma unroll
    for (int q = 0; q < NC; ++q) any_live |= live[q];
    if (!any_live) return;

    const double* Y = arr(w, p.lay.y0, 0);
    double* Ynew = arr(w, p.lay.y1, 0);
    const double* aux = arr(w, p.lay.aux, 0);
    double* K = arr(w, p.lay.k, 0);
    const double* fcn = arr(w, p.lay.fcn0, 0);
    const long long kst = (long long)nvar * TSN;
    for (int s = 0; s < r.S; ++s) {
      if (s > 0 && r.NewF[s]) {
        for (int i = 0; i < nvar; ++i) {
#pragma unroll
          for (int q = 0; q < NC; ++q) {
            double y = Y[i * TSN + q * TS];
            for (int t = 0; t < r.a_n[s]; ++t) {
              const int j = r.a_j[s][t];
              const double a = r.A[(s * (s - 1)) / 2 + j];
              const double kj = K[j * kst + i * TSN + q * TS];
              y = STRICT ? y + a * kj : fma(a, kj, y);
            }
            Ynew[i * TSN + q * TS] = y;
          }
        }
        b_products<NC>(m, Ynew, aux, arr(w, p.lay.b, 0));
        fun_split<STRICT, NC>(m, Ynew, aux, arr(w, p.lay.a, 0), arr(w, p.lay.b, 0), arr(w, p.lay.fcn, 0));
#pragma unroll
        for (int q = 0; q < NC; ++q)
          if (live[q]) L[q].nfun += 1;
        fcn = arr(w, p.lay.fcn, 0);
      }
      double hc[NC][SMAX], hg[NC];
      unsigned hbits[NC];  // WAXPY's alpha = 0 skip, tested once per stage: bit j set if hc(j) != 0
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        hbits[q] = 0u;
        for (int j = 0; j < s; ++j) {
          hc[q][j] = r.C[(s * (s - 1)) / 2 + j] / (dir * L[q].H);
          if (hc[q][j] != 0.0) hbits[q] |= 1u << j;
        }
        hg[q] = dir * L[q].H * r.Gamma[s];
      }
      const bool use_dfdt = (!p.autonomous) && (r.Gamma[s] != 0.0);
      const double* dfdt = arr(w, p.lay.dfdt, 0);
      double* Ks = K + s * kst;
      for (int i = 0; i < nvar; ++i) {
#pragma unroll
        for (int q = 0; q < NC; ++q) {
          double k = fcn[i * TSN + q * TS];
          for (int j = 0; j < s; ++j) {
            if (!((hbits[q] >> j) & 1u)) continue;
            const double kj = K[j * kst + i * TSN + q * TS];
            k = STRICT ? k + hc[q][j] * kj : fma(hc[q][j], kj, k);
          }
          if (use_dfdt && hg[q] != 0.0) {
            const double dd = dfdt[i * TSN + q * TS];
            k = STRICT ? k + hg[q] * dd : fma(hg[q], dd, k);
          }
          if constexpr (AR) {
            // a frozen species' stage vector stays 0 (:704-728 loop over kept ones)
            if (arr(w, p.lay.slv, q)[i * TSN] < 0.0) k = 0.0;
          }
          Ks[i * TSN + q * TS] = k;
        }
      }
      solve<STRICT, NC>(m, G, Ks);
#pragma unroll
      for (int q = 0; q < NC; ++q)
        if (live[q]) L[q].nsol += 1;
    }
    // new solution, error estimate and norm (:729-740, :1715-1745)
    double err[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) err[q] = 0.0;
    for (int i = 0; i < nvar; ++i) {
      const double at = p.vector_tol ? __ldg(p.atol + i) : __ldg(p.atol);
      const double rt = p.vector_tol ? __ldg(p.rtol + i) : __ldg(p.rtol);
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        const double y0 = Y[i * TSN + q * TS];
        double y = y0;
        double yerr = 0.0;
        // the M and E terms in ascending j, each sum in its own order
        for (int t = 0; t < r.m_n; ++t) {
          const int j = r.m_j[t];
          const double kj = K[j * kst + i * TSN + q * TS];
          y = STRICT ? y + r.M[j] * kj : fma(r.M[j], kj, y);
        }
        for (int t = 0; t < r.e_n; ++t) {
          const int j = r.e_j[t];
          const double kj = K[j * kst + i * TSN + q * TS];
          yerr = STRICT ? yerr + r.E[j] * kj : fma(r.E[j], kj, yerr);
        }
        Ynew[i * TSN + q * TS] = y;
        const double ymax = fmax(fabs(y0), fabs(y));
        const double scale = STRICT ? at + rt * ymax : fma(rt, ymax, at);
        const double e = yerr / scale;
        err[q] = STRICT ? err[q] + e * e : fma(e, e, err[q]);
      }
    }
    // step size control (:742-778)
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      if (!live[q]) continue;
      if (control(L[q], err[q], dir)) {
        double* yq = arr(w, p.lay.y0, q);
        const double* ynq = arr(w, p.lay.y1, q);
        for (int i = 0; i < nvar; ++i) {
          const double v = ynq[i * TSN];
          yq[i * TSN] = (!AR && p.clamp_negative) ? fmax(v, 0.0) : v;  // ros_yIntegrator does not clamp
        }
      }
    }
  }
};

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Queue positions held by one cell slot of a lane: the next one, the
// distance to the one after it, and how many of its last claim remain.
struct QueueSlot {
  int next, stride, left;
};

// Next queue position of a slot.  A slot with none left claims `chunk`
// positions per calling lane in one warp-aggregated atomic: the n calling
// lanes reserve n*chunk consecutive positions and lane r of them takes
// positions r, r+n, r+2n, ... of that range, so lanes that claim together
// start on consecutive positions.  chunk 1 is one position per claim.
__device__ __forceinline__ int queue_take(int* counter, int chunk, QueueSlot& s) {
  if (s.left <= 0) {
    const unsigned mask = __activemask();
    const int leader = __ffs(mask) - 1;
    const unsigned lt = mask & ((1u << lane_id()) - 1u);
    const int n = __popc(mask);
    int base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(counter, n * chunk);
    base = __shfl_sync(mask, base, leader);
    s.next = base + __popc(lt);
    s.stride = n;
    s.left = chunk;
  }
  const int idx = s.next;
  s.next += s.stride;
  --s.left;
  return idx;
}

template <bool STRICT, bool QUEUE, int NC, bool AR = false>
__device__ void ros_driver(const MechDev& m, const RosMethod& r, const RosParams& p) {
  constexpr int TSN = TS * NC;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long warp = tid / TS;
  const int lane = (int)(tid % TS);
  Rosenbrock<STRICT, NC, AR> ros(m, r, p);
  double* w = p.ws + warp * (long long)p.lay.total * TSN + lane;
  Lane L[NC];
  bool has[NC];
  QueueSlot qs[NC];
  const int chunk = p.queue_chunk > 1 ? p.queue_chunk : 1;
  int qlo = 0, qhi = p.ncell;
  if (p.qrange) {
    qlo = p.qrange[0];
    qhi = p.qrange[1];
  }
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    long long idx;
    qs[q].left = 0;
    if (QUEUE) {
      idx = (long long)qlo + queue_take(p.queue_counter, chunk, qs[q]);
    } else {
      idx = (long long)qlo + warp * TSN + q * TS + lane;
    }
    has[q] = false;
    if (idx < qhi) {
      const int cell = p.order ? p.order[idx] : idx;
      has[q] = (unsigned)cell < (unsigned)p.cell_limit;
      if (has[q]) ros.load_cell(w, q, L[q], cell);
    }
  }
  while (true) {
    bool any = false;
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      if (has[q] && (L[q].phase == PH_DONE || L[q].phase == PH_EVICTED)) {
        if (L[q].phase == PH_DONE)
          ros.store_cell(w, q, L[q]);
        else
          ros.evict_cell(w, q, L[q]);
        has[q] = false;
        if (QUEUE) {
          const long long idx = (long long)qlo + queue_take(p.queue_counter, chunk, qs[q]);
          if (idx < qhi) {
            const int cell = p.order ? p.order[idx] : idx;
            if ((unsigned)cell < (unsigned)p.cell_limit) {
              ros.load_cell(w, q, L[q], cell);
              has[q] = true;
            }
          }
        }
      }
      any |= has[q];
    }
    if (!any) break;
    bool need = false;
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      if (has[q] && L[q].phase == PH_NEWSTEP) {
        ros.step_checks(L[q]);
        if (p.evict_after > 0 && L[q].phase == PH_NEWSTEP && L[q].nstp >= p.evict_after &&
            (!p.evict_drained || (long long)qlo + *(volatile int*)p.queue_counter >= qhi))
          L[q].phase = PH_EVICTED;
        need |= L[q].phase == PH_NEWSTEP;
      }
    }
    if (need) {
      ros.fun0_jac0(w, L);
#pragma unroll
      for (int q = 0; q < NC; ++q) {
        if (has[q] && L[q].phase == PH_NEWSTEP) {
          L[q].nfun += p.autonomous ? 1 : 2;
          L[q].njac += 1;
          L[q].phase = PH_ATTEMPT;
        }
      }
    }
    bool act[NC];
    bool any_act = false;
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      act[q] = has[q] && L[q].phase == PH_ATTEMPT;
      any_act |= act[q];
    }
    if (any_act) ros.attempt(w, L, act);
  }
}

}  // namespace gckpp
