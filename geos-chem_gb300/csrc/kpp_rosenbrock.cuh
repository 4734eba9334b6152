// Rosenbrock integrator for one cell per thread, written as a per-lane state
// machine so that a warp always executes the same phase code: every loop
// iteration is one step attempt for every active lane.
//
// The control flow restates ros_Integrator
// (KPP/fullchem/gckpp_Integrator.F90:578-786) with the method tables of
// Ros2/Ros3/Ros4/Rodas3/Rodas4/Rang3 (:2060-2480), ros_ErrorNorm (:1715-1745),
// ros_FunTimeDerivative (:1748-1769) and ros_PrepareMatrix's singular-matrix
// retry (:1921-1999).  ICNTRL/RCNTRL are resolved on the host exactly as
// Rosenbrock does (:333-477) and passed in RosParams.
//
// Two schedules share the state machine:
//   plain  - thread i integrates cell i, workspace slot i;
//   queue  - persistent threads; when a lane's cell finishes it claims the
//            next cell of a device work queue (warp-aggregated atomics), so
//            lanes never idle while cells remain.
#pragma once
#include "kpp_mech.cuh"

namespace gckpp {

constexpr int SMAX = 6;

struct RosMethod {
  int S;
  double A[15], C[15], M[SMAX], E[SMAX], Alpha[SMAX], Gamma[SMAX], ELO;
  int NewF[SMAX];
};

struct WsLayout {
  int aux, y0, y1, fcn0, fcn, dfdt, k, a, b, j0, g, total;
};

struct RosParams {
  // cells
  int ncell;
  const int* order;       // optional queue order (cell ids), length ncell
  int* queue_counter;     // queue schedule: next queue position
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
  // workspace
  double* ws;
  WsLayout lay;
  long long nslot;
};

__device__ __forceinline__ double* slot_base(const RosParams& p, long long slot) {
  return p.ws + (slot / TS) * (long long)p.lay.total * TS + (slot % TS);
}

enum : int { PH_DONE = 0, PH_NEWSTEP = 1, PH_ATTEMPT = 2 };

struct Lane {
  int cell;
  int phase;
  double T, H;
  int rej_last, rej_more;
  int nfun, njac, nstp, nacc, nrej, ndec, nsol, nsng;
  double texit, hexit, hnew_out;
  int ierr;
  int ybuf;  // which of y0/y1 holds Y
};

template <bool STRICT>
struct Rosenbrock {
  const MechDev& m;
  const RosMethod& r;
  const RosParams& p;

  __device__ Rosenbrock(const MechDev& m_, const RosMethod& r_, const RosParams& p_) : m(m_), r(r_), p(p_) {}

  __device__ void load_cell(double* w, Lane& L, int cell) {
    const int nvar = m.nvar;
    // aux = [RCT | constant-rate literals]; Y buffers = [V | F]
    double* aux = w + p.lay.aux * TS;
    for (int q = 0; q < m.nreact; ++q) aux[q * TS] = p.rconst[(long long)q * p.ldr + cell];
    for (int q = m.nreact; q < m.naux; ++q) aux[q * TS] = __ldg(m.pre_lit + (q - m.nreact));
    double* y = w + p.lay.y0 * TS;
    double* y1 = w + p.lay.y1 * TS;
    for (int i = 0; i < nvar; ++i) y[i * TS] = p.c_in[(long long)i * p.ldc + cell];
    for (int f = 0; f < m.nfix; ++f) {
      const double v = p.c_in[(long long)(nvar + f) * p.ldc + cell];
      y[(nvar + f) * TS] = v;
      y1[(nvar + f) * TS] = v;
    }
    L.cell = cell;
    L.ybuf = 0;
    L.nfun = L.njac = L.nstp = L.nacc = L.nrej = L.ndec = L.nsol = L.nsng = 0;
    L.texit = 0.0;
    L.hexit = 0.0;
    L.hnew_out = 0.0;
    L.ierr = 0;
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

  __device__ void store_cell(double* w, const Lane& L) {
    const int nvar = m.nvar;
    const double* y = w + (L.ybuf ? p.lay.y1 : p.lay.y0) * TS;
    const int cell = L.cell;
    for (int i = 0; i < nvar; ++i) p.c_out[(long long)i * p.ldc + cell] = y[i * TS];
    if (p.c_out != p.c_in)
      for (int f = 0; f < m.nfix; ++f)
        p.c_out[(long long)(nvar + f) * p.ldc + cell] = p.c_in[(long long)(nvar + f) * p.ldc + cell];
    if (p.istatus) {
      const int v[8] = {L.nfun, L.njac, L.nstp, L.nacc, L.nrej, L.ndec, L.nsol, L.nsng};
      for (int q = 0; q < 20; ++q) p.istatus[(long long)q * p.ldo + cell] = q < 8 ? v[q] : 0;
    }
    if (p.rstatus) {
      for (int q = 0; q < 20; ++q) {
        double v = 0.0;
        if (q == 0) v = L.texit;
        if (q == 1) v = L.hexit;
        if (q == 2) v = L.hnew_out;
        p.rstatus[(long long)q * p.ldo + cell] = v;
      }
    }
    if (p.ierr) p.ierr[cell] = L.ierr;
  }

  // TimeLoop head + Fun0 + Jac0 (ros_Integrator :652-677)
  __device__ void new_step(double* w, Lane& L) {
    const double dir = (p.tend >= p.tstart) ? 1.0 : -1.0;
    const bool go = (dir > 0.0) ? ((L.T - p.tend) + p.roundoff <= 0.0) : ((p.tend - L.T) + p.roundoff <= 0.0);
    if (!go) {
      L.ierr = 1;
      L.phase = PH_DONE;
      return;
    }
    if (L.nstp > p.max_steps) {
      L.ierr = -6;
      L.phase = PH_DONE;
      return;
    }
    if (((L.T + 0.1 * L.H) == L.T) || (L.H <= p.roundoff)) {
      L.ierr = -7;
      L.phase = PH_DONE;
      return;
    }
    L.H = fmin(L.H, fabs(p.tend - L.T));
    const double* aux = w + p.lay.aux * TS;
    const double* Y = w + (L.ybuf ? p.lay.y1 : p.lay.y0) * TS;
    double* B = w + p.lay.b * TS;
    // B products once for both Jac_SP and Fun0's D_VAR terms.
    b_products(m, Y, aux, B);
    jac_sp<STRICT>(m, B, w + p.lay.j0 * TS);
    fun_split<STRICT>(m, Y, aux, w + p.lay.a * TS, B, w + p.lay.fcn0 * TS);
    L.nfun += 1;
    if (!p.autonomous) {
      // ros_FunTimeDerivative (:1748-1769); rates are frozen for the step
      // (ICNTRL(15)=-1) so FunTemplate(T+Delta) evaluates the same point.
      double* dfdt = w + p.lay.dfdt * TS;
      const double* f0 = w + p.lay.fcn0 * TS;
      const double delta = sqrt(p.roundoff) * fmax(1.0e-6, fabs(L.T));
      fun_split<STRICT>(m, Y, aux, w + p.lay.a * TS, B, dfdt);
      L.nfun += 1;
      const double rd = 1.0 / delta;
      for (int i = 0; i < m.nvar; ++i) {
        double v = dfdt[i * TS] + (-1.0) * f0[i * TS];
        if (rd != 1.0) v = rd * v;
        dfdt[i * TS] = v;
      }
    }
    L.njac += 1;
    L.phase = PH_ATTEMPT;
  }

  // One pass of UntilAccepted (:681-778)
  __device__ void attempt(double* w, Lane& L, int& ier_out) {
    const double dir = (p.tend >= p.tstart) ? 1.0 : -1.0;
    const int nvar = m.nvar;
    double* G = w + p.lay.g * TS;
    const double* J0 = w + p.lay.j0 * TS;
    // ros_PrepareMatrix with singular retry (:1921-1999)
    int nconsec = 0;
    while (true) {
      const double ghinv = 1.0 / (dir * L.H * r.Gamma[0]);
      const int ier = p.lu_form ? decomp<STRICT>(m, J0, ghinv, G) : decomp_rows<STRICT>(m, J0, ghinv, G);
      L.ndec += 1;
      if (ier == 0) break;
      L.nsng += 1;
      nconsec += 1;
      if (nconsec <= 5) {
        L.H = L.H * 0.5;
      } else {
        L.ierr = -8;
        L.phase = PH_DONE;
        ier_out = ier;
        return;
      }
    }
    const double* Y = w + (L.ybuf ? p.lay.y1 : p.lay.y0) * TS;
    double* Ynew = w + (L.ybuf ? p.lay.y0 : p.lay.y1) * TS;
    const double* aux = w + p.lay.aux * TS;
    double* K = w + p.lay.k * TS;
    const double* fcn = w + p.lay.fcn0 * TS;
    const long long kst = (long long)nvar * TS;
    for (int s = 0; s < r.S; ++s) {
      if (s > 0 && r.NewF[s]) {
        for (int i = 0; i < nvar; ++i) {
          double y = Y[i * TS];
          for (int j = 0; j < s; ++j) {
            const double a = r.A[(s * (s - 1)) / 2 + j];
            if (a != 0.0) y = STRICT ? y + a * K[j * kst + i * TS] : fma(a, K[j * kst + i * TS], y);
          }
          Ynew[i * TS] = y;
        }
        b_products(m, Ynew, aux, w + p.lay.b * TS);
        fun_split<STRICT>(m, Ynew, aux, w + p.lay.a * TS, w + p.lay.b * TS, w + p.lay.fcn * TS);
        L.nfun += 1;
        fcn = w + p.lay.fcn * TS;
      }
      double hc[SMAX];
      for (int j = 0; j < s; ++j) hc[j] = r.C[(s * (s - 1)) / 2 + j] / (dir * L.H);
      const bool use_dfdt = (!p.autonomous) && (r.Gamma[s] != 0.0);
      const double hg = dir * L.H * r.Gamma[s];
      const double* dfdt = w + p.lay.dfdt * TS;
      double* Ks = K + s * kst;
      for (int i = 0; i < nvar; ++i) {
        double k = fcn[i * TS];
        for (int j = 0; j < s; ++j)
          if (hc[j] != 0.0) k = STRICT ? k + hc[j] * K[j * kst + i * TS] : fma(hc[j], K[j * kst + i * TS], k);
        if (use_dfdt && hg != 0.0) k = STRICT ? k + hg * dfdt[i * TS] : fma(hg, dfdt[i * TS], k);
        Ks[i * TS] = k;
      }
      solve<STRICT>(m, G, Ks);
      L.nsol += 1;
    }
    // new solution, error estimate and norm (:729-740, :1715-1745)
    const double* atol = p.atol;
    const double* rtol = p.rtol;
    double err = 0.0;
    for (int i = 0; i < nvar; ++i) {
      double y = Y[i * TS];
      double yerr = 0.0;
      for (int j = 0; j < r.S; ++j) {
        const double kj = K[j * kst + i * TS];
        if (r.M[j] != 0.0) y = STRICT ? y + r.M[j] * kj : fma(r.M[j], kj, y);
        if (r.E[j] != 0.0) yerr = STRICT ? yerr + r.E[j] * kj : fma(r.E[j], kj, yerr);
      }
      Ynew[i * TS] = y;
      const double ymax = fmax(fabs(Y[i * TS]), fabs(y));
      const double at = p.vector_tol ? __ldg(atol + i) : __ldg(atol);
      const double rt = p.vector_tol ? __ldg(rtol + i) : __ldg(rtol);
      const double scale = STRICT ? at + rt * ymax : fma(rt, ymax, at);
      const double q = yerr / scale;
      err = STRICT ? err + q * q : fma(q, q, err);
    }
    err = sqrt(err / (double)nvar);
    err = fmax(err, 1.0e-10);
    // step size control (:742-778)
    const double fac = fmin(r_facmax(), fmax(p.facmin, p.facsafe / pow(err, 1.0 / r.ELO)));
    double hnew = L.H * fac;
    L.nstp += 1;
    if ((err <= 1.0) || (L.H <= p.hmin)) {
      L.nacc += 1;
      if (p.clamp_negative)
        for (int i = 0; i < nvar; ++i) Ynew[i * TS] = fmax(Ynew[i * TS], 0.0);
      L.ybuf ^= 1;
      L.T = L.T + dir * L.H;
      hnew = fmax(p.hmin, fmin(hnew, p.hmax));
      if (L.rej_last) hnew = fmin(hnew, L.H);
      L.hexit = L.H;
      L.hnew_out = hnew;
      L.texit = L.T;
      L.rej_last = 0;
      L.rej_more = 0;
      L.H = hnew;
      L.phase = PH_NEWSTEP;
    } else {
      if (L.rej_more) hnew = L.H * p.facrej;
      L.rej_more = L.rej_last;
      L.rej_last = 1;
      L.H = hnew;
      if (L.nacc >= 1) L.nrej += 1;
    }
  }

  __device__ __forceinline__ double r_facmax() const { return p.facmax; }
};

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Claim the next queue position for each calling lane (warp-aggregated).
__device__ __forceinline__ int queue_claim(int* counter) {
  const unsigned mask = __activemask();
  const int leader = __ffs(mask) - 1;
  const unsigned lt = mask & ((1u << lane_id()) - 1u);
  const int n = __popc(mask);
  int base = 0;
  if ((int)lane_id() == leader) base = atomicAdd(counter, n);
  base = __shfl_sync(mask, base, leader);
  return base + __popc(lt);
}

template <bool STRICT, bool QUEUE>
__device__ void ros_driver(const MechDev& m, const RosMethod& r, const RosParams& p) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Rosenbrock<STRICT> ros(m, r, p);
  double* w = slot_base(p, tid);
  Lane L;
  bool active = true;
  if (QUEUE) {
    const int q = queue_claim(p.queue_counter);
    if (q >= p.ncell) return;
    ros.load_cell(w, L, p.order ? p.order[q] : q);
  } else {
    if (tid >= p.ncell) return;
    ros.load_cell(w, L, p.order ? p.order[tid] : (int)tid);
  }
  while (active) {
    if (L.phase == PH_DONE) {
      ros.store_cell(w, L);
      if (QUEUE) {
        const int q = queue_claim(p.queue_counter);
        if (q < p.ncell) ros.load_cell(w, L, p.order ? p.order[q] : q);
        else active = false;
      } else {
        active = false;
      }
    }
    if (active && L.phase == PH_NEWSTEP) ros.new_step(w, L);
    if (active && L.phase == PH_ATTEMPT) {
      int ier = 0;
      ros.attempt(w, L, ier);
    }
  }
}

}  // namespace gckpp
