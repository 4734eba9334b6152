// Host build of the thread-per-cell Rosenbrock driver (ros_driver of
// geos-chem_gb300/csrc/kpp_rosenbrock.cuh, plain schedule, strict or fast
// arithmetic) for tests/test_ros_host.py: the CUDA qualifiers become plain
// C++, the launch becomes a loop over the threads of the grid (in the plain
// schedule a thread owns its cell and its lane of the workspace, so the
// threads are independent), CUDA's math functions glibc's.  Built
// -ffp-contract=off, it performs the kernel's arithmetic operation for
// operation, so the kernel's integration logic -- the step control, the
// auto-reduction mask, APPEND, the first-order update -- can be checked
// against the oracle without a GPU.
//
// argv: ncell tout ar append thr target ratio [percell] [keep] [strict] [queue]
// (strict = 0: the fast arithmetic, FMA through std::fma, which rounds once
// as the GPU's does; queue = 1: the work-queue schedule over the cells in
// reverse order -- emulated one thread after the other, the first thread
// claims every cell, so one workspace slot serves them all in turn)
// Inputs (float64/int32, cell-interleaved): c.bin [nspec][n], r.bin
// [nreact][n], atol.bin/rtol.bin [nvar]; with percell: pthr.bin [n],
// ptgt.bin (int32) [n], pratio.bin [n]; with keep: keep.bin (uint8) [nvar].
// Outputs: c_out.bin [nspec][n], ist.bin (int32) [20][n], rst.bin [20][n],
// ierr.bin (int32) [n].
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define __device__
#define __global__
#define __host__
#define __forceinline__ inline
#define __noinline__
#define __launch_bounds__(...)

struct HostDim {
  unsigned x, y, z;
};
static HostDim threadIdx, blockIdx, blockDim;

template <class T>
static inline T __ldg(const T* p) {
  return *p;
}
template <class T>
static inline T __ldcg(const T* p) {
  return *p;
}
static inline long long __double_as_longlong(double d) {
  long long v;
  memcpy(&v, &d, 8);
  return v;
}
// one emulated thread runs at a time: it is the only active lane of its warp
static inline unsigned __activemask() { return 1u << (threadIdx.x & 31u); }
static inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
// round-to-nearest products and sums (built -ffp-contract=off: never fused)
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
static inline int __shfl_sync(unsigned, int v, int) { return v; }
static inline int atomicAdd(int* p, int v) {
  const int o = *p;
  *p += v;
  return o;
}
using std::exp;
using std::fabs;
using std::fma;
using std::fmax;
using std::fmin;
using std::pow;
using std::sqrt;

#include "mech_tables.inc"
#include "ros_methods.h"

namespace T = gcmech_tables;

template <class X>
static std::vector<X> rd(const char* f, size_t n) {
  std::vector<X> v(n);
  FILE* p = fopen(f, "rb");
  if (!p || fread(v.data(), sizeof(X), n, p) != n) {
    fprintf(stderr, "cannot read %s\n", f);
    exit(1);
  }
  fclose(p);
  return v;
}

template <class X>
static void wr(const char* f, const std::vector<X>& v) {
  FILE* p = fopen(f, "wb");
  fwrite(v.data(), sizeof(X), v.size(), p);
  fclose(p);
}

int main(int argc, char** argv) {
  if (argc < 8) return 2;
  const int n = atoi(argv[1]);
  const double tout = atof(argv[2]);
  const int ar = atoi(argv[3]), append = atoi(argv[4]);
  const double thr = atof(argv[5]);
  const int target = atoi(argv[6]);
  const double ratio = atof(argv[7]);
  const int percell = argc > 8 ? atoi(argv[8]) : 0;
  const int with_keep = argc > 9 ? atoi(argv[9]) : 0;
  const int strict = argc > 10 ? atoi(argv[10]) : 1;
  const int queue = argc > 11 ? atoi(argv[11]) : 0;

  gckpp::MechDev m{};
  m.nvar = T::NVAR;
  m.nfix = T::NFIX;
  m.nreact = T::NREACT;
  m.nspec = T::NSPEC;
  m.lu_nonzero = T::LU_NONZERO;
  m.nb = T::NB;
  m.lit0 = T::LIT0;
  m.prod_packed = reinterpret_cast<const uint2*>(T::prod_packed);
  m.prod_ids_a = T::prod_ids_a;
  m.prod_ids_b = T::prod_ids_b;
  for (int i = 0; i < 9; ++i) {
    m.a_cls[i] = T::a_cls_start[i];
    m.b_cls[i] = T::b_cls_start[i];
  }
  m.naux = T::NAUX;
  m.pre_lit = T::pre_literals;
  m.p_start = T::p_start;
  m.p_sterm = T::p_sterm;
  m.slit = T::slit;
  m.d_start = T::d_start;
  m.d_sterm = T::d_sterm;
  m.j_start = T::j_start;
  m.j_sterm = T::j_sterm;
  m.lu_crow = T::lu_crow;
  m.lu_diag = T::lu_diag;
  m.lu_icol = T::lu_icol;
  m.lrow_start = T::lrow_start;
  m.lop_kk = T::lop_kk;
  m.lop_dj = T::lop_dj;
  m.lop_u = T::lop_u;
  m.uop = T::uop;
  m.lit = T::lit;
  m.dot_start = T::dot_start;
  m.dot_term = T::dot_term;
  m.lu_irow = T::lu_irow;

  gckpp::RosMethod meth{};
  if (!gckpp::method_table(4, meth)) return 3;  // Rodas3, ICNTRL(3) = 4

  // the thread workspace of the auto-reduce layout (make_layout(true) of the C ABI)
  gckpp::WsLayout l{};
  int o = 0;
  l.aux = o; o += T::NAUX;
  l.y0 = o; o += T::NSPEC;
  l.y1 = o; o += T::NSPEC;
  l.fcn0 = o; o += T::NVAR;
  l.fcn = o; o += T::NVAR;
  l.dfdt = o; o += T::NVAR;
  l.k = o; o += gckpp::SMAX * T::NVAR;
  l.a = o; o += T::NREACT;
  l.b = o; o += T::NB;
  l.j0 = o; o += T::LU_NONZERO;
  l.g = o; o += T::LU_NONZERO;
  l.slv = o; o += T::NVAR;
  l.prod = o; o += T::NVAR;
  l.loss = o; o += T::NVAR;
  l.pcur = o; o += T::NVAR;
  l.dcur = o; o += T::NVAR;
  l.total = o;

  auto c_in = rd<double>("c.bin", (size_t)T::NSPEC * n);
  auto rc = rd<double>("r.bin", (size_t)T::NREACT * n);
  auto atol = rd<double>("atol.bin", T::NVAR), rtol = rd<double>("rtol.bin", T::NVAR);
  std::vector<double> pthr, pratio;
  std::vector<int> ptgt;
  std::vector<unsigned char> keep;
  if (percell) {
    pthr = rd<double>("pthr.bin", n);
    ptgt = rd<int>("ptgt.bin", n);
    pratio = rd<double>("pratio.bin", n);
  }
  if (with_keep) keep = rd<unsigned char>("keep.bin", T::NVAR);
  std::vector<double> c_out(c_in), rst((size_t)20 * n);
  std::vector<int> ist((size_t)20 * n), ierr(n);
  const int block = 128;
  const int nthread = (n + block - 1) / block * block;
  std::vector<double> ws((size_t)nthread * l.total);
  int counter = 0;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = n - 1 - i;

  gckpp::RosParams p{};
  p.ncell = n;
  p.cell_limit = n;
  p.queue_counter = &counter;
  p.c_in = c_in.data();
  p.c_out = c_out.data();
  p.ldc = n;
  p.rconst = rc.data();
  p.ldr = n;
  p.istatus = ist.data();
  p.rstatus = rst.data();
  p.ldo = n;
  p.ierr = ierr.data();
  p.atol = atol.data();
  p.rtol = rtol.data();
  p.vector_tol = 1;
  p.tstart = 0.0;
  p.tend = tout;
  p.hmin = 0.0;
  p.hmax = tout;
  p.hstart_default = 1.0e-5;
  p.facmin = 0.2;
  p.facmax = 6.0;
  p.facrej = 0.1;
  p.facsafe = 0.9;
  p.roundoff = 2.220446049250313e-16;
  p.autonomous = 1;
  p.max_steps = 200000;
  p.clamp_negative = 0;
  p.lu_form = 0;
  p.ar_target = target;
  p.ar_append = append;
  p.ar_thr = thr > 0.0 ? thr : 1.0e2;
  p.ar_ratio = ratio > 0.0 ? ratio : 0.0;
  if (percell) {
    p.ar_thr_cell = pthr.data();
    p.ar_target_cell = ptgt.data();
    p.ar_ratio_cell = pratio.data();
  }
  if (with_keep) p.ar_keep = keep.data();
  if (queue) p.order = order.data();
  p.ws = ws.data();
  p.lay = l;
  p.nslot = nthread;

  blockDim = HostDim{(unsigned)block, 1, 1};
  for (int t = 0; t < nthread; ++t) {
    blockIdx = HostDim{(unsigned)(t / block), 0, 0};
    threadIdx = HostDim{(unsigned)(t % block), 0, 0};
    if (queue) {
      if (strict) {
        if (ar)
          gckpp::ros_driver<true, true, 1, true>(m, meth, p);
        else
          gckpp::ros_driver<true, true, 1, false>(m, meth, p);
      } else {
        if (ar)
          gckpp::ros_driver<false, true, 1, true>(m, meth, p);
        else
          gckpp::ros_driver<false, true, 1, false>(m, meth, p);
      }
    } else if (strict) {
      if (ar)
        gckpp::ros_driver<true, false, 1, true>(m, meth, p);
      else
        gckpp::ros_driver<true, false, 1, false>(m, meth, p);
    } else {
      if (ar)
        gckpp::ros_driver<false, false, 1, true>(m, meth, p);
      else
        gckpp::ros_driver<false, false, 1, false>(m, meth, p);
    }
  }
  wr("c_out.bin", c_out);
  wr("ist.bin", ist);
  wr("rst.bin", rst);
  wr("ierr.bin", ierr);
  return 0;
}
