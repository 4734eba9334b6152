// C ABI of the GB300 KPP fullchem solve (include/gckpp_gb300.h).
//
// Host side of INTEGRATE/Rosenbrock (KPP/fullchem/gckpp_Integrator.F90:
// 80-162, 333-477): merges ICNTRL_U/RCNTRL_U over the defaults, selects the
// method, validates tolerances, then launches the per-cell kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gckpp_gb300.h"
#include "mech_tables.inc"  // generated per mechanism (csrc/_gen/<mechanism>/)
#include "rates_program.inc"
#include "het_layout.h"
#include "kpp_rates.h"
#include "kpp_launch.h"
#include "kpp_util.h"
#include "het_state.h"
#include "kpp_block.cuh"
#include "kpp_rosenbrock.cuh"
#include "ros_methods.h"

using namespace gckpp;
namespace T = gcmech_tables;
namespace RT = gcrates_tables;


namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define GC_TRY(call)            \
  do {                          \
    int _rc = (call);           \
    if (_rc != GC_KPP_OK) return _rc; \
  } while (0)

int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? GC_KPP_ENOMEM : GC_KPP_ECUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define GC_CUDA(call)                                   \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return cuda_fail(_e, #call); \
  } while (0)

template <typename X>
cudaError_t upload(const X* host, size_t n, const X** dev, std::vector<void*>& owned) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, n * sizeof(X) + 16);
  if (e != cudaSuccess) return e;
  owned.push_back(p);
  e = cudaMemcpy(p, host, n * sizeof(X), cudaMemcpyHostToDevice);
  *dev = static_cast<const X*>(p);
  return e;
}

// Workspace layout of one cell of the thread-per-cell kernel; ar adds the
// auto-reduction arrays (order of entry, P_VAR and D_VAR at Tstart and at
// the current step).
WsLayout make_layout(bool ar = false) {
  WsLayout l;
  int o = 0;
  l.aux = o; o += T::NAUX;
  l.y0 = o; o += T::NSPEC;
  l.y1 = o; o += T::NSPEC;
  l.fcn0 = o; o += T::NVAR;
  l.fcn = o; o += T::NVAR;
  l.dfdt = o; o += T::NVAR;
  l.k = o; o += SMAX * T::NVAR;
  l.a = o; o += T::NREACT;
  l.b = o; o += T::NB;
  l.j0 = o; o += T::LU_NONZERO;
  l.g = o; o += T::LU_NONZERO;
  l.slv = l.prod = l.loss = l.pcur = l.dcur = -1;
  if (ar) {
    l.slv = o; o += T::NVAR;
    l.prod = o; o += T::NVAR;
    l.loss = o; o += T::NVAR;
    l.pcur = o; o += T::NVAR;
    l.dcur = o; o += T::NVAR;
  }
  l.total = o;
  return l;
}

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

}  // namespace

struct gc_kpp_ctx {
  int device = 0;
  int nsm = 0;
  MechDev mech{};
  gcrates::RatesDev rates{};
  std::vector<void*> owned;
  WsLayout lay{};
  DevBuf ws, counter;
  DevBuf h_c, h_r, h_at, h_rt, h_hs, h_is, h_rs, h_ie;  // staging for host-memory calls
  DevBuf h_met, h_ph, h_ord, h_het;
  DevBuf h_hetin;  // staging of fullchem_SetStateHet inputs for host-memory calls
  // HetState of the chemistry steps (gc_kpp_ctx_set_hetstate): device rows
  DevBuf step_het;
  const double* het = nullptr;
  long long het_ld = 0;
  int het_ncell = 0;
  DevBuf rc_buf, cb_buf, ord_buf;  // chemistry-step scratch: RCONST, C_before, retry list
  // auto-reduction controls (gc_kpp_ctx_set_autoreduce): per-cell RCNTRL(12),
  // ICNTRL(14), RCNTRL(14) for ar_ncell cells, and keepSpcActive
  DevBuf ar_thr, ar_tgt, ar_ratio, ar_keep;
  int ar_ncell = 0, ar_has_thr = 0, ar_has_tgt = 0, ar_has_ratio = 0, ar_keep_on = 0;
  int last_launches = 0;
  // optional CUDA-event timing of the Rosenbrock launches (GC_KPP_OPT_TIMING)
  int timing = 0;
  int lu_form = 0;  // 0 row-wise dot products, 1 KppDecomp right-looking order
  int async = 0;    // chemistry steps never synchronise the host (GC_KPP_OPT_ASYNC)
  int occ_arith = -1, occ_block = -1, occ_value = 1;  // cached occupancy query
  int evict_after = 0;  // hand cells over to the block-per-cell kernel after this many steps
  int evict_drained = 0;  // ... only once the queue has no unclaimed cell left
  int queue_chunk = 1;    // queue positions a lane takes per claim
  DevBuf evict_buf;     // ids of the handed-over cells
  DevBuf bws;           // Jac0 slots of the block-per-cell kernel, one per block of its grid
  int bocc_key = -1, bocc_value = 1;  // cached occupancy of the block-per-cell kernel
  DevBuf ranges;    // device queue ranges: [0,1] block-per-cell, [2,3] thread-per-cell, [4,5] retry
  // tolerance arrays validated by the last synchronous step (async steps reuse them)
  const void* tol_at = nullptr;
  const void* tol_rt = nullptr;
  int tol_vec = -1;
  int ntimed = 0;
  cudaEvent_t ev[8] = {};
  int arith = 0;     // 0 fast, 1 strict
  int schedule = 0;  // 0 plain, 1 queue
  int block = 128;
  int cell_block = 256;  // threads of the block-per-cell kernel
  int block_split = 1;   // fast arithmetic: the split block-per-cell form
  int rates_direct = 1;  // Update_RCONST as straight-line code (0: the interpreter)
  cudaStream_t side = nullptr;  // block-per-cell launches run beside the queue kernel
  cudaEvent_t fork = nullptr, join = nullptr;
  int blocks_per_sm = 0;
  long long max_slots = 0;
};

extern "C" {

int gc_kpp_mechanism_dims(int* nspec, int* nvar, int* nfix, int* nreact, int* lu_nonzero) {
  if (nspec) *nspec = T::NSPEC;
  if (nvar) *nvar = T::NVAR;
  if (nfix) *nfix = T::NFIX;
  if (nreact) *nreact = T::NREACT;
  if (lu_nonzero) *lu_nonzero = T::LU_NONZERO;
  return GC_KPP_OK;
}

const char* gc_kpp_last_error(void) { return g_last_error.c_str(); }

int gc_kpp_ctx_create(gc_kpp_ctx** out, int device) {
  if (!out) return fail(GC_KPP_EINVAL, "ctx pointer is NULL");
  *out = nullptr;
  GC_CUDA(cudaSetDevice(device));
  gc_kpp_ctx* c = new gc_kpp_ctx();
  c->device = device;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaGetDeviceProperties");
  }
  c->nsm = prop.multiProcessorCount;
  // side stream and events of block-per-cell launches, made here so that no
  // later call (possibly inside a stream capture) has to create them
  e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    gc_kpp_ctx_destroy(c);
    return cuda_fail(e, "stream/event creation");
  }
  MechDev& m = c->mech;
  m.nvar = T::NVAR; m.nfix = T::NFIX; m.nreact = T::NREACT; m.nspec = T::NSPEC;
  m.lu_nonzero = T::LU_NONZERO; m.nb = T::NB; m.lit0 = T::LIT0;
#define UP(field, arr)                                                         \
  e = upload(T::arr, sizeof(T::arr) / sizeof(T::arr[0]), &m.field, c->owned); \
  if (e != cudaSuccess) { gc_kpp_ctx_destroy(c); return cuda_fail(e, "upload " #arr); }
  e = upload(reinterpret_cast<const uint2*>(T::prod_packed), sizeof(T::prod_packed) / (2 * sizeof(unsigned)),
             &m.prod_packed, c->owned);
  if (e != cudaSuccess) { gc_kpp_ctx_destroy(c); return cuda_fail(e, "upload prod_packed"); }
  m.naux = T::NAUX;
  UP(prod_ids_a, prod_ids_a) UP(prod_ids_b, prod_ids_b)
  for (int i = 0; i < 9; ++i) {
    m.a_cls[i] = T::a_cls_start[i];
    m.b_cls[i] = T::b_cls_start[i];
  }
  UP(pre_lit, pre_literals) UP(p_start, p_start) UP(p_sterm, p_sterm) UP(slit, slit)
  UP(d_start, d_start) UP(d_sterm, d_sterm) UP(j_start, j_start) UP(j_sterm, j_sterm)
  UP(lu_crow, lu_crow) UP(lu_diag, lu_diag) UP(lu_icol, lu_icol) UP(lrow_start, lrow_start)
  UP(lop_kk, lop_kk) UP(lop_dj, lop_dj) UP(lop_u, lop_u) UP(uop, uop) UP(lit, lit)
  UP(dot_start, dot_start) UP(dot_term, dot_term)
  UP(lu_irow, lu_irow) UP(lu_lvl_start, lu_lvl_start) UP(lu_lvl_entry, lu_lvl_entry)
  UP(fs_lvl_start, fs_lvl_start) UP(fs_lvl_row, fs_lvl_row) UP(bs_lvl_start, bs_lvl_start)
  UP(bs_lvl_row, bs_lvl_row) UP(fun_rows_by_len, fun_rows_by_len) UP(jac_by_len, jac_by_len)
  m.lu_nlvl = T::LU_NLVL; m.fs_nlvl = T::FS_NLVL; m.bs_nlvl = T::BS_NLVL;
#undef UP
#define UPSPLIT(ph, name, NAME)                                                                                \
  e = upload(reinterpret_cast<const uint4*>(T::split_##name##_task), sizeof(T::split_##name##_task) / 16,    \
             &m.sp_task[ph], c->owned);                                                                      \
  if (e == cudaSuccess)                                                                                      \
    e = upload(T::split_##name##_pass, sizeof(T::split_##name##_pass) / 4, &m.sp_pass[ph], c->owned);        \
  if (e != cudaSuccess) { gc_kpp_ctx_destroy(c); return cuda_fail(e, "upload split schedule " #name); }      \
  m.sp_npass[ph] = T::SPLIT_##NAME##_NPASS;                                                                   \
  m.sp_nt[ph] = T::SPLIT_##NAME##_NT;
  UPSPLIT(gckpp::SP_LU, lu, LU) UPSPLIT(gckpp::SP_FS, fs, FS) UPSPLIT(gckpp::SP_BS, bs, BS)
  UPSPLIT(gckpp::SP_FUN, fun, FUN) UPSPLIT(gckpp::SP_JAC, jac, JAC)
#undef UPSPLIT
  e = upload(reinterpret_cast<const uint4*>(T::split_fs_rec), sizeof(T::split_fs_rec) / 16, &m.sp_rec[0], c->owned);
  if (e == cudaSuccess)
    e = upload(reinterpret_cast<const uint4*>(T::split_bs_rec), sizeof(T::split_bs_rec) / 16, &m.sp_rec[1],
               c->owned);
  if (e != cudaSuccess) { gc_kpp_ctx_destroy(c); return cuda_fail(e, "upload split substitution records"); }
  gcrates::RatesDev& rp = c->rates;
  rp.nreact = T::NREACT;
  rp.nmet = RT::NMET;
  e = upload(RT::code, sizeof(RT::code) / sizeof(int), &rp.code, c->owned);
  if (e == cudaSuccess) e = upload(RT::start, sizeof(RT::start) / sizeof(int), &rp.start, c->owned);
  if (e == cudaSuccess) e = upload(RT::consts, sizeof(RT::consts) / sizeof(double), &rp.consts, c->owned);
  if (e == cudaSuccess) e = upload(RT::law_nargs, sizeof(RT::law_nargs) / sizeof(int), &rp.law_nargs, c->owned);
  if (e == cudaSuccess) e = upload(RT::het_nargs, sizeof(RT::het_nargs) / sizeof(int), &rp.het_nargs, c->owned);
  if (e == cudaSuccess) e = upload(RT::hs_ind, sizeof(RT::hs_ind) / sizeof(int), &rp.hs_ind, c->owned);
  if (e == cudaSuccess) e = upload(RT::hs_mw, sizeof(RT::hs_mw) / sizeof(double), &rp.hs_mw, c->owned);
  if (e == cudaSuccess) e = upload(RT::hs_srmw, sizeof(RT::hs_srmw) / sizeof(double), &rp.hs_srmw, c->owned);
  if (e == cudaSuccess) e = upload(RT::hs_hk0, sizeof(RT::hs_hk0) / sizeof(double), &rp.hs_hk0, c->owned);
  if (e == cudaSuccess) e = upload(RT::hs_hcr, sizeof(RT::hs_hcr) / sizeof(double), &rp.hs_hcr, c->owned);
  if (e != cudaSuccess) {
    gc_kpp_ctx_destroy(c);
    return cuda_fail(e, "upload rate program");
  }
  c->lay = make_layout();
  *out = c;
  return GC_KPP_OK;
}

int gc_kpp_ctx_destroy(gc_kpp_ctx* c) {
  if (!c) return GC_KPP_OK;
  cudaSetDevice(c->device);
  for (void* p : c->owned) cudaFree(p);
  for (cudaEvent_t ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  if (c->fork) cudaEventDestroy(c->fork);
  if (c->join) cudaEventDestroy(c->join);
  if (c->side) cudaStreamDestroy(c->side);
  DevBuf* bufs[] = {&c->ws,   &c->counter, &c->h_c,  &c->h_r,  &c->h_at,  &c->h_rt,
                    &c->h_hs, &c->h_is,    &c->h_rs, &c->h_ie, &c->h_met, &c->h_ph,
                    &c->rc_buf, &c->cb_buf, &c->ord_buf, &c->h_ord, &c->ranges, &c->evict_buf, &c->bws,
                    &c->h_het, &c->step_het, &c->ar_thr, &c->ar_tgt, &c->ar_ratio, &c->ar_keep,
                    &c->h_hetin};
  for (DevBuf* b : bufs) b->release();
  delete c;
  return GC_KPP_OK;
}

int gc_kpp_ctx_set_option(gc_kpp_ctx* c, int key, long long v) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  switch (key) {
    case GC_KPP_OPT_ARITH:
      if (v < 0 || v > 3)
        return fail(GC_KPP_EINVAL, "arith must be 0 (fast), 1 (strict), 2 (fast, 2 cells per thread) or 3 (fast, 4)");
      c->arith = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_SCHEDULE:
      if (v != 0 && v != 1) return fail(GC_KPP_EINVAL, "schedule must be 0 or 1");
      c->schedule = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_BLOCK:
      if (v == 0) v = 128;
      if (v < 32 || v > 1024 || v % 32) return fail(GC_KPP_EINVAL, "block must be a multiple of 32 in [32,1024]");
      c->block = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_BLOCKS_PER_SM:
      if (v < 0 || v > 64) return fail(GC_KPP_EINVAL, "blocks per SM out of range");
      c->blocks_per_sm = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_LU:
      if (v != 0 && v != 1) return fail(GC_KPP_EINVAL, "lu form must be 0 or 1");
      c->lu_form = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_EVICT_AFTER:
      if (v < 0 || v > 1000000) return fail(GC_KPP_EINVAL, "evict-after steps out of range");
      c->evict_after = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_QUEUE_CHUNK:
      if (v == 0) v = 1;
      if (v < 1 || v > 64) return fail(GC_KPP_EINVAL, "queue chunk must be in [1, 64]");
      c->queue_chunk = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_EVICT_DRAINED:
      if (v != 0 && v != 1) return fail(GC_KPP_EINVAL, "evict-drained must be 0 or 1");
      c->evict_drained = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_ASYNC:
      if (v != 0 && v != 1) return fail(GC_KPP_EINVAL, "async must be 0 or 1");
      c->async = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_TIMING:
      c->timing = v ? 1 : 0;
      return GC_KPP_OK;
    case GC_KPP_OPT_CELL_BLOCK:
      if (v == 0) v = 256;
      if (v < 32 || v > 1024 || v % 32)
        return fail(GC_KPP_EINVAL, "block-per-cell threads must be a multiple of 32 in [32,1024]");
      c->cell_block = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_RATES_DIRECT:
      if (v != 0 && v != 1) return fail(GC_KPP_EINVAL, "rates-direct must be 0 or 1");
      c->rates_direct = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_BLOCK_SPLIT:
      if (v != 0 && v != 1) return fail(GC_KPP_EINVAL, "block-split must be 0 or 1");
      c->block_split = (int)v;
      return GC_KPP_OK;
    case GC_KPP_OPT_MAX_SLOTS:
      if (v < 0) return fail(GC_KPP_EINVAL, "max slots must be >= 0");
      c->max_slots = v;
      return GC_KPP_OK;
    default:
      return fail(GC_KPP_EINVAL, "unknown option key");
  }
}

}  // extern "C"

namespace {

// Options of INTEGRATE/Rosenbrock after merging the caller's ICNTRL_U/RCNTRL_U
// (gckpp_Integrator.F90:101-117, :333-477).
struct Resolved {
  int code = 0;  // per-cell IERR for an option error, 0 if none
  RosMethod meth{};
  bool vector_tol = true;
  int max_steps = 200000;
  double hmin = 0, hmax = 0, hstart_default = 0, facmin = 0, facmax = 0, facrej = 0, facsafe = 0;
  int autonomous = 1, clamp = 0;
  // auto-reduction (Rosenbrock :388-394, :478-487): ICNTRL(12) = 1
  int autoreduce = 0, ar_target = 0, ar_append = 0;
  double ar_thr = 1.0e2, ar_ratio = 0.0;
};

int resolve(const int* icntrl_u, const double* rcntrl_u, double tin, double tout, Resolved& R) {
  int icntrl[20] = {0};
  double rcntrl[20] = {0.0};
  icntrl[14] = 5;
  if (icntrl_u)
    for (int i = 0; i < 20; ++i)
      if (icntrl_u[i] != 0) icntrl[i] = icntrl_u[i];
  if (rcntrl_u)
    for (int i = 0; i < 20; ++i)
      if (rcntrl_u[i] > 0) rcntrl[i] = rcntrl_u[i];
  // Integrator_Update_Options (gckpp_Util.F90:179-205): rate or sun updates
  // inside the integrator need the met state, which this path does not take.
  if (icntrl[14] != -1 && (icntrl[14] & 5))
    return fail(GC_KPP_EUNSUPPORTED, "ICNTRL(15) requests Update_RCONST/Update_SUN inside the integrator");
  if (icntrl[11] == 1) {
    if (icntrl[13] < 0 || icntrl[13] > T::NVAR)
      return fail(GC_KPP_EUNSUPPORTED, "auto-reduce target species ICNTRL(14) out of range");
    R.autoreduce = 1;
    R.ar_target = icntrl[13];
    R.ar_append = icntrl[12] == 1 ? 1 : 0;  // ros_yIntegratorA
    if (rcntrl[11] > 0.0) R.ar_thr = rcntrl[11];
    R.ar_ratio = rcntrl[13];
  }
  R.vector_tol = icntrl[1] == 0;
  if (!method_table(icntrl[2], R.meth)) R.code = -2;
  if (!R.code) {
    if (icntrl[3] > 0) R.max_steps = icntrl[3];
    else if (icntrl[3] < 0) R.code = -1;
  }
  const double span = std::fabs(tout - tin);
  R.hmin = rcntrl[0];
  R.hmax = rcntrl[1] == 0.0 ? span : std::min(std::fabs(rcntrl[1]), span);
  R.hstart_default = rcntrl[2] == 0.0 ? std::max(R.hmin, 1.0e-5) : std::min(std::fabs(rcntrl[2]), span);
  R.facmin = rcntrl[3] == 0.0 ? 0.2 : rcntrl[3];
  R.facmax = rcntrl[4] == 0.0 ? 6.0 : rcntrl[4];
  R.facrej = rcntrl[5] == 0.0 ? 0.1 : rcntrl[5];
  R.facsafe = rcntrl[6] == 0.0 ? 0.9 : rcntrl[6];
  R.autonomous = icntrl[0] != 0 ? 1 : 0;
  R.clamp = icntrl[15] == 1 ? 1 : 0;
  return GC_KPP_OK;
}

// Tolerance check of Rosenbrock (:464-472) on host copies.
int check_tolerances(const double* atol, const double* rtol, int mem, bool vector_tol, cudaStream_t s, Resolved& R) {
  const size_t ntol = vector_tol ? T::NVAR : 1;
  std::vector<double> at(ntol), rt(ntol);
  if (mem == GC_KPP_MEM_HOST) {
    std::memcpy(at.data(), atol, ntol * sizeof(double));
    std::memcpy(rt.data(), rtol, ntol * sizeof(double));
  } else {
    GC_CUDA(cudaMemcpyAsync(at.data(), atol, ntol * sizeof(double), cudaMemcpyDeviceToHost, s));
    GC_CUDA(cudaMemcpyAsync(rt.data(), rtol, ntol * sizeof(double), cudaMemcpyDeviceToHost, s));
    GC_CUDA(cudaStreamSynchronize(s));
  }
  for (size_t i = 0; i < ntol; ++i)
    if (!(at[i] > 0.0) || rt[i] <= 10.0 * DBL_EPSILON || rt[i] >= 1.0) R.code = -5;
  return GC_KPP_OK;
}

struct DevArgs {
  int ncell;
  const int* order;  // optional cell list
  int cell_limit;    // cell ids lie in [0, cell_limit); 0 = ncell
  int nblock;        // the first nblock cells of order run block-per-cell
  const int* nblock_dev;  // or: that count in device memory (no host synchronisation)
  const int* qrange;      // or: device {begin, end} of the order positions to integrate
  int block_only;         // every cell of the range block-per-cell (no queue kernel)
  const double* c_in;
  double* c_out;
  long long ldc;
  const double* rconst;
  long long ldr;
  const double* atol;
  const double* rtol;
  const double* hstart;
  int* istatus;
  double* rstatus;
  long long ldo;
  int* ierr;
};

// Kernel variant by GC_KPP_OPT_ARITH: 0 fast, 1 strict (both 1 cell per
// thread), 2 fast with 2 cells per thread, 3 fast with 4.
cudaError_t variant_launch(int arith, int queue, int grid, int block, const MechDev& m, const RosMethod& r,
                           const RosParams& p, cudaStream_t s, int ar = 0) {
  switch (arith) {
    case 1: return gckpp_launch_ros_strict(queue, grid, block, m, r, p, s, ar);
    case 2: return gckpp_launch_ros_fast2(queue, grid, block, m, r, p, s, ar);
    case 3: return gckpp_launch_ros_fast4(queue, grid, block, m, r, p, s, ar);
    default: return gckpp_launch_ros_fast(queue, grid, block, m, r, p, s, ar);
  }
}

cudaError_t variant_occupancy(int arith, int block, int* nblocks) {
  switch (arith) {
    case 1: return gckpp_occupancy_strict(1, block, nblocks);
    case 2: return gckpp_occupancy_fast2(1, block, nblocks);
    case 3: return gckpp_occupancy_fast4(1, block, nblocks);
    default: return gckpp_occupancy_fast(1, block, nblocks);
  }
}

int variant_cells_per_thread(int arith) {
  switch (arith) {
    case 1: return gckpp_cells_per_thread_strict();
    case 2: return gckpp_cells_per_thread_fast2();
    case 3: return gckpp_cells_per_thread_fast4();
    default: return gckpp_cells_per_thread_fast();
  }
}

// Grid of the block-per-cell kernel (resident blocks per SM x SMs, at most
// `want` if positive) and its Jac0 slots.
int block_grid(gc_kpp_ctx* c, const Resolved& R, int autonomous, long long want, int* grid, double** ws) {
  const bool split = c->arith != 1 && c->block_split;
  const size_t smem = c->arith == 1 ? gckpp_block_smem_strict(c->mech, R.meth, autonomous)
                      : split       ? gckpp_block_smem_split(c->mech, R.meth, autonomous)
                                    : gckpp_block_smem_fast(c->mech, R.meth, autonomous);
  // smem < 2^18 bytes, arith < 4, cell_block / 32 <= 32
  const int key = (int)smem + (c->arith << 18) + ((c->cell_block / 32) << 20) + ((split ? 1 : 0) << 26);
  if (c->bocc_key != key) {
    int occ = 0;
    cudaError_t e = c->arith == 1 ? gckpp_block_occupancy_strict(c->cell_block, smem, &occ)
                    : split       ? gckpp_block_occupancy_split(smem, &occ)
                                  : gckpp_block_occupancy_fast(c->cell_block, smem, &occ);
    if (e != cudaSuccess) return cuda_fail(e, "block-per-cell occupancy");
    if (occ < 1) return fail(GC_KPP_EUNSUPPORTED, "block-per-cell kernel does not fit an SM");
    c->bocc_key = key;
    c->bocc_value = occ;
  }
  long long g = (long long)c->nsm * c->bocc_value;
  if (want > 0 && want < g) g = want;
  *grid = (int)g;
  const BlockLayout bl = block_layout(T::NAUX, T::NSPEC, T::NVAR, T::NREACT, T::NB, T::LU_NONZERO, R.meth.S,
                                      autonomous);
  GC_CUDA(c->bws.ensure((size_t)g * bl.slot * sizeof(double)));
  *ws = (double*)c->bws.p;
  return GC_KPP_OK;
}

// Launch of the block-per-cell kernel of the context's arithmetic.
cudaError_t launch_block(gc_kpp_ctx* c, int grid, const Resolved& R, const RosParams& p, cudaStream_t s) {
  if (c->arith == 1) return gckpp_launch_block_strict(grid, c->cell_block, c->mech, R.meth, p, s);
  if (c->block_split) return gckpp_launch_block_split(grid, c->mech, R.meth, p, s);
  return gckpp_launch_block_fast(grid, c->cell_block, c->mech, R.meth, p, s);
}

// Launch the Rosenbrock kernel over device arrays.  A thread holds `nc`
// cells, so a block covers block*nc workspace slots.
int launch_integrate(gc_kpp_ctx* c, const Resolved& R, double tin, double tout, const DevArgs& a, cudaStream_t s,
                     int* launches) {
  const int queue = c->schedule;
  const int block = c->block;
  const int nc = variant_cells_per_thread(c->arith);
  const long long per_block = (long long)block * nc;
  // the first a.nblock cells of a.order run block-per-cell, the rest on the
  // thread-per-cell kernel
  const int nb = a.nblock;
  if (nb < 0 || nb > a.ncell) return fail(GC_KPP_EINVAL, "block-per-cell count outside [0, ncell]");
  if (nb > 0 && !a.order) return fail(GC_KPP_EINVAL, "block-per-cell cells need a cell order");
  const bool dev_split = a.nblock_dev != nullptr;
  if ((nb > 0 || dev_split) && (c->arith > 1 || c->lu_form != 0))
    return fail(GC_KPP_EUNSUPPORTED, "block-per-cell cells need ARITH 0 or 1 and the row-wise LU");
  if ((dev_split || a.qrange) && !queue)
    return fail(GC_KPP_EINVAL, "cell counts held on the device need the queue schedule");
  // auto-reduction runs on the thread-per-cell kernel alone (1 cell per
  // thread, row-wise LU): no block-per-cell routing, no hand-over
  if (R.autoreduce && (nb > 0 || dev_split || a.block_only || c->arith > 1 || c->lu_form != 0))
    return fail(GC_KPP_EUNSUPPORTED,
                "auto-reduce needs ARITH 0 or 1, the row-wise LU and no block-per-cell cells");
  if (R.autoreduce && c->ar_ncell > 0 && (a.cell_limit > 0 ? a.cell_limit : a.ncell) != c->ar_ncell)
    return fail(GC_KPP_EINVAL, "auto-reduce controls were set for a different number of cells");
  const WsLayout lay = make_layout(R.autoreduce != 0);
  if (dev_split && (!a.order || nb != 0)) return fail(GC_KPP_EINVAL, "device block-per-cell count needs an order");
  // with counts on the device, size for every cell; the kernels read the ranges
  const long long nthread = (dev_split || a.qrange) ? (long long)a.ncell : (long long)a.ncell - nb;
  long long nslot, ws_slots = 0;
  int grid;
  if (queue) {
    int per_sm = c->blocks_per_sm;
    if (per_sm == 0) {
      // resident blocks per SM of this variant and block size (cached)
      if (c->occ_arith != c->arith || c->occ_block != block) {
        cudaError_t e = variant_occupancy(c->arith, block, &c->occ_value);
        if (e != cudaSuccess) return cuda_fail(e, "occupancy");
        c->occ_arith = c->arith;
        c->occ_block = block;
      }
      per_sm = std::max(c->occ_value, 1);
    }
    grid = c->nsm * per_sm;
    const long long need_blocks = std::max(1LL, (nthread + per_block - 1) / per_block);
    if (grid > need_blocks) grid = (int)need_blocks;
    if (c->max_slots > 0 && (long long)grid * per_block > c->max_slots)
      grid = (int)std::max(1LL, c->max_slots / per_block);
    nslot = (long long)grid * per_block;
    // the workspace is sized for every cell of the call on the queue kernel,
    // whatever share goes block-per-cell, so that an asynchronous call of the
    // same batch (possibly inside a capture) never has to grow it
    long long all = std::min<long long>((long long)c->nsm * per_sm,
                                        std::max(1LL, ((long long)a.ncell + per_block - 1) / per_block));
    if (c->max_slots > 0 && all * per_block > c->max_slots) all = std::max(1LL, c->max_slots / per_block);
    ws_slots = std::max(nslot, all * per_block);
  } else {
    grid = (int)std::max(1LL, (nthread + per_block - 1) / per_block);
    nslot = (long long)grid * per_block;
    if (c->max_slots > 0 && nslot > c->max_slots)
      return fail(GC_KPP_EINVAL, "plain schedule needs one workspace slot per cell; raise MAX_SLOTS or use the queue");
  }
  const size_t ws_bytes = (size_t)std::max(nslot, ws_slots) * (size_t)lay.total * sizeof(double);
  GC_CUDA(c->ws.ensure(ws_bytes));
  GC_CUDA(c->counter.ensure(2 * sizeof(int)));
  GC_CUDA(cudaMemsetAsync(c->counter.p, 0, 2 * sizeof(int), s));
  GC_CUDA(c->ranges.ensure(8 * sizeof(int)));
  int* ranges = (int*)c->ranges.p;
  if (dev_split) {
    cudaError_t e = gcutil::split_ranges(a.nblock_dev, a.ncell, ranges, s);
    if (e != cudaSuccess) return cuda_fail(e, "range kernel launch");
    if (launches) *launches += 1;
  }
  RosParams p{};
  p.ncell = (int)nthread;
  p.order = a.order ? a.order + nb : nullptr;
  p.qrange = dev_split ? ranges + 2 : a.qrange;
  // hand-over of long-running cells (needs the status rows to carry their state)
  const bool evict = c->evict_after > 0 && queue && c->arith <= 1 && c->lu_form == 0 && a.istatus && a.rstatus &&
                     !R.autoreduce;
  if (evict) {
    GC_CUDA(c->evict_buf.ensure((size_t)std::max(a.ncell, 1) * sizeof(int)));
    GC_CUDA(cudaMemsetAsync(ranges + 6, 0, 2 * sizeof(int), s));
    p.evict_after = c->evict_after;
    p.evict_drained = c->evict_drained;
    p.evict_list = (int*)c->evict_buf.p;
    p.evict_count = ranges + 7;
  }
  p.cell_limit = a.cell_limit > 0 ? a.cell_limit : a.ncell;
  p.queue_counter = (int*)c->counter.p;
  p.queue_chunk = c->queue_chunk;
  p.c_in = a.c_in;
  p.c_out = a.c_out;
  p.ldc = a.ldc;
  p.rconst = a.rconst;
  p.ldr = a.ldr;
  p.hstart = a.hstart;
  p.istatus = a.istatus;
  p.rstatus = a.rstatus;
  p.ldo = a.ldo;
  p.ierr = a.ierr;
  p.atol = a.atol;
  p.rtol = a.rtol;
  p.vector_tol = R.vector_tol ? 1 : 0;
  p.tstart = tin;
  p.tend = tout;
  p.hmin = R.hmin;
  p.hmax = R.hmax;
  p.hstart_default = R.hstart_default;
  p.facmin = R.facmin;
  p.facmax = R.facmax;
  p.facrej = R.facrej;
  p.facsafe = R.facsafe;
  p.roundoff = DBL_EPSILON;  // WLAMCH('E') = 2**-52
  p.autonomous = R.autonomous;
  p.max_steps = R.max_steps;
  p.clamp_negative = R.clamp;
  p.lu_form = c->lu_form;
  p.ar_target = R.ar_target;
  p.ar_append = R.ar_append;
  p.ar_thr = R.ar_thr;
  p.ar_ratio = R.ar_ratio;
  if (R.autoreduce) {
    p.ar_thr_cell = c->ar_has_thr ? (const double*)c->ar_thr.p : nullptr;
    p.ar_target_cell = c->ar_has_tgt ? (const int*)c->ar_tgt.p : nullptr;
    p.ar_ratio_cell = c->ar_has_ratio ? (const double*)c->ar_ratio.p : nullptr;
    p.ar_keep = c->ar_keep_on ? (const unsigned char*)c->ar_keep.p : nullptr;
  }
  p.ws = (double*)c->ws.p;
  p.lay = lay;
  p.nslot = nslot;
  const bool timed = c->timing && !c->async && c->ntimed < 4;
  if (timed) {
    for (int i = 2 * c->ntimed; i < 2 * c->ntimed + 2; ++i)
      if (!c->ev[i]) GC_CUDA(cudaEventCreate(&c->ev[i]));
    GC_CUDA(cudaEventRecord(c->ev[2 * c->ntimed], s));
  }
  if (nb > 0 || dev_split) {
    if (!c->side) GC_CUDA(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    if (!c->fork) GC_CUDA(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
    if (!c->join) GC_CUDA(cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming));
    GC_CUDA(cudaEventRecord(c->fork, s));
    GC_CUDA(cudaStreamWaitEvent(c->side, c->fork, 0));
    RosParams pb = p;
    pb.ncell = dev_split ? a.ncell : nb;
    pb.order = a.order;
    pb.qrange = dev_split ? ranges : nullptr;
    pb.queue_counter = (int*)c->counter.p + 1;
    pb.nslot = 0;
    int bgrid = 0;
    GC_TRY(block_grid(c, R, p.autonomous, dev_split ? 0 : nb, &bgrid, &pb.ws));
    cudaError_t eb = launch_block(c, bgrid, R, pb, c->side);
    if (eb != cudaSuccess) return cuda_fail(eb, "block-per-cell kernel launch");
    GC_CUDA(cudaEventRecord(c->join, c->side));
    if (launches) *launches += 1;
  }
  if (a.block_only) {
    if (c->arith > 1 || c->lu_form != 0 || !a.qrange)
      return fail(GC_KPP_EINVAL, "block-only launches need a device range, ARITH 0 or 1 and the row-wise LU");
    RosParams pb = p;
    pb.queue_counter = (int*)c->counter.p + 1;
    pb.evict_after = 0;
    pb.nslot = 0;
    int bgrid = 0;
    GC_TRY(block_grid(c, R, p.autonomous, 0, &bgrid, &pb.ws));
    cudaError_t eb = launch_block(c, bgrid, R, pb, s);
    if (eb != cudaSuccess) return cuda_fail(eb, "block-per-cell kernel launch");
    if (launches) *launches += 1;
    if (timed) {
      GC_CUDA(cudaEventRecord(c->ev[2 * c->ntimed + 1], s));
      c->ntimed += 1;
    }
    return GC_KPP_OK;
  }
  if (nthread > 0) {
    cudaError_t e = variant_launch(c->arith, queue, grid, block, c->mech, R.meth, p, s, R.autoreduce);
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    if (launches) *launches += 1;
  }
  if (nb > 0 || dev_split) GC_CUDA(cudaStreamWaitEvent(s, c->join, 0));
  if (evict) {
    // the handed-over cells continue block-per-cell from their saved state
    RosParams pr = p;
    pr.resume = 1;
    pr.evict_after = 0;
    pr.order = (const int*)c->evict_buf.p;
    pr.qrange = ranges + 6;
    pr.ncell = a.ncell;
    pr.c_in = p.c_out;
    pr.hstart = nullptr;
    pr.queue_counter = (int*)c->counter.p + 1;
    pr.nslot = 0;
    int rgrid = 0;
    GC_TRY(block_grid(c, R, p.autonomous, 0, &rgrid, &pr.ws));
    GC_CUDA(cudaMemsetAsync(pr.queue_counter, 0, sizeof(int), s));
    cudaError_t er = launch_block(c, rgrid, R, pr, s);
    if (er != cudaSuccess) return cuda_fail(er, "block-per-cell continuation launch");
    if (launches) *launches += 1;
  }
  if (timed) {
    GC_CUDA(cudaEventRecord(c->ev[2 * c->ntimed + 1], s));
    c->ntimed += 1;
  }
  return GC_KPP_OK;
}

// Write the per-call option error into every cell's outputs (device arrays).
int fill_option_error(int code, int ncell, int* ierr, int* istatus, double* rstatus, long long ldo, cudaStream_t s) {
  std::vector<int> e(ncell, code);
  GC_CUDA(cudaMemcpyAsync(ierr, e.data(), ncell * sizeof(int), cudaMemcpyHostToDevice, s));
  if (istatus) GC_CUDA(cudaMemset2DAsync(istatus, ldo * sizeof(int), 0, ncell * sizeof(int), 20, s));
  if (rstatus) GC_CUDA(cudaMemset2DAsync(rstatus, ldo * sizeof(double), 0, ncell * sizeof(double), 20, s));
  GC_CUDA(cudaStreamSynchronize(s));
  return GC_KPP_OK;
}

template <typename X>
int stage_in(DevBuf& buf, const X* host, long long ld, size_t ncell, size_t rows, cudaStream_t s, X** dev) {
  GC_CUDA(buf.ensure(rows * ncell * sizeof(X)));
  *dev = (X*)buf.p;
  if (host)
    GC_CUDA(gcutil::copy_rows(buf.p, ncell * sizeof(X), host, ld * sizeof(X), ncell * sizeof(X), rows, s));
  return GC_KPP_OK;
}

// The PHOTOL rows that the rate program reads, staged into a device buffer
// of all GC_KPP_NPHOTOL rows (the others are never read).
int stage_photol(DevBuf& buf, const double* host, long long ld, size_t ncell, cudaStream_t s, double** dev) {
  GC_TRY(stage_in<double>(buf, nullptr, ld, ncell, GC_KPP_NPHOTOL, s, dev));
  for (int r = 0; r < RT::NPHOTOL_RUNS; ++r) {
    const int a = RT::photol_runs[2 * r], b = RT::photol_runs[2 * r + 1];
    GC_CUDA(gcutil::copy_rows(*dev + (size_t)a * ncell, ncell * sizeof(double), host + (long long)a * ld,
                              ld * sizeof(double), ncell * sizeof(double), b - a, s));
  }
  return GC_KPP_OK;
}

template <typename X>
int stage_out(X* host, long long ld, const X* dev, size_t ncell, size_t rows, cudaStream_t s) {
  GC_CUDA(gcutil::copy_rows(host, ld * sizeof(X), dev, ncell * sizeof(X), ncell * sizeof(X), rows, s));
  return GC_KPP_OK;
}


}  // namespace

extern "C" {

int gc_kpp_integrate_batch(gc_kpp_ctx* c, int ncell, double tin, double tout, double* cc, long long ldc,
                           const double* rconst, long long ldr, const double* atol, const double* rtol,
                           const int* icntrl_u, const double* rcntrl_u, const double* hstart, int* istatus,
                           double* rstatus, long long ldo, int* ierr, int mem, void* stream) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  if (ncell < 0) return fail(GC_KPP_EINVAL, "ncell < 0");
  if (ncell == 0) return GC_KPP_OK;
  if (!cc || !rconst || !atol || !rtol || !ierr) return fail(GC_KPP_EINVAL, "required array is NULL");
  if (ldc < ncell || ldr < ncell || ((istatus || rstatus) && ldo < ncell))
    return fail(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  GC_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  c->ntimed = 0;
  Resolved R;
  GC_TRY(resolve(icntrl_u, rcntrl_u, tin, tout, R));
  if (!R.code) GC_TRY(check_tolerances(atol, rtol, mem, R.vector_tol, s, R));
  const size_t n = (size_t)ncell, ntol = R.vector_tol ? T::NVAR : 1;
  DevArgs a{};
  a.ncell = ncell;
  if (mem == GC_KPP_MEM_HOST) {
    double *dc, *dr, *dat, *drt, *dhs = nullptr, *drs = nullptr;
    int *dis = nullptr, *die;
    GC_TRY(stage_in(c->h_c, cc, ldc, n, T::NSPEC, s, &dc));
    GC_TRY(stage_in(c->h_r, rconst, ldr, n, T::NREACT, s, &dr));
    GC_TRY(stage_in(c->h_at, atol, (long long)ntol, ntol, 1, s, &dat));
    GC_TRY(stage_in(c->h_rt, rtol, (long long)ntol, ntol, 1, s, &drt));
    if (hstart) GC_TRY(stage_in(c->h_hs, hstart, ncell, n, 1, s, &dhs));
    if (istatus) GC_TRY(stage_in<int>(c->h_is, nullptr, ncell, n, 20, s, &dis));
    if (rstatus) GC_TRY(stage_in<double>(c->h_rs, nullptr, ncell, n, 20, s, &drs));
    GC_TRY(stage_in<int>(c->h_ie, nullptr, ncell, n, 1, s, &die));
    a.c_in = dc; a.c_out = dc; a.ldc = ncell; a.rconst = dr; a.ldr = ncell; a.atol = dat; a.rtol = drt;
    a.hstart = dhs; a.istatus = dis; a.rstatus = drs; a.ldo = ncell; a.ierr = die;
  } else {
    a.c_in = cc; a.c_out = cc; a.ldc = ldc; a.rconst = rconst; a.ldr = ldr; a.atol = atol; a.rtol = rtol;
    a.hstart = hstart; a.istatus = istatus; a.rstatus = rstatus; a.ldo = ldo; a.ierr = ierr;
  }
  if (R.code) {
    GC_TRY(fill_option_error(R.code, ncell, a.ierr, a.istatus, a.rstatus, a.ldo, s));
  } else {
    GC_TRY(launch_integrate(c, R, tin, tout, a, s, nullptr));
  }
  if (mem == GC_KPP_MEM_HOST) {
    GC_TRY(stage_out(cc, ldc, (const double*)a.c_out, n, T::NVAR, s));
    GC_TRY(stage_out(ierr, ncell, (const int*)a.ierr, n, 1, s));
    if (istatus) GC_TRY(stage_out(istatus, ldo, (const int*)a.istatus, n, 20, s));
    if (rstatus) GC_TRY(stage_out(rstatus, ldo, (const double*)a.rstatus, n, 20, s));
    GC_CUDA(cudaStreamSynchronize(s));
  }
  return GC_KPP_OK;
}

static int fullchem_step_impl(gc_kpp_ctx* c, int ncell, double dt, const double* met, long long ldm,
                              const double* photol, long long ldp, double* cc, long long ldc, const double* atol,
                              const double* rtol, const int* icntrl_u, const double* rcntrl_u, double* hstart,
                              int* istatus, double* rstatus, long long ldo, int* ierr, int* nretry,
                              const int* order, int nblock, const int* nblock_dev, int mem, void* stream) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  if (ncell < 0) return fail(GC_KPP_EINVAL, "ncell < 0");
  if (nretry) *nretry = 0;
  if (ncell == 0) return GC_KPP_OK;
  if (!met || !photol || !cc || !atol || !rtol || !ierr) return fail(GC_KPP_EINVAL, "required array is NULL");
  if (ldm < ncell || ldp < ncell || ldc < ncell || ((istatus || rstatus) && ldo < ncell))
    return fail(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  GC_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  c->ntimed = 0;
  Resolved R;
  GC_TRY(resolve(icntrl_u, rcntrl_u, 0.0, dt, R));
  const bool async = c->async != 0;
  if (async && (mem != GC_KPP_MEM_DEVICE || !c->schedule))
    return fail(GC_KPP_EINVAL, "asynchronous steps need device memory and the queue schedule");
  if (!R.code) {
    if (async) {
      // the tolerance check reads the arrays on the host; asynchronous steps
      // reuse arrays that a synchronous step has checked
      if (atol != c->tol_at || rtol != c->tol_rt || (int)R.vector_tol != c->tol_vec)
        return fail(GC_KPP_EINVAL, "asynchronous steps need tolerance arrays checked by a synchronous step first");
    } else {
      GC_TRY(check_tolerances(atol, rtol, mem, R.vector_tol, s, R));
      if (!R.code && mem == GC_KPP_MEM_DEVICE) {
        c->tol_at = atol;
        c->tol_rt = rtol;
        c->tol_vec = R.vector_tol ? 1 : 0;
      }
    }
  }
  const size_t n = (size_t)ncell, ntol = R.vector_tol ? T::NVAR : 1;
  GC_CUDA(c->ord_buf.ensure(n * sizeof(int)));  // retry list, sized before any capture
  if (c->arith <= 1 && c->lu_form == 0 && !R.code) {
    // the block-per-cell kernel's attributes and slots (asynchronous retries
    // use it), set up by synchronous calls so that a capture never allocates
    int g = 0;
    double* w = nullptr;
    GC_TRY(block_grid(c, R, R.autonomous, 0, &g, &w));
  }
  const double *dmet, *dph, *dat, *drt;
  double *dc, *dhs = nullptr, *drs;
  int *dis, *die;
  const int* dorder = nullptr;
  long long lm, lp, lc, lo;
  if (order && mem == GC_KPP_MEM_HOST) {
    // a host order list must be a permutation of the cells
    std::vector<char> seen(n, 0);
    for (int i = 0; i < ncell; ++i) {
      if (order[i] < 0 || order[i] >= ncell || seen[order[i]])
        return fail(GC_KPP_EINVAL, "order is not a permutation of 0..ncell-1");
      seen[order[i]] = 1;
    }
  }
  if (mem == GC_KPP_MEM_HOST) {
    double* tmp;
    if (order) {
      int* t;
      GC_TRY(stage_in<int>(c->h_ord, order, ncell, n, 1, s, &t));
      dorder = t;
    }
    GC_TRY(stage_in(c->h_met, met, ldm, n, RT::NMET, s, &tmp)); dmet = tmp;
    GC_TRY(stage_photol(c->h_ph, photol, ldp, n, s, &tmp)); dph = tmp;
    GC_TRY(stage_in(c->h_c, (const double*)cc, ldc, n, T::NSPEC, s, &dc));
    GC_TRY(stage_in(c->h_at, atol, (long long)ntol, ntol, 1, s, &tmp)); dat = tmp;
    GC_TRY(stage_in(c->h_rt, rtol, (long long)ntol, ntol, 1, s, &tmp)); drt = tmp;
    if (hstart) GC_TRY(stage_in(c->h_hs, (const double*)hstart, ncell, n, 1, s, &dhs));
    GC_TRY(stage_in<int>(c->h_is, nullptr, ncell, n, 20, s, &dis));
    GC_TRY(stage_in<double>(c->h_rs, nullptr, ncell, n, 20, s, &drs));
    GC_TRY(stage_in<int>(c->h_ie, nullptr, ncell, n, 1, s, &die));
    lm = lp = lc = lo = ncell;
  } else {
    dmet = met; dph = photol; dc = cc; dat = atol; drt = rtol; dhs = hstart; lm = ldm; lp = ldp; lc = ldc;
    die = ierr;
    dorder = order;
    if (istatus && rstatus) {
      dis = istatus; drs = rstatus; lo = ldo;
    } else {
      GC_TRY(stage_in<int>(c->h_is, nullptr, ncell, n, 20, s, &dis));
      GC_TRY(stage_in<double>(c->h_rs, nullptr, ncell, n, 20, s, &drs));
      lo = ncell;
    }
  }
  // zero the prod/loss family dummies (fullchem_mod.F90:943-946)
  for (int f = 0; f < (int)(sizeof(T::family_species) / sizeof(int)); ++f)
    GC_CUDA(cudaMemsetAsync(dc + (long long)T::family_species[f] * lc, 0, n * sizeof(double), s));
  // Update_RCONST (fullchem_mod.F90:953)
  double* drc;
  GC_TRY(stage_in<double>(c->rc_buf, nullptr, ncell, n, T::NREACT, s, &drc));
  gcrates::RatesArgs ra{};
  ra.ncell = ncell; ra.met = dmet; ra.ldm = lm; ra.photol = dph; ra.ldp = lp; ra.c = dc; ra.ldc = lc;
  ra.rconst = drc; ra.ldr = ncell;
  if (c->het) {
    if (c->het_ncell != ncell) return fail(GC_KPP_EINVAL, "HetState was set for a different number of cells");
    ra.het = c->het;
    ra.ldh = c->het_ld;
  }
  cudaError_t e = c->rates_direct ? gcrates::launch_rates_direct(c->rates, ra, s) : gcrates::launch_rates(c->rates, ra, s);
  if (e != cudaSuccess) return cuda_fail(e, "rates kernel launch");
  c->last_launches = 1;
  if (R.code && async) {
    e = gcutil::fill_error(R.code, ncell, die, dis, drs, lo, s);
    if (e != cudaSuccess) return cuda_fail(e, "error fill kernel launch");
    c->last_launches += 1;
  } else if (R.code) {
    GC_TRY(fill_option_error(R.code, ncell, die, dis, drs, lo, s));
  } else {
    // C_before_integrate (fullchem_mod.F90:1023), same leading dimension as C
    double* dcb;
    GC_TRY(stage_in<double>(c->cb_buf, nullptr, lc, (size_t)lc, T::NSPEC, s, &dcb));
    GC_CUDA(cudaMemcpyAsync(dcb, dc, (size_t)lc * T::NSPEC * sizeof(double), cudaMemcpyDeviceToDevice, s));
    DevArgs a{};
    a.ncell = ncell; a.c_in = dc; a.c_out = dc; a.ldc = lc; a.rconst = drc; a.ldr = ncell; a.atol = dat;
    a.rtol = drt; a.hstart = dhs; a.istatus = dis; a.rstatus = drs; a.ldo = lo; a.ierr = die;
    a.order = dorder; a.cell_limit = ncell; a.nblock = nblock; a.nblock_dev = nblock_dev;
    GC_TRY(launch_integrate(c, R, 0.0, dt, a, s, &c->last_launches));
    if (async) {
      // retry list built on the device; the retry launch reads its length there
      int* ranges = (int*)c->ranges.p;
      e = gcutil::collect_failed(die, ncell, (int*)c->ord_buf.p, ranges + 4, s);
      if (e != cudaSuccess) return cuda_fail(e, "retry list kernel launch");
      c->last_launches += 1;
      DevArgs b = a;
      b.order = (const int*)c->ord_buf.p;
      b.qrange = ranges + 4;
      b.nblock = 0;
      b.nblock_dev = nullptr;
      // retries are few: latency form (auto-reduction runs on the thread kernel)
      b.block_only = (c->arith <= 1 && c->lu_form == 0 && !R.autoreduce) ? 1 : 0;
      b.cell_limit = ncell;
      b.c_in = dcb;
      b.hstart = nullptr;
      Resolved R2 = R;
      R2.hstart_default = std::max(R.hmin, 1.0e-5);
      if (nretry) *nretry = -1;
      GC_TRY(launch_integrate(c, R2, 0.0, dt, b, s, &c->last_launches));
    }
    // retry failed cells once with Hstart = 0 from C_before
    // (fullchem_mod.F90:1138-1162)
    std::vector<int> hier(async ? 0 : n);
    if (!async) {
    GC_CUDA(cudaMemcpyAsync(hier.data(), die, n * sizeof(int), cudaMemcpyDeviceToHost, s));
    GC_CUDA(cudaStreamSynchronize(s));
    std::vector<int> failed;
    for (int i = 0; i < ncell; ++i)
      if (hier[i] < 0) failed.push_back(i);
    if (!failed.empty()) {
      int* dord;
      GC_TRY(stage_in<int>(c->ord_buf, failed.data(), (long long)failed.size(), failed.size(), 1, s, &dord));
      // the failed cells restart from C_before (c_in) and overwrite their
      // entries of C (c_out); Hstart = RCNTRL(3) = 0 -> DeltaMin
      DevArgs b = a;
      b.ncell = (int)failed.size();
      b.order = dord;
      b.cell_limit = ncell;
      // a few cells integrate faster one per block than on the queue kernel
      b.nblock = (c->arith <= 1 && c->lu_form == 0 && !R.autoreduce && (long long)failed.size() <= 4LL * c->nsm)
                     ? (int)failed.size() : 0;
      b.nblock_dev = nullptr;
      b.qrange = nullptr;
      b.c_in = dcb;
      b.hstart = nullptr;
      Resolved R2 = R;
      R2.hstart_default = std::max(R.hmin, 1.0e-5);
      if (nretry) *nretry = (int)failed.size();
      GC_TRY(launch_integrate(c, R2, 0.0, dt, b, s, &c->last_launches));
    }
    }
    // C = MAX(C, 0) (fullchem_mod.F90:1329-1350)
    e = gcutil::clamp_nonneg(dc, lc, T::NSPEC, ncell, s);
    if (e != cudaSuccess) return cuda_fail(e, "clamp kernel launch");
    c->last_launches += 1;
    // KPPHvalue = RSTATE(Nhnew) (fullchem_mod.F90:1294)
    if (dhs)
      GC_CUDA(cudaMemcpyAsync(dhs, drs + 2 * lo, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  if (mem == GC_KPP_MEM_HOST) {
    GC_TRY(stage_out(cc, ldc, (const double*)dc, n, T::NSPEC, s));
    GC_TRY(stage_out(ierr, ncell, (const int*)die, n, 1, s));
    if (istatus) GC_TRY(stage_out(istatus, ldo, (const int*)dis, n, 20, s));
    if (rstatus) GC_TRY(stage_out(rstatus, ldo, (const double*)drs, n, 20, s));
    if (hstart) GC_TRY(stage_out(hstart, ncell, (const double*)dhs, n, 1, s));
    GC_CUDA(cudaStreamSynchronize(s));
  }
  return GC_KPP_OK;
}

int gc_kpp_fullchem_step(gc_kpp_ctx* c, int ncell, double dt, const double* met, long long ldm,
                         const double* photol, long long ldp, double* cc, long long ldc, const double* atol,
                         const double* rtol, const int* icntrl_u, const double* rcntrl_u, double* hstart,
                         int* istatus, double* rstatus, long long ldo, int* ierr, int* nretry, int mem,
                         void* stream) {
  return fullchem_step_impl(c, ncell, dt, met, ldm, photol, ldp, cc, ldc, atol, rtol, icntrl_u, rcntrl_u, hstart,
                            istatus, rstatus, ldo, ierr, nretry, nullptr, 0, nullptr, mem, stream);
}

int gc_kpp_fullchem_step_ordered(gc_kpp_ctx* c, int ncell, double dt, const double* met, long long ldm,
                                 const double* photol, long long ldp, double* cc, long long ldc,
                                 const double* atol, const double* rtol, const int* icntrl_u,
                                 const double* rcntrl_u, double* hstart, int* istatus, double* rstatus,
                                 long long ldo, int* ierr, int* nretry, const int* order, int mem, void* stream) {
  return fullchem_step_impl(c, ncell, dt, met, ldm, photol, ldp, cc, ldc, atol, rtol, icntrl_u, rcntrl_u, hstart,
                            istatus, rstatus, ldo, ierr, nretry, order, 0, nullptr, mem, stream);
}

int gc_kpp_fullchem_step_binned(gc_kpp_ctx* c, int ncell, double dt, const double* met, long long ldm,
                                const double* photol, long long ldp, double* cc, long long ldc, const double* atol,
                                const double* rtol, const int* icntrl_u, const double* rcntrl_u, double* hstart,
                                int* istatus, double* rstatus, long long ldo, int* ierr, int* nretry,
                                const int* order, int nblock, int mem, void* stream) {
  if (nblock < 0 || nblock > ncell) return fail(GC_KPP_EINVAL, "nblock outside [0, ncell]");
  if (nblock > 0 && !order) return fail(GC_KPP_EINVAL, "nblock > 0 needs an order");
  return fullchem_step_impl(c, ncell, dt, met, ldm, photol, ldp, cc, ldc, atol, rtol, icntrl_u, rcntrl_u, hstart,
                            istatus, rstatus, ldo, ierr, nretry, order, nblock, nullptr, mem, stream);
}

int gc_kpp_last_launch_count(gc_kpp_ctx* c) { return c ? c->last_launches : 0; }

int gc_kpp_last_kernel_ms(gc_kpp_ctx* c, double* ms, int* nlaunch) {
  if (!c || !ms) return fail(GC_KPP_EINVAL, "NULL argument");
  double total = 0.0;
  for (int i = 0; i < c->ntimed; ++i) {
    GC_CUDA(cudaEventSynchronize(c->ev[2 * i + 1]));
    float t = 0.f;
    GC_CUDA(cudaEventElapsedTime(&t, c->ev[2 * i], c->ev[2 * i + 1]));
    total += t;
  }
  *ms = total;
  if (nlaunch) *nlaunch = c->ntimed;
  c->ntimed = 0;
  return GC_KPP_OK;
}

int gc_kpp_ctx_set_hetstate(gc_kpp_ctx* c, int ncell, const double* het, long long ldh, int mem) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  if (!het) {
    c->het = nullptr;
    c->het_ncell = 0;
    return GC_KPP_OK;
  }
  if (ncell <= 0 || ldh < ncell) return fail(GC_KPP_EINVAL, "bad ncell or leading dimension");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  GC_CUDA(cudaSetDevice(c->device));
  if (mem == GC_KPP_MEM_DEVICE) {
    c->het = het;
    c->het_ld = ldh;
  } else {
    const size_t n = (size_t)ncell;
    GC_CUDA(c->step_het.ensure((size_t)HET_NFIELD * n * sizeof(double)));
    GC_CUDA(cudaMemcpy2D(c->step_het.p, n * sizeof(double), het, ldh * sizeof(double), n * sizeof(double),
                         HET_NFIELD, cudaMemcpyHostToDevice));
    c->het = (const double*)c->step_het.p;
    c->het_ld = ncell;
  }
  c->het_ncell = ncell;
  return GC_KPP_OK;
}

int gc_kpp_ctx_set_autoreduce(gc_kpp_ctx* c, int ncell, const double* thr, const int* target, const double* ratio,
                              const unsigned char* keep, int mem) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  const bool cells = thr || target || ratio;
  if (cells && ncell <= 0) return fail(GC_KPP_EINVAL, "per-cell controls need ncell > 0");
  if (cells && mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  GC_CUDA(cudaSetDevice(c->device));
  const size_t n = cells ? (size_t)ncell : 0;
  const cudaMemcpyKind kind = mem == GC_KPP_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (target) {
    // ICNTRL(14) must name a variable species (or be 0) in every cell
    std::vector<int> t(n);
    GC_CUDA(cudaMemcpy(t.data(), target, n * sizeof(int),
                       mem == GC_KPP_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
    for (size_t i = 0; i < n; ++i)
      if (t[i] < 0 || t[i] > T::NVAR) return fail(GC_KPP_EUNSUPPORTED, "auto-reduce target species out of range");
    GC_CUDA(c->ar_tgt.ensure(n * sizeof(int)));
    GC_CUDA(cudaMemcpy(c->ar_tgt.p, t.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (thr) {
    GC_CUDA(c->ar_thr.ensure(n * sizeof(double)));
    GC_CUDA(cudaMemcpy(c->ar_thr.p, thr, n * sizeof(double), kind));
  }
  if (ratio) {
    GC_CUDA(c->ar_ratio.ensure(n * sizeof(double)));
    GC_CUDA(cudaMemcpy(c->ar_ratio.p, ratio, n * sizeof(double), kind));
  }
  if (keep) {
    unsigned char k[T::NVAR];
    for (int i = 0; i < T::NVAR; ++i) k[i] = keep[i] ? 1 : 0;
    GC_CUDA(c->ar_keep.ensure(sizeof(k)));
    GC_CUDA(cudaMemcpy(c->ar_keep.p, k, sizeof(k), cudaMemcpyHostToDevice));
  }
  c->ar_ncell = (int)n;
  c->ar_has_thr = thr != nullptr;
  c->ar_has_tgt = target != nullptr;
  c->ar_has_ratio = ratio != nullptr;
  c->ar_keep_on = keep != nullptr;
  return GC_KPP_OK;
}

int gc_kpp_update_rconst_batch(gc_kpp_ctx* c, int ncell, const double* met, long long ldm, const double* photol,
                               long long ldp, const double* conc, long long ldc, double* rconst, long long ldr, int mem,
                               void* stream) {
  return gc_kpp_update_rconst_het_batch(c, ncell, met, ldm, photol, ldp, conc, ldc, nullptr, 0, rconst, ldr, mem,
                                        stream);
}

int gc_kpp_update_rconst_het_batch(gc_kpp_ctx* c, int ncell, const double* met, long long ldm, const double* photol,
                                   long long ldp, const double* conc, long long ldc, const double* het, long long ldh,
                                   double* rconst, long long ldr, int mem, void* stream) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  if (ncell < 0) return fail(GC_KPP_EINVAL, "ncell < 0");
  if (ncell == 0) return GC_KPP_OK;
  if (!met || !photol || !conc || !rconst) return fail(GC_KPP_EINVAL, "required array is NULL");
  if (ldm < ncell || ldp < ncell || ldc < ncell || ldr < ncell || (het && ldh < ncell))
    return fail(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  GC_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gcrates::RatesArgs a{};
  a.ncell = ncell;
  const size_t n = (size_t)ncell;
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(c->h_met.ensure(RT::NMET * n * sizeof(double)));
    GC_CUDA(c->h_ph.ensure(GC_KPP_NPHOTOL * n * sizeof(double)));
    GC_CUDA(c->h_c.ensure(T::NSPEC * n * sizeof(double)));
    GC_CUDA(c->h_r.ensure(T::NREACT * n * sizeof(double)));
    GC_CUDA(gcutil::copy_rows(c->h_met.p, n * sizeof(double), met, ldm * sizeof(double), n * sizeof(double),
                              RT::NMET, s));
    GC_CUDA(gcutil::copy_rows(c->h_ph.p, n * sizeof(double), photol, ldp * sizeof(double), n * sizeof(double),
                              GC_KPP_NPHOTOL, s));
    GC_CUDA(gcutil::copy_rows(c->h_c.p, n * sizeof(double), conc, ldc * sizeof(double), n * sizeof(double),
                              T::NSPEC, s));
    a.met = (const double*)c->h_met.p;
    a.photol = (const double*)c->h_ph.p;
    a.c = (const double*)c->h_c.p;
    a.rconst = (double*)c->h_r.p;
    a.ldm = a.ldp = a.ldc = a.ldr = ncell;
    if (het) {
      GC_CUDA(c->h_het.ensure((size_t)HET_NFIELD * n * sizeof(double)));
      GC_CUDA(gcutil::copy_rows(c->h_het.p, n * sizeof(double), het, ldh * sizeof(double), n * sizeof(double),
                                HET_NFIELD, s));
      a.het = (const double*)c->h_het.p;
      a.ldh = ncell;
    }
  } else {
    a.het = het;
    a.ldh = ldh;
    a.met = met;
    a.ldm = ldm;
    a.photol = photol;
    a.ldp = ldp;
    a.c = conc;
    a.ldc = ldc;
    a.rconst = rconst;
    a.ldr = ldr;
  }
  cudaError_t e = c->rates_direct ? gcrates::launch_rates_direct(c->rates, a, s) : gcrates::launch_rates(c->rates, a, s);
  if (e != cudaSuccess) return cuda_fail(e, "rates kernel launch");
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(gcutil::copy_rows(rconst, ldr * sizeof(double), a.rconst, n * sizeof(double), n * sizeof(double),
                              T::NREACT, s));
    GC_CUDA(cudaStreamSynchronize(s));
  }
  return GC_KPP_OK;
}

int gc_kpp_set_state_het_batch(gc_kpp_ctx* c, int ncell, const double* hetin, long long ldi, const double* conc,
                               long long ldc, double gamma_ho2, int lpscchem, int turn_off_het_rates, double* het,
                               long long ldh, int mem, void* stream) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  if (ncell < 0) return fail(GC_KPP_EINVAL, "ncell < 0");
  if (ncell == 0) return GC_KPP_OK;
  if (!hetin || !conc || !het) return fail(GC_KPP_EINVAL, "required array is NULL");
  if (ldi < ncell || ldc < ncell || ldh < ncell) return fail(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  GC_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gchet::SetStateArgs a{};
  a.ncell = ncell;
  for (int k = 0; k < HSS_N; ++k) a.ind[k] = RT::hss_ind[k];
  a.gamma_ho2 = gamma_ho2;
  a.lpscchem = lpscchem;
  a.turn_off_het_rates = turn_off_het_rates;
  const size_t n = (size_t)ncell;
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(c->h_hetin.ensure((size_t)HETIN_NFIELD * n * sizeof(double)));
    GC_CUDA(c->h_c.ensure(T::NSPEC * n * sizeof(double)));
    GC_CUDA(c->h_het.ensure((size_t)HET_NFIELD * n * sizeof(double)));
    GC_CUDA(gcutil::copy_rows(c->h_hetin.p, n * sizeof(double), hetin, ldi * sizeof(double), n * sizeof(double),
                              HETIN_NFIELD, s));
    GC_CUDA(gcutil::copy_rows(c->h_c.p, n * sizeof(double), conc, ldc * sizeof(double), n * sizeof(double),
                              T::NSPEC, s));
    a.in = (const double*)c->h_hetin.p;
    a.c = (const double*)c->h_c.p;
    a.het = (double*)c->h_het.p;
    a.ldi = a.ldc = a.ldh = ncell;
  } else {
    a.in = hetin;
    a.ldi = ldi;
    a.c = conc;
    a.ldc = ldc;
    a.het = het;
    a.ldh = ldh;
  }
  cudaError_t e = gchet::set_state_het(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "SetStateHet kernel launch");
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(gcutil::copy_rows(het, ldh * sizeof(double), a.het, n * sizeof(double), n * sizeof(double), HET_NFIELD, s));
    GC_CUDA(cudaStreamSynchronize(s));
  }
  return GC_KPP_OK;
}

int gc_kpp_sulfur_aq_rates_batch(gc_kpp_ctx* c, int ncell, const double* hetin, long long ldi, const double* conc,
                                 long long ldc, double* met, long long ldm, int mem, void* stream) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  if (ncell < 0) return fail(GC_KPP_EINVAL, "ncell < 0");
  if (ncell == 0) return GC_KPP_OK;
  if (!hetin || !conc || !met) return fail(GC_KPP_EINVAL, "required array is NULL");
  if (ldi < ncell || ldc < ncell || ldm < ncell) return fail(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  GC_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gchet::SulfurAqArgs a{};
  a.ncell = ncell;
  for (int k = 0; k < HSS_N; ++k) {
    a.ind[k] = RT::hss_ind[k];
    a.srmw[k] = RT::hss_srmw[k];
  }
  a.row_temp = GC_KPP_MET_TEMP;
  a.row_numden = GC_KPP_MET_NUMDEN;
  a.row_kmt = GC_KPP_MET_K_MT;
  const size_t n = (size_t)ncell;
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(c->h_hetin.ensure((size_t)HETIN_NFIELD * n * sizeof(double)));
    GC_CUDA(c->h_c.ensure(T::NSPEC * n * sizeof(double)));
    GC_CUDA(c->h_met.ensure(RT::NMET * n * sizeof(double)));
    GC_CUDA(gcutil::copy_rows(c->h_hetin.p, n * sizeof(double), hetin, ldi * sizeof(double), n * sizeof(double),
                              HETIN_NFIELD, s));
    GC_CUDA(gcutil::copy_rows(c->h_c.p, n * sizeof(double), conc, ldc * sizeof(double), n * sizeof(double),
                              T::NSPEC, s));
    GC_CUDA(gcutil::copy_rows(c->h_met.p, n * sizeof(double), met, ldm * sizeof(double), n * sizeof(double),
                              RT::NMET, s));
    a.in = (const double*)c->h_hetin.p;
    a.c = (const double*)c->h_c.p;
    a.met = (double*)c->h_met.p;
    a.ldi = a.ldc = a.ldm = ncell;
  } else {
    a.in = hetin;
    a.ldi = ldi;
    a.c = conc;
    a.ldc = ldc;
    a.met = met;
    a.ldm = ldm;
  }
  cudaError_t e = gchet::sulfur_aq_rates(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "SulfurAqChem kernel launch");
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(gcutil::copy_rows(met + (long long)GC_KPP_MET_K_MT * ldm, ldm * sizeof(double),
                              a.met + (long long)GC_KPP_MET_K_MT * ncell, n * sizeof(double), n * sizeof(double), 6, s));
    GC_CUDA(cudaStreamSynchronize(s));
  }
  return GC_KPP_OK;
}

int gc_kpp_het_drop_chem_batch(gc_kpp_ctx* c, int ncell, double dt, const double* hetin, long long ldi,
                               const double* conc, long long ldc, const double* het, long long ldh, const int* size_res,
                               double* met, long long ldm, int mem, void* stream) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  if (ncell < 0) return fail(GC_KPP_EINVAL, "ncell < 0");
  if (ncell == 0) return GC_KPP_OK;
  if (!hetin || !conc || !het || !size_res || !met) return fail(GC_KPP_EINVAL, "required array is NULL");
  if (ldi < ncell || ldc < ncell || ldh < ncell || ldm < ncell)
    return fail(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  if (!(dt > 0.0)) return fail(GC_KPP_EINVAL, "dt must be positive");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  GC_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gchet::HetDropArgs a{};
  a.ncell = ncell;
  a.dt = dt;
  for (int k = 0; k < HSS_N; ++k) a.ind[k] = RT::hss_ind[k];
  const gcrates::RatesDev& rp = c->rates;
  a.hs_ind = rp.hs_ind;
  a.hs_mw = rp.hs_mw;
  a.hs_srmw = rp.hs_srmw;
  a.hs_hk0 = rp.hs_hk0;
  a.hs_hcr = rp.hs_hcr;
  const size_t n = (size_t)ncell;
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(c->h_hetin.ensure((size_t)HETIN_NFIELD * n * sizeof(double)));
    GC_CUDA(c->h_c.ensure(T::NSPEC * n * sizeof(double)));
    GC_CUDA(c->h_het.ensure((size_t)HET_NFIELD * n * sizeof(double)));
    GC_CUDA(c->h_met.ensure(RT::NMET * n * sizeof(double)));
    GC_CUDA(c->h_ie.ensure(n * sizeof(int)));
    GC_CUDA(gcutil::copy_rows(c->h_hetin.p, n * sizeof(double), hetin, ldi * sizeof(double), n * sizeof(double),
                              HETIN_NFIELD, s));
    GC_CUDA(gcutil::copy_rows(c->h_c.p, n * sizeof(double), conc, ldc * sizeof(double), n * sizeof(double),
                              T::NSPEC, s));
    GC_CUDA(gcutil::copy_rows(c->h_het.p, n * sizeof(double), het, ldh * sizeof(double), n * sizeof(double),
                              HET_NFIELD, s));
    GC_CUDA(gcutil::copy_rows(c->h_met.p, n * sizeof(double), met, ldm * sizeof(double), n * sizeof(double),
                              RT::NMET, s));
    GC_CUDA(gcutil::copy_rows(c->h_ie.p, n * sizeof(int), size_res, n * sizeof(int), n * sizeof(int), 1, s));
    a.in = (const double*)c->h_hetin.p;
    a.c = (const double*)c->h_c.p;
    a.het = (const double*)c->h_het.p;
    a.met = (double*)c->h_met.p;
    a.size_res = (const int*)c->h_ie.p;
    a.ldi = a.ldc = a.ldh = a.ldm = ncell;
  } else {
    a.in = hetin;
    a.ldi = ldi;
    a.c = conc;
    a.ldc = ldc;
    a.het = het;
    a.ldh = ldh;
    a.met = met;
    a.ldm = ldm;
    a.size_res = size_res;
  }
  cudaError_t e = gchet::het_drop_chem(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "HetDropChem kernel launch");
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(gcutil::copy_rows(met + (long long)GC_KPP_MET_SRHOCL * ldm, ldm * sizeof(double),
                              a.met + (long long)GC_KPP_MET_SRHOCL * ncell, n * sizeof(double), n * sizeof(double), 2,
                              s));
    GC_CUDA(cudaStreamSynchronize(s));
  }
  return GC_KPP_OK;
}

int gc_kpp_sulfur_cld_rates_batch(gc_kpp_ctx* c, int ncell, double* hetin, long long ldi, const double* conc,
                                  long long ldc, double* met, long long ldm, int lmetalcatso2, int* size_res, int mem,
                                  void* stream) {
  if (!c) return fail(GC_KPP_EINVAL, "ctx is NULL");
  if (ncell < 0) return fail(GC_KPP_EINVAL, "ncell < 0");
  if (ncell == 0) return GC_KPP_OK;
  if (!hetin || !conc || !met) return fail(GC_KPP_EINVAL, "required array is NULL");
  if (ldi < ncell || ldc < ncell || ldm < ncell) return fail(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return fail(GC_KPP_EINVAL, "bad mem kind");
  if (lmetalcatso2 != 0 && lmetalcatso2 != 1) return fail(GC_KPP_EINVAL, "lmetalcatso2 must be 0 or 1");
  GC_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gchet::SulfurCldArgs a{};
  a.ncell = ncell;
  for (int k = 0; k < HSS_N; ++k) a.ind[k] = RT::hss_ind[k];
  a.row_kcld = GC_KPP_MET_K_CLD;
  a.lmetalcatso2 = lmetalcatso2;
  const size_t n = (size_t)ncell;
  // the rows SET_SO2 (and Set_Sulfur_Chem_Rates) write back into hetin
  const int out_rows[] = {HETIN_HSO3_aq, HETIN_SO3_aq, HETIN_pHCloud, HETIN_fupdateHOBr, HETIN_fupdateHOCl};
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(c->h_hetin.ensure((size_t)HETIN_NFIELD * n * sizeof(double)));
    GC_CUDA(c->h_c.ensure(T::NSPEC * n * sizeof(double)));
    GC_CUDA(c->h_met.ensure(RT::NMET * n * sizeof(double)));
    GC_CUDA(c->h_ie.ensure(n * sizeof(int)));
    GC_CUDA(gcutil::copy_rows(c->h_hetin.p, n * sizeof(double), hetin, ldi * sizeof(double), n * sizeof(double),
                              HETIN_NFIELD, s));
    GC_CUDA(gcutil::copy_rows(c->h_c.p, n * sizeof(double), conc, ldc * sizeof(double), n * sizeof(double),
                              T::NSPEC, s));
    a.in = (double*)c->h_hetin.p;
    a.c = (const double*)c->h_c.p;
    a.met = (double*)c->h_met.p;
    a.ldi = a.ldc = a.ldm = ncell;
    a.size_res = size_res ? (int*)c->h_ie.p : nullptr;
  } else {
    a.in = hetin;
    a.ldi = ldi;
    a.c = conc;
    a.ldc = ldc;
    a.met = met;
    a.ldm = ldm;
    a.size_res = size_res;
  }
  cudaError_t e = gchet::sulfur_cld_rates(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "SulfurCldChem kernel launch");
  if (mem == GC_KPP_MEM_HOST) {
    GC_CUDA(gcutil::copy_rows(met + (long long)GC_KPP_MET_K_CLD * ldm, ldm * sizeof(double),
                              a.met + (long long)GC_KPP_MET_K_CLD * ncell, n * sizeof(double), n * sizeof(double), 6,
                              s));
    for (int r : out_rows)
      GC_CUDA(gcutil::copy_rows(hetin + (long long)r * ldi, ldi * sizeof(double), a.in + (long long)r * ncell,
                                n * sizeof(double), n * sizeof(double), 1, s));
    if (size_res) GC_CUDA(gcutil::copy_rows(size_res, n * sizeof(int), a.size_res, n * sizeof(int), n * sizeof(int), 1, s));
    GC_CUDA(cudaStreamSynchronize(s));
  }
  return GC_KPP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// No-allocation entry point.  Everything it needs on the device lives in
// file-scope __device__ arrays of this translation unit: the workspace for at
// most NOALLOC_MAX_CELLS cells and copies of the mechanism tables.  Host code
// cannot use those arrays' names as device addresses, so the first call on
// each device, with that device current, copies the tables in with
// cudaMemcpyToSymbol and takes every address with cudaGetSymbolAddress.
namespace {

constexpr int NOALLOC_MAX_CELLS = 1024;
constexpr int NOALLOC_BLOCK = 128;
constexpr int NOALLOC_WS_TOTAL = T::NAUX + 2 * T::NSPEC + 3 * T::NVAR + SMAX * T::NVAR + T::NREACT + T::NB +
                                 2 * T::LU_NONZERO;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_ws[(size_t)NOALLOC_MAX_CELLS * NOALLOC_WS_TOTAL];

#define GC_NA_TABLE(type, name) static __device__ type g_na_##name[sizeof(T::name) / sizeof(T::name[0])];
GC_NA_TABLE(unsigned, prod_packed)
GC_NA_TABLE(int, prod_ids_a)
GC_NA_TABLE(int, prod_ids_b)
GC_NA_TABLE(double, pre_literals)
GC_NA_TABLE(int, p_start)
GC_NA_TABLE(unsigned, p_sterm)
GC_NA_TABLE(int, d_start)
GC_NA_TABLE(unsigned, d_sterm)
GC_NA_TABLE(int, j_start)
GC_NA_TABLE(unsigned, j_sterm)
GC_NA_TABLE(double, slit)
GC_NA_TABLE(int, lu_crow)
GC_NA_TABLE(int, lu_diag)
GC_NA_TABLE(int, lu_icol)
GC_NA_TABLE(int, lrow_start)
GC_NA_TABLE(int, lop_kk)
GC_NA_TABLE(int, lop_dj)
GC_NA_TABLE(int, lop_u)
GC_NA_TABLE(unsigned, uop)
GC_NA_TABLE(int, dot_start)
GC_NA_TABLE(unsigned, dot_term)
GC_NA_TABLE(double, lit)
#undef GC_NA_TABLE

struct NoAllocDevice {
  bool ready = false;
  MechDev mech{};
  double* ws = nullptr;
};
NoAllocDevice g_noalloc[NOALLOC_MAX_DEVICES];
std::mutex g_noalloc_mutex;

// Per-device set-up (the current device): fill the table copies and take the
// device addresses of the tables and of the workspace.
int noalloc_setup(int dev, NoAllocDevice** out) {
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(GC_KPP_EINVAL, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocDevice& d = g_noalloc[dev];
  if (!d.ready) {
    if (make_layout().total != NOALLOC_WS_TOTAL) return fail(GC_KPP_EINVAL, "workspace layout mismatch");
    MechDev& m = d.mech;
    m.nvar = T::NVAR; m.nfix = T::NFIX; m.nreact = T::NREACT; m.nspec = T::NSPEC;
    m.lu_nonzero = T::LU_NONZERO; m.nb = T::NB; m.lit0 = T::LIT0; m.naux = T::NAUX;
    void* p = nullptr;
#define GC_NA_FILL(field, name, type)                                                        \
    GC_CUDA(cudaMemcpyToSymbol(g_na_##name, T::name, sizeof(T::name)));                      \
    GC_CUDA(cudaGetSymbolAddress(&p, g_na_##name));                                          \
    m.field = reinterpret_cast<type>(p);
    GC_NA_FILL(prod_packed, prod_packed, const uint2*)
    GC_NA_FILL(prod_ids_a, prod_ids_a, const int*)
    GC_NA_FILL(prod_ids_b, prod_ids_b, const int*)
    for (int i = 0; i < 9; ++i) {
      m.a_cls[i] = T::a_cls_start[i];
      m.b_cls[i] = T::b_cls_start[i];
    }
    GC_NA_FILL(pre_lit, pre_literals, const double*)
    GC_NA_FILL(p_start, p_start, const int*)
    GC_NA_FILL(p_sterm, p_sterm, const unsigned*)
    GC_NA_FILL(d_start, d_start, const int*)
    GC_NA_FILL(d_sterm, d_sterm, const unsigned*)
    GC_NA_FILL(j_start, j_start, const int*)
    GC_NA_FILL(j_sterm, j_sterm, const unsigned*)
    GC_NA_FILL(slit, slit, const double*)
    GC_NA_FILL(lu_crow, lu_crow, const int*)
    GC_NA_FILL(lu_diag, lu_diag, const int*)
    GC_NA_FILL(lu_icol, lu_icol, const int*)
    GC_NA_FILL(lrow_start, lrow_start, const int*)
    GC_NA_FILL(lop_kk, lop_kk, const int*)
    GC_NA_FILL(lop_dj, lop_dj, const int*)
    GC_NA_FILL(lop_u, lop_u, const int*)
    GC_NA_FILL(uop, uop, const unsigned*)
    GC_NA_FILL(dot_start, dot_start, const int*)
    GC_NA_FILL(dot_term, dot_term, const unsigned*)
    GC_NA_FILL(lit, lit, const double*)
#undef GC_NA_FILL
    double* ws = nullptr;
    GC_CUDA(cudaGetSymbolAddress((void**)&ws, g_noalloc_ws));
    d.ws = ws;
    d.ready = true;
  }
  *out = &d;
  return GC_KPP_OK;
}

}  // namespace

void gckpp_photol_rows(unsigned char* mask);

extern "C" {

int gc_kpp_integrate_batch_noalloc(int ncell, double tin, double tout, double* c, long long ldc, const double* rconst,
                                   long long ldr, const double* atol, const double* rtol, const int* icntrl_u,
                                   const double* rcntrl_u, const double* hstart, int* istatus, double* rstatus,
                                   long long ldo, int* ierr, void* stream) {
  if (ncell < 0) return fail(GC_KPP_EINVAL, "ncell < 0");
  if (ncell > NOALLOC_MAX_CELLS)
    return fail(GC_KPP_EINVAL, "ncell exceeds the no-allocation workspace (GC_KPP_NOALLOC_MAX_CELLS = 1024 cells "
                               "per call); split the batch");
  if (ncell == 0) return GC_KPP_OK;
  if (!c || !rconst || !atol || !rtol || !ierr) return fail(GC_KPP_EINVAL, "required array is NULL");
  if (ldc < ncell || ldr < ncell || ((istatus || rstatus) && ldo < ncell))
    return fail(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  int dev = 0;
  GC_CUDA(cudaGetDevice(&dev));
  NoAllocDevice* d = nullptr;
  GC_TRY(noalloc_setup(dev, &d));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Resolved R;
  GC_TRY(resolve(icntrl_u, rcntrl_u, tin, tout, R));
  // auto-reduction needs the per-cell mask rows of a context's workspace
  if (R.autoreduce)
    return fail(GC_KPP_EUNSUPPORTED, "the no-allocation entry point does not run auto-reduction (ICNTRL(12) = 1)");
  if (!R.code) {
    // Rosenbrock's tolerance check (:464-472) on host copies held on the stack
    const int ntol = R.vector_tol ? T::NVAR : 1;
    double at[T::NVAR], rt[T::NVAR];
    GC_CUDA(cudaMemcpyAsync(at, atol, ntol * sizeof(double), cudaMemcpyDeviceToHost, s));
    GC_CUDA(cudaMemcpyAsync(rt, rtol, ntol * sizeof(double), cudaMemcpyDeviceToHost, s));
    GC_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < ntol; ++i)
      if (!(at[i] > 0.0) || rt[i] <= 10.0 * DBL_EPSILON || rt[i] >= 1.0) R.code = -5;
  }
  if (R.code) {
    // every cell gets the option error, ISTATUS/RSTATUS zeroed, on the device
    GC_CUDA(gcutil::fill_error(R.code, ncell, ierr, istatus, rstatus, ldo, s));
    return GC_KPP_OK;
  }
  // One thread and one workspace slot per cell (plain schedule).  Every slot
  // entry the kernel reads it has written earlier in the same call, so the
  // previous call's contents need no clearing.
  const int nc = gckpp_cells_per_thread_fast();
  const int grid = (ncell + NOALLOC_BLOCK * nc - 1) / (NOALLOC_BLOCK * nc);
  RosParams p{};
  p.ncell = ncell;
  p.cell_limit = ncell;
  p.c_in = c;
  p.c_out = c;
  p.ldc = ldc;
  p.rconst = rconst;
  p.ldr = ldr;
  p.hstart = hstart;
  p.istatus = istatus;
  p.rstatus = rstatus;
  p.ldo = ldo;
  p.ierr = ierr;
  p.atol = atol;
  p.rtol = rtol;
  p.vector_tol = R.vector_tol ? 1 : 0;
  p.tstart = tin;
  p.tend = tout;
  p.hmin = R.hmin;
  p.hmax = R.hmax;
  p.hstart_default = R.hstart_default;
  p.facmin = R.facmin;
  p.facmax = R.facmax;
  p.facrej = R.facrej;
  p.facsafe = R.facsafe;
  p.roundoff = DBL_EPSILON;
  p.autonomous = R.autonomous;
  p.max_steps = R.max_steps;
  p.clamp_negative = R.clamp;
  p.lu_form = 0;
  p.ws = d->ws;
  p.lay = make_layout();
  p.nslot = (long long)grid * NOALLOC_BLOCK * nc;
  if (p.nslot > NOALLOC_MAX_CELLS) return fail(GC_KPP_EINVAL, "no-allocation workspace too small");
  cudaError_t e = gckpp_launch_ros_fast(0, grid, NOALLOC_BLOCK, d->mech, R.meth, p, s, 0);
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  return GC_KPP_OK;
}

int gc_kpp_copy_rows(void* dst, long long dpitch, const void* src, long long spitch, long long width, long long rows,
                     void* stream) {
  if (rows < 0 || width < 0 || dpitch < width || spitch < width) return fail(GC_KPP_EINVAL, "bad copy shape");
  if (rows > 0 && width > 0 && (!dst || !src)) return fail(GC_KPP_EINVAL, "NULL array");
  cudaError_t e = gcutil::copy_rows(dst, (size_t)dpitch, src, (size_t)spitch, (size_t)width, (size_t)rows,
                                    (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "row copy");
  return GC_KPP_OK;
}

int gc_kpp_photol_rows(unsigned char* mask) {
  if (!mask) return fail(GC_KPP_EINVAL, "NULL mask");
  gckpp_photol_rows(mask);
  return GC_KPP_OK;
}

}  // extern "C"

// Error text for the library's other translation units (gckpp_learned_capi.cu).
int gckpp_set_error(int code, const char* msg) {
  g_last_error = msg;
  return code;
}

// The binned step with the block-per-cell count in device memory (the learned
// step's asynchronous path, gckpp_learned_capi.cu).
int gckpp_step_binned_dev(gc_kpp_ctx* c, int ncell, double dt, const double* met, long long ldm, const double* photol,
                          long long ldp, double* cc, long long ldc, const double* atol, const double* rtol,
                          const int* icntrl_u, const double* rcntrl_u, double* hstart, int* istatus, double* rstatus,
                          long long ldo, int* ierr, int* nretry, const int* order, const int* nblock_dev, void* stream) {
  return fullchem_step_impl(c, ncell, dt, met, ldm, photol, ldp, cc, ldc, atol, rtol, icntrl_u, rcntrl_u, hstart,
                            istatus, rstatus, ldo, ierr, nretry, order, 0, nblock_dev, GC_KPP_MEM_DEVICE, stream);
}

int gckpp_ctx_async(const gc_kpp_ctx* c) { return c ? c->async : 0; }

// mask[r] = 1 for the PHOTOL rows r that the rate program reads (GC_KPP_NPHOTOL entries).
void gckpp_photol_rows(unsigned char* mask) {
  for (int r = 0; r < GC_KPP_NPHOTOL; ++r) mask[r] = 0;
  for (int k = 0; k < RT::NPHOTOL_RUNS; ++k)
    for (int r = RT::photol_runs[2 * k]; r < RT::photol_runs[2 * k + 1]; ++r) mask[r] = 1;
}
