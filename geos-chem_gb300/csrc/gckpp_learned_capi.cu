// The learned chemistry step behind the C ABI (include/gckpp_gb300.h,
// gc_kpp_proposer_* and gc_kpp_fullchem_step_learned): features -> MLP ->
// H0 proposals and stiffness bins -> stable bin order -> the binned step, so
// that a Fortran caller gets the learned form with the same call shape as
// gc_kpp_fullchem_step.  Built on the public entry points of gckpp_capi.cu
// and the proposer kernels of kpp_mlp.cu.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "../../include/gckpp_gb300.h"
#include "kpp_mlp.h"
#include "kpp_util.h"

using namespace gcmlp;

struct gc_kpp_proposer {
  int device = 0;
  double scale = 1.0;
  double h0_cap = 0.0;  // largest proposed H0 [s]; 0 = the step length
  __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w3 = nullptr;
  float *b1 = nullptr, *b2 = nullptr, *b3 = nullptr;
  double *mean = nullptr, *inv_std = nullptr;
  int *jrows = nullptr, *srows = nullptr;
  // PHOTOL rows a host-memory call stages: the rate program's and the features'
  unsigned char photol_rows[GC_KPP_NPHOTOL] = {};
  // per-call buffers, grown to the largest batch seen
  size_t cap = 0;
  float *x = nullptr, *h1 = nullptr, *h2 = nullptr, *out = nullptr;
  int *bins = nullptr, *order = nullptr, *counts = nullptr, *scratch = nullptr;
  // staging of host-memory calls
  size_t hcap = 0;
  double *met = nullptr, *ph = nullptr, *c = nullptr, *hs = nullptr, *rs = nullptr, *tol = nullptr;
  int *is = nullptr, *ie = nullptr;
};

namespace {

template <typename X>
cudaError_t dalloc(X** p, size_t n) {
  return cudaMalloc((void**)p, n * sizeof(X));
}

template <typename X>
cudaError_t upload(X** p, const X* host, size_t n) {
  cudaError_t e = dalloc(p, n);
  if (e == cudaSuccess) e = cudaMemcpy(*p, host, n * sizeof(X), cudaMemcpyHostToDevice);
  return e;
}

cudaError_t upload_bf16(__nv_bfloat16** p, const float* host, size_t n) {
  std::vector<__nv_bfloat16> b(n);
  for (size_t i = 0; i < n; ++i) b[i] = __float2bfloat16_rn(host[i]);
  return upload(p, b.data(), n);
}

void release(gc_kpp_proposer* q) {
  void* ptrs[] = {q->w1, q->w2, q->w3, q->b1, q->b2, q->b3, q->mean, q->inv_std, q->jrows, q->srows, q->x,
                  q->h1, q->h2, q->out, q->bins, q->order, q->counts, q->scratch, q->met, q->ph, q->c, q->hs,
                  q->rs, q->tol, q->is, q->ie};
  for (void* p : ptrs)
    if (p) cudaFree(p);
}

cudaError_t ensure_plan(gc_kpp_proposer* q, size_t n) {
  if (n <= q->cap) return cudaSuccess;
  void* old[] = {q->x, q->h1, q->h2, q->out, q->bins, q->order, q->counts, q->scratch};
  for (void* p : old)
    if (p) cudaFree(p);
  cudaError_t e = dalloc(&q->x, n * NFEAT);
  if (e == cudaSuccess) e = dalloc(&q->h1, n * HID);
  if (e == cudaSuccess) e = dalloc(&q->h2, n * HID);
  if (e == cudaSuccess) e = dalloc(&q->out, n * NOUT);
  if (e == cudaSuccess) e = dalloc(&q->bins, n);
  if (e == cudaSuccess) e = dalloc(&q->order, n);
  if (e == cudaSuccess) e = dalloc(&q->counts, (size_t)NBIN);
  if (e == cudaSuccess) e = dalloc(&q->scratch, (size_t)bin_order_scratch((int)n));
  q->cap = e == cudaSuccess ? n : 0;
  return e;
}

cudaError_t ensure_host_staging(gc_kpp_proposer* q, size_t n, int nspec, int nvar) {
  if (n <= q->hcap) return cudaSuccess;
  void* old[] = {q->met, q->ph, q->c, q->hs, q->rs, q->tol, q->is, q->ie};
  for (void* p : old)
    if (p) cudaFree(p);
  cudaError_t e = dalloc(&q->met, n * GC_KPP_NMET);
  if (e == cudaSuccess) e = dalloc(&q->ph, n * GC_KPP_NPHOTOL);
  if (e == cudaSuccess) e = dalloc(&q->c, n * nspec);
  if (e == cudaSuccess) e = dalloc(&q->hs, n);
  if (e == cudaSuccess) e = dalloc(&q->rs, n * 20);
  if (e == cudaSuccess) e = dalloc(&q->tol, 2 * (size_t)nvar);
  if (e == cudaSuccess) e = dalloc(&q->is, n * 20);
  if (e == cudaSuccess) e = dalloc(&q->ie, n);
  q->hcap = e == cudaSuccess ? n : 0;
  return e;
}

}  // namespace

#define GC_L_CUDA(x)                              \
  do {                                            \
    if ((x) != cudaSuccess) return GC_KPP_ECUDA;  \
  } while (0)

int gckpp_set_error(int code, const char* msg);
int gckpp_ctx_async(const gc_kpp_ctx* c);
void gckpp_photol_rows(unsigned char* mask);
int gckpp_step_binned_dev(gc_kpp_ctx* c, int ncell, double dt, const double* met, long long ldm, const double* photol,
                          long long ldp, double* cc, long long ldc, const double* atol, const double* rtol,
                          const int* icntrl_u, const double* rcntrl_u, double* hstart, int* istatus, double* rstatus,
                          long long ldo, int* ierr, int* nretry, const int* order, const int* nblock_dev, void* stream);

extern "C" {

int gc_kpp_proposer_create(int device, const float* w1, const float* b1, const float* w2, const float* b2,
                           const float* w3, const float* b3, const double* mean, const double* inv_std,
                           const int* jrows, const int* srows, double scale, gc_kpp_proposer** out) {
  if (!out || !w1 || !b1 || !w2 || !b2 || !w3 || !b3 || !mean || !inv_std || !jrows || !srows)
    return gckpp_set_error(GC_KPP_EINVAL, "NULL argument");
  if (!(scale > 0.0)) return gckpp_set_error(GC_KPP_EINVAL, "scale must be positive");
  int nspec = 0;
  gc_kpp_mechanism_dims(&nspec, nullptr, nullptr, nullptr, nullptr);
  for (int k = 0; k < NJ; ++k)
    if (jrows[k] < 0 || jrows[k] >= GC_KPP_NPHOTOL) return gckpp_set_error(GC_KPP_EINVAL, "jrows outside PHOTOL");
  for (int k = 0; k < NSPC; ++k)
    if (srows[k] < 0 || srows[k] >= nspec) return gckpp_set_error(GC_KPP_EINVAL, "srows outside the species");
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return gckpp_set_error(GC_KPP_ECUDA, "cudaSetDevice");
  gc_kpp_proposer* q = new gc_kpp_proposer();
  q->device = device;
  q->scale = scale;
  gckpp_photol_rows(q->photol_rows);
  for (int k = 0; k < NJ; ++k) q->photol_rows[jrows[k]] = 1;
  cudaError_t e = upload_bf16(&q->w1, w1, (size_t)HID * NFEAT);
  if (e == cudaSuccess) e = upload_bf16(&q->w2, w2, (size_t)HID * HID);
  if (e == cudaSuccess) e = upload_bf16(&q->w3, w3, (size_t)NOUT * HID);
  if (e == cudaSuccess) e = upload(&q->b1, b1, (size_t)HID);
  if (e == cudaSuccess) e = upload(&q->b2, b2, (size_t)HID);
  if (e == cudaSuccess) e = upload(&q->b3, b3, (size_t)NOUT);
  if (e == cudaSuccess) e = upload(&q->mean, mean, (size_t)NFEAT);
  if (e == cudaSuccess) e = upload(&q->inv_std, inv_std, (size_t)NFEAT);
  if (e == cudaSuccess) e = upload(&q->jrows, jrows, (size_t)NJ);
  if (e == cudaSuccess) e = upload(&q->srows, srows, (size_t)NSPC);
  if (e != cudaSuccess) {
    release(q);
    delete q;
    return gckpp_set_error(GC_KPP_ECUDA, "proposer upload failed");
  }
  *out = q;
  return GC_KPP_OK;
}

int gc_kpp_proposer_set_h0_cap(gc_kpp_proposer* q, double cap) {
  if (!q) return gckpp_set_error(GC_KPP_EINVAL, "proposer is NULL");
  if (!(cap >= 0.0)) return gckpp_set_error(GC_KPP_EINVAL, "H0 cap must be >= 0");
  q->h0_cap = cap;
  return GC_KPP_OK;
}

int gc_kpp_proposer_destroy(gc_kpp_proposer* q) {
  if (!q) return GC_KPP_OK;
  cudaSetDevice(q->device);
  release(q);
  delete q;
  return GC_KPP_OK;
}

int gc_kpp_fullchem_step_learned(gc_kpp_ctx* ctx, gc_kpp_proposer* q, int ncell, double dt, const double* met,
                                 long long ldm, const double* photol, long long ldp, double* c, long long ldc,
                                 const double* atol, const double* rtol, const int* icntrl, const double* rcntrl,
                                 double* hstart, int* istatus, double* rstatus, long long ldo, int* ierr,
                                 int* nretry, int* nblock, int mem, void* stream) {
  if (!ctx || !q) return gckpp_set_error(GC_KPP_EINVAL, "ctx or proposer is NULL");
  if (nblock) *nblock = 0;
  if (ncell < 0) return gckpp_set_error(GC_KPP_EINVAL, "ncell < 0");
  if (ncell == 0) return gc_kpp_fullchem_step(ctx, 0, dt, met, ldm, photol, ldp, c, ldc, atol, rtol, icntrl,
                                              rcntrl, hstart, istatus, rstatus, ldo, ierr, nretry, mem, stream);
  if (!met || !photol || !c || !atol || !rtol || !ierr) return gckpp_set_error(GC_KPP_EINVAL, "NULL array");
  if (ldm < ncell || ldp < ncell || ldc < ncell || ((istatus || rstatus) && ldo < ncell))
    return gckpp_set_error(GC_KPP_EINVAL, "leading dimension smaller than ncell");
  if (mem != GC_KPP_MEM_HOST && mem != GC_KPP_MEM_DEVICE) return gckpp_set_error(GC_KPP_EINVAL, "bad mem kind");
  int nspec = 0, nvar = 0;
  gc_kpp_mechanism_dims(&nspec, &nvar, nullptr, nullptr, nullptr);
  const bool vector_tol = !(icntrl && icntrl[1] != 0);  // ICNTRL(2) = 0: vector tolerances
  const size_t ntol = vector_tol ? (size_t)nvar : 1;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaSetDevice(q->device) != cudaSuccess) return gckpp_set_error(GC_KPP_ECUDA, "cudaSetDevice");
  const size_t n = (size_t)ncell;
  if (ensure_plan(q, n) != cudaSuccess) return gckpp_set_error(GC_KPP_ENOMEM, "proposer buffers");
  // device views of the inputs
  const double *dmet = met, *dph = photol, *dat = atol, *drt = rtol;
  double *dc = c, *dhs = hstart, *drs = rstatus;
  int *dis = istatus, *die = ierr;
  long long lm = ldm, lp = ldp, lc = ldc, lo = ldo;
  const bool host = mem == GC_KPP_MEM_HOST;
  if (host) {
    if (ensure_host_staging(q, n, nspec, nvar) != cudaSuccess)
      return gckpp_set_error(GC_KPP_ENOMEM, "proposer staging buffers");
    GC_L_CUDA(gcutil::copy_rows(q->met, n * 8, met, ldm * 8, n * 8, GC_KPP_NMET, s));
    // only the PHOTOL rows that the rates and the features read
    for (int r0 = 0; r0 < GC_KPP_NPHOTOL;) {
      if (!q->photol_rows[r0]) {
        ++r0;
        continue;
      }
      int r1 = r0 + 1;
      while (r1 < GC_KPP_NPHOTOL && q->photol_rows[r1]) ++r1;
      GC_L_CUDA(gcutil::copy_rows(q->ph + (size_t)r0 * n, n * 8, photol + (long long)r0 * ldp, ldp * 8, n * 8,
                                  r1 - r0, s));
      r0 = r1;
    }
    GC_L_CUDA(gcutil::copy_rows(q->c, n * 8, c, ldc * 8, n * 8, nspec, s));
    GC_L_CUDA(cudaMemcpyAsync(q->tol, atol, ntol * 8, cudaMemcpyHostToDevice, s));
    GC_L_CUDA(cudaMemcpyAsync(q->tol + nvar, rtol, ntol * 8, cudaMemcpyHostToDevice, s));
    if (hstart) GC_L_CUDA(gcutil::copy_rows(q->hs, n * 8, hstart, n * 8, n * 8, 1, s));
    dmet = q->met; dph = q->ph; dc = q->c; dat = q->tol; drt = q->tol + nvar;
    dhs = q->hs; dis = q->is; drs = q->rs; die = q->ie;
    lm = lp = lc = lo = ncell;
  } else if (!hstart) {
    return gckpp_set_error(GC_KPP_EINVAL, "device-memory calls need an hstart array (zeros for a cold start)");
  }
  if (host && !hstart) GC_L_CUDA(cudaMemsetAsync(q->hs, 0, n * 8, s));
  // plan: features, MLP, proposals (kept KPPHvalues win), stable bin order
  FeatureArgs fa{ncell, dmet, lm, dph, lp, dc, lc, nullptr, q->jrows, q->srows, q->mean, q->inv_std, q->x};
  GC_L_CUDA(features(fa, s));
  GC_L_CUDA(gemm_fwd(q->x, q->w1, q->b1, nullptr, q->h1, ncell, NFEAT, HID, 1, s));
  GC_L_CUDA(gemm_fwd(q->h1, q->w2, q->b2, nullptr, q->h2, ncell, HID, HID, 1, s));
  GC_L_CUDA(gemm_fwd(q->h2, q->w3, q->b3, nullptr, q->out, ncell, HID, NOUT, 0, s));
  const double hmax = (q->h0_cap > 0.0 && q->h0_cap < dt) ? q->h0_cap : dt;
  GC_L_CUDA(propose(q->out, ncell, q->scale, 1.0e-5, hmax, dhs, q->bins, 1, s));
  GC_L_CUDA(bin_order(q->bins, ncell, q->counts, q->scratch, q->order, s));
  if (gckpp_ctx_async(ctx)) {
    // the top bin's size stays on the device (no host synchronisation)
    if (host) return gckpp_set_error(GC_KPP_EINVAL, "asynchronous steps need device memory");
    if (nblock) *nblock = -1;
    return gckpp_step_binned_dev(ctx, ncell, dt, dmet, lm, dph, lp, dc, lc, dat, drt, icntrl, rcntrl, dhs, dis, drs,
                                 lo, die, nretry, q->order, q->counts + (NBIN - 1), stream);
  }
  int counts[NBIN];
  GC_L_CUDA(cudaMemcpyAsync(counts, q->counts, sizeof(counts), cudaMemcpyDeviceToHost, s));
  GC_L_CUDA(cudaStreamSynchronize(s));
  const int nb = counts[NBIN - 1];
  if (nblock) *nblock = nb;
  int rc = gc_kpp_fullchem_step_binned(ctx, ncell, dt, dmet, lm, dph, lp, dc, lc, dat, drt, icntrl, rcntrl, dhs,
                                       dis, drs, lo, die, nretry, q->order, nb, GC_KPP_MEM_DEVICE, stream);
  if (rc != GC_KPP_OK) return rc;
  if (host) {
    GC_L_CUDA(gcutil::copy_rows(c, ldc * 8, q->c, n * 8, n * 8, nspec, s));
    GC_L_CUDA(gcutil::copy_rows(ierr, n * 4, q->ie, n * 4, n * 4, 1, s));
    if (istatus) GC_L_CUDA(gcutil::copy_rows(istatus, ldo * 4, q->is, n * 4, n * 4, 20, s));
    if (rstatus) GC_L_CUDA(gcutil::copy_rows(rstatus, ldo * 8, q->rs, n * 8, n * 8, 20, s));
    if (hstart) GC_L_CUDA(gcutil::copy_rows(hstart, n * 8, q->hs, n * 8, n * 8, 1, s));
    GC_L_CUDA(cudaStreamSynchronize(s));
  }
  return GC_KPP_OK;
}

}  // extern "C"
