// C ABI of the learned step-size / stiffness proposer (include/gckpp_gb300_mlp.h).
// All pointers are device pointers; calls are asynchronous on `stream`.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/gckpp_gb300_mlp.h"
#include "kpp_mlp.h"

using namespace gcmlp;

static int rc(cudaError_t e) { return e == cudaSuccess ? 0 : -102; }
#define GC_MLP_TRY(x)                     \
  do {                                    \
    cudaError_t _e = (x);                 \
    if (_e != cudaSuccess) return rc(_e); \
  } while (0)

extern "C" {

int gc_mlp_dims(int* nfeat, int* hidden, int* nout, int* nj, int* nspc) {
  if (nfeat) *nfeat = NFEAT;
  if (hidden) *hidden = HID;
  if (nout) *nout = NOUT;
  if (nj) *nj = NJ;
  if (nspc) *nspc = NSPC;
  return 0;
}

int gc_mlp_features(int ncell, const double* met, long long ldm, const double* photol, long long ldp,
                    const double* c, long long ldc, const double* suncos, const int* jslot, const int* spc,
                    const double* mean, const double* inv_std, float* x, void* stream) {
  if (ncell < 0 || !met || !photol || !c || !jslot || !spc || !mean || !inv_std || !x) return -101;
  FeatureArgs a{ncell, met, ldm, photol, ldp, c, ldc, suncos, jslot, spc, mean, inv_std, x};
  return rc(features(a, (cudaStream_t)stream));
}

int gc_mlp_forward(int M, const float* x, const void* w1, const float* b1, const void* w2, const float* b2,
                   const void* w3, const float* b3, float* z1, float* h1, float* z2, float* h2, float* out,
                   void* stream) {
  if (M < 0 || !x || !w1 || !b1 || !w2 || !b2 || !w3 || !b3 || !h1 || !h2 || !out) return -101;
  cudaStream_t s = (cudaStream_t)stream;
  GC_MLP_TRY(gemm_fwd(x, (const __nv_bfloat16*)w1, b1, z1, h1, M, NFEAT, HID, 1, s));
  GC_MLP_TRY(gemm_fwd(h1, (const __nv_bfloat16*)w2, b2, z2, h2, M, HID, HID, 1, s));
  GC_MLP_TRY(gemm_fwd(h2, (const __nv_bfloat16*)w3, b3, nullptr, out, M, HID, NOUT, 0, s));
  return 0;
}

int gc_mlp_loss(int M, const float* out, const float* y_h, const int* y_bin, float w_ce, float* dout, float* loss,
                void* stream) {
  if (M < 0 || !out || !y_h || !y_bin || !dout || !loss) return -101;
  return rc(head_loss(out, y_h, y_bin, dout, loss, M, w_ce, (cudaStream_t)stream));
}

int gc_mlp_backward(int M, const float* x, const void* w1, const void* w2, const void* w3, const float* z1,
                    const float* h1, const float* z2, const float* h2, const float* dout, float* g_w1, float* g_b1,
                    float* g_w2, float* g_b2, float* g_w3, float* g_b3, float* scratch, void* stream) {
  if (M < 0 || !x || !w1 || !w2 || !w3 || !z1 || !h1 || !z2 || !h2 || !dout || !scratch) return -101;
  cudaStream_t s = (cudaStream_t)stream;
  float* dz3 = scratch;
  float* dh2 = dz3 + (size_t)M * NOUT;
  float* dz2 = dh2 + (size_t)M * HID;
  float* dh1 = dz2 + (size_t)M * HID;
  float* dz1 = dh1 + (size_t)M * HID;
  GC_MLP_TRY(gemm_dx(dout, nullptr, (const __nv_bfloat16*)w3, dz3, dh2, M, HID, NOUT, 0, s));
  GC_MLP_TRY(gemm_dw(dz3, h2, g_w3, g_b3, M, HID, NOUT, s));
  GC_MLP_TRY(gemm_dx(dh2, z2, (const __nv_bfloat16*)w2, dz2, dh1, M, HID, HID, 1, s));
  GC_MLP_TRY(gemm_dw(dz2, h1, g_w2, g_b2, M, HID, HID, s));
  GC_MLP_TRY(gemm_dx(dh1, z1, (const __nv_bfloat16*)w1, dz1, nullptr, M, NFEAT, HID, 1, s));
  GC_MLP_TRY(gemm_dw(dz1, x, g_w1, g_b1, M, NFEAT, HID, s));
  return 0;
}

int gc_mlp_adam(int n, float* w, void* w_bf16, float* g, float* m1, float* m2, float lr, float b1, float b2,
                float eps, int step, void* stream) {
  if (n < 0 || !w || !g || !m1 || !m2 || step < 1) return -101;
  return rc(adam(w, (__nv_bfloat16*)w_bf16, g, m1, m2, n, lr, b1, b2, eps, step, (cudaStream_t)stream));
}

int gc_mlp_propose(int M, const float* out, double scale, double hmin, double hmax, double* h0, int* bin,
                   int keep, void* stream) {
  if (M < 0 || !out) return -101;
  return rc(propose(out, M, scale, hmin, hmax, h0, bin, keep, (cudaStream_t)stream));
}

int gc_mlp_bin_order_scratch(int M) { return M < 0 ? -101 : bin_order_scratch(M); }

int gc_mlp_bin_order(int M, const int* bin, int* counts, int* scratch, int* order, void* stream) {
  if (M < 0 || !bin || !counts || !scratch || !order) return -101;
  return rc(bin_order(bin, M, counts, scratch, order, (cudaStream_t)stream));
}

}  // extern "C"
