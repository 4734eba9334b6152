// Learned proposer kernels (kpp_mlp.cu): shapes and launch interface.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace gcmlp {

constexpr int NJ = 20;                      // log J-value inputs
constexpr int NSPC = 32;                    // log key-species inputs
constexpr int NFEAT = 4 + NJ + NSPC;        // log T, log P, log H2O vmr, cos SZA, J, species
constexpr int HID = 128;                    // hidden width
constexpr int NBIN = 4;                     // stiffness bins
constexpr int NOUT = 1 + NBIN;              // log H0 + bin logits

struct FeatureArgs {
  int ncell;
  const double* met;
  long long ldm;
  const double* photol;
  long long ldp;
  const double* c;
  long long ldc;
  const double* suncos;   // [ncell] or null
  const int* jslot;       // [NJ] PHOTOL rows
  const int* spc;         // [NSPC] species rows
  const double* mean;     // [NFEAT]
  const double* inv_std;  // [NFEAT]
  float* x;               // [ncell][NFEAT]
};

cudaError_t features(const FeatureArgs& a, cudaStream_t s);
cudaError_t gemm_fwd(const float* X, const __nv_bfloat16* W, const float* b, float* Z, float* Y, int M, int K, int N,
                     int act, cudaStream_t s);
cudaError_t gemm_dx(const float* dY, const float* Z, const __nv_bfloat16* W, float* dZ, float* dX, int M, int K,
                    int N, int act, cudaStream_t s);
cudaError_t gemm_dw(const float* dZ, const float* X, float* dW, float* db, int M, int K, int N, cudaStream_t s);
cudaError_t head_loss(const float* out, const float* y_h, const int* y_bin, float* dout, float* loss, int M,
                      float w_ce, cudaStream_t s);
cudaError_t adam(float* w, __nv_bfloat16* wb, float* g, float* m1, float* m2, int n, float lr, float b1, float b2,
                 float eps, int step, cudaStream_t s);
cudaError_t propose(const float* out, int M, double scale, double hmin, double hmax, double* h0, int* bin,
                    int keep, cudaStream_t s);
cudaError_t bin_order(const int* bin, int M, int* counts, int* scratch, int* order, cudaStream_t s);
int bin_order_scratch(int M);

}  // namespace gcmlp
