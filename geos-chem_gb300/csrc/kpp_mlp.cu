// Learned step-size / stiffness proposer: a 56 -> 128 -> 128 -> 5 MLP with
// GELU, BF16 weights and FP32 activations/accumulation, trained and run on
// the GPU by these kernels.
//
//   features   cell state (met, J-values, key species) -> normalised inputs
//   gemm_fwd   Y = act(X W^T + b)         (W [N][K] bf16, K, N <= 128)
//   gemm_dx    dX = dZ W                   (dZ = dY * act'(Z) fused in)
//   gemm_dw    dW += dZ^T X, db += sum dZ  (block partials, atomicAdd)
//   head_loss  outputs [M][5]: squared error on log H0, softmax
//              cross-entropy on 4 stiffness bins; writes dOut
//   adam       fp32 master weights, bf16 copy for the forward pass
//
// Tiles: a 256-thread block computes 64 rows x up to 128 columns, each thread
// a 4 x 8 register tile; X and W tiles are staged in shared memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "kpp_mlp.h"

namespace gcmlp {

constexpr int TM = 64;     // rows per block
constexpr int KMAX = 128;  // max input width
constexpr int NMAX = 128;  // max output width

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
  return cdf + z * pdf;
}

// ---------------------------------------------------------------- features
__global__ void features_kernel(FeatureArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= a.ncell) return;
  float* x = a.x + (long long)cell * NFEAT;
  const double t = a.met[0 * a.ldm + cell];
  const double nd = a.met[1 * a.ldm + cell];
  const double h2o = a.met[2 * a.ldm + cell];
  const double p = a.met[3 * a.ldm + cell];
  double f[NFEAT];
  f[0] = log(t);
  f[1] = log(fmax(p, 1e-6));
  f[2] = log(fmax(h2o / fmax(nd, 1.0), 1e-12));
  f[3] = a.suncos ? a.suncos[cell] : 0.0;
  for (int j = 0; j < NJ; ++j) f[4 + j] = log(fmax(a.photol[(long long)a.jslot[j] * a.ldp + cell], 1e-20));
  for (int s = 0; s < NSPC; ++s)
    f[4 + NJ + s] = log(fmax(a.c[(long long)a.spc[s] * a.ldc + cell] / fmax(nd, 1.0), 1e-30));
  for (int i = 0; i < NFEAT; ++i) x[i] = (float)((f[i] - a.mean[i]) * a.inv_std[i]);
}

// ---------------------------------------------------------------- forward
// Y[M][N] = act(X[M][K] W[N][K]^T + b); Z (pre-activation) kept if non-null.
__global__ void __launch_bounds__(256) gemm_fwd_kernel(const float* __restrict__ X, const __nv_bfloat16* __restrict__ W,
                                                       const float* __restrict__ b, float* __restrict__ Z,
                                                       float* __restrict__ Y, int M, int K, int N, int act) {
  extern __shared__ float smem[];
  float (*xs)[KMAX + 1] = reinterpret_cast<float (*)[KMAX + 1]>(smem);
  float (*ws)[KMAX + 1] = reinterpret_cast<float (*)[KMAX + 1]>(smem + TM * (KMAX + 1));
  const int row0 = blockIdx.x * TM;
  for (int i = threadIdx.x; i < TM * K; i += blockDim.x) {
    const int r = i / K, k = i % K;
    xs[r][k] = (row0 + r < M) ? X[(long long)(row0 + r) * K + k] : 0.0f;
  }
  for (int i = threadIdx.x; i < N * K; i += blockDim.x) ws[i / K][i % K] = __bfloat162float(W[i]);
  __syncthreads();
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;  // 16 x 16 threads, 4 rows x 8 cols each
  float acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
  for (int k = 0; k < K; ++k) {
    float xr[4], wc[8];
#pragma unroll
    for (int i = 0; i < 4; ++i) xr[i] = xs[ty * 4 + i][k];
#pragma unroll
    for (int j = 0; j < 8; ++j) wc[j] = (tx * 8 + j < N) ? ws[tx * 8 + j][k] : 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(xr[i], wc[j], acc[i][j]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = row0 + ty * 4 + i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n = tx * 8 + j;
      if (n >= N) continue;
      const float z = acc[i][j] + b[n];
      if (Z) Z[(long long)r * N + n] = z;
      Y[(long long)r * N + n] = act ? gelu(z) : z;
    }
  }
}

// ---------------------------------------------------------------- backward
// dX[M][K] = (dY * act'(Z))[M][N] W[N][K]; also writes dZ for gemm_dw.
__global__ void __launch_bounds__(256) gemm_dx_kernel(const float* __restrict__ dY, const float* __restrict__ Z,
                                                      const __nv_bfloat16* __restrict__ W, float* __restrict__ dZ,
                                                      float* __restrict__ dX, int M, int K, int N, int act) {
  extern __shared__ float smem[];
  float (*gs)[NMAX + 1] = reinterpret_cast<float (*)[NMAX + 1]>(smem);
  float (*ws)[KMAX + 1] = reinterpret_cast<float (*)[KMAX + 1]>(smem + TM * (NMAX + 1));
  const int row0 = blockIdx.x * TM;
  for (int i = threadIdx.x; i < TM * N; i += blockDim.x) {
    const int r = i / N, n = i % N;
    float g = 0.0f;
    if (row0 + r < M) {
      g = dY[(long long)(row0 + r) * N + n];
      if (act) g *= gelu_grad(Z[(long long)(row0 + r) * N + n]);
      dZ[(long long)(row0 + r) * N + n] = g;
    }
    gs[r][n] = g;
  }
  if (dX) {
    for (int i = threadIdx.x; i < N * K; i += blockDim.x) ws[i / K][i % K] = __bfloat162float(W[i]);
  }
  __syncthreads();
  if (!dX) return;
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
  float acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
  for (int n = 0; n < N; ++n) {
    float gr[4], wk[8];
#pragma unroll
    for (int i = 0; i < 4; ++i) gr[i] = gs[ty * 4 + i][n];
#pragma unroll
    for (int j = 0; j < 8; ++j) wk[j] = (tx * 8 + j < K) ? ws[n][tx * 8 + j] : 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(gr[i], wk[j], acc[i][j]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = row0 + ty * 4 + i;
    if (r >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = tx * 8 + j;
      if (k < K) dX[(long long)r * K + k] = acc[i][j];
    }
  }
}

// dW[N][K] += dZ^T X over this block's rows; db[N] += column sums of dZ.
__global__ void __launch_bounds__(256) gemm_dw_kernel(const float* __restrict__ dZ, const float* __restrict__ X,
                                                      float* __restrict__ dW, float* __restrict__ db, int M, int K,
                                                      int N, int rows_per_block) {
  extern __shared__ float smem[];
  float (*gs)[NMAX + 1] = reinterpret_cast<float (*)[NMAX + 1]>(smem);
  float (*xs)[KMAX + 1] = reinterpret_cast<float (*)[KMAX + 1]>(smem + TM * (NMAX + 1));
  const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;  // thread tile: 8 n x 8 k
  float acc[8][8];
  float bacc[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    bacc[i] = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
  }
  const int r_begin = blockIdx.x * rows_per_block;
  const int r_end = min(M, r_begin + rows_per_block);
  for (int r0 = r_begin; r0 < r_end; r0 += TM) {
    __syncthreads();
    for (int i = threadIdx.x; i < TM * N; i += blockDim.x) {
      const int r = i / N, n = i % N;
      gs[r][n] = (r0 + r < r_end) ? dZ[(long long)(r0 + r) * N + n] : 0.0f;
    }
    for (int i = threadIdx.x; i < TM * K; i += blockDim.x) {
      const int r = i / K, k = i % K;
      xs[r][k] = (r0 + r < r_end) ? X[(long long)(r0 + r) * K + k] : 0.0f;
    }
    __syncthreads();
    for (int r = 0; r < TM; ++r) {
      float gn[8], xk[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) gn[i] = (ty * 8 + i < N) ? gs[r][ty * 8 + i] : 0.0f;
#pragma unroll
      for (int j = 0; j < 8; ++j) xk[j] = (tx * 8 + j < K) ? xs[r][tx * 8 + j] : 0.0f;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if (tx == 0) bacc[i] += gn[i];
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(gn[i], xk[j], acc[i][j]);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int n = ty * 8 + i;
    if (n >= N) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = tx * 8 + j;
      if (k < K) atomicAdd(dW + (long long)n * K + k, acc[i][j]);
    }
    if (tx == 0 && db) atomicAdd(db + n, bacc[i]);
  }
}

// ---------------------------------------------------------------- loss head
// out[M][5]: out[:,0] predicts log H0 (target y_h), out[:,1:5] bin logits
// (target y_bin).  loss = mean((out0-y_h)^2) + w_ce * mean(CE).
__global__ void head_loss_kernel(const float* __restrict__ out, const float* __restrict__ y_h,
                                 const int* __restrict__ y_bin, float* __restrict__ dout, float* __restrict__ loss,
                                 int M, float w_ce) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (r < M) {
    const float* o = out + (long long)r * NOUT;
    float* d = dout + (long long)r * NOUT;
    const float e = o[0] - y_h[r];
    d[0] = 2.0f * e / M;
    l = e * e;
    float mx = o[1];
    for (int k = 2; k < NOUT; ++k) mx = fmaxf(mx, o[k]);
    float s = 0.0f, p[NOUT];
    for (int k = 1; k < NOUT; ++k) {
      p[k] = expf(o[k] - mx);
      s += p[k];
    }
    const int y = y_bin[r];
    for (int k = 1; k < NOUT; ++k) {
      const float q = p[k] / s;
      d[k] = w_ce * (q - (k - 1 == y ? 1.0f : 0.0f)) / M;
    }
    l += w_ce * -(o[1 + y] - mx - logf(s));
  }
  // block reduction of the loss
  __shared__ float red[256];
  red[threadIdx.x] = l;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, red[0] / M);
}

// ---------------------------------------------------------------- optimiser
__global__ void adam_kernel(float* __restrict__ w, __nv_bfloat16* __restrict__ wb, float* __restrict__ g,
                            float* __restrict__ m1, float* __restrict__ m2, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.0f - b1) * gi;
  const float v = b2 * m2[i] + (1.0f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = v;
  const float upd = lr * (a / c1) / (sqrtf(v / c2) + eps);
  const float nw = w[i] - upd;
  w[i] = nw;
  if (wb) wb[i] = __float2bfloat16_rn(nw);
  g[i] = 0.0f;
}

// ---------------------------------------------------------------- proposals
// From the head outputs: H0 = scale * exp(out0), bin = argmax(out1..4).
// With keep, an H0 entry that is already positive (a KPPHvalue) stays.
__global__ void propose_kernel(const float* __restrict__ out, int M, double scale, double hmin, double hmax,
                               double* __restrict__ h0, int* __restrict__ bin, int keep) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= M) return;
  const float* o = out + (long long)r * NOUT;
  double h = scale * exp((double)o[0]);
  h = fmin(fmax(h, hmin), hmax);
  if (h0 && !(keep && h0[r] > 0.0)) h0[r] = h;
  int b = 0;
  for (int k = 1; k < NBIN; ++k)
    if (o[1 + k] > o[1 + b]) b = k;
  if (bin) bin[r] = b;
}

// Stable counting sort of cells by bin, heaviest bin first (work-queue
// order).  Cells keep ascending index order inside a bin, so that a warp of
// the queue kernel that claims 32 consecutive positions of a dense bin reads
// mostly consecutive cells, and the order is the same on every run.
// Pass 1: per-block bin counts; pass 2: exclusive scan over (bin descending,
// block ascending); pass 3: scatter with each cell's rank inside its block.
constexpr int BO_BLOCK = 256;

__global__ void bin_block_count_kernel(const int* __restrict__ bin, int M, int* __restrict__ blk) {
  __shared__ int local[NBIN];
  if (threadIdx.x < NBIN) local[threadIdx.x] = 0;
  __syncthreads();
  const int r = blockIdx.x * BO_BLOCK + threadIdx.x;
  if (r < M) atomicAdd(&local[bin[r]], 1);
  __syncthreads();
  if (threadIdx.x < NBIN) blk[blockIdx.x * NBIN + threadIdx.x] = local[threadIdx.x];
}

// One block of 1024 threads: blk[j*NBIN+b] <- start of block j's cells of
// bin b in the order; counts[b] <- cells in bin b.
__global__ void bin_block_scan_kernel(int* __restrict__ blk, int nblk, int* __restrict__ counts) {
  __shared__ int part[1024];
  __shared__ int base;
  const int t = threadIdx.x;
  const int per = (nblk + 1023) / 1024;
  const int j0 = t * per, j1 = min(nblk, j0 + per);
  if (t == 0) base = 0;
  __syncthreads();
  for (int b = NBIN - 1; b >= 0; --b) {
    int sum = 0;
    for (int j = j0; j < j1; ++j) sum += blk[j * NBIN + b];
    part[t] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
      const int v = t >= off ? part[t - off] : 0;
      __syncthreads();
      part[t] += v;
      __syncthreads();
    }
    int run = base + part[t] - sum;
    for (int j = j0; j < j1; ++j) {
      const int c = blk[j * NBIN + b];
      blk[j * NBIN + b] = run;
      run += c;
    }
    __syncthreads();
    if (t == 1023) {
      counts[b] = part[1023];
      base += part[1023];
    }
    __syncthreads();
  }
}

__global__ void bin_stable_scatter_kernel(const int* __restrict__ bin, int M, const int* __restrict__ blk,
                                          int* __restrict__ order) {
  __shared__ int wcnt[BO_BLOCK / 32][NBIN];
  const int r = blockIdx.x * BO_BLOCK + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = r < M ? bin[r] : -1;
  const unsigned lt = (1u << lane) - 1u;
  int rank = 0;
  for (int k = 0; k < NBIN; ++k) {
    const unsigned mk = __ballot_sync(0xffffffffu, b == k);
    if (lane == 0) wcnt[warp][k] = __popc(mk);
    if (b == k) rank = __popc(mk & lt);
  }
  __syncthreads();
  if (b >= 0) {
    int pos = blk[blockIdx.x * NBIN + b] + rank;
    for (int w = 0; w < warp; ++w) pos += wcnt[w][b];
    order[pos] = r;
  }
}

// ---------------------------------------------------------------- launchers
constexpr size_t SMEM_FWD = (size_t)(TM + NMAX) * (KMAX + 1) * sizeof(float);
constexpr size_t SMEM_DX = (size_t)TM * (NMAX + 1) * sizeof(float) + (size_t)NMAX * (KMAX + 1) * sizeof(float);
constexpr size_t SMEM_DW = (size_t)TM * (NMAX + 1) * sizeof(float) + (size_t)TM * (KMAX + 1) * sizeof(float);

static cudaError_t smem_attrs() {
  static bool done = false;
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(gemm_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_FWD);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(gemm_dx_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_DX);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(gemm_dw_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_DW);
  if (e == cudaSuccess) done = true;
  return e;
}

cudaError_t features(const FeatureArgs& a, cudaStream_t s) {
  if (a.ncell > 0) features_kernel<<<(a.ncell + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}
cudaError_t gemm_fwd(const float* X, const __nv_bfloat16* W, const float* b, float* Z, float* Y, int M, int K, int N,
                     int act, cudaStream_t s) {
  if (K > KMAX || N > NMAX) return cudaErrorInvalidValue;
  cudaError_t e = smem_attrs();
  if (e != cudaSuccess) return e;
  if (M > 0) gemm_fwd_kernel<<<(M + TM - 1) / TM, 256, SMEM_FWD, s>>>(X, W, b, Z, Y, M, K, N, act);
  return cudaGetLastError();
}
cudaError_t gemm_dx(const float* dY, const float* Z, const __nv_bfloat16* W, float* dZ, float* dX, int M, int K,
                    int N, int act, cudaStream_t s) {
  if (K > KMAX || N > NMAX) return cudaErrorInvalidValue;
  cudaError_t e = smem_attrs();
  if (e != cudaSuccess) return e;
  if (M > 0) gemm_dx_kernel<<<(M + TM - 1) / TM, 256, SMEM_DX, s>>>(dY, Z, W, dZ, dX, M, K, N, act);
  return cudaGetLastError();
}
cudaError_t gemm_dw(const float* dZ, const float* X, float* dW, float* db, int M, int K, int N, cudaStream_t s) {
  if (K > KMAX || N > NMAX) return cudaErrorInvalidValue;
  cudaError_t e = smem_attrs();
  if (e != cudaSuccess) return e;
  const int rows = 1024;
  if (M > 0) gemm_dw_kernel<<<(M + rows - 1) / rows, 256, SMEM_DW, s>>>(dZ, X, dW, db, M, K, N, rows);
  return cudaGetLastError();
}
cudaError_t head_loss(const float* out, const float* y_h, const int* y_bin, float* dout, float* loss, int M,
                      float w_ce, cudaStream_t s) {
  if (M > 0) head_loss_kernel<<<(M + 255) / 256, 256, 0, s>>>(out, y_h, y_bin, dout, loss, M, w_ce);
  return cudaGetLastError();
}
cudaError_t adam(float* w, __nv_bfloat16* wb, float* g, float* m1, float* m2, int n, float lr, float b1, float b2,
                 float eps, int step, cudaStream_t s) {
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  if (n > 0) adam_kernel<<<(n + 255) / 256, 256, 0, s>>>(w, wb, g, m1, m2, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}
cudaError_t propose(const float* out, int M, double scale, double hmin, double hmax, double* h0, int* bin,
                    int keep, cudaStream_t s) {
  if (M > 0) propose_kernel<<<(M + 255) / 256, 256, 0, s>>>(out, M, scale, hmin, hmax, h0, bin, keep);
  return cudaGetLastError();
}
int bin_order_scratch(int M) { return NBIN * std::max(1, (M + BO_BLOCK - 1) / BO_BLOCK); }

cudaError_t bin_order(const int* bin, int M, int* counts, int* scratch, int* order, cudaStream_t s) {
  if (M == 0) return cudaMemsetAsync(counts, 0, NBIN * sizeof(int), s);
  const int nblk = (M + BO_BLOCK - 1) / BO_BLOCK;
  bin_block_count_kernel<<<nblk, BO_BLOCK, 0, s>>>(bin, M, scratch);
  bin_block_scan_kernel<<<1, 1024, 0, s>>>(scratch, nblk, counts);
  bin_stable_scatter_kernel<<<nblk, BO_BLOCK, 0, s>>>(bin, M, scratch, order);
  return cudaGetLastError();
}

}  // namespace gcmlp
