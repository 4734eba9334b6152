// Small element-wise kernels of the chemistry-step boundary.
#include "kpp_util.h"

namespace gcutil {

// C(k, cell) = MAX(C(k, cell), 0) for all species (fullchem_mod.F90:1329-1350)
__global__ void clamp_nonneg_kernel(double* c, long long ldc, int nrows, int ncell) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)nrows * ncell;
  if (i >= total) return;
  const long long k = i / ncell, cell = i % ncell;
  double* p = c + k * ldc + cell;
  *p = fmax(*p, 0.0);
}

cudaError_t clamp_nonneg(double* c, long long ldc, int nrows, int ncell, cudaStream_t s) {
  const long long total = (long long)nrows * ncell;
  if (total == 0) return cudaSuccess;
  const int block = 256;
  const long long grid = (total + block - 1) / block;
  clamp_nonneg_kernel<<<(unsigned)grid, block, 0, s>>>(c, ldc, nrows, ncell);
  return cudaGetLastError();
}

}  // namespace gcutil
