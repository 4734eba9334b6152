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

namespace {

// ranges[0..3] = {0, nblock, nblock, ncell}: queue ranges of the
// block-per-cell and thread-per-cell kernels for a device-side nblock.
__global__ void split_ranges_kernel(const int* nblock, int ncell, int* ranges) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const int nb = min(max(*nblock, 0), ncell);
    ranges[0] = 0;
    ranges[1] = nb;
    ranges[2] = nb;
    ranges[3] = ncell;
  }
}

// Append the cells with ierr < 0 to list; range = {0, count} must start at
// {0, 0}.  Warp-aggregated: one atomic per warp.
__global__ void collect_failed_kernel(const int* ierr, int ncell, int* list, int* range) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool bad = i < ncell && ierr[i] < 0;
  const unsigned m = __ballot_sync(0xffffffffu, bad);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(range + 1, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (bad) list[base + __popc(m & ((1u << lane) - 1u))] = i;
}

// Per-call option error (:538-575 codes) for every cell, on the device.
__global__ void fill_error_kernel(int code, int ncell, int* ierr, int* istatus, double* rstatus, long long ldo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncell) return;
  ierr[i] = code;
  for (int k = 0; k < 20; ++k) {
    if (istatus) istatus[(long long)k * ldo + i] = 0;
    if (rstatus) rstatus[(long long)k * ldo + i] = 0.0;
  }
}

}  // namespace

namespace gcutil {

cudaError_t split_ranges(const int* nblock, int ncell, int* ranges, cudaStream_t s) {
  split_ranges_kernel<<<1, 32, 0, s>>>(nblock, ncell, ranges);
  return cudaGetLastError();
}

cudaError_t collect_failed(const int* ierr, int ncell, int* list, int* range, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(range, 0, 2 * sizeof(int), s);
  if (e != cudaSuccess || ncell == 0) return e;
  collect_failed_kernel<<<(ncell + 255) / 256, 256, 0, s>>>(ierr, ncell, list, range);
  return cudaGetLastError();
}

cudaError_t fill_error(int code, int ncell, int* ierr, int* istatus, double* rstatus, long long ldo, cudaStream_t s) {
  if (ncell > 0) fill_error_kernel<<<(ncell + 255) / 256, 256, 0, s>>>(code, ncell, ierr, istatus, rstatus, ldo);
  return cudaGetLastError();
}

}  // namespace gcutil
