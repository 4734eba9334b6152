// Small element-wise kernels of the chemistry-step boundary.
#include "kpp_util.h"

#include <algorithm>
#include <cstdint>

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

// Rows of m elements of type V; each thread keeps four loads in flight.
template <typename V>
__global__ void copy_rows_kernel(char* dst, size_t dpitch, const char* src, size_t spitch, long long m,
                                 long long rows) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long r = blockIdx.y; r < rows; r += gridDim.y) {
    V* d = reinterpret_cast<V*>(dst + r * (long long)dpitch);
    const V* s = reinterpret_cast<const V*>(src + r * (long long)spitch);
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < m; i += 4 * stride) {
      const V a = s[i], b = s[i + stride], c = s[i + 2 * stride], e = s[i + 3 * stride];
      d[i] = a;
      d[i + stride] = b;
      d[i + 2 * stride] = c;
      d[i + 3 * stride] = e;
    }
    for (; i < m; i += stride) d[i] = s[i];
  }
}

// The address at which the current device reaches p, or nullptr when it
// cannot (pageable host memory).
static void* device_alias(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return const_cast<void*>(p);
  if (a.type == cudaMemoryTypeHost && a.devicePointer) {
    // offset of p within what the attributes describe (0 when they describe p itself)
    const char* hp = a.hostPointer ? static_cast<const char*>(a.hostPointer) : static_cast<const char*>(p);
    return static_cast<char*>(a.devicePointer) + (static_cast<const char*>(p) - hp);
  }
  return nullptr;
}

cudaError_t copy_rows(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t rows,
                      cudaStream_t s) {
  if (rows == 0 || width == 0) return cudaSuccess;
  void* d = device_alias(dst);
  const void* sp = device_alias(src);
  const size_t bits = (size_t)(uintptr_t)d | (size_t)(uintptr_t)sp | dpitch | spitch | width;
  if (!d || !sp || (bits & 3)) return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, cudaMemcpyDefault, s);
  const int g = (bits & 15) == 0 ? 16 : (bits & 7) == 0 ? 8 : 4;
  const long long m = (long long)(width / g);
  const int threads = 256;
  const long long gx = std::min<long long>((m + 4LL * threads - 1) / (4LL * threads), 65535LL);
  const dim3 grid((unsigned)gx, (unsigned)std::min<size_t>(rows, 65535));
  char* dc = static_cast<char*>(d);
  const char* sc = static_cast<const char*>(sp);
  if (g == 16)
    copy_rows_kernel<uint4><<<grid, threads, 0, s>>>(dc, dpitch, sc, spitch, m, (long long)rows);
  else if (g == 8)
    copy_rows_kernel<uint2><<<grid, threads, 0, s>>>(dc, dpitch, sc, spitch, m, (long long)rows);
  else
    copy_rows_kernel<unsigned><<<grid, threads, 0, s>>>(dc, dpitch, sc, spitch, m, (long long)rows);
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
