// FP64 FMA throughput probe: the denominator of the solver's FP64 roofline.
// Independent DFMA chains per thread over a grid of a few waves; returns the
// best of several timed launches in GFLOP/s (an FMA counts as 2 flops).
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256) dfma_chains(double* sink, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  if (s == -1.2345) sink[0] = s;  // keeps the chains live
}

}  // namespace

extern "C" int gc_probe_fp64_gflops(int device, double* gflops) {
  if (!gflops) return -1;
  if (cudaSetDevice(device) != cudaSuccess) return -2;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return -2;
  double* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return -3;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int block = 256, grid = prop.multiProcessorCount * 4, iters = 4096;
  double best = 0.0;
  dfma_chains<<<grid, block>>>(sink, iters, 0.999999, 1e-7);
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    dfma_chains<<<grid, block>>>(sink, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double g = 2.0 * 8.0 * iters * (double)grid * block / (ms * 1e-3) / 1e9;
    if (g > best) best = g;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  *gflops = best;
  return cudaGetLastError() == cudaSuccess ? 0 : -4;
}
