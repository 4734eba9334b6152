// Rosenbrock kernels, compiled once per variant (build.py):
//   strict   -DGCKPP_STRICT=1 -fmad=false   reference evaluation order, 1 cell/thread
//   fast     -DGCKPP_STRICT=0               FMA, reciprocal pivots, 1 cell/thread
//   fast2    fast with 2 cells per thread
//   fast4    fast with 4 cells per thread
// On the 4x5x72 grid step the 1-cell form is the fastest (the 2- and 4-cell
// forms spill registers and hold fewer warps per SM).
#include "kpp_launch.h"
#include "kpp_block.cuh"
#include "kpp_rosenbrock.cuh"

#ifndef GCKPP_MAX_THREADS
#define GCKPP_MAX_THREADS 1024  // 1024 threads x 64 registers fill an SM
#endif
#ifndef GCKPP_NC
#define GCKPP_NC 1  // cells per thread
#endif
#ifndef GCKPP_SPLIT_NT
#define GCKPP_SPLIT_NT 256  // threads of the split block-per-cell kernel (tables.py SPLIT_NT)
#endif
#ifndef GCKPP_VARIANT
#define GCKPP_VARIANT fast
#endif
#define GCKPP_CAT2(a, b) a##b
#define GCKPP_CAT(a, b) GCKPP_CAT2(a, b)

namespace gckpp {

template <bool QUEUE, bool AR>
__global__ void __launch_bounds__(GCKPP_MAX_THREADS, 1) ros_kernel(MechDev m, RosMethod r, RosParams p) {
  ros_driver<GCKPP_STRICT != 0, QUEUE, GCKPP_NC, AR>(m, r, p);
}

// ar = 1: the auto-reducing integrator (one cell per thread only)
cudaError_t GCKPP_CAT(gckpp_launch_ros_, GCKPP_VARIANT)(int queue, int grid, int block, const MechDev& m,
                                                        const RosMethod& r, const RosParams& p, cudaStream_t s,
                                                        int ar) {
  if (block > GCKPP_MAX_THREADS) return cudaErrorInvalidConfiguration;
#if GCKPP_NC == 1
  if (ar) {
    if (queue)
      ros_kernel<true, true><<<grid, block, 0, s>>>(m, r, p);
    else
      ros_kernel<false, true><<<grid, block, 0, s>>>(m, r, p);
    return cudaGetLastError();
  }
#else
  if (ar) return cudaErrorInvalidConfiguration;
#endif
  if (queue)
    ros_kernel<true, false><<<grid, block, 0, s>>>(m, r, p);
  else
    ros_kernel<false, false><<<grid, block, 0, s>>>(m, r, p);
  return cudaGetLastError();
}

int GCKPP_CAT(gckpp_cells_per_thread_, GCKPP_VARIANT)() { return GCKPP_NC; }

cudaError_t GCKPP_CAT(gckpp_occupancy_, GCKPP_VARIANT)(int queue, int block, int* nblocks) {
  if (queue) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_kernel<true, false>, block, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_kernel<false, false>, block, 0);
}

#if GCKPP_NC == 1
// Block-per-cell form (kpp_block.cuh), built in the 1-cell-per-thread units.
// (a template, so that each variant's translation unit keeps its own kernel)
template <bool STRICT>
__global__ void __launch_bounds__(1024) ros_block_kernel(MechDev m, RosMethod r, RosParams p) {
  ros_block_driver<STRICT>(m, r, p);
}

size_t GCKPP_CAT(gckpp_block_smem_, GCKPP_VARIANT)(const MechDev& m, const RosMethod& r, int autonomous) {
  return sizeof(double) *
         (size_t)block_layout(m.naux, m.nspec, m.nvar, m.nreact, m.nb, m.lu_nonzero, r.S, autonomous).total;
}

// resident blocks per SM of the block-per-cell kernel
cudaError_t GCKPP_CAT(gckpp_block_occupancy_, GCKPP_VARIANT)(int block, size_t smem, int* nblocks) {
  static int smem_set[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64 || smem_set[dev] < (int)smem) {
    e = cudaFuncSetAttribute(ros_block_kernel<GCKPP_STRICT != 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) smem_set[dev] = (int)smem;
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_block_kernel<GCKPP_STRICT != 0>, block, smem);
}

cudaError_t GCKPP_CAT(gckpp_launch_block_, GCKPP_VARIANT)(int grid, int block, const MechDev& m, const RosMethod& r,
                                                          const RosParams& p, cudaStream_t s) {
  if (block < 32 || block > 1024 || block % 32) return cudaErrorInvalidConfiguration;
  const size_t smem = GCKPP_CAT(gckpp_block_smem_, GCKPP_VARIANT)(m, r, p.autonomous);
  int nblk = 0;  // also sets the shared-memory attribute
  cudaError_t e = GCKPP_CAT(gckpp_block_occupancy_, GCKPP_VARIANT)(block, smem, &nblk);
  if (e != cudaSuccess) return e;
  if (nblk < 1) return cudaErrorInvalidConfiguration;
  ros_block_kernel<GCKPP_STRICT != 0><<<grid, block, smem, s>>>(m, r, p);
  return cudaGetLastError();
}
#endif

#if GCKPP_NC == 1 && GCKPP_STRICT == 0
// Split block-per-cell form: SPLIT_NT threads, sums cut across warp lanes.
__global__ void __launch_bounds__(GCKPP_SPLIT_NT, 3) ros_block_split_kernel(MechDev m, RosMethod r, RosParams p) {
  GCKPP_PHASE_BEGIN();
  ros_block_driver<false, true>(m, r, p);
  GCKPP_PHASE_END(7, threadIdx.x == 0)
}

#ifdef GCKPP_PHASE_CYCLES
// Profiling build only: copies the split kernel's phase counters (16
// values: cycles of LU, forward and backward substitution, Fun_SPLIT,
// Jac_SP, -, -, whole kernel; then the call counts) and optionally clears
// them.  Synchronises the device.
extern "C" int gc_kpp_phase_cycles(unsigned long long* out, int reset) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(out, g_phase_cycles, sizeof(g_phase_cycles));
  if (e == cudaSuccess && reset) {
    const unsigned long long zero[16] = {};
    e = cudaMemcpyToSymbol(g_phase_cycles, zero, sizeof(zero));
  }
  return (int)e;
}
#endif

// the cell's arrays, 16-byte aligned, and the ring of staged substitution
// records
size_t gckpp_block_smem_split(const MechDev& m, const RosMethod& r, int autonomous) {
  const int total = block_layout(m.naux, m.nspec, m.nvar, m.nreact, m.nb, m.lu_nonzero, r.S, autonomous).total;
  return sizeof(double) * (size_t)((total + 1) & ~1) + SPLIT_RING_BYTES;
}

cudaError_t gckpp_block_occupancy_split(size_t smem, int* nblocks) {
  static int smem_set[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64 || smem_set[dev] < (int)smem) {
    e = cudaFuncSetAttribute(ros_block_split_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) smem_set[dev] = (int)smem;
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_block_split_kernel, GCKPP_SPLIT_NT, smem);
}

cudaError_t gckpp_launch_block_split(int grid, const MechDev& m, const RosMethod& r, const RosParams& p,
                                     cudaStream_t s) {
  for (int ph = 0; ph < 5; ++ph)  // each phase runs on one warp or on the whole block
    if (m.sp_nt[ph] != 32 && m.sp_nt[ph] != GCKPP_SPLIT_NT) return cudaErrorInvalidConfiguration;
  if (m.sp_nt[SP_FS] != 32 || m.sp_nt[SP_BS] != 32) return cudaErrorInvalidConfiguration;  // staged records
  const size_t smem = gckpp_block_smem_split(m, r, p.autonomous);
  int nblk = 0;  // also sets the shared-memory attribute
  cudaError_t e = gckpp_block_occupancy_split(smem, &nblk);
  if (e != cudaSuccess) return e;
  if (nblk < 1) return cudaErrorInvalidConfiguration;
  ros_block_split_kernel<<<grid, GCKPP_SPLIT_NT, smem, s>>>(m, r, p);
  return cudaGetLastError();
}
#endif

}  // namespace gckpp
