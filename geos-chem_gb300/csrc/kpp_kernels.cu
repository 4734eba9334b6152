// Rosenbrock kernels, compiled once per variant (build.py):
//   strict   -DGCKPP_STRICT=1 -fmad=false   reference evaluation order
//   fast     -DGCKPP_STRICT=0               FMA, reciprocal pivots
//   fastcg   fast + per-cell reads bypass L1 (GCKPP_LDCG)
//   fast128  fast with a 128-register budget (half the resident warps)
#include "kpp_launch.h"
#include "kpp_rosenbrock.cuh"

#ifndef GCKPP_MAX_THREADS
#define GCKPP_MAX_THREADS 1024  // 1024 threads x 64 registers fill an SM
#endif
#ifndef GCKPP_VARIANT
#define GCKPP_VARIANT fast
#endif
#define GCKPP_CAT2(a, b) a##b
#define GCKPP_CAT(a, b) GCKPP_CAT2(a, b)

namespace gckpp {

template <bool QUEUE>
__global__ void __launch_bounds__(GCKPP_MAX_THREADS, 1) ros_kernel(MechDev m, RosMethod r, RosParams p) {
  ros_driver<GCKPP_STRICT != 0, QUEUE>(m, r, p);
}

cudaError_t GCKPP_CAT(gckpp_launch_ros_, GCKPP_VARIANT)(int queue, int grid, int block, const MechDev& m,
                                                        const RosMethod& r, const RosParams& p, cudaStream_t s) {
  if (block > GCKPP_MAX_THREADS) return cudaErrorInvalidConfiguration;
  if (queue)
    ros_kernel<true><<<grid, block, 0, s>>>(m, r, p);
  else
    ros_kernel<false><<<grid, block, 0, s>>>(m, r, p);
  return cudaGetLastError();
}

cudaError_t GCKPP_CAT(gckpp_occupancy_, GCKPP_VARIANT)(int queue, int block, int* nblocks) {
  if (queue) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_kernel<true>, block, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_kernel<false>, block, 0);
}

}  // namespace gckpp
