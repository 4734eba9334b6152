// Rosenbrock kernels, compiled once per variant (build.py):
//   strict   -DGCKPP_STRICT=1 -fmad=false   reference evaluation order, 1 cell/thread
//   fast     -DGCKPP_STRICT=0               FMA, reciprocal pivots, GCKPP_NC cells/thread
//   fast1    fast with 1 cell per thread
//   fast4    fast with 4 cells per thread
#include "kpp_launch.h"
#include "kpp_rosenbrock.cuh"

#ifndef GCKPP_MAX_THREADS
#define GCKPP_MAX_THREADS 1024  // 1024 threads x 64 registers fill an SM
#endif
#ifndef GCKPP_NC
#define GCKPP_NC 1  // cells per thread
#endif
#ifndef GCKPP_VARIANT
#define GCKPP_VARIANT fast
#endif
#define GCKPP_CAT2(a, b) a##b
#define GCKPP_CAT(a, b) GCKPP_CAT2(a, b)

namespace gckpp {

template <bool QUEUE>
__global__ void __launch_bounds__(GCKPP_MAX_THREADS, 1) ros_kernel(MechDev m, RosMethod r, RosParams p) {
  ros_driver<GCKPP_STRICT != 0, QUEUE, GCKPP_NC>(m, r, p);
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

int GCKPP_CAT(gckpp_cells_per_thread_, GCKPP_VARIANT)() { return GCKPP_NC; }

cudaError_t GCKPP_CAT(gckpp_occupancy_, GCKPP_VARIANT)(int queue, int block, int* nblocks) {
  if (queue) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_kernel<true>, block, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_kernel<false>, block, 0);
}

}  // namespace gckpp
