// Rosenbrock kernels, compiled twice: -DGCKPP_STRICT=1 with -fmad=false
// (reference evaluation order, no contraction) and -DGCKPP_STRICT=0 (fast).
#include "kpp_launch.h"
#include "kpp_rosenbrock.cuh"

#if GCKPP_STRICT
#define GCKPP_ARITH true
#define GCKPP_LAUNCH gckpp_launch_ros_strict
#define GCKPP_OCC gckpp_occupancy_strict
#else
#define GCKPP_ARITH false
#define GCKPP_LAUNCH gckpp_launch_ros_fast
#define GCKPP_OCC gckpp_occupancy_fast
#endif

#ifndef GCKPP_MAX_BLOCK
#define GCKPP_MAX_BLOCK 128
#endif
#ifndef GCKPP_MIN_BLOCKS
#define GCKPP_MIN_BLOCKS 8
#endif

namespace gckpp {

template <bool QUEUE>
__global__ void __launch_bounds__(GCKPP_MAX_BLOCK, GCKPP_MIN_BLOCKS) ros_kernel(MechDev m, RosMethod r, RosParams p) {
  ros_driver<GCKPP_ARITH, QUEUE>(m, r, p);
}

cudaError_t GCKPP_LAUNCH(int queue, int grid, int block, const MechDev& m, const RosMethod& r,
                         const RosParams& p, cudaStream_t s) {
  if (queue)
    ros_kernel<true><<<grid, block, 0, s>>>(m, r, p);
  else
    ros_kernel<false><<<grid, block, 0, s>>>(m, r, p);
  return cudaGetLastError();
}

cudaError_t GCKPP_OCC(int queue, int block, int* nblocks) {
  if (queue) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_kernel<true>, block, 0);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(nblocks, ros_kernel<false>, block, 0);
}

}  // namespace gckpp
