// Host-side launch interface between the C ABI and the kernel translation
// units (one per arithmetic mode).
#pragma once
#include <cuda_runtime.h>

namespace gckpp {
struct MechDev;
struct RosMethod;
struct RosParams;
cudaError_t gckpp_launch_ros_strict(int queue, int grid, int block, const MechDev& m, const RosMethod& r,
                                    const RosParams& p, cudaStream_t s);
cudaError_t gckpp_launch_ros_fast(int queue, int grid, int block, const MechDev& m, const RosMethod& r,
                                  const RosParams& p, cudaStream_t s);
cudaError_t gckpp_occupancy_strict(int queue, int block, int* nblocks);
cudaError_t gckpp_occupancy_fast(int queue, int block, int* nblocks);
}  // namespace gckpp
