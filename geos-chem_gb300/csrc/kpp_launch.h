// Host-side launch interface between the C ABI and the kernel translation
// units (one per arithmetic/code variant, see kpp_kernels.cu).
#pragma once
#include <cuda_runtime.h>

namespace gckpp {
struct MechDev;
struct RosMethod;
struct RosParams;

#define GCKPP_DECLARE_VARIANT(name)                                                                        \
  cudaError_t gckpp_launch_ros_##name(int queue, int grid, int block, const MechDev& m, const RosMethod& r, \
                                      const RosParams& p, cudaStream_t s, int ar);                         \
  cudaError_t gckpp_occupancy_##name(int queue, int block, int* nblocks);                                    \
  int gckpp_cells_per_thread_##name();

GCKPP_DECLARE_VARIANT(strict)
GCKPP_DECLARE_VARIANT(fast)
GCKPP_DECLARE_VARIANT(fast2)
GCKPP_DECLARE_VARIANT(fast4)
#undef GCKPP_DECLARE_VARIANT

// block-per-cell kernels (one block integrates one cell in shared memory)
cudaError_t gckpp_launch_block_strict(int grid, int block, const MechDev& m, const RosMethod& r, const RosParams& p,
                                      cudaStream_t s);
cudaError_t gckpp_launch_block_fast(int grid, int block, const MechDev& m, const RosMethod& r, const RosParams& p,
                                    cudaStream_t s);
size_t gckpp_block_smem_strict(const MechDev& m, const RosMethod& r, int autonomous);
size_t gckpp_block_smem_fast(const MechDev& m, const RosMethod& r, int autonomous);
size_t gckpp_block_smem_split(const MechDev& m, const RosMethod& r, int autonomous);
cudaError_t gckpp_block_occupancy_strict(int block, size_t smem, int* nblocks);
cudaError_t gckpp_block_occupancy_fast(int block, size_t smem, int* nblocks);
// split form (fast arithmetic, SPLIT_NT threads per block)
cudaError_t gckpp_launch_block_split(int grid, const MechDev& m, const RosMethod& r, const RosParams& p,
                                     cudaStream_t s);
cudaError_t gckpp_block_occupancy_split(size_t smem, int* nblocks);
}  // namespace gckpp
