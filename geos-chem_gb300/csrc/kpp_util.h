#pragma once
#include <cuda_runtime.h>

namespace gcutil {
cudaError_t clamp_nonneg(double* c, long long ldc, int nrows, int ncell, cudaStream_t s);
}
