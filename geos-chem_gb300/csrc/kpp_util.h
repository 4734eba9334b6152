#pragma once
#include <cuda_runtime.h>

namespace gcutil {
cudaError_t clamp_nonneg(double* c, long long ldc, int nrows, int ncell, cudaStream_t s);
// device-side step plumbing (no host synchronisation; capturable in a graph)
cudaError_t split_ranges(const int* nblock, int ncell, int* ranges, cudaStream_t s);
cudaError_t collect_failed(const int* ierr, int ncell, int* list, int* range, cudaStream_t s);
cudaError_t fill_error(int code, int ncell, int* ierr, int* istatus, double* rstatus, long long ldo, cudaStream_t s);
}
