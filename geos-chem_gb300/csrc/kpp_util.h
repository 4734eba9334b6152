#pragma once
#include <cuda_runtime.h>

namespace gcutil {
cudaError_t clamp_nonneg(double* c, long long ldc, int nrows, int ncell, cudaStream_t s);
// device-side step plumbing (no host synchronisation; capturable in a graph)
cudaError_t split_ranges(const int* nblock, int ncell, int* ranges, cudaStream_t s);
cudaError_t collect_failed(const int* ierr, int ncell, int* list, int* range, cudaStream_t s);
cudaError_t fill_error(int code, int ncell, int* ierr, int* istatus, double* rstatus, long long ldo, cudaStream_t s);
// Stream-ordered copy of `rows` rows of `width` bytes from src (row pitch
// spitch bytes) to dst (pitch dpitch), either side in host or device memory.
// When both sides are device-accessible -- device memory, or page-locked host
// memory (cudaHostAlloc, cudaHostRegister) through its device alias -- the
// SMs copy with 16-, 8- or 4-byte loads and stores; otherwise (pageable host
// memory, or addresses not 4-byte aligned) cudaMemcpy2DAsync does.
cudaError_t copy_rows(void* dst, size_t dpitch, const void* src, size_t spitch, size_t width, size_t rows,
                      cudaStream_t s);
}
