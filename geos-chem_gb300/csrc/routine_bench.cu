// Profiling aid, not part of the C ABI: one launch per mechanism routine of
// the thread-per-cell kernel (KppDecomp in its row-wise form, KppSolve,
// Fun_SPLIT with its A and B products, the B products alone, Jac_SP), each
// on its own workspace tile of nthreads cells filled with positive values,
// so that a profiler can count the FP64 instructions every routine executes
// per cell (the fast arithmetic, one cell per thread, the library's tables).
#include <cuda_runtime.h>

#include "kpp_mech.cuh"
#include "mech_tables.inc"

namespace {

using namespace gckpp;
namespace T = gcmech_tables;

// entries of one cell's tile: aux, Y, A, B, Fun output / J0, G, X
constexpr int SLOT = T::NAUX + T::NSPEC + T::NREACT + T::NB + 2 * T::LU_NONZERO + T::NVAR;

__device__ __forceinline__ double* tile(double* ws) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  return ws + (t / TS) * (long long)SLOT * TS + (t % TS);
}

__global__ void rb_decomp(MechDev m, double* ws, int* ier) {
  double* w = tile(ws);
  double ghinv[1] = {4.0};
  int e[1];
  decomp_rows<false, 1>(m, w, ghinv, w + T::LU_NONZERO * TS, e);
  ier[blockIdx.x * blockDim.x + threadIdx.x] = e[0];
}

__global__ void rb_solve(MechDev m, double* ws) {
  double* w = tile(ws);
  solve<false, 1>(m, w, w + 2 * T::LU_NONZERO * TS);
}

__global__ void rb_fun(MechDev m, double* ws) {
  double* w = tile(ws);
  double* aux = w;
  double* Y = aux + T::NAUX * TS;
  double* A = Y + T::NSPEC * TS;
  double* B = A + T::NREACT * TS;
  b_products<1>(m, Y, aux, B);
  fun_split<false, 1>(m, Y, aux, A, B, B + T::NB * TS);
}

__global__ void rb_bprod(MechDev m, double* ws) {
  double* w = tile(ws);
  b_products<1>(m, w + T::NAUX * TS, w, w + (T::NAUX + T::NSPEC + T::NREACT) * TS);
}

__global__ void rb_jac(MechDev m, double* ws) {
  double* w = tile(ws);
  jac_sp<false, 1>(m, w, w + T::NB * TS);
}

__global__ void rb_fill(double* p, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 1.0 + 1.0e-3 * (double)(i % 97);
}

template <class X>
cudaError_t up(const X* h, size_t n, const X** d) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, n * sizeof(X));
  if (e == cudaSuccess) e = cudaMemcpy(p, h, n * sizeof(X), cudaMemcpyHostToDevice);
  *d = static_cast<const X*>(p);
  return e;
}

}  // namespace

// Runs the routines once each, in the order decomp, solve, fun, bprod, jac,
// over nthreads cells (a multiple of 128).  Returns 0 or a CUDA error code.
extern "C" int gc_routine_bench(int device, int nthreads) {
  if (nthreads <= 0 || nthreads % 128) return -1;
  if (cudaSetDevice(device) != cudaSuccess) return -2;
  MechDev m{};
  m.nvar = T::NVAR; m.nfix = T::NFIX; m.nreact = T::NREACT; m.nspec = T::NSPEC;
  m.lu_nonzero = T::LU_NONZERO; m.nb = T::NB; m.lit0 = T::LIT0; m.naux = T::NAUX;
  cudaError_t e = up(reinterpret_cast<const uint2*>(T::prod_packed), sizeof(T::prod_packed) / 8, &m.prod_packed);
#define RB_UP(f, a) \
  if (e == cudaSuccess) e = up(T::a, sizeof(T::a) / sizeof(T::a[0]), &m.f);
  RB_UP(prod_ids_a, prod_ids_a) RB_UP(prod_ids_b, prod_ids_b) RB_UP(p_start, p_start) RB_UP(p_sterm, p_sterm)
  RB_UP(slit, slit) RB_UP(d_start, d_start) RB_UP(d_sterm, d_sterm) RB_UP(j_start, j_start)
  RB_UP(j_sterm, j_sterm) RB_UP(lu_crow, lu_crow) RB_UP(lu_diag, lu_diag) RB_UP(lu_icol, lu_icol)
  RB_UP(dot_start, dot_start) RB_UP(dot_term, dot_term)
#undef RB_UP
  for (int i = 0; i < 9; ++i) {
    m.a_cls[i] = T::a_cls_start[i];
    m.b_cls[i] = T::b_cls_start[i];
  }
  const long long n = (long long)nthreads * SLOT;
  double* ws = nullptr;
  int* ier = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&ws, n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&ier, nthreads * sizeof(int));
  const int fb = (int)((n + 255) / 256), g = nthreads / 128;
  if (e == cudaSuccess) {
    rb_fill<<<fb, 256>>>(ws, n);
    rb_decomp<<<g, 128>>>(m, ws, ier);
    rb_fill<<<fb, 256>>>(ws, n);
    rb_solve<<<g, 128>>>(m, ws);
    rb_fill<<<fb, 256>>>(ws, n);
    rb_fun<<<g, 128>>>(m, ws);
    rb_bprod<<<g, 128>>>(m, ws);
    rb_jac<<<g, 128>>>(m, ws);
    e = cudaDeviceSynchronize();
  }
  const void* tabs[] = {m.prod_packed, m.prod_ids_a, m.prod_ids_b, m.p_start, m.p_sterm, m.slit, m.d_start,
                        m.d_sterm, m.j_start, m.j_sterm, m.lu_crow, m.lu_diag, m.lu_icol, m.dot_start, m.dot_term};
  for (const void* p : tabs) cudaFree(const_cast<void*>(p));
  cudaFree(ws);
  cudaFree(ier);
  return e == cudaSuccess ? 0 : (int)e;
}
