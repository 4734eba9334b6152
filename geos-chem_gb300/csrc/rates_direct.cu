// Update_RCONST as straight-line code of one mechanism's rate program
// (rates_direct.inc, gcchem.rates_program emit_direct), compiled once per
// mechanism with that mechanism's generated directory on the include path:
// the operations of gcrates::rates_kernel in the same order, without its
// opcode dispatch and local-memory stack.  Results agree with the
// interpreter to rounding (a few libm calls with literal arguments are
// specialised by the compiler), within the 1e-13 parity bar of both.
#include <cuda_runtime.h>

#include "het_rates.cuh"
#include "kpp_rates.h"
#include "rate_laws.cuh"

namespace gcrates {
template <typename... A>
__device__ __forceinline__ double lawv(int id, const Env& E, A... v) {
  const double t[] = {double(v)...};
  return law(id, t, E);
}
template <typename... A>
__device__ __forceinline__ double hetv(int id, bool has_het, const HetCell& X, A... v) {
  if (!has_het) return 0.0;
  const double t[] = {double(v)..., 0.0};
  return het_law(id, t, X);
}

__global__ void __launch_bounds__(128) rates_direct_kernel(RatesDev rp, RatesArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= a.ncell) return;
#define M(f) a.met[(long long)(f) * a.ldm + cell]
#define PH(j) a.photol[(long long)(j) * a.ldp + cell]
#define CC(i) a.c[(long long)(i) * a.ldc + cell]
#define OUT(r) a.rconst[(long long)(r) * a.ldr + cell]
  Env E;
  env_init(E, M(0), M(1), M(2), M(3), M(4), M(5));
  const bool has_het = a.het != nullptr;
  HetCell X;
  X.H = a.het;
  X.ldh = a.ldh;
  X.C = a.c;
  X.ldc = a.ldc;
  X.cell = cell;
  X.sp = HetSpecies{rp.hs_ind, rp.hs_mw, rp.hs_srmw, rp.hs_hk0, rp.hs_hcr};
  if (has_het) het_cell_init(X, E);
#include "rates_direct.inc"
#undef M
#undef PH
#undef CC
#undef OUT
}

cudaError_t launch_rates_direct(const RatesDev& rp, const RatesArgs& a, cudaStream_t s) {
  const int block = 128;
  const int grid = (a.ncell + block - 1) / block;
  if (grid > 0) rates_direct_kernel<<<grid, block, 0, s>>>(rp, a);
  return cudaGetLastError();
}
}  // namespace gcrates
