// Launch interface of the Update_RCONST kernel.
#pragma once
#include <cuda_runtime.h>

namespace gcrates {
struct RatesDev {
  const int* code;
  const int* start;
  const double* consts;
  const int* law_nargs;
  const int* het_nargs;
  // species table of the heterogeneous laws (het_rates.cuh HetSpc order)
  const int* hs_ind;
  const double* hs_mw;
  const double* hs_srmw;
  const double* hs_hk0;
  const double* hs_hcr;
  int nreact, nmet;
};
struct RatesArgs {
  int ncell;
  const double* met;
  long long ldm;
  const double* photol;
  long long ldp;
  const double* c;
  long long ldc;
  double* rconst;
  long long ldr;
  const double* het;  // HetState rows (het_layout.h) or NULL for the zeroed HetState
  long long ldh;
};
cudaError_t launch_rates(const RatesDev& rp, const RatesArgs& a, cudaStream_t s);
// the generated straight-line form (rates_direct.cu, one object per mechanism)
cudaError_t launch_rates_direct(const RatesDev& rp, const RatesArgs& a, cudaStream_t s);
}  // namespace gcrates
