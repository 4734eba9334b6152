// Launch interface of the Update_RCONST kernel.
#pragma once
#include <cuda_runtime.h>

namespace gcrates {
struct RatesDev {
  const int* code;
  const int* start;
  const double* consts;
  const int* law_nargs;
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
};
cudaError_t launch_rates(const RatesDev& rp, const RatesArgs& a, cudaStream_t s);
}  // namespace gcrates
