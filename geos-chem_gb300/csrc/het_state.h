// fullchem_SetStateHet on the GPU (het_state.cu): launcher and arguments.
#pragma once
#include <cuda_runtime.h>

#include "het_layout.h"

namespace gchet {

struct SetStateArgs {
  int ncell;
  const double* in;  // HETIN_NFIELD rows, cell-interleaved
  long long ldi;
  const double* c;   // NSPEC rows (KPP concentrations)
  long long ldc;
  int ind[HSS_N];    // KPP index of each HSS_* species, -1 if the mechanism lacks it
  double gamma_ho2;  // Input_Opt%gamma_HO2
  int lpscchem;      // Input_Opt%LPSCCHEM
  int turn_off_het_rates;  // Input_Opt%TurnOffHetRates
  double* het;       // HET_NFIELD rows out
  long long ldh;
};

cudaError_t set_state_het(const SetStateArgs& a, cudaStream_t s);

}  // namespace gchet
