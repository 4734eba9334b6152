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

// fullchem_SulfurAqChem: K_MT(1:6) from the fine and coarse alkaline sea
// salt (types 11 and 12 of the aerosol rows of `in`), written to the K_MT
// rows of the met array, whose TEMP and NUMDEN rows it reads.
struct SulfurAqArgs {
  int ncell;
  const double* in;  // HETIN_NFIELD rows (WetAeroArea, AeroRadi read)
  long long ldi;
  const double* c;   // NSPEC rows
  long long ldc;
  int ind[HSS_N];    // KPP index of each HSS_* species
  double srmw[HSS_N];  // SR_MW of each HSS_* species
  double* met;       // met rows: TEMP, NUMDEN in; K_MT out
  long long ldm;
  int row_temp, row_numden, row_kmt;
};

cudaError_t sulfur_aq_rates(const SulfurAqArgs& a, cudaStream_t s);

// SET_SO2 (fullchem_SulfurCldChem): K_CLD(1:6) of the in-cloud sulfur
// chemistry into the K_CLD rows of met; the cloud water's HSO3-, SO3-- and
// pH into the HSO3_aq, SO3_aq and pHCloud rows of `in` (which
// fullchem_SetStateHet reads next) and fupdateHOBr/HOCl = 1 there, as
// Set_Sulfur_Chem_Rates leaves them; Fahey and Seinfeld's size_res (whether
// HetDropChem would run) per cell.
struct SulfurCldArgs {
  int ncell;
  double* in;        // HETIN_NFIELD rows: read, and the rows above written
  long long ldi;
  const double* c;   // NSPEC rows
  long long ldc;
  int ind[HSS_N];    // KPP index of each HSS_* species
  double* met;       // K_CLD rows written, the others untouched
  long long ldm;
  int row_kcld;
  int* size_res;     // [ncell] out, or nullptr
  int* niter;        // [ncell] GET_HPLUS Newton iterations (0 outside cloud), or nullptr
  int lmetalcatso2;  // Input_Opt%LMETALCATSO2
};

cudaError_t sulfur_cld_rates(const SulfurCldArgs& a, cudaStream_t s);

// fullchem_HetDropChem under Do_FullChem's call conditions: SRHOCl and
// SRHOBr, the size-resolved cloud-droplet S(IV) oxidation by HOCl and HOBr
// (Yuen et al. 1996), into their met rows (0 where it is not called).
struct HetDropArgs {
  int ncell;
  double dt;             // chemistry time step [s]
  const double* in;      // HETIN_NFIELD rows (after SET_SO2)
  long long ldi;
  const double* c;       // NSPEC rows
  long long ldc;
  const double* het;     // HET_NFIELD rows of fullchem_SetStateHet
  long long ldh;
  const int* size_res;   // [ncell] from SET_SO2
  double* met;           // TEMP, NUMDEN, H2O, PRESS and K_CLD read; SRHOCl, SRHOBr written
  long long ldm;
  int ind[HSS_N];        // KPP index of each HSS_* species
  const int* hs_ind;     // the heterogeneous laws' species tables (gcrates::HetSpecies)
  const double *hs_mw, *hs_srmw, *hs_hk0, *hs_hcr;
};

cudaError_t het_drop_chem(const HetDropArgs& a, cudaStream_t s);

}  // namespace gchet
