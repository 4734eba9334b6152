// fullchem_SetStateHet on the GPU: the per-cell HetState that Update_RCONST's
// heterogeneous rate laws read, computed from the grid box's meteorology,
// aerosol and cloud-chemistry fields and its KPP concentrations.
//
//   fullChem_SetStateHet            KPP/fullchem/fullchem_HetStateFuncs.F90:48-244
//   Get_Theta_Ice                   :268-310
//   Halide_Conc, Get_Halide_CldConc,
//   Get_Halide_SsaConc,
//   Compute_L2G_Local               :325-650
//   Cld_Params                      KPP/fullchem/rateLawUtilFuncs.F90:281-417
//   CALC_KH, CALC_HEFF              GeosUtil/henry_mod.F90:74-204
//   fullchem_SulfurAqChem (K_MT)    KPP/fullchem/fullchem_SulfurChemFuncs.F90:120-305
//
// One thread per cell.  Inputs are rows of a cell-interleaved array
// (HETIN_* of het_layout.h); outputs the HET_NFIELD rows of the HetState
// array that gc_kpp_update_rconst_het_batch and gc_kpp_ctx_set_hetstate
// take.  Every statement follows the Fortran in the same evaluation order;
// logical fields are written as 0.0 / 1.0.  The fields fullchem_SetStateHet
// leaves alone (H2O, and cloudBox / fracOrgAer / fracInorgAer, which only the
// Hg simulation sets) are written as 0.
#include <cuda_runtime.h>

#include "het_rates.cuh"
#include "het_state.h"

namespace gchet {

namespace {

constexpr double AVO = 6.022140857e+23;  // Headers/physconstants.F90:32
constexpr double PI = 3.14159265358979323;
constexpr double HENRY_TREF = 298.15, HENRY_R = 8.3144598, HENRY_ATM = 101.325;

struct Cell {
  const SetStateArgs* a;
  int cell;
  __device__ double in(int f) const { return a->in[(long long)f * a->ldi + cell]; }
  __device__ double c(int s) const {
    const int i = a->ind[s];
    return i >= 0 ? a->c[(long long)i * a->ldc + cell] : 0.0;
  }
  __device__ void out(int f, double v) const { a->het[(long long)f * a->ldh + cell] = v; }
};

// CALC_KH then CALC_HEFF then L2G = HEFF * H2OLIQ (Compute_L2G_Local)
__device__ __forceinline__ double l2g_local(double k0, double cr, double pka, double tk, double h2oliq, double ph) {
  double kh = k0 * exp(cr * (1.0 / tk - 1.0 / HENRY_TREF)) * HENRY_R * tk / HENRY_ATM;
  double heff = kh;
  if (ph > 0.0 && pka > -100.0) heff = heff * (1.0 + pow(10.0, ph - pka));
  return heff * h2oliq;
}

// Get_Halide_SsaConc
__device__ __forceinline__ double halide_ssa_conc(double n_x, double surf_area, double r_w) {
  const double v_tot = (surf_area * r_w / 3.0) * 1e-3;
  if (v_tot <= 1.0e-20) return 0.0;
  const double conc = (n_x / AVO) / v_tot;
  return fmax(conc, 0.0);
}

__global__ void set_state_het_kernel(SetStateArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= a.ncell) return;
  const Cell X{&a, cell};
  using gcrates::SafeDiv;

  X.out(HET_AVO, AVO);
  X.out(HET_PI, PI);

  // meteorology
  const double cldf_met = X.in(HETIN_CLDF);
  const double cldfr = fmin(fmax(cldf_met, 0.0), 1.0);
  X.out(HET_cldFr, cldfr);
  X.out(HET_clearFr, 1.0 - cldfr);
  const double qi = X.in(HETIN_QI), ql = X.in(HETIN_QL);
  X.out(HET_qIce, qi);
  X.out(HET_qLiq, ql);
  const double vair = X.in(HETIN_AIRVOL) * 1.0e6;
  X.out(HET_vAir, vair);

  // aerosol fields
  X.out(HET_NAEROTYPE, 14.0);
  const double acl_area = X.in(HETIN_aClArea), acl_radi = X.in(HETIN_aClRadi);
  X.out(HET_aClArea, acl_area);
  X.out(HET_aClRadi, acl_radi);
  X.out(HET_aClVol, acl_area * acl_radi / 3.0);
  X.out(HET_aWater, X.in(HETIN_IsorropAeroH2O));
  X.out(HET_aWater + 1, X.in(HETIN_IsorropAeroH2O + 1));
  for (int t = 0; t < 14; ++t) {
    const double area = X.in(HETIN_AeroArea + t), radi = X.in(HETIN_AeroRadi + t);
    X.out(HET_xArea + t, area);
    X.out(HET_xRadi + t, radi);
    X.out(HET_xVol + t, area * radi / 3.0);
    X.out(HET_wetArea + t, X.in(HETIN_WetAeroArea + t));
    X.out(HET_xH2O + t, X.in(HETIN_AeroH2O + t) * 1.0e-6);
  }
  X.out(HET_OMOC_POA, X.in(HETIN_OMOC_POA));
  X.out(HET_OMOC_OPOA, X.in(HETIN_OMOC_OPOA));

  // HSO3- and SO3-- in cloud [mol/L]
  const double hso3 = X.in(HETIN_HSO3_aq), so3 = X.in(HETIN_SO3_aq);
  const double tso3 = hso3 + so3;
  X.out(HET_HSO3_aq, hso3);
  X.out(HET_SO3_aq, so3);
  X.out(HET_TSO3_aq, tso3);
  X.out(HET_frac_HSO3_aq, SafeDiv(hso3, tso3, 0.0));
  X.out(HET_frac_SO3_aq, SafeDiv(so3, tso3, 0.0));

  // ISORROPIA/HETP concentrations, pH and alkalinity
  X.out(HET_HSO4_molal, X.in(HETIN_IsorropBisulfate));
  X.out(HET_NO3_molal, X.in(HETIN_IsorropNitrate));
  X.out(HET_SO4_molal, X.in(HETIN_IsorropSulfate));
  X.out(HET_H_plus, X.in(HETIN_IsorropHplus));
  const double ph_cloud = X.in(HETIN_pHCloud);
  const double ph_ssa1 = X.in(HETIN_IsorropAeropH);
  X.out(HET_pHCloud, ph_cloud);
  X.out(HET_pHSSA, ph_ssa1);
  X.out(HET_pHSSA + 1, X.in(HETIN_IsorropAeropH + 1));
  const double h_sul = pow(10.0, -1.0 * ph_ssa1);
  X.out(HET_H_conc_Sul, h_sul);
  X.out(HET_H_conc_LCl, pow(10.0, -1.0 * ph_cloud));
  X.out(HET_H_conc_ICl, pow(10.0, -4.5));
  X.out(HET_H_conc_SSA, h_sul);
  X.out(HET_H_conc_SSC, pow(10.0, -5.0));
  double f_alk_ssa = SafeDiv(X.in(HETIN_SALAAL), X.in(HETIN_SALA), 0.0);
  f_alk_ssa = fmax(fmin(f_alk_ssa, 1.0), 0.0);
  double f_alk_ssc = SafeDiv(X.in(HETIN_SALCAL), X.in(HETIN_SALC), 0.0);
  f_alk_ssc = fmax(fmin(f_alk_ssc, 1.0), 0.0);
  X.out(HET_f_Alk_SSA, f_alk_ssa);
  X.out(HET_f_Acid_SSA, 1.0 - f_alk_ssa);
  X.out(HET_f_Alk_SSC, f_alk_ssc);
  X.out(HET_f_Acid_SSC, 1.0 - f_alk_ssc);
  const bool ssa_alk = fabs(f_alk_ssa) > 0.01, ssc_alk = fabs(f_alk_ssc) > 0.01;
  X.out(HET_SSA_is_Alk, ssa_alk ? 1.0 : 0.0);
  X.out(HET_SSA_is_Acid, ssa_alk ? 0.0 : 1.0);
  X.out(HET_SSC_is_Alk, ssc_alk ? 1.0 : 0.0);
  X.out(HET_SSC_is_Acid, ssc_alk ? 0.0 : 1.0);

  X.out(HET_gamma_HO2, a.gamma_ho2);
  X.out(HET_fupdateHOBr, X.in(HETIN_fupdateHOBr));
  X.out(HET_fupdateHOCl, X.in(HETIN_fupdateHOCl));

  // aqueous S(IV) in cloud water as ratios to SO2 [1]
  const double airden = X.in(HETIN_AIRDEN);
  const double so2 = X.c(HSS_SO2);
  double hso3m = SafeDiv(hso3 * 1.0e-3 * AVO * ql * airden * 1.0e-3, cldf_met, 0.0);
  X.out(HET_HSO3m, SafeDiv(hso3m, so2, 0.0));
  double so3mm = SafeDiv(so3 * 1.0e-3 * AVO * ql * airden * 1.0e-3, cldf_met, 0.0);
  X.out(HET_SO3mm, SafeDiv(so3mm, so2, 0.0));

  // Cld_Params(AD, CLDF, FRLAND, FROCEAN, QI, QL, T)
  const double temp = X.in(HETIN_T);
  double rliq, rice, aliq, vliq, aice, vice;
  if ((ql + qi <= 0.0) || (cldf_met <= 0.0)) {
    rliq = 6.0e-4;
    rice = 38.5e-4;
    aliq = vliq = aice = vice = 0.0;
  } else {
    const double ad = X.in(HETIN_AD);
    rliq = (X.in(HETIN_FRLAND) > X.in(HETIN_FROCEAN)) ? 6.0e-4 : 10.0e-4;
    vliq = ql * ad / 0.001 / vair;
    vice = qi * ad / 0.91e-3 / vair;
    aliq = 3.0 * vliq / rliq;
    double alpha, beta;
    if (temp < 202.0) {
      alpha = 83.3;
      beta = 0.0184;
    } else if (temp < 217.0) {
      alpha = 9.1744e+4;
      beta = 0.117;
    } else {
      alpha = 308.4;
      beta = 0.0152;
    }
    rice = 0.5 * alpha * exp(beta * (temp - 273.15)) / 1e+4;
    aice = 3.0 * vice / rice * 2.25;
  }
  X.out(HET_rLiq, rliq);
  X.out(HET_rIce, rice);
  X.out(HET_aLiq, aliq);
  X.out(HET_vLiq, vliq);
  X.out(HET_aIce, aice);
  X.out(HET_vIce, vice);

  // Get_Theta_Ice(HNO3, HCl, HBr) at TEMP
  {
    const double hno3 = X.c(HSS_HNO3), hcl = X.c(HSS_HCl), hbr = X.c(HSS_HBr);
    double klin = 7.5e-5 * exp(4585.0 / temp);
    const double klang1 = klin / 2.7e+14;
    klin = 1.3e-5 * exp(4600.0 / temp);
    const double klang2 = klin / 3.0e+14;
    const double denom = 1.0 + klang1 * hno3 + klang2 * hcl;
    X.out(HET_HNO3_theta, klang1 * hno3 / denom);
    X.out(HET_HCl_theta, klang2 * hcl / denom);
    X.out(HET_HBr_theta, fmin(4.14e-10 * pow(hbr, 0.88), 1.0));
  }

  // Halide_Conc
  {
    const double c_hbr = X.c(HSS_HBr), c_brsala = X.c(HSS_BrSALA), c_brsalc = X.c(HSS_BrSALC);
    const double c_hcl = X.c(HSS_HCl), c_salacl = X.c(HSS_SALACL), c_salccl = X.c(HSS_SALCCL);
    const double hbr = c_hbr + (c_brsala * 0.7) + c_brsalc;
    const double hcl = c_hcl + (c_salacl * 0.7) + c_salccl;
    // Get_Halide_CldConc
    double br_conc = 0.0, cl_conc = 0.0;
    const double v_tot = SafeDiv(vliq, cldfr, 0.0);
    if (!(v_tot < 1.0e-20)) {
      double l2g = l2g_local(1.0, 9000.0, -6.3, temp, v_tot, ph_cloud);
      double f_l = l2g / (1.0 + l2g);
      cl_conc = f_l * hcl / (v_tot * AVO * 1.0e-3);
      l2g = l2g_local(7.5e-1, 10200.0, -9.0, temp, v_tot, ph_cloud);
      f_l = l2g / (1.0 + l2g);
      br_conc = f_l * hbr / (v_tot * AVO * 1.0e-3);
    }
    double br_a = 0.0, br_c = 0.0, br_g = 0.0, cl_a = 0.0, cl_c = 0.0, cl_g = 0.0;
    double denom = c_hbr + (c_brsala * 0.7) + c_brsalc;
    if (denom > 0.0) {
      br_g = (br_conc * c_hbr) / denom;
      br_a = (br_conc * c_brsala * 0.7) / denom;
      br_c = (br_conc * c_brsalc) / denom;
    }
    denom = c_hcl + (c_salacl * 0.7) + c_salccl;
    if (denom > 0.0) {
      cl_g = (cl_conc * c_hcl) / denom;
      cl_a = (cl_conc * c_salacl * 0.7) / denom;
      cl_c = (cl_conc * c_salccl) / denom;
    }
    const double br_cld = br_a + br_c + br_g, cl_cld = cl_a + cl_c + cl_g;
    X.out(HET_Br_conc_CldA, br_a);
    X.out(HET_Br_conc_CldC, br_c);
    X.out(HET_Br_conc_CldG, br_g);
    X.out(HET_Br_conc_Cld, br_cld);
    X.out(HET_Cl_conc_CldA, cl_a);
    X.out(HET_Cl_conc_CldC, cl_c);
    X.out(HET_Cl_conc_CldG, cl_g);
    X.out(HET_Cl_conc_Cld, cl_cld);
    X.out(HET_frac_Br_CldA, br_cld > 0.0 ? br_a / br_cld : 0.0);
    X.out(HET_frac_Br_CldC, br_cld > 0.0 ? br_c / br_cld : 0.0);
    X.out(HET_frac_Br_CldG, br_cld > 0.0 ? br_g / br_cld : 0.0);
    X.out(HET_frac_Cl_CldA, cl_cld > 0.0 ? cl_a / cl_cld : 0.0);
    X.out(HET_frac_Cl_CldC, cl_cld > 0.0 ? cl_c / cl_cld : 0.0);
    X.out(HET_frac_Cl_CldG, cl_cld > 0.0 ? cl_g / cl_cld : 0.0);
    const double area12 = X.in(HETIN_AeroArea + 11), radi12 = X.in(HETIN_AeroRadi + 11);
    const double br_ssa = halide_ssa_conc(c_brsala, acl_area, acl_radi);
    const double br_ssc = halide_ssa_conc(c_brsalc, area12, radi12);
    const double cl_ssa = halide_ssa_conc(c_salacl, acl_area, acl_radi);
    const double cl_ssc = halide_ssa_conc(c_salccl, area12, radi12);
    X.out(HET_Br_conc_SSA, br_ssa);
    X.out(HET_Br_conc_SSC, br_ssc);
    X.out(HET_Cl_conc_SSA, cl_ssa);
    X.out(HET_Cl_conc_SSC, cl_ssc);
    const double c_nit = X.c(HSS_NIT);
    X.out(HET_NIT_conc_SSA, halide_ssa_conc(c_nit, acl_area, acl_radi));
    X.out(HET_NIT_conc_SSC, halide_ssa_conc(X.c(HSS_NITs), area12, radi12));
    X.out(HET_Br_over_Cl_Cld, cl_cld > 0.0 ? br_cld / cl_cld : 0.0);
    X.out(HET_Br_over_Cl_SSA, cl_ssa > 0.0 ? br_ssa / cl_ssa : 0.0);
    X.out(HET_Br_over_Cl_SSC, cl_ssc > 0.0 ? br_ssc / cl_ssc : 0.0);
    const double s = c_salacl + c_nit + X.c(HSS_SO4);
    X.out(HET_frac_SALACL, s > 0.0 ? c_salacl / (c_salacl + c_nit + X.c(HSS_SO4)) : 0.0);
  }

  // UCX: PSC uptake probabilities, stratosphere and PSC flags
  for (int r = 0; r < 11; ++r) X.out(HET_KHETI_SLA + r, X.in(HETIN_KHETI_SLA + r));
  const bool strat = X.in(HETIN_InStratosphere) != 0.0;
  const bool psc = (a.lpscchem != 0) && (X.in(HETIN_STATE_PSC) >= 2.0) && strat;
  X.out(HET_stratBox, strat ? 1.0 : 0.0);
  X.out(HET_pscBox, psc ? 1.0 : 0.0);
  X.out(HET_natSurface, (psc && (X.c(HSS_NIT) > 0.0)) ? 1.0 : 0.0);
  X.out(HET_TurnOffHetRates, a.turn_off_het_rates ? 1.0 : 0.0);

  // fields fullchem_SetStateHet does not set
  X.out(HET_H2O, 0.0);
  X.out(HET_cloudBox, 0.0);
  X.out(HET_fracOrgAer, 0.0);
  X.out(HET_fracInorgAer, 0.0);
  X.out(HET_SUNCOS, X.in(HETIN_SUNCOS));
}

// fullchem_SulfurAqChem (KPP/fullchem/fullchem_SulfurChemFuncs.F90:120-305):
// uptake of SO2 (with O3), HCl and HNO3 on alkaline fine (type 11) and coarse
// (type 12) sea salt, K_MT(1:6) [1/s or cm3/molec/s], through Ars_L1K and
// kIIR1Ltd (rateLawUtilFuncs.F90:77-160) at the cell's TEMP and NUMDEN.
__global__ void sulfur_aq_kernel(SulfurAqArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= a.ncell) return;
  auto in = [&](int f) { return a.in[(long long)f * a.ldi + cell]; };
  auto c = [&](int sp) {
    const int i = a.ind[sp];
    return i >= 0 ? a.c[(long long)i * a.ldc + cell] : 0.0;
  };
  gcrates::HetCell X{};
  X.NUMDEN = a.met[(long long)a.row_numden * a.ldm + cell];
  X.SR_TEMP = sqrt(a.met[(long long)a.row_temp * a.ldm + cell]);
  double k_mt[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const bool salaal = c(HSS_SALAAL) > 0.1, salcal = c(HSS_SALCAL) > 0.1, o3 = c(HSS_O3) > 1.0e+10;
  // fine (t = 0, type 11, eductor SALAAL) then coarse (t = 1, type 12, SALCAL)
  for (int t = 0; t < 2; ++t) {
    const bool alk = t == 0 ? salaal : salcal;
    const double educt = c(t == 0 ? HSS_SALAAL : HSS_SALCAL);
    const double area = in(HETIN_WetAeroArea + 10 + t), radius = in(HETIN_AeroRadi + 10 + t);
    double k_ex;
    if (alk && o3) {
      k_ex = gcrates::Ars_L1k(X, area, radius, 0.11, a.srmw[HSS_SO2]);
      k_mt[3 * t] = gcrates::kIIR1Ltd(c(HSS_SO2), educt, k_ex) / c(HSS_O3);
    }
    if (alk) {
      k_ex = gcrates::Ars_L1k(X, area, radius, 0.07, a.srmw[HSS_HCl]);
      k_mt[3 * t + 1] = gcrates::kIIR1Ltd(c(HSS_HCl), educt, k_ex);
      k_ex = gcrates::Ars_L1k(X, area, radius, 0.5, a.srmw[HSS_HNO3]);
      k_mt[3 * t + 2] = gcrates::kIIR1Ltd(c(HSS_HNO3), educt, k_ex);
    }
  }
  for (int k = 0; k < 6; ++k) a.met[(long long)(a.row_kmt + k) * a.ldm + cell] = k_mt[k];
}

}  // namespace

cudaError_t sulfur_aq_rates(const SulfurAqArgs& a, cudaStream_t s) {
  if (a.ncell <= 0) return cudaSuccess;
  const int block = 128;
  sulfur_aq_kernel<<<(a.ncell + block - 1) / block, block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t set_state_het(const SetStateArgs& a, cudaStream_t s) {
  if (a.ncell <= 0) return cudaSuccess;
  const int block = 128;
  set_state_het_kernel<<<(a.ncell + block - 1) / block, block, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace gchet
