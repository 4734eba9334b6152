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
//   fullchem_SulfurCldChem / SET_SO2 (K_CLD, cloud pH, HSO3_aq, SO3_aq)
//                                   :320-398, 865-1620, 1635-3549
//   fullchem_HetDropChem (SRHOCl, SRHOBr)  :414-790, 808-849
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

// ---------------------------------------------------------------------------
// SET_SO2, the in-cloud branch of fullchem_SulfurCldChem
// (KPP/fullchem/fullchem_SulfurChemFuncs.F90:865-1620): cloud pH from
// GET_HPLUS (:1635-1853, Newton's method on the cloud water's
// electroneutrality with the Henry/dissociation functions kCO21..dkAA and
// CaCO3_PRECIP, :1867-3156), the aqueous S(IV) oxidation rates of
// AQCHEM_SO2 (:3171-3549) and the Fahey and Seinfeld size_res decision.
//
// The Fortran functions re-evaluate their temperature-dependent constants
// (about 40 exp() calls) at every Newton iteration; here they, and every
// [H+]-independent leading product of the functions' expressions, are
// evaluated once per cell (SO2Equil), and each iteration only does the
// [H+]-dependent rest in the Fortran's order, so the values are the ones the
// per-call evaluation gives.  Literals the Fortran writes without a kind
// (Kc1 = 4.3e-7 ...) are default REAL there: their single-precision value.
namespace so2 {

constexpr double AIRMW = 28.9644;  // Headers/physconstants.F90:26
constexpr double ATM = 1.01325e+5;  // :70
constexpr double RL = 0.08205;      // the functions' gas constant [L atm/mol/K]

__device__ __forceinline__ double tf(double D, double T) { return exp(D * ((1.0 / T) - (1.0 / 298.0))); }
__device__ __forceinline__ double sq(double x) { return x * x; }

// one acid (or base) with a single dissociation: kHNO3/dkHNO3, kHCl/dkHCl,
// kFA/dkFA, kAA/dkAA share this form
struct Mono {
  double H_T, K_T, HK;         // Henry and dissociation constants at T; H_T * K_T
  double XP, num_d, a1, a2;    // X*P; dk numerator; K_T*H_T*RL*T*LWC; H_T*RL*T*LWC
  __device__ void init(double H_T_, double K_T_, double X, double P, double T, double LWC) {
    H_T = H_T_;
    K_T = K_T_;
    HK = H_T * K_T;
    XP = X * P;
    num_d = -1.0 * K_T * H_T * X * P * (1.0 + H_T * RL * T * LWC);
    a1 = K_T * H_T * RL * T * LWC;
    a2 = H_T * RL * T * LWC;
  }
  __device__ double f(double H, double T, double LWC) const {
    const double Heff = H_T * (1.0 + (K_T / H));
    const double x = 1.0 / (1.0 + (Heff * RL * T * LWC));
    return HK * (XP * x) / H;
  }
  __device__ double df(double H) const { return num_d / sq(a1 + a2 * H + H); }
};

// H2CO3 (CO2) or H2SO3 (SO2) with two dissociations: kCO21/kCO22/dkCO21/
// dkCO22, kSO21/kSO22/dkSO21/dkSO22
struct Di {
  double H_T, K1_T, K2_T, K12, HK1, HK12;  // Henry, K1, K2 at T; K1*K2; H*K1 or K1*H; K1*K2*H
  double XP, pre1, pre2;                   // X*P; K1*H*X*P; -1*K1*K2*H*X*P
  double a1, a2, a3, b2;                   // K1*K2*H*RL*T*LWC; H*RL*T*LWC; K1*H*RL*T*LWC; 2*H*RL*T*LWC
  __device__ void init(double H_T_, double K1_T_, double K2_T_, double X, double P, double T, double LWC, bool so2) {
    H_T = H_T_;
    K1_T = K1_T_;
    K2_T = K2_T_;
    K12 = K1_T * K2_T;
    HK1 = so2 ? H_T * K1_T : 0.0;  // kSO21 multiplies Hso2_T * Ks1_T first
    HK12 = K1_T * K2_T * H_T;
    XP = X * P;
    pre1 = K1_T * H_T * X * P;
    pre2 = -1.0 * K1_T * K2_T * H_T * X * P;
    a1 = K1_T * K2_T * H_T * RL * T * LWC;
    a2 = H_T * RL * T * LWC;
    a3 = K1_T * H_T * RL * T * LWC;
    b2 = 2.0 * H_T * RL * T * LWC;
  }
  // partial pressure X * P * x of the gas at [H+] = H
  __device__ double pgas(double H, double T, double LWC) const {
    const double Heff = H_T * (1.0 + (K1_T / H) + (K12 / (H * H)));
    const double x = 1.0 / (1.0 + (Heff * RL * T * LWC));
    return XP * x;
  }
  __device__ double den(double H) const { return sq(a1 + a3 * H + a2 * H * H + H * H); }
  __device__ double d1(double H, double dn) const { return pre1 * (a1 - a2 * H * H - H * H) / dn; }
  __device__ double d2(double H, double dn) const { return pre2 * (a3 + b2 * H + 2.0 * H) / dn; }
};

// The [H+]-independent part of GET_HPLUS's functions for one cell.
struct SO2Equil {
  Di co2, so2;
  Mono hno3, hcl, fa, aa;
  double Hnh3_T, Ka1_T, NH3P, nh3_num, nh3_a2;  // kNH3 / dkNH3
  double Ksp_T, ca_den, Ksp2;                    // CaCO3_PRECIP
  double Kw_T;
};

__device__ void equil_init(SO2Equil& E, double T, double P, double LWC, double SO2, double TNO3, double TNH3,
                           double CL, double TFA, double TAA) {
  const double CO2 = 390.0e-6;
  // kCO2x: Kc1 = 4.3e-7, Kc2 = 4.68e-11, Hco2 = 3.4e-2 (single precision)
  E.co2.init((double)3.4e-2f * tf(2.44e+3, T), (double)4.3e-7f * tf(-1000.0, T), (double)4.68e-11f * tf(-1760.0, T),
             CO2, P, T, LWC, false);
  // kSO2x: Ks1 = 1.3e-2, Ks2 = 6.6e-8, Hso2 = 1.23 (single precision)
  E.so2.init((double)1.23f * tf(3.14e+3, T), (double)1.3e-2f * tf(1960.0, T), (double)6.6e-8f * tf(1500.0, T), SO2,
             P, T, LWC, true);
  // kHNO3: Kn1 = 15.4, Hhno3 = 2.1e5 (single precision), Dhhno3 = 0
  E.hno3.init((double)2.1e5f * tf(0.0, T), (double)15.4f * tf(8700.0, T), TNO3, P, T, LWC);
  E.hcl.init(1.5e+3 * tf(2.3e+3, T), 1.74e+6 * tf(6900.0, T), CL, P, T, LWC);
  E.fa.init(8800.0 * tf(6100.0, T), 1.8e-4 * tf(151.0, T), TFA, P, T, LWC);
  E.aa.init(4100.0 * tf(6200.0, T), 1.75e-5 * tf(50.0, T), TAA, P, T, LWC);
  // kNH3: Ka1 = 1.7e-5 (single precision), Hnh3 = 60
  E.Kw_T = 1.0e-14 * exp(-6710.0 * ((1.0 / T) - (1.0 / 298.0)));
  E.Hnh3_T = 60.0 * tf(4200.0, T);
  E.Ka1_T = (double)1.7e-5f * tf(-450.0, T);
  E.NH3P = TNH3 * P;
  E.nh3_num = E.Ka1_T * E.Hnh3_T * TNH3 * E.Kw_T * P * (1.0 + E.Hnh3_T * RL * T * LWC);
  E.nh3_a2 = E.Hnh3_T * RL * T * LWC;
  // CaCO3_PRECIP (double-precision constants)
  const double Hco2_T = 3.4e-2 * tf(2.44e+3, T), Kc1_T = 4.3e-7 * tf(-1000.0, T), Kc2_T = 4.68e-11 * tf(-1760.0, T);
  E.Ksp_T = 3.3e-9 * tf(-1200.0, T);
  E.ca_den = Kc1_T * Kc2_T * Hco2_T * CO2 * P;
  E.Ksp2 = 2.0 * E.Ksp_T;
}

// GET_HPLUS: [H+] of the cloud water; *niter = Newton iterations
__device__ double get_hplus(const SO2Equil& E, double SO4nss, double TNA, double TDCA, double T, double LWC,
                            double iHPLUS, int* niter) {
  const double Kw = 1.0e-14, MINVAL_ = (double)0.01f;
  double ipH = -log10(iHPLUS), newpH = 0.0;
  int count = 0;
  while (fabs(ipH - newpH) > MINVAL_) {
    count = count + 1;
    if (count != 1) ipH = newpH;
    const double H = pow(10.0, -ipH);
    // f(x) terms
    const double pco2 = E.co2.pgas(H, T, LWC);
    const double fHCO3 = E.co2.H_T / H * E.co2.K1_T * pco2;
    const double fCO3 = E.co2.HK12 / H / H * pco2;
    const double pso2 = E.so2.pgas(H, T, LWC);
    const double fHSO3 = E.so2.HK1 * pso2 / H;
    const double fSO3 = E.so2.HK12 / H / H * pso2;
    const double fHNO3 = E.hno3.f(H, T, LWC);
    const double Hnh3eff = E.Hnh3_T * (1.0 + ((E.Ka1_T * H) / E.Kw_T));
    const double xNH3 = 1.0 / (1.0 + (Hnh3eff * RL * T * LWC));
    const double fNH4 = H * E.Hnh3_T * E.Ka1_T * (E.NH3P * xNH3) / E.Kw_T;
    const double fHCl = E.hcl.f(H, T, LWC);
    const double fFA = E.fa.f(H, T, LWC);
    const double fAA = E.aa.f(H, T, LWC);
    // f'(x) terms
    const double dnc = E.co2.den(H), dns = E.so2.den(H);
    const double dHCO3 = E.co2.d1(H, dnc), dCO3 = E.co2.d2(H, dnc);
    const double dHSO3 = E.so2.d1(H, dns), dSO3 = E.so2.d2(H, dns);
    const double dHNO3 = E.hno3.df(H);
    const double dNH4 = E.nh3_num / sq(E.nh3_a2 * (E.Kw_T + E.Ka1_T * H) + E.Kw_T);
    const double dHCl = E.hcl.df(H), dFA = E.fa.df(H), dAA = E.aa.df(H);
    // CaCO3_PRECIP
    const double fCa = E.Ksp_T * H * H / E.ca_den;
    const double dCa = E.Ksp2 * H / E.ca_den;
    double f, df;
    if (fCa >= TDCA) {
      const double D = (2.0 * SO4nss) - (TNA + 2.0 * TDCA);
      f = D - H + Kw / H + fHCO3 + 2.0 * fCO3 + fHSO3 + 2.0 * fSO3 + fHNO3 - fNH4 + fHCl + fFA + fAA;
      df = -1.0 - Kw / H / H + dHCO3 + 2.0 * dCO3 + dHSO3 + 2.0 * dSO3 + dHNO3 - dNH4 + dHCl + dFA + dAA;
    } else {
      const double D = (2.0 * SO4nss) - TNA;
      f = D - H + Kw / H + fHCO3 + 2.0 * fCO3 + fHSO3 + 2.0 * fSO3 + fHNO3 - fNH4 + fHCl + fFA + fAA - 2.0 * fCa;
      df = -1.0 - Kw / H / H + dHCO3 + 2.0 * dCO3 + dHSO3 + 2.0 * dSO3 + dHNO3 - dNH4 + dHCl + dFA + dAA - 2.0 * dCa;
    }
    double nn = H - f / df;
    nn = fmax(nn, 1.0e-14);
    nn = fmin(nn, 1.0e-1);
    if (count > 50) {
      newpH = ((-log10(nn)) + (-log10(H))) / 2.0;
      break;
    }
    newpH = -log10(nn);
    if (isnan(newpH)) break;  // the reference stops the model here
  }
  *niter = count;
  return pow(10.0, -newpH);
}

__global__ void sulfur_cld_kernel(SulfurCldArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= a.ncell) return;
  auto in = [&](int f) { return a.in[(long long)f * a.ldi + cell]; };
  auto c = [&](int sp) {
    const int i = a.ind[sp];
    return i >= 0 ? a.c[(long long)i * a.ldc + cell] : 0.0;
  };
  double kcld[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double hso3 = 1.0e-32, so3 = 1.0e-32, phcloud = 0.0;
  int size_res = 0, niter = 0;
  const double RHO = in(HETIN_AIRDEN);
  const double CNVFAC = 1.E3 * AIRMW / (RHO * AVO);  // molec/cm3 -> v/v
  const double SO2_AfterSS = c(HSS_SO2) * CNVFAC;
  const double H2O20 = c(HSS_H2O2) * CNVFAC;
  const double PATM = in(HETIN_PMID_DRY) / (ATM * 1.e-2);
  const double TK = in(HETIN_T), FC = in(HETIN_CLDF);
  double LWC = in(HETIN_QL) * in(HETIN_AIRDEN) * 1e-3;
  LWC = fmax(0.0, LWC);
  LWC = gcrates::SafeDiv(LWC, FC, 0.0);
  if ((FC > 1.0e-4) && (SO2_AfterSS > 1.e-20) && (TK > 258.0) && (LWC > 1.0e-20)) {
    const double SO4nss = 1.e+3 * (c(HSS_SO4) * 0.7 + c(HSS_SO4s)) / (LWC * AVO);
    const double TNH3 = ((in(HETIN_NH4) * 0.7) + in(HETIN_NH3)) * CNVFAC;
    double CL = (c(HSS_SALACL) * 0.7) + c(HSS_SALCCL);
    CL = (CL + c(HSS_HCl)) * CNVFAC;
    const double TFA = c(HSS_HCOOH) * CNVFAC, TAA = c(HSS_ACTA) * CNVFAC;
    const double TNA = 1.e3 * (in(HETIN_SALA) * 0.7 + in(HETIN_SALC)) * (31.6 * 0.359 / 23.0) / (LWC * AVO);
    double dsum = in(HETIN_DSTbin);
    for (int b = 1; b < 7; ++b) dsum = dsum + in(HETIN_DSTbin + b);
    const double DUST = dsum * 1.e+15 * HSS_MW_DSTbin1 / AVO;
    const double TDCA = DUST * 2.22e-15 / LWC;
    const double TNO3 = (c(HSS_HNO3) + (c(HSS_NIT) * 0.7) + c(HSS_NITs)) * CNVFAC;
    SO2Equil E;
    equil_init(E, TK, PATM, LWC, SO2_AfterSS, TNO3, TNH3, CL, TFA, TAA);
    const double HPLUS = get_hplus(E, SO4nss, TNA, TDCA, TK, LWC, 3.16227766016837953e-5, &niter);
    phcloud = -1.0 * log10(HPLUS);
    double FeIII = 0.0, MnII = 0.0;
    if (a.lmetalcatso2) {
      const double Fe_nat = DUST * 35e-3;
      const double Mn_nat = Fe_nat / 50.0;
      const double Fe_ant = in(HETIN_pFe) * CNVFAC * 1.e+12 * in(HETIN_AD) / (AIRMW / HSS_MW_pFe) / in(HETIN_AIRVOL);
      const double Mn_ant = Fe_ant / 10.0;
      const double Mn_tot = Mn_ant + Mn_nat;
      const double Mn_d = Mn_tot * 1e-9 / 54.94 / LWC * 1e-3 * 0.5;  // LWC > 0 in this branch
      const double Fe_d_ant = Fe_ant * 1e-9 / HSS_MW_pFe / LWC * 1e-3;
      const double Fe_d_nat = Fe_nat * 1e-9 / HSS_MW_pFe / LWC * 1e-3;
      const double Fe_d = Fe_d_ant * 0.1 + Fe_d_nat * 0.01;
      FeIII = in(HETIN_SUNCOS) > 0.0 ? Fe_d * 0.1 : Fe_d * 0.9;
      MnII = Mn_d;
    }
    // AQCHEM_SO2
    const double T = TK, P = PATM, Hplus = HPLUS;
    const double KH2O2 = 6.31e+14 * exp(-4.76e+3 / T);
    const double Ks1 = 1.30e-2 * exp(6.75 * (298.15 / T - 1.0));
    const double Ks2 = 6.31e-8 * exp(5.05 * (298.15 / T - 1.0));
    const double XSO2aq = 1.0 / (1.0 + Ks1 / Hplus + Ks1 * Ks2 / (Hplus * Hplus));
    const double XHSO3 = 1.0 / (1.0 + Hplus / Ks1 + Ks2 / Hplus);
    const double XSO3 = 1.0 / (1.0 + Hplus / Ks2 + Hplus * Hplus / (Ks1 * Ks2));
    const double HCSO2 = 1.22 * exp(10.55 * (298.15 / T - 1.0));
    const double FHCSO2 = HCSO2 * (1.0 + (Ks1 / Hplus) + (Ks1 * Ks2 / (Hplus * Hplus)));
    const double XSO2g = 1.0 / (1.0 + (FHCSO2 * RL * T * LWC));
    const double SIV = FHCSO2 * XSO2g * SO2_AfterSS * P;
    const double Kh1 = 2.20e-12 * exp(-12.52 * (298.15 / T - 1.0));
    const double HCH2O2 = 7.45e+4 * exp(22.21 * (298.15 / T - 1.0));
    const double FHCH2O2 = HCH2O2 * (1.0 + (Kh1 / Hplus));
    const double XH2O2g = 1.0 / (1.0 + (FHCH2O2 * RL * T * LWC));
    const double KaqH2O2 = KH2O2 * Ks1 * FHCH2O2 * HCSO2 * XH2O2g * XSO2g * P * LWC * RL * T;
    const double KO0 = 2.40e+4, KO1 = 3.49e+12 * exp(-4.83e+3 / T), KO2 = 7.32e+14 * exp(-4.03e+3 / T);
    const double HCO3 = 1.13e-2 * exp(8.51 * (298.15 / T - 1.0));
    const double XO3g = 1.0 / (1.0 + (HCO3 * RL * T * LWC));
    const double KaqO3 = (KO0 * XSO2aq + KO1 * XHSO3 + KO2 * XSO3) * FHCSO2 * XSO2g * P * HCO3 * XO3g * LWC * RL * T;
    const double KaqO2 = FHCSO2 * XSO2g * ((750.0 * MnII) + (2600.0 * FeIII) + (1e+10 * MnII * FeIII)) * LWC * RL * T;
    const double KHCHO1 = 7.9e+2 * exp(-16.44 * (298.15 / T - 1.0));
    const double KHCHO2 = 2.5e+7 * exp(-6.04 * (298.15 / T - 1.0));
    const double KHMS = 3.6e+3 * exp(-15.09 * (298.15 / T - 1.0));
    const double KHMS2 = 2.65e+8 * exp(-5.03 * (298.15 / T - 1.0));
    const double Khc1 = 2.53e+3 * exp(13.48 * (298.15 / T - 1.0));
    const double Kw1 = 1e-14 * exp(-22.51 * (298.15 / T - 1.0));
    const double HCHCHO = 2.5 * exp(21.6 * (298.15 / T - 1.0));
    const double FHCHCHO = HCHCHO * (1.0 + Khc1);
    const double XHCHOg = 1.0 / (1.0 + (FHCHCHO * RL * T * LWC));
    const double KaqHCHO = (KHCHO1 * XHSO3 + KHCHO2 * XSO3) * FHCSO2 * XSO2g * P * HCHCHO * XHCHOg * LWC * RL * T;
    const double KaqHMS = KHMS * (Kw1 / Hplus) * 0.7;
    const double KaqHMS2 = KHMS2 * 1.0e-19 * 0.7;
    kcld[0] = KaqH2O2 * FC * CNVFAC;
    kcld[1] = KaqO3 * FC * CNVFAC;
    kcld[2] = KaqO2 * FC;
    kcld[3] = KaqHCHO * FC * CNVFAC;
    kcld[4] = KaqHMS * FC;
    kcld[5] = KaqHMS2 * FC / c(HSS_SO2);
    // Fahey and Seinfeld's decision (:1421-1540).  size_res starts false;
    // the first branch keeps it false, the second (LWC < 0.1e-6) sets it,
    // and every other branch only ever sets it false again (its final ELSE
    // is unreachable: LWC is a number > 1e-20 here).  So the alkalinity,
    // NH3 and HNO3 tests of those branches cannot change the result and are
    // not evaluated.
    size_res = (!(H2O20 > SO2_AfterSS + 1e-9) && LWC < 0.1e-6) ? 1 : 0;
    hso3 = SIV * XHSO3;
    so3 = SIV * XSO3;
  }
  for (int k = 0; k < 6; ++k) a.met[(long long)(a.row_kcld + k) * a.ldm + cell] = kcld[k];
  a.in[(long long)HETIN_HSO3_aq * a.ldi + cell] = hso3;
  a.in[(long long)HETIN_SO3_aq * a.ldi + cell] = so3;
  a.in[(long long)HETIN_pHCloud * a.ldi + cell] = phcloud;
  a.in[(long long)HETIN_fupdateHOBr * a.ldi + cell] = 1.0;
  a.in[(long long)HETIN_fupdateHOCl * a.ldi + cell] = 1.0;
  if (a.size_res) a.size_res[cell] = size_res;
  if (a.niter) a.niter[cell] = niter;
}

}  // namespace so2

// ---------------------------------------------------------------------------
// fullchem_HetDropChem (KPP/fullchem/fullchem_SulfurChemFuncs.F90:414-790,
// WhenExpCantBeDone :808-849) where Do_FullChem calls it
// (GeosCore/fullchem_mod.F90:913-934): the share of SO2 that the
// size-resolved droplet chemistry (Yuen et al. 1996) adds to the HOCl and
// HOBr oxidation, as the rate coefficients SRHOCl and SRHOBr.
namespace drop {

constexpr double AIRMW = 28.9644, G0 = 9.80665, PI_PHYS = 3.14159265358979323;
constexpr double SS_DEN = 2200.0;
// RG_S**3 and NINE_HALVES * LOG(SIG_S)**2 of the Fortran are constant
// expressions of PARAMETERs, folded by the compiler with correct rounding of
// each operation: (0.4e-6)**3 and 4.5 * log(1.8)**2
constexpr double RG_S3 = 0x1.2e3b40a0e9b4fp-64, ARG_SS = 0x1.8e02146ec938fp+0;

// second-order loss of R1 with R2 over DT at rate K, or WhenExpCantBeDone
__device__ __forceinline__ double loss2(double R1, double R2, double K, double DT) {
  const double Arg = (R1 - R2) * (K * DT);
  if (fabs(Arg) < 709.0 && fabs(Arg) > 0.0) {
    const double XX = exp(Arg);
    return (R1 * R2) * (XX - 1.0) / ((R1 * XX) - R2);
  }
  const double DIFF = R1 - R2;
  if (DIFF < 0.0) return R1;
  if (DIFF > 0.0) return R2;
  return R1 - 1.0 / (K * DT + (1.0 / R1));
}

__global__ void het_drop_kernel(HetDropArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= a.ncell) return;
  auto in = [&](int f) { return a.in[(long long)f * a.ldi + cell]; };
  auto c = [&](int sp) {
    const int i = a.ind[sp];
    return i >= 0 ? a.c[(long long)i * a.ldc + cell] : 0.0;
  };
  auto met = [&](int f) { return a.met[(long long)f * a.ldm + cell]; };
  double srhocl = 0.0, srhobr = 0.0;
  const double FC = in(HETIN_CLDF), TEMP = met(0);
  if (FC > 1.0e-4) {
    const double LWC = (in(HETIN_QL) * in(HETIN_AIRDEN) * 1.0e-3 / FC);
    if (a.size_res[cell] && in(HETIN_IsWater) != 0.0 && TEMP > 268.15 && LWC > 1.0e-20) {
      // the four sulfite uptake laws at this cell's HetState
      gcrates::Env E;
      gcrates::env_init(E, met(0), met(1), met(2), met(3), met(4), met(5));
      gcrates::HetCell X;
      X.H = a.het;
      X.ldh = a.ldh;
      X.C = a.c;
      X.ldc = a.ldc;
      X.cell = cell;
      X.sp = gcrates::HetSpecies{a.hs_ind, a.hs_mw, a.hs_srmw, a.hs_hk0, a.hs_hcr};
      gcrates::het_cell_init(X, E);
      const double CVF = 1.0e3 * AIRMW / (in(HETIN_AIRDEN) * AVO);
      const double DT = a.dt;
      const double so2 = c(HSS_SO2) * CVF;
      const double XX1 = loss2(so2, c(HSS_H2O2) * CVF, met(12) / CVF / FC, DT);
      const double XX2 = loss2(so2, c(HSS_O3) * CVF, met(13) / CVF / FC, DT);
      double XX3 = 0.0;
      const double Arg3 = (-met(14) / FC) * DT;
      if (fabs(Arg3) < 709.0) XX3 = so2 * (1.0 - exp(Arg3));
      const double r_hso3 = c(HSS_SO2) * CVF * in(HETIN_HSO3_aq);
      const double r_so3 = c(HSS_SO2) * CVF * in(HETIN_SO3_aq);
      const double hocl = c(HSS_HOCl) * CVF, hobr = c(HSS_HOBr) * CVF;
      double XX4 = loss2(r_hso3, hocl, gcrates::HOClUptkByHSO3m(X) / CVF, DT);
      XX4 = XX4 + loss2(r_so3, hocl, gcrates::HOClUptkBySO3mm(X) / CVF, DT);
      double XX5 = loss2(r_hso3, hobr, gcrates::HOBrUptkByHSO3m(X) / CVF, DT);
      XX5 = XX5 + loss2(r_so3, hobr, gcrates::HOBrUptkBySO3mm(X) / CVF, DT);
      // the Fortran's R1 is the SO3-- term at this point
      double xx[5] = {XX1, XX2, XX3, XX4, XX5};
      double LST = xx[0] + xx[1] + xx[2] + xx[3] + xx[4];
      if (LST > r_so3) {
        for (int k = 0; k < 5; ++k) xx[k] = (r_so3 * xx[k]) / LST;
        LST = xx[0] + xx[1] + xx[2] + xx[3] + xx[4];
      }
      const double NH3 = in(HETIN_NH3) * CVF * 1.0e+12;
      const double SO2 = fmax(c(HSS_SO2) * CVF - (LST * FC), 1.0e-20) * 1.0e+12;
      const double H2O2 = c(HSS_H2O2) * CVF * 1.0e12;
      const double HNO3 = c(HSS_HNO3) * CVF * 1.0e12;
      const double AD = in(HETIN_AD), AIRVOL = in(HETIN_AIRVOL);
      const double SO4 = (c(HSS_SO4) * CVF * AD * 1.0e+9) / ((AIRMW / HSS_MW_SO4) * AIRVOL);
      const double B = (LST * AD * 1.0e+9) / ((AIRMW / HSS_MW_SO4) * AIRVOL);
      const double CNss = in(HETIN_SALC) * CVF * AD / ((AIRMW / HSS_MW_SALC) * AIRVOL);
      const double CN = (0.75 * CNss) / (PI_PHYS * SS_DEN * RG_S3 * exp(ARG_SS)) * 1.e-6;
      // Yuen et al.'s coefficients by SO2 [pptv]: B, NH3, SO2, H2O2, HNO3, W, CN, SO4
      static constexpr double AL[4][8] = {
          {0.5318, -1.67e-7, 2.59e-6, -1.77e-7, -1.72e-7, 1.22e-6, 4.58e-6, -1.00e-5},
          {0.5591, 3.62e-6, 1.66e-6, 1.06e-7, -5.45e-7, -5.79e-7, 1.63e-5, -7.40e-6},
          {1.1547, -4.28e-8, -1.23e-7, -9.05e-7, 1.73e-7, 7.22e-6, 2.44e-5, 3.25e-5},
          {1.1795, 2.57e-7, -5.54e-7, -1.08e-6, 1.95e-6, 6.14e-6, 1.64e-5, 2.48e-6}};
      const int bin = SO2 <= 200.0 ? 0 : SO2 <= 500.0 ? 1 : SO2 < 1000.0 ? 2 : 3;
      const double* al = AL[bin];
      const double W = -in(HETIN_OMEGA) / (in(HETIN_AIRDEN) * G0) * 100.0;
      const double APV = sqrt(in(HETIN_U) * in(HETIN_U) + in(HETIN_V) * in(HETIN_V)) + (W * W * 1.0e-4);
      const double H = DT * APV;
      const double sum_gas = (al[1] * NH3) + (al[2] * SO2) + (al[3] * H2O2) + (al[4] * HNO3);
      const double DSVI = (al[0] * B) + (((al[6] * CN) + (al[5] * W) + (al[7] * SO4) + sum_gas) * H);
      double SR = 0.0;
      if (W > 0.0 && c(HSS_SO2) > 0.0) {
        SR = fmax((DSVI - B), 0.0);
        if (SR > 0.0) {
          SR = SR * (AIRMW / HSS_MW_SO4) * 1.e-9 / in(HETIN_AIRDEN);
          SR = fmin(SR, SO2 / 1.0e12);
        }
      }
      SR = SR / CVF / DT;
      const double DENOM = xx[1] + xx[3] + xx[4];
      srhocl = SR * gcrates::SafeDiv(xx[3], DENOM, 0.0);
      srhobr = SR * gcrates::SafeDiv(xx[4], DENOM, 0.0);
      srhocl = gcrates::SafeDiv(srhocl, (c(HSS_SO2) * c(HSS_HOCl)), 0.0);
      srhobr = gcrates::SafeDiv(srhobr, (c(HSS_SO2) * c(HSS_HOBr)), 0.0);
    }
  }
  a.met[(long long)4 * a.ldm + cell] = srhocl;
  a.met[(long long)5 * a.ldm + cell] = srhobr;
}

}  // namespace drop

}  // namespace

cudaError_t het_drop_chem(const HetDropArgs& a, cudaStream_t s) {
  if (a.ncell <= 0) return cudaSuccess;
  const int block = 128;
  drop::het_drop_kernel<<<(a.ncell + block - 1) / block, block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t sulfur_cld_rates(const SulfurCldArgs& a, cudaStream_t s) {
  if (a.ncell <= 0) return cudaSuccess;
  const int block = 128;
  so2::sulfur_cld_kernel<<<(a.ncell + block - 1) / block, block, 0, s>>>(a);
  return cudaGetLastError();
}

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
