// Heterogeneous rate laws of the fullchem Update_RCONST (device code).
//
//   Ars_L1k, kIIR1Ltd, CloudHet, ReactoDiff_Corr, SafeDiv, Is_SafeDiv
//                         KPP/fullchem/rateLawUtilFuncs.F90:77-522
//   the 60 uptake / hydrolysis rate functions and their gamma routines
//                         KPP/fullchem/fullchem_RateLawFuncs.F90:795-3460
//   TEMP-derived terms, RELHUM
//                         GeosCore/fullchem_mod.F90:2147-2165
//
// The per-cell HetState arrives as rows of a cell-interleaved array (row
// offsets HET_* from gcchem.hetstate, with SUNCOS as the last row), the
// species the laws read through C(ind_X), MW, SR_MW and HENRY_K0/CR are
// addressed through HetSpc (a per-mechanism index and constant table).
// Each function follows its Fortran statement by statement, in the same
// evaluation order; logical HetState fields are 0.0 / 1.0.
#pragma once
#include <cuda_runtime.h>

#include "het_layout.h"
#include "rate_laws.cuh"

namespace gcrates {

// Species that the heterogeneous laws reference.
enum HetSpc : int {
  HS_BrNO3 = 0, HS_H2O, HS_HCl, HS_ClNO2, HS_BrSALA, HS_BrSALC, HS_HBr, HS_SALACL, HS_SALCCL, HS_ClNO3,
  HS_HOBr, HS_SO2, HS_HOCl, HS_HO2, HS_IONO2, HS_N2O5, HS_NIT, HS_NITs, HS_NO2, HS_NO3, HS_O3, HS_OH, HS_N
};

// Per-mechanism species data of the heterogeneous laws: KPP index (-1 if
// the mechanism lacks the species), MW, SR_MW, HENRY_K0, HENRY_CR.
struct HetSpecies {
  const int* ind;
  const double* mw;
  const double* srmw;
  const double* hk0;
  const double* hcr;
};

// aerosol types (1-based, as the Fortran indexes xArea/xRadi/...)
constexpr int DU1 = 1, SUL = 8, BKC = 9, ORC = 10, SSA = 11, SSC = 12, SLA = 13, IIC = 14;
// KHETI_SLA reactions (1-based)
constexpr int N2O5_plus_H2O = 1, N2O5_plus_HCl = 2, ClNO3_plus_H2O = 3, ClNO3_plus_HCl = 4, ClNO3_plus_HBr = 5,
              BrNO3_plus_H2O = 6, BrNO3_plus_HCl = 7, HOCl_plus_HCl = 8, HOCl_plus_HBr = 9, HOBr_plus_HCl = 10,
              HOBr_plus_HBr = 11;
constexpr double CON_R = 0.083144598;
constexpr double RSTARG = 8.3144598;
constexpr double RGASLATM = 8.2057e-2;
constexpr double BOLTZ = 1.38064852e-23;
constexpr double CRITRH = 35.0;
constexpr double CON_ATM_BAR = 1.0 / 1.01325;
constexpr double INV_T298 = 1.0 / 298.15;
constexpr double HET_MIN_LIFE = 1.e-3;
constexpr double HET_MIN_RATE = 1.0 / HET_MIN_LIFE;

struct HetCell {
  const double* H;
  long long ldh;
  const double* C;
  long long ldc;
  int cell;
  HetSpecies sp;
  double TEMP, NUMDEN, INV_TEMP, SR_TEMP, FOUR_R_T, FOUR_RGASLATM_T, EIGHT_RSTARG_T, RELHUM, SUNCOS;

  __device__ double h(int f) const { return H[(long long)f * ldh + cell]; }
  __device__ bool b(int f) const { return h(f) != 0.0; }
  __device__ double xArea(int t) const { return h(HET_xArea + t - 1); }
  __device__ double xRadi(int t) const { return h(HET_xRadi + t - 1); }
  __device__ double xVol(int t) const { return h(HET_xVol + t - 1); }
  __device__ double xH2O(int t) const { return h(HET_xH2O + t - 1); }
  __device__ double kheti(int r) const { return h(HET_KHETI_SLA + r - 1); }
  __device__ double c(int s) const {
    const int i = __ldg(sp.ind + s);
    return i >= 0 ? C[(long long)i * ldc + cell] : 0.0;
  }
  __device__ double mw(int s) const { return __ldg(sp.mw + s); }
  __device__ double srmw(int s) const { return __ldg(sp.srmw + s); }
};

// Set_Kpp_GridBox_Values' temperature and humidity terms
// (GeosCore/fullchem_mod.F90:2152-2165).
__device__ __forceinline__ void het_cell_init(HetCell& X, const Env& E) {
  X.TEMP = E.TEMP;
  X.NUMDEN = E.NUMDEN;
  X.INV_TEMP = E.INV_TEMP;
  X.SR_TEMP = E.SR_TEMP;
  X.FOUR_R_T = 4.0 * CON_R * E.TEMP;
  X.FOUR_RGASLATM_T = 4.0 * RGASLATM * E.TEMP;
  X.EIGHT_RSTARG_T = 8.0 * RSTARG * E.TEMP;
  const double consvap = 6.1078e+03 / (BOLTZ * 1e+7);
  const double consexp = 17.2693882 * (E.TEMP - 273.16) / (E.TEMP - 35.86);
  const double vpresh2o = consvap * exp(consexp) / E.TEMP;
  X.RELHUM = (E.H2O / vpresh2o) * 100.0;
  X.SUNCOS = X.h(HET_SUNCOS);
}

// Fortran EXPONENT(x): e with x = f * 2**e, 0.5 <= |f| < 1; 0 for x = 0.
__device__ __forceinline__ int f_exponent(double x) {
  if (x == 0.0) return 0;
  int e;
  frexp(x, &e);
  return e;
}

__device__ __forceinline__ double SafeDiv(double num, double denom, double alt) {
  const int ediff = f_exponent(num) - f_exponent(denom);
  if (ediff > 1023 || denom == 0.0) return alt;
  if (ediff < -1020) return 0.0;
  return num / denom;
}

__device__ __forceinline__ bool Is_SafeDiv(double num, double denom) {
  const int ediff = f_exponent(num) - f_exponent(denom);
  return !(ediff < -1020 || ediff > 1023 || denom == 0.0);
}

__device__ __forceinline__ double Ars_L1k(const HetCell& X, double area, double radius, double gamma, double srMw) {
  if (gamma < 1.0e-30 || radius < 1.0e-30) return 0.0;
  const double dfkg = (9.45E+17 / X.NUMDEN) * X.SR_TEMP * sqrt(3.472E-2 + 1.0 / (srMw * srMw));
  return area / ((radius / dfkg) + 2.749064E-4 * srMw / (gamma * X.SR_TEMP));
}

__device__ __forceinline__ double kIIR1Ltd(double concGas, double concEduct, double kISource) {
  double kII = 0.0;
  if (concEduct < 1.0) return kII;
  if (!Is_SafeDiv(concGas * kISource, concEduct)) return kII;
  const double kIGas = kISource;
  const double kIEduct = kIGas * concGas / concEduct;
  kII = kIGas / concEduct;
  if (kIGas > 0.0) {
    const double lifeA = SafeDiv(1.0, kIGas, 0.0);
    const double lifeB = SafeDiv(1.0, kIEduct, 0.0);
    if ((lifeA < lifeB) && (lifeA < HET_MIN_LIFE))
      kII = SafeDiv(HET_MIN_RATE, concEduct, 0.0);
    else if (lifeB < HET_MIN_LIFE)
      kII = SafeDiv(HET_MIN_RATE, concGas, 0.0);
  }
  return kII;
}

__device__ __forceinline__ double CloudHet(const HetCell& X, double srMw, double gamLiq, double gamIce, double brLiq,
                                           double brIce) {
  const double tauc = 3600.0;
  const double cldfr = X.h(HET_cldFr), aliq = X.h(HET_aLiq), aice = X.h(HET_aIce);
  if ((cldfr < 0.0001) || (aliq + aice <= 0.0)) return 0.0;
  double kI = 0.0, kIb = 0.0, ktmp;
  if (brLiq > 0.0) {
    const double area = SafeDiv(aliq, cldfr, 0.0);
    if (area > 0.0) {
      ktmp = Ars_L1k(X, area, X.h(HET_rLiq), gamLiq, srMw);
      kI = kI + ktmp;
      kIb = kIb + (ktmp * brLiq);
    }
  }
  if (brIce > 0.0) {
    const double area = SafeDiv(aice, cldfr, 0.0);
    if (area > 0.0) {
      ktmp = Ars_L1k(X, area, X.h(HET_rIce), gamIce, srMw);
      kI = kI + ktmp;
      kIb = kIb + (ktmp * brIce);
    }
  }
  const double branch = SafeDiv(kIb, kI, 0.0);
  if (!(branch > 0.0)) return 0.0;
  const double kk = kI * tauc;
  double ff = SafeDiv(cldfr, X.h(HET_clearFr), 1.0e+30);
  ff = fmin(ff, 1.0e+30);
  double xx = (ff - kk - 1.0) / 2.0 + sqrt(1.0 + ff * ff + kk * kk + 2.0 * ff + 2.0 * kk - 2.0 * ff * kk) / 2.0;
  xx = fmax(xx, 0.0);
  double kHet = kI / (1.0 + SafeDiv(1.0, xx, 1.0e+30));
  return kHet * branch;
}

__device__ __forceinline__ double coth(double x) {
  const double y = exp(-2.0 * x);
  return (1.0 + y) / (1.0 - y);
}

__device__ __forceinline__ double ReactoDiff_Corr(double radius, double l) {
  const double x = radius / l;
  if (x > 1000.0) return 1.0;
  if (x < 0.1) return x / 3.0;
  return coth(x) - (1.0 / x);
}

// thermal velocity [cm/s] of species s
__device__ __forceinline__ double het_cavg(const HetCell& X, int s) {
  const double M_X = X.mw(s) * 1.0e-3;
  return sqrt(X.EIGHT_RSTARG_T / (X.h(HET_PI) * M_X)) * 100.0;
}


// ---- BrNO3 (fullchem_RateLawFuncs.F90:803-866) ----------------------------
__device__ __forceinline__ double BrNO3uptkByH2O(const HetCell& X) {
  double k = 0.0;
  const double gamLiq = 0.0021 * X.TEMP - 0.561;
  const double gamIce = 5.3e-4 * exp(1100.0 / X.TEMP);
  const double srMw = X.srmw(HS_BrNO3);
  const double clr = X.h(HET_clearFr);
  double gamma = gamLiq;
  k = k + Ars_L1k(X, clr * X.xArea(SUL), X.xRadi(SUL), gamma, srMw);
  k = k + Ars_L1k(X, clr * X.xArea(SSA), X.xRadi(SSA), gamma, srMw);
  k = k + Ars_L1k(X, clr * X.xArea(SSC), X.xRadi(SSC), gamma, srMw);
  k = k + X.xArea(SLA) * X.kheti(BrNO3_plus_H2O);
  gamma = 0.3;
  if (X.b(HET_natSurface)) gamma = 0.001;
  k = k + Ars_L1k(X, clr * X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
  k = k + CloudHet(X, srMw, gamLiq, gamIce, 1.0, 1.0);
  return kIIR1Ltd(X.c(HS_BrNO3), X.c(HS_H2O), k);
}

__device__ __forceinline__ double BrNO3uptkByHCl(const HetCell& X) {
  double k = 0.0;
  const double srMw = X.srmw(HS_BrNO3);
  if (X.b(HET_stratBox)) {
    k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), 0.9, srMw);
    k = k + X.xArea(SLA) * X.kheti(BrNO3_plus_HCl);
    k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), 0.3, srMw);
  }
  k = kIIR1Ltd(X.c(HS_BrNO3), X.c(HS_HCl), k);
  if (X.b(HET_TurnOffHetRates)) k = 0.0;
  return k;
}

// ---- ClNO2 (fullchem_RateLawFuncs.F90:872-1108) ---------------------------
__device__ __forceinline__ void Gam_ClNO2(const HetCell& X, double radius, double pH, double C_Cl, double C_Br,
                                          double& gamma, double& branchCl, double& branchBr) {
  const double INV_AB = 1.0 / 0.01;
  const double D_l = 1.0e-5;
  const double cavg = het_cavg(X, HS_ClNO2);
  const double H_X = 4.5e-2 * CON_ATM_BAR;
  double k_Cl = 1.0e+7 * C_Cl;
  if (pH >= 2.0) k_Cl = 0.0;
  const double k_Br = (1.01e-1 / (H_X * H_X * D_l)) * C_Br;
  const double k_tot = k_Cl + k_Br;
  gamma = 0.0;
  branchCl = 0.0;
  branchBr = 0.0;
  if (k_tot > 0.0) {
    const double l_r = sqrt(D_l / k_tot);
    double gb_tot = X.FOUR_R_T * H_X * l_r * k_tot / cavg;
    gb_tot = gb_tot * ReactoDiff_Corr(radius, l_r);
    gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
    branchCl = k_Cl / k_tot;
    branchBr = k_Br / k_tot;
  }
}

// ClNO2 + (Br or Cl) in tropospheric cloud, branch of the given fraction
__device__ __forceinline__ double clno2_cloud(const HetCell& X, bool br, double frac) {
  double gamma, bCl, bBr;
  Gam_ClNO2(X, X.h(HET_rLiq), X.h(HET_pHCloud), X.h(HET_Cl_conc_Cld), X.h(HET_Br_conc_Cld), gamma, bCl, bBr);
  const double branch = (br ? bBr : bCl) * frac;
  return CloudHet(X, X.srmw(HS_ClNO2), gamma, 0.0, branch, 0.0);
}

__device__ __forceinline__ double ClNO2uptkByBrSALA(const HetCell& X) {
  double k = 0.0, gamma, dummy, branchBr;
  const double srMw = X.srmw(HS_ClNO2);
  if (!X.b(HET_stratBox)) k = k + clno2_cloud(X, true, X.h(HET_frac_Br_CldA));
  Gam_ClNO2(X, X.h(HET_aClRadi), X.h(HET_pHSSA), X.h(HET_Cl_conc_SSA), X.h(HET_Br_conc_SSA), gamma, dummy,
            branchBr);
  const double area = X.h(HET_clearFr) * X.h(HET_aClArea);
  k = k + Ars_L1k(X, area, X.h(HET_aClRadi), gamma, srMw) * branchBr;
  return kIIR1Ltd(X.c(HS_ClNO2), X.c(HS_BrSALA), k);
}

__device__ __forceinline__ double ClNO2uptkByBrSALC(const HetCell& X) {
  double k = 0.0, gamma, dummy, branchBr;
  const double srMw = X.srmw(HS_ClNO2);
  if (!X.b(HET_stratBox)) k = k + clno2_cloud(X, true, X.h(HET_frac_Br_CldC));
  Gam_ClNO2(X, X.xRadi(SSC), X.h(HET_pHSSA + 1), X.h(HET_Cl_conc_SSC), X.h(HET_Br_conc_SSC), gamma, dummy,
            branchBr);
  const double area = X.h(HET_clearFr) * X.xArea(SSC);
  k = k + Ars_L1k(X, area, X.xRadi(SSC), gamma, srMw) * branchBr;
  return kIIR1Ltd(X.c(HS_ClNO2), X.c(HS_BrSALC), k);
}

__device__ __forceinline__ double ClNO2uptkByHBr(const HetCell& X) {
  double k = 0.0;
  if (!X.b(HET_stratBox)) k = k + clno2_cloud(X, true, X.h(HET_frac_Br_CldG));
  return kIIR1Ltd(X.c(HS_ClNO2), X.c(HS_HBr), k);
}

__device__ __forceinline__ double ClNO2uptkBySALACL(const HetCell& X) {
  double k = 0.0, gamma, branchCl, dummy;
  const double srMw = X.srmw(HS_ClNO2);
  if (!X.b(HET_stratBox)) k = k + clno2_cloud(X, false, X.h(HET_frac_Cl_CldA));
  Gam_ClNO2(X, X.h(HET_aClRadi), X.h(HET_pHSSA), X.h(HET_Cl_conc_SSA), X.h(HET_Br_conc_SSA), gamma, branchCl,
            dummy);
  const double area = X.h(HET_clearFr) * X.h(HET_aClArea);
  k = k + Ars_L1k(X, area, X.h(HET_aClRadi), gamma, srMw) * branchCl;
  return kIIR1Ltd(X.c(HS_ClNO2), X.c(HS_SALACL), k);
}

__device__ __forceinline__ double ClNO2uptkBySALCCL(const HetCell& X) {
  double k = 0.0;
  if (!X.b(HET_stratBox)) k = k + clno2_cloud(X, false, X.h(HET_frac_Cl_CldC));
  return kIIR1Ltd(X.c(HS_ClNO2), X.c(HS_SALCCL), k);
}

__device__ __forceinline__ double ClNO2uptkByHCl(const HetCell& X) {
  double k = 0.0;
  if (!X.b(HET_stratBox)) k = k + clno2_cloud(X, false, X.h(HET_frac_Cl_CldG));
  return kIIR1Ltd(X.c(HS_ClNO2), X.c(HS_HCl), k);
}

// ---- ClNO3 (fullchem_RateLawFuncs.F90:1114-1420) --------------------------
__device__ __forceinline__ void Gam_ClNO3_Aer(const HetCell& X, double C_Br, double& gamma, double& branchBr) {
  const double INV_AB = 1.0 / 0.108;
  const double K_0 = 1.2e+5 * 1.2e+5;  // 1.2e+5_dp ** 2.0_dp
  const double D_l = 5.0e-6;
  const double cavg = het_cavg(X, HS_ClNO3);
  const double k_Br = 1.0e+12 * C_Br;
  const double k_tot = K_0 + k_Br;
  const double gb_tot = X.FOUR_R_T * sqrt(k_tot * D_l) / cavg;
  gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
  branchBr = k_Br / k_tot;
}

__device__ __forceinline__ void Gam_ClNO3_Ice(const HetCell& X, double& gamma, double& brHCl, double& brHBr,
                                              double& brH2O) {
  const double twenty = 1.0 / 0.5;
  const double g1 = 0.24 * X.h(HET_HCl_theta);
  const double g2 = 0.56 * X.h(HET_HBr_theta);
  const double cavg = het_cavg(X, HS_ClNO3);
  const double H2Os = 1e+15 - (3.0 * 2.7e+14 * X.h(HET_HNO3_theta));
  const double kks = 4.0 * 5.2e-17 * exp(2032.0 / X.TEMP);
  const double g3 = 1.0 / (twenty + cavg / (kks * H2Os));
  gamma = g1 + g2 + g3;
  brHCl = g1 / gamma;
  brHBr = g2 / gamma;
  brH2O = g3 / gamma;
}

__device__ __forceinline__ double ClNO3uptkByH2O(const HetCell& X) {
  double k = 0.0, gamma, branchBr, gammaIce, dum1, dum2, branchIce;
  const double srMw = X.srmw(HS_ClNO3);
  Gam_ClNO3_Aer(X, X.h(HET_Br_conc_SSA), gamma, branchBr);
  const double area = X.h(HET_clearFr) * X.h(HET_aClArea);
  double branchLiq = (1.0 - branchBr) * (1.0 - X.h(HET_frac_SALACL));
  k = k + Ars_L1k(X, area, X.h(HET_aClRadi), gamma, srMw) * branchLiq;
  k = k + X.xArea(SLA) * X.kheti(ClNO3_plus_H2O);
  gamma = 0.3;
  if (X.b(HET_natSurface)) gamma = 0.004;
  k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
  if (!X.b(HET_stratBox)) {
    Gam_ClNO3_Aer(X, X.h(HET_Br_conc_Cld), gamma, branchBr);
    branchLiq = 1.0 - branchBr;
    Gam_ClNO3_Ice(X, gammaIce, dum1, dum2, branchIce);
    k = k + CloudHet(X, srMw, gamma, gammaIce, branchLiq, branchIce);
  }
  return kIIR1Ltd(X.c(HS_ClNO3), X.c(HS_H2O), k);
}

__device__ __forceinline__ double ClNO3uptkByHCl(const HetCell& X) {
  double k = 0.0, gamma, gammaIce, branchIce, dum1, dum2;
  const double srMw = X.srmw(HS_ClNO3);
  if (X.b(HET_stratBox)) {
    gamma = 0.1e-4;
    k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gamma, srMw);
    k = k + X.xArea(SLA) * X.kheti(ClNO3_plus_HCl);
    gamma = 0.3;
    if (X.b(HET_natSurface)) gamma = 0.2;
    k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
  } else {
    Gam_ClNO3_Ice(X, gammaIce, branchIce, dum1, dum2);
    k = k + CloudHet(X, srMw, 0.0, gammaIce, 0.0, branchIce);
  }
  return kIIR1Ltd(X.c(HS_ClNO3), X.c(HS_HCl), k);
}

__device__ __forceinline__ double ClNO3uptkByHBr(const HetCell& X) {
  double k = 0.0, gamma, branchBr, gammaIce, dum1, branchIce, dum2;
  const double srMw = X.srmw(HS_ClNO3);
  if (X.b(HET_stratBox)) {
    k = k + X.xArea(SLA) * X.kheti(ClNO3_plus_HBr);
    gamma = 0.3;
    k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
  } else {
    Gam_ClNO3_Aer(X, X.h(HET_Br_conc_Cld), gamma, branchBr);
    const double branchLiq = branchBr * X.h(HET_frac_Br_CldG);
    Gam_ClNO3_Ice(X, gammaIce, dum1, branchIce, dum2);
    k = CloudHet(X, srMw, gamma, gammaIce, branchLiq, branchIce);
  }
  k = kIIR1Ltd(X.c(HS_ClNO3), X.c(HS_HBr), k);
  if (X.b(HET_TurnOffHetRates)) k = 0.0;
  return k;
}

__device__ __forceinline__ double ClNO3uptkByBrSALA(const HetCell& X) {
  double k = 0.0, gamma, branchBr;
  const double srMw = X.srmw(HS_ClNO3);
  if (!X.b(HET_stratBox)) {
    Gam_ClNO3_Aer(X, X.h(HET_Br_conc_Cld), gamma, branchBr);
    const double branch = branchBr * X.h(HET_frac_Br_CldA);
    k = k + CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  Gam_ClNO3_Aer(X, X.h(HET_Br_conc_SSA), gamma, branchBr);
  const double area = X.h(HET_clearFr) * X.h(HET_aClArea);
  k = k + Ars_L1k(X, area, X.h(HET_aClRadi), gamma, srMw) * branchBr;
  k = kIIR1Ltd(X.c(HS_ClNO3), X.c(HS_BrSALA), k);
  if (X.b(HET_TurnOffHetRates)) k = 0.0;
  return k;
}

__device__ __forceinline__ double ClNO3uptkByBrSALC(const HetCell& X) {
  double k = 0.0, gamma, branchBr;
  const double srMw = X.srmw(HS_ClNO3);
  if (!X.b(HET_stratBox)) {
    Gam_ClNO3_Aer(X, X.h(HET_Br_conc_Cld), gamma, branchBr);
    const double branch = branchBr * X.h(HET_frac_Br_CldC);
    k = k + CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  Gam_ClNO3_Aer(X, X.h(HET_Br_conc_SSC), gamma, branchBr);
  const double area = X.h(HET_clearFr) * X.xArea(SSC);
  k = k + Ars_L1k(X, area, X.xRadi(SSC), gamma, srMw) * branchBr;
  k = kIIR1Ltd(X.c(HS_ClNO3), X.c(HS_BrSALC), k);
  if (X.b(HET_TurnOffHetRates)) k = 0.0;
  return k;
}

__device__ __forceinline__ double ClNO3uptkBySALACL(const HetCell& X) {
  if (X.b(HET_stratBox)) return 0.0;
  double gamma, branchBr;
  Gam_ClNO3_Aer(X, X.h(HET_Br_conc_SSA), gamma, branchBr);
  const double srMw = X.srmw(HS_ClNO3);
  const double area = X.h(HET_clearFr) * X.h(HET_aClArea);
  const double branch = (1.0 - branchBr) * X.h(HET_frac_SALACL);
  double k = 0.0;
  k = k + Ars_L1k(X, area, X.h(HET_aClRadi), gamma, srMw) * branch;
  return kIIR1Ltd(X.c(HS_ClNO3), X.c(HS_SALACL), k);
}

__device__ __forceinline__ double ClNO3uptkBySALCCL(const HetCell& X) {
  if (X.b(HET_stratBox)) return 0.0;
  double gamma, branchBr;
  Gam_ClNO3_Aer(X, X.h(HET_Br_conc_SSC), gamma, branchBr);
  const double srMw = X.srmw(HS_ClNO3);
  const double area = X.h(HET_clearFr) * X.xArea(SSC);
  const double branch = 1.0 - branchBr;
  double k = 0.0;
  k = k + Ars_L1k(X, area, X.xRadi(SSC), gamma, srMw) * branch;
  return kIIR1Ltd(X.c(HS_ClNO3), X.c(HS_SALCCL), k);
}

// ---- HBr, HO2 (fullchem_RateLawFuncs.F90:1423-1488) -----------------------
__device__ __forceinline__ double HBrUptkBySALA(const HetCell& X) {
  if (X.b(HET_stratBox)) return 0.0;
  const double area = X.h(HET_clearFr) * X.h(HET_aClArea);
  const double gamma = 1.3e-8 * exp(4290.0 / X.TEMP);
  return Ars_L1k(X, area, X.h(HET_aClRadi), gamma, X.srmw(HS_HBr));
}

__device__ __forceinline__ double HBrUptkBySALC(const HetCell& X) {
  if (X.b(HET_stratBox)) return 0.0;
  const double area = X.h(HET_clearFr) * X.xArea(SSC);
  const double gamma = 1.3e-8 * exp(4290.0 / X.TEMP);
  return Ars_L1k(X, area, X.xRadi(SSC), gamma, X.srmw(HS_HBr));
}

__device__ __forceinline__ double HO2uptk1stOrd(const HetCell& X) {
  double k = 0.0;
  const double srMw = X.srmw(HS_HO2);
  const double g = X.h(HET_gamma_HO2);
  for (int t = DU1; t <= SSC; ++t) k = k + Ars_L1k(X, X.xArea(t), X.xRadi(t), g, srMw);  // types 1..12 in order
  return k;
}

// ---- HOBr (fullchem_RateLawFuncs.F90:1490-2050) ---------------------------
__device__ __forceinline__ double Br2_Yield(double Br_over_Cl) {
  double Y_Br2 = 0.0;
  if (Br_over_Cl > 0.0) {
    Y_Br2 = 0.41 * log10(Br_over_Cl) + 2.25;
    Y_Br2 = fmax(fmin(Y_Br2, 0.9), 0.0);
  }
  return Y_Br2;
}

__device__ __forceinline__ double hobr_henry(const HetCell& X) {
  return (__ldg(X.sp.hk0 + HS_HOBr) * CON_ATM_BAR) * exp(__ldg(X.sp.hcr + HS_HOBr) * (1.0 / X.TEMP - INV_T298));
}

__device__ __forceinline__ double Gam_HOBr_Aer(const HetCell& X, double radius, double C_Hp, double C_Clm,
                                               double C_Brm) {
  const double INV_AB = 1.0 / 0.6;
  const double D_l = 1.4e-5;
  const double H_X = hobr_henry(X);
  const double cavg = het_cavg(X, HS_HOBr);
  const double C_Hp1 = fmax(fmin(C_Hp, 1.0e-6), 1.0e-9);
  const double C_Hp2 = fmax(fmin(C_Hp, 1.0e-2), 1.0e-6);
  const double k_HOBr_Cl = 2.3e+10 * C_Clm * C_Hp1;
  const double k_HOBr_Br = 1.6e+10 * C_Brm * C_Hp2;
  const double k_tot = k_HOBr_Cl + k_HOBr_Br;
  double gamma = 0.0;
  if (k_tot > 0.0) {
    const double l_r = sqrt(D_l / k_tot);
    double gb_tot = X.FOUR_R_T * H_X * l_r * k_tot / cavg;
    gb_tot = gb_tot * ReactoDiff_Corr(radius, l_r);
    gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
  }
  return gamma;
}

struct HobrCld {
  double gamma, k_tot, k_Cl, k_Br, k_HSO3, k_SO3;
};

__device__ __forceinline__ HobrCld Gam_HOBr_Cld(const HetCell& X) {
  const double INV_AB = 1.0 / 0.6;
  const double D_l = 1.4e-5;
  HobrCld g;
  const double H_X = hobr_henry(X);
  const double cavg = het_cavg(X, HS_HOBr);
  double C_Hp1 = fmin(X.h(HET_H_conc_LCl), 1.0e-6);
  double C_Hp2 = fmin(X.h(HET_H_conc_LCl), 1.0e-2);
  C_Hp1 = fmax(C_Hp1, 1.0e-9);
  C_Hp2 = fmax(C_Hp2, 1.0e-6);
  g.k_Cl = 2.3e+10 * X.h(HET_Cl_conc_Cld) * C_Hp1;
  g.k_Br = 1.6e+10 * X.h(HET_Br_conc_Cld) * C_Hp2;
  g.k_HSO3 = 2.6e+7 * X.h(HET_HSO3_aq);
  g.k_SO3 = 5.0e+9 * X.h(HET_SO3_aq);
  g.k_tot = g.k_Cl + g.k_Br + g.k_HSO3 + g.k_SO3;
  g.gamma = 0.0;
  if (g.k_tot > 0.0) {
    const double l_r = sqrt(D_l / g.k_tot);
    double gb_tot = X.FOUR_R_T * H_X * l_r * g.k_tot / cavg;
    gb_tot = gb_tot * ReactoDiff_Corr(X.h(HET_rLiq), l_r);
    g.gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
  }
  return g;
}

__device__ __forceinline__ void Gam_HOBr_Ice(const HetCell& X, double& gamma, double& branch_HCl,
                                             double& branch_HBr) {
  const double gamma_HCl = X.h(HET_HCl_theta) * 0.25;
  const double gamma_HBr = X.h(HET_HBr_theta) * 4.8e-4 * exp(1240.0 / X.TEMP);
  gamma = gamma_HCl + gamma_HBr;
  branch_HCl = 0.0;
  branch_HBr = 0.0;
  if (gamma > 0.0) {
    branch_HCl = gamma_HCl / gamma;
    branch_HBr = gamma_HBr / gamma;
  }
}

// cloud branch of HOBr + Br- (toBr) or + Cl- (!toBr): branch_0 * 0.9 (0.1),
// or by the Br2 yield when Br/Cl <= 5e-4
__device__ __forceinline__ double hobr_cloud_branch(const HetCell& X, const HobrCld& g, bool toBr) {
  const double branch_0 = (g.k_Cl + g.k_Br) / g.k_tot;
  double branch = branch_0 * (toBr ? 0.9 : 0.1);
  if (X.h(HET_Br_over_Cl_Cld) <= 5.0e-4)
    branch = toBr ? branch_0 * Br2_Yield(X.h(HET_Br_over_Cl_Cld))
                  : branch_0 * (1.0 - Br2_Yield(X.h(HET_Br_over_Cl_Cld)));
  return branch;
}

__device__ __forceinline__ double HOBrUptkByHBr(const HetCell& X) {
  double k = 0.0, brIce = 0.0, brLiq = 0.0, gammaIce = 0.0, gammaLiq = 0.0, dummy;
  const double srMw = X.srmw(HS_HOBr);
  if (X.b(HET_stratBox)) {
    gammaLiq = 0.25;
    k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gammaLiq, srMw);
    k = k + X.xArea(SLA) * X.kheti(HOBr_plus_HBr);
    gammaIce = 0.3;
    if (X.b(HET_natSurface)) gammaIce = 0.001;
    k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gammaIce, srMw);
  } else {
    const HobrCld g = Gam_HOBr_Cld(X);
    gammaLiq = g.gamma;
    brLiq = hobr_cloud_branch(X, g, true) * X.h(HET_frac_Br_CldG);
    Gam_HOBr_Ice(X, gammaIce, dummy, brIce);
    k = k + CloudHet(X, srMw, gammaLiq, gammaIce, brLiq, brIce);
  }
  return kIIR1Ltd(X.c(HS_HOBr), X.c(HS_HBr), k);
}

__device__ __forceinline__ double HOBrUptkByHCl(const HetCell& X) {
  double k = 0.0, brIce = 0.0, brLiq = 0.0, gammaIce = 0.0, gammaLiq = 0.0, dummy;
  const double srMw = X.srmw(HS_HOBr);
  if (X.b(HET_stratBox)) {
    gammaLiq = 0.2;
    k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gammaLiq, srMw);
    k = k + X.xArea(SLA) * X.kheti(HOBr_plus_HCl);
    gammaIce = 0.3;
    if (X.b(HET_natSurface)) gammaIce = 0.1;
    k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gammaIce, srMw);
  } else {
    const HobrCld g = Gam_HOBr_Cld(X);
    gammaLiq = g.gamma;
    brLiq = hobr_cloud_branch(X, g, false) * X.h(HET_frac_Cl_CldG);
    Gam_HOBr_Ice(X, gammaIce, brIce, dummy);
    k = k + CloudHet(X, srMw, gammaLiq, gammaIce, brLiq, brIce);
  }
  return kIIR1Ltd(X.c(HS_HOBr), X.c(HS_HCl), k);
}

// HOBr on sea salt: cloud part (fraction frac of the Br or Cl branch) and
// the acidic aerosol part (fine: aClArea/aClRadi, coarse: SSC)
__device__ __forceinline__ double hobr_seasalt(const HetCell& X, bool toBr, bool fine, double frac) {
  double k = 0.0;
  const double srMw = X.srmw(HS_HOBr);
  if (!X.b(HET_stratBox)) {
    const HobrCld g = Gam_HOBr_Cld(X);
    const double brLiq = hobr_cloud_branch(X, g, toBr) * frac;
    k = k + CloudHet(X, srMw, g.gamma, 0.0, brLiq, 0.0);
  }
  if (X.b(fine ? HET_SSA_is_Acid : HET_SSC_is_Acid)) {
    const double radi = fine ? X.h(HET_aClRadi) : X.xRadi(SSC);
    const double gammaAer =
        fine ? Gam_HOBr_Aer(X, radi, X.h(HET_H_conc_SSA), X.h(HET_Cl_conc_SSA), X.h(HET_Br_conc_SSA))
             : Gam_HOBr_Aer(X, radi, X.h(HET_H_conc_SSC), X.h(HET_Cl_conc_SSC), X.h(HET_Br_conc_SSC));
    const double ratio = X.h(fine ? HET_Br_over_Cl_SSA : HET_Br_over_Cl_SSC);
    double branch = toBr ? 0.9 : 0.1;
    if (ratio <= 5.0e-4) branch = toBr ? Br2_Yield(ratio) : 1.0 - Br2_Yield(ratio);
    const double area = fine ? X.h(HET_clearFr) * X.h(HET_aClArea) * X.h(HET_f_Acid_SSA)
                             : X.h(HET_clearFr) * X.xArea(SSC) * X.h(HET_f_Acid_SSC);
    k = k + Ars_L1k(X, area, radi, gammaAer, srMw) * branch;
  }
  return k;
}

__device__ __forceinline__ double HOBrUptkByBrSALA(const HetCell& X) {
  return kIIR1Ltd(X.c(HS_HOBr), X.c(HS_BrSALA), hobr_seasalt(X, true, true, X.h(HET_frac_Br_CldA)));
}
__device__ __forceinline__ double HOBrUptkByBrSALC(const HetCell& X) {
  return kIIR1Ltd(X.c(HS_HOBr), X.c(HS_BrSALC), hobr_seasalt(X, true, false, X.h(HET_frac_Br_CldC)));
}
__device__ __forceinline__ double HOBrUptkBySALACL(const HetCell& X) {
  return kIIR1Ltd(X.c(HS_HOBr), X.c(HS_SALACL), hobr_seasalt(X, false, true, X.h(HET_frac_Cl_CldA)));
}
__device__ __forceinline__ double HOBrUptkBySALCCL(const HetCell& X) {
  return kIIR1Ltd(X.c(HS_HOBr), X.c(HS_SALCCL), hobr_seasalt(X, false, false, X.h(HET_frac_Cl_CldC)));
}

__device__ __forceinline__ double HOBrUptkByHSO3m(const HetCell& X) {
  double k = 0.0;
  if (!X.b(HET_stratBox)) {
    const HobrCld g = Gam_HOBr_Cld(X);
    const double brLiq = g.k_HSO3 / g.k_tot;
    k = k + CloudHet(X, X.srmw(HS_HOBr), g.gamma, 0.0, brLiq, 0.0);
  }
  return kIIR1Ltd(X.c(HS_HOBr), X.c(HS_SO2), k);
}

__device__ __forceinline__ double HOBrUptkBySO3mm(const HetCell& X) {
  double k = 0.0;
  if (!X.b(HET_stratBox)) {
    const HobrCld g = Gam_HOBr_Cld(X);
    const double brLiq = g.k_SO3 / g.k_tot;
    k = k + CloudHet(X, X.srmw(HS_HOBr), g.gamma, 0.0, brLiq, 0.0);
  }
  return kIIR1Ltd(X.c(HS_HOBr), X.c(HS_SO2), k);
}

// ---- HOCl (fullchem_RateLawFuncs.F90:2075-2364) ---------------------------
__device__ __forceinline__ double hocl_henry(const HetCell& X) {
  return (__ldg(X.sp.hk0 + HS_HOCl) * CON_ATM_BAR) * exp(__ldg(X.sp.hcr + HS_HOCl) * (X.INV_TEMP - INV_T298));
}

__device__ __forceinline__ void Gam_HOCl_Cld(const HetCell& X, double& gamma, double& branchCl,
                                             double& branchSO3) {
  const double INV_AB = 1.0 / 0.8;
  const double D_l = 2.0e-5;
  const double k_Cl = 1.5e+4 * X.h(HET_H_conc_LCl) * X.h(HET_Cl_conc_Cld);
  const double k_SO3 = 2.8e+5 * X.h(HET_TSO3_aq);
  const double k_tot = k_Cl + k_SO3;
  gamma = 0.0;
  branchCl = 0.0;
  branchSO3 = 0.0;
  if (k_tot > 0.0) {
    const double cavg = het_cavg(X, HS_HOCl);
    const double H_X = hocl_henry(X);
    const double l_r = sqrt(D_l / k_tot);
    double gb_tot = X.FOUR_R_T * H_X * l_r * k_tot / cavg;
    gb_tot = gb_tot * ReactoDiff_Corr(X.h(HET_rLiq), l_r);
    gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
    branchCl = k_Cl / k_tot;
    branchSO3 = k_SO3 / k_tot;
  }
}

__device__ __forceinline__ double Gam_HOCl_Aer(const HetCell& X, double radius, double C_Hp, double C_Cl) {
  const double INV_AB = 1.0 / 0.8;
  const double D_l = 2.0e-5;
  const double K_TER = 1.5e+4;
  if (!(C_Cl > 0.0)) return 0.0;
  const double cavg = het_cavg(X, HS_HOCl);
  const double H_X = hocl_henry(X);
  const double l_r = sqrt(D_l / (K_TER * C_Hp * C_Cl));
  double gb = X.FOUR_R_T * H_X * l_r * K_TER * C_Hp * C_Cl / cavg;
  gb = gb * ReactoDiff_Corr(radius, l_r);
  return 1.0 / (INV_AB + 1.0 / gb);
}

__device__ __forceinline__ double HOClUptkByHCl(const HetCell& X) {
  double k = 0.0, gamma, branchCl, dummy;
  const double srMw = X.srmw(HS_HOCl);
  if (X.b(HET_stratBox)) {
    gamma = 0.8;
    k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gamma, srMw);
    k = k + X.xArea(SLA) * X.kheti(HOCl_plus_HCl);
    gamma = 0.2;
    if (X.b(HET_natSurface)) gamma = 0.1;
    k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
    return kIIR1Ltd(X.c(HS_HOCl), X.c(HS_HCl), k);
  }
  Gam_HOCl_Cld(X, gamma, branchCl, dummy);
  const double branch = branchCl * X.h(HET_frac_Cl_CldG);
  const double gammaIce = 0.22 * X.h(HET_HCl_theta);
  const double brIce = 1.0;
  k = k + CloudHet(X, srMw, gamma, gammaIce, branch, brIce);
  return kIIR1Ltd(X.c(HS_HOCl), X.c(HS_HCl), k);
}

__device__ __forceinline__ double HOClUptkByHBr(const HetCell& X) {
  double k = 0.0, gamma;
  const double srMw = X.srmw(HS_HOCl);
  if (X.b(HET_stratBox)) {
    gamma = 0.8;
    k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gamma, srMw);
    k = k + X.xArea(SLA) * X.kheti(HOCl_plus_HBr);
    gamma = 0.3;
    k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
  }
  k = kIIR1Ltd(X.c(HS_HOCl), X.c(HS_HBr), k);
  if (X.b(HET_TurnOffHetRates)) k = 0.0;
  return k;
}

__device__ __forceinline__ double hocl_seasalt(const HetCell& X, bool fine, double frac) {
  double k = 0.0, gamma, branchCl, dummy;
  const double srMw = X.srmw(HS_HOCl);
  if (!X.b(HET_stratBox)) {
    Gam_HOCl_Cld(X, gamma, branchCl, dummy);
    const double branch = branchCl * frac;
    k = k + CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  if (X.b(fine ? HET_SSA_is_Acid : HET_SSC_is_Acid)) {
    const double radi = fine ? X.h(HET_aClRadi) : X.xRadi(SSC);
    gamma = fine ? Gam_HOCl_Aer(X, radi, X.h(HET_H_conc_SSA), X.h(HET_Cl_conc_SSA))
                 : Gam_HOCl_Aer(X, radi, X.h(HET_H_conc_SSC), X.h(HET_Cl_conc_SSC));
    const double area = fine ? X.h(HET_clearFr) * X.h(HET_aClArea) * X.h(HET_f_Acid_SSA)
                             : X.h(HET_clearFr) * X.xArea(SSC) * X.h(HET_f_Acid_SSC);
    k = k + Ars_L1k(X, area, radi, gamma, srMw);
  }
  return k;
}

__device__ __forceinline__ double HOClUptkBySALACL(const HetCell& X) {
  return kIIR1Ltd(X.c(HS_HOCl), X.c(HS_SALACL), hocl_seasalt(X, true, X.h(HET_frac_Cl_CldA)));
}
__device__ __forceinline__ double HOClUptkBySALCCL(const HetCell& X) {
  return kIIR1Ltd(X.c(HS_HOCl), X.c(HS_SALCCL), hocl_seasalt(X, false, X.h(HET_frac_Cl_CldC)));
}

__device__ __forceinline__ double hocl_sulfite(const HetCell& X, double frac, double ratio) {
  double k = 0.0, gamma, dummy, branchSO3;
  if (!X.b(HET_stratBox)) {
    Gam_HOCl_Cld(X, gamma, dummy, branchSO3);
    const double branch = branchSO3 * frac;
    k = k + CloudHet(X, X.srmw(HS_HOCl), gamma, 0.0, branch, 0.0);
  }
  return kIIR1Ltd(X.c(HS_HOCl), X.c(HS_SO2), k) * ratio;
}
__device__ __forceinline__ double HOClUptkByHSO3m(const HetCell& X) {
  return hocl_sulfite(X, X.h(HET_frac_HSO3_aq), X.h(HET_HSO3m));
}
__device__ __forceinline__ double HOClUptkBySO3mm(const HetCell& X) {
  return hocl_sulfite(X, X.h(HET_frac_SO3_aq), X.h(HET_SO3mm));
}

// ---- iodine (fullchem_RateLawFuncs.F90:2371-2541) -------------------------
__device__ __forceinline__ double IuptkBySulf1stOrd(const HetCell& X, double srMw, double gamma) {
  double k = Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gamma, srMw);
  return k + Ars_L1k(X, X.xArea(SLA), X.xRadi(SLA), gamma, srMw);
}
__device__ __forceinline__ double IuptkBySALA1stOrd(const HetCell& X, double srMw, double gamma) {
  if (X.b(HET_stratBox)) return 0.0;
  return Ars_L1k(X, X.xArea(SSA), X.xRadi(SSA), gamma, srMw);
}
__device__ __forceinline__ double IuptkByAlkSALA1stOrd(const HetCell& X, double srMw, double gamma) {
  if (X.b(HET_stratBox) || !X.b(HET_SSA_is_Alk)) return 0.0;
  const double ssarea = X.h(HET_f_Alk_SSA) * X.xArea(SSA);
  return Ars_L1k(X, ssarea, X.xRadi(SSA), gamma, srMw);
}
__device__ __forceinline__ double IuptkBySALC1stOrd(const HetCell& X, double srMw, double gamma) {
  if (X.b(HET_stratBox)) return 0.0;
  return Ars_L1k(X, X.xArea(SSC), X.xRadi(SSC), gamma, srMw);
}
__device__ __forceinline__ double IuptkByAlkSALC1stOrd(const HetCell& X, double srMw, double gamma) {
  if (X.b(HET_stratBox) || !X.b(HET_SSC_is_Alk)) return 0.0;
  const double ssarea = X.h(HET_f_Alk_SSC) * X.xArea(SSC);
  return Ars_L1k(X, ssarea, X.xRadi(SSC), gamma, srMw);
}
// acid-catalysed breakdown on sea salt: share of the uptake (0.15 Br, 0.85 Cl)
__device__ __forceinline__ double ibrkdn(const HetCell& X, double srMw, double conc, double gamma, bool fine,
                                         double share, int educt) {
  if (X.b(HET_stratBox) || !X.b(fine ? HET_SSA_is_Acid : HET_SSC_is_Acid)) return 0.0;
  const int t = fine ? SSA : SSC;
  const double ssarea = X.h(fine ? HET_f_Acid_SSA : HET_f_Acid_SSC) * X.xArea(t);
  const double k = share * Ars_L1k(X, ssarea, X.xRadi(t), gamma, srMw);
  return kIIR1Ltd(conc, X.c(educt), k);
}

// ---- IONO2, N2O5 (fullchem_RateLawFuncs.F90:2544-2897) --------------------
__device__ __forceinline__ double IONO2uptkByH2O(const HetCell& X) {
  double k = 0.0;
  const double srMw = X.srmw(HS_IONO2);
  const double clr = X.h(HET_clearFr);
  double area = clr * X.xArea(SUL);
  double gamma = fmax((0.0021 * X.TEMP - 0.561), 0.0);
  k = k + Ars_L1k(X, area, X.xRadi(SUL), gamma, srMw);
  k = k + X.xArea(SLA) * X.kheti(BrNO3_plus_H2O);
  area = clr * X.xArea(IIC);
  gamma = 0.3;
  if (X.b(HET_natSurface)) gamma = 0.001;
  k = k + Ars_L1k(X, area, X.xRadi(IIC), gamma, srMw);
  k = k + CloudHet(X, srMw, 0.01, 0.01, 1.0, 1.0);
  return kIIR1Ltd(X.c(HS_IONO2), X.c(HS_H2O), k);
}

__device__ __forceinline__ double ClNO2_BT(double Cl, double H2O) {
  const double k2k3 = 1.0 / 4.5e+2;
  if (H2O < 0.1) return Cl > 1e-3 ? 1.0 : 0.0;
  return 1.0 / (1.0 + k2k3 * SafeDiv(H2O, Cl, 1.0e+30));
}

struct N2O5Uptake {
  double gamma, Y_ClNO2, Rp, SA;
};

__device__ __forceinline__ N2O5Uptake N2O5_InorgOrg(const HetCell& X, double volInorg, double volOrg,
                                                     double H2Oinorg, double H2Oorg, double Rcore, double NIT,
                                                     double Cl) {
  const double KH = 5.1e+1, k3k2b = 4.0e-2, beta = 1.15e+6, delta = 1.3e-1, Haq = 5e+3, Daq = 1e-9;
  const double ONE_THIRD = 1.0 / 3.0;
  N2O5Uptake u;
  const double volTotal = volInorg + volOrg;
  const double H2Ototal = H2Oinorg + H2Oorg;
  const double volRatioDry = SafeDiv(fmax(volInorg - H2Oinorg, 0.0), fmax(volTotal - H2Ototal, 0.0), 0.0);
  const double Rp = SafeDiv(Rcore, pow(volRatioDry, ONE_THIRD), Rcore);
  const double l = Rp - Rcore;
  const double M_N2O5 = X.mw(HS_N2O5) * 1.0e-3;
  double speed = sqrt(X.EIGHT_RSTARG_T / (X.h(HET_PI) * M_N2O5));
  const double avo = X.h(HET_AVO);
  const double M_H2O = H2Ototal / 18e+0 / volTotal * 1000.0;
  const double M_NIT = NIT / volTotal / avo * 1000.0;
  const double M_Cl = Cl / volTotal / avo * 1000.0;
  const double OCratio = (((X.h(HET_OMOC_POA) + X.h(HET_OMOC_OPOA)) / 2.0) - 1.17) / 1.29;
  const double eps = 1.5e-1 * OCratio + 1.6e-3 * X.RELHUM;
  double gamma_coat;
  if (l <= 0.0e+0)
    gamma_coat = 0.0;
  else
    gamma_coat = (X.FOUR_RGASLATM_T * 1.0e-3 * eps * Haq * Daq * Rcore / 100.0) / (speed * l / 100.0 * Rp / 100.0);
  const double areaTotal = 3.0 * volTotal / Rp;
  double gamma_core;
  if (M_H2O < 0.1) {
    gamma_core = 0.005;
  } else {
    speed = speed * 1e+2;
    double A = ((4.0 * volTotal) / (speed * areaTotal)) * KH;
    A = fmin(A, 3.2e-8);
    double k2f;
    if (delta * M_H2O < 1e-2)
      k2f = beta * (delta * M_H2O);
    else
      k2f = beta * (1e+0 - exp(-delta * M_H2O));
    gamma_core = A * k2f * (1.0 - 1.0 / (1.0 + SafeDiv(k3k2b * M_H2O, M_NIT, 1.0e+30)));
  }
  if (gamma_coat <= 0.0)
    u.gamma = gamma_core;
  else if (gamma_core <= 0.0)
    u.gamma = 0.0;
  else
    u.gamma = 1.0 / ((1.0 / gamma_core) + (1.0 / gamma_coat));
  u.Y_ClNO2 = ClNO2_BT(M_Cl, M_H2O);
  u.Rp = Rp;
  u.SA = areaTotal;
  return u;
}

__device__ __forceinline__ N2O5Uptake n2o5_fine(const HetCell& X) {
  return N2O5_InorgOrg(X, X.h(HET_aClVol), X.xVol(ORC), X.xH2O(SUL), X.xH2O(ORC), X.h(HET_aClRadi), X.c(HS_NIT),
                       X.c(HS_SALACL));
}
__device__ __forceinline__ N2O5Uptake n2o5_coarse(const HetCell& X) {
  return N2O5_InorgOrg(X, X.xVol(SSC), 0.0, X.xH2O(SSC), 0.0, X.xRadi(SSC), X.c(HS_NITs), X.c(HS_SALCCL));
}

__device__ __forceinline__ double N2O5uptkByH2O(const HetCell& X) {
  double k = 0.0, ktmp;
  const double srMw = X.srmw(HS_N2O5);
  const double clr = X.h(HET_clearFr);
  double gamma = 0.02;
  for (int t = DU1; t <= DU1 + 6; ++t) k = k + Ars_L1k(X, clr * X.xArea(t), X.xRadi(t), gamma, srMw);
  N2O5Uptake u = n2o5_fine(X);
  ktmp = Ars_L1k(X, clr * u.SA, u.Rp, u.gamma, srMw);
  k = k + ktmp - (ktmp * u.Y_ClNO2 * 0.25);
  gamma = 0.005;
  k = k + Ars_L1k(X, clr * X.xArea(BKC), X.xRadi(BKC), gamma, srMw);
  u = n2o5_coarse(X);
  ktmp = Ars_L1k(X, clr * u.SA, u.Rp, u.gamma, srMw);
  k = k + ktmp - (ktmp * u.Y_ClNO2);
  k = k + X.xArea(SLA) * X.kheti(N2O5_plus_H2O);
  gamma = 0.02;
  if (X.b(HET_natSurface)) gamma = 4.0e-4;
  k = k + Ars_L1k(X, clr * X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
  return kIIR1Ltd(X.c(HS_N2O5), X.c(HS_H2O), k);
}

__device__ __forceinline__ double N2O5uptkBySALACl(const HetCell& X) {
  if (X.b(HET_stratBox)) return 0.0;
  const N2O5Uptake u = n2o5_fine(X);
  double k = Ars_L1k(X, X.h(HET_clearFr) * u.SA, u.Rp, u.gamma, X.srmw(HS_N2O5));
  k = k * u.Y_ClNO2 * 0.25;
  return kIIR1Ltd(X.c(HS_N2O5), X.c(HS_SALACL), k);
}

__device__ __forceinline__ double N2O5uptkBySALCCl(const HetCell& X) {
  if (X.b(HET_stratBox)) return 0.0;
  const N2O5Uptake u = n2o5_coarse(X);
  double k = Ars_L1k(X, X.h(HET_clearFr) * u.SA, u.Rp, u.gamma, X.srmw(HS_N2O5));
  k = k * u.Y_ClNO2;
  return kIIR1Ltd(X.c(HS_N2O5), X.c(HS_SALCCL), k);
}

__device__ __forceinline__ double N2O5uptkByCloud(const HetCell& X) {
  const double cst = 0.03 / 0.019;
  const double gamma = cst * exp(-25.5265 + 9283.76 / X.TEMP - 851801.0 / (X.TEMP * X.TEMP));
  return CloudHet(X, X.srmw(HS_N2O5), gamma, 0.02, 1.0, 1.0);
}

__device__ __forceinline__ double N2O5uptkByStratHCl(const HetCell& X) {
  double k = 0.0;
  if (X.b(HET_stratBox)) {
    k = k + (X.xArea(SLA) * X.kheti(N2O5_plus_HCl));
    double gamma = 0.03;
    if (X.b(HET_natSurface)) gamma = 0.003;
    k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gamma, X.srmw(HS_N2O5));
  }
  return kIIR1Ltd(X.c(HS_N2O5), X.c(HS_HCl), k);
}

// ---- NO2, NO3 (fullchem_RateLawFuncs.F90:2928-3104) -----------------------
__device__ __forceinline__ double NO2uptk1stOrdAndCloud(const HetCell& X) {
  double k = 0.0;
  const double srMw = X.srmw(HS_NO2);
  double gamma = 1.0e-8;
  for (int t = DU1; t <= DU1 + 6; ++t) k = k + Ars_L1k(X, X.xArea(t), X.xRadi(t), gamma, srMw);
  gamma = 5e-6;
  k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gamma, srMw);
  gamma = 1e-4;
  k = k + Ars_L1k(X, X.xArea(BKC), X.xRadi(BKC), gamma, srMw);
  gamma = 1e-6;
  k = k + Ars_L1k(X, X.xArea(ORC), X.xRadi(ORC), gamma, srMw);
  if (X.RELHUM < 40.0)
    gamma = 1.0e-8;
  else if (X.RELHUM > 70.0)
    gamma = 1.0e-4;
  else
    gamma = 1.0e-8 + (1e-4 - 1e-8) * (X.RELHUM - 40.0) / 30.0;
  k = k + Ars_L1k(X, X.xArea(SSA), X.xRadi(SSA), gamma, srMw);
  k = k + Ars_L1k(X, X.xArea(SSC), X.xRadi(SSC), gamma, srMw);
  gamma = 1.0e-4;
  k = k + Ars_L1k(X, X.xArea(SLA), X.xRadi(SLA), gamma, srMw);
  k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
  k = k + CloudHet(X, X.srmw(HS_NO2), 1.0e-8, 0.0, 1.0, 0.0);
  return k;
}

__device__ __forceinline__ double Gam_NO3(const HetCell& X, double aArea, double aRadi, double aWater, double C_X) {
  const double INV_AB = 1.0 / 1.3e-2;
  const double Vol = aArea * aRadi * 1.0e-3 / 3.0;
  const double WaterC = aWater / 18.0e+12 / Vol;
  const double M_X = X.mw(HS_NO3) * 1.0e-3;
  const double cavg = sqrt(X.EIGHT_RSTARG_T / (X.h(HET_PI) * M_X)) * 1.0e2;
  const double k_tot = (2.76e+6 * C_X) + (23.0 * WaterC);
  double gamma = 0.0;
  if (k_tot > 0.0) {
    const double H_X = 0.6 * CON_ATM_BAR;
    const double l_r = sqrt(1.0e-5 / k_tot);
    double gb = X.FOUR_R_T * H_X * l_r * k_tot / cavg;
    const double corr = ReactoDiff_Corr(aRadi, l_r);
    gb = gb * corr;
    gamma = 1.0 / (INV_AB + 1.0 / gb);
  }
  return gamma;
}

__device__ __forceinline__ double NO3uptk1stOrdAndCloud(const HetCell& X) {
  double k = 0.0;
  const double srMw = X.srmw(HS_NO3);
  double gamma = 0.01;
  for (int t = DU1; t <= DU1 + 6; ++t) k = k + Ars_L1k(X, X.xArea(t), X.xRadi(t), gamma, srMw);
  gamma = X.RELHUM < 50.0 ? 2.0e-4 : 1.0e-3;
  k = k + Ars_L1k(X, X.xArea(BKC), X.xRadi(BKC), gamma, srMw);
  gamma = 0.005;
  k = k + Ars_L1k(X, X.xArea(ORC), X.xRadi(ORC), gamma, srMw);
  gamma = 0.1;
  k = k + Ars_L1k(X, X.xArea(SLA), X.xRadi(SLA), gamma, srMw);
  k = k + Ars_L1k(X, X.xArea(IIC), X.xRadi(IIC), gamma, srMw);
  k = k + CloudHet(X, X.srmw(HS_NO3), 0.002, 0.001, 1.0, 1.0);
  return k;
}

__device__ __forceinline__ double no3_hydrolysis(const HetCell& X, bool fine) {
  const double area = fine ? X.h(HET_aClArea) : X.xArea(SSC);
  const double radi = fine ? X.h(HET_aClRadi) : X.xRadi(SSC);
  const double water = X.h(HET_aWater + (fine ? 0 : 1));
  const double conc = X.h(fine ? HET_Cl_conc_SSA : HET_Cl_conc_SSC);
  const double gamma = Gam_NO3(X, area, radi, water, conc) * 0.01;
  return Ars_L1k(X, X.h(HET_clearFr) * area, radi, gamma, X.srmw(HS_NO3));
}

// ---- O3 + Br- (fullchem_RateLawFuncs.F90:3106-3240) -----------------------
__device__ __forceinline__ double Gamma_O3_Br(const HetCell& X, double Radius, double C_Br) {
  const double K0_O3 = 1.1e-2 * CON_ATM_BAR;
  if (!(C_Br > 0.0)) return 0.0;
  const double H_X = K0_O3 * exp(2300.0 * (X.INV_TEMP - INV_T298));
  const double cavg = het_cavg(X, HS_O3);
  const double Nmax = 3.0e+14, KLangC = 1.0e-13, k_s = 1.0e-16;
  const double C_Br_surf = fmin(3.41e+14 * C_Br, Nmax);
  const double gs = (4.0 * k_s * C_Br_surf * KLangC * Nmax) / (cavg * (1.0 + KLangC * X.c(HS_O3)));
  const double k_b = 6.3e+8 * exp(-4.45e+3 / X.TEMP);
  const double D_l = 8.9e-6;
  const double l_r = sqrt(D_l / (k_b * C_Br));
  double gb = X.FOUR_R_T * H_X * l_r * k_b * C_Br / cavg;
  gb = gb * ReactoDiff_Corr(Radius, l_r);
  return gb + gs;
}

__device__ __forceinline__ double O3uptkByBrInTropCloud(const HetCell& X, double Br_branch) {
  if (X.b(HET_stratBox)) return 0.0;
  const double gamma = Gamma_O3_Br(X, X.h(HET_rLiq), X.h(HET_Br_conc_Cld));
  return CloudHet(X, X.srmw(HS_O3), gamma, 0.0, Br_branch, 0.0);
}

__device__ __forceinline__ double O3uptkByHBr(const HetCell& X) {
  const double k = O3uptkByBrInTropCloud(X, X.h(HET_frac_Br_CldG));
  return kIIR1Ltd(X.c(HS_O3), X.c(HS_HBr), k);
}

__device__ __forceinline__ double o3_seasalt(const HetCell& X, bool fine) {
  if (X.b(HET_stratBox)) return 0.0;
  double k = 0.0;
  k = k + O3uptkByBrInTropCloud(X, X.h(fine ? HET_frac_Br_CldA : HET_frac_Br_CldC));
  if (X.b(fine ? HET_SSA_is_Acid : HET_SSC_is_Acid)) {
    const double radi = fine ? X.h(HET_aClRadi) : X.xRadi(SSC);
    const double area = fine ? X.h(HET_clearFr) * X.h(HET_aClArea) * X.h(HET_f_Acid_SSA)
                             : X.h(HET_clearFr) * X.xArea(SSC) * X.h(HET_f_Acid_SSC);
    const double gamma = Gamma_O3_Br(X, radi, X.h(fine ? HET_Br_conc_SSA : HET_Br_conc_SSC));
    k = k + Ars_L1k(X, area, radi, gamma, X.srmw(HS_O3));
  }
  return kIIR1Ltd(X.c(HS_O3), X.c(fine ? HS_BrSALA : HS_BrSALC), k);
}

// ---- OH, organics (fullchem_RateLawFuncs.F90:3244-3458) -------------------
__device__ __forceinline__ double oh_seasalt(const HetCell& X, bool fine) {
  if (X.b(HET_stratBox)) return 0.0;
  const double gamma = 0.04 * X.h(fine ? HET_Cl_conc_SSA : HET_Cl_conc_SSC);
  const double k = fine ? Ars_L1k(X, X.h(HET_aClArea), X.h(HET_aClRadi), gamma, X.srmw(HS_OH))
                        : Ars_L1k(X, X.xArea(SSC), X.xRadi(SSC), gamma, X.srmw(HS_OH));
  return kIIR1Ltd(X.c(HS_OH), X.c(fine ? HS_SALACL : HS_SALCCL), k);
}

__device__ __forceinline__ double GLYXuptk1stOrd(const HetCell& X, double srMw) {
  double k = 0.0;
  if (X.RELHUM >= CRITRH) {
    const double gamma = X.SUNCOS > 0.0 ? 4.4e-3 : 8.0e-6;
    k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gamma, srMw);
  }
  return k;
}

__device__ __forceinline__ double EpoxUptkGamma(const HetCell& X, double srMw) {
  const double DIFF_N2O5_STD = 1.0e-1, MACOEFF = 1.0e-1, K_HPLUS = 3.6e-2, K_NUC = 2.0e-4, K_HSO4 = 7.3e-4,
               K_HYDRO = 0.0e+0, HSTAR_EPOX = 1.7e+7;
  double valTmp = 0.0;
  const double areaS = X.xArea(SUL), radiS = X.xRadi(SUL);
  const double aerVol = (areaS * radiS) / 3.0;
  const double xmms = sqrt((2.117e+8 * X.TEMP) / (srMw * srMw));
  const double hp = X.h(HET_H_plus);
  const double kPart = (K_HPLUS * hp) + (K_NUC * hp * (X.h(HET_NO3_molal) + X.h(HET_SO4_molal))) +
                       (K_HSO4 * X.h(HET_HSO4_molal)) + (K_HYDRO);
  const double val1 = (radiS * xmms) / (4.0 * DIFF_N2O5_STD);
  const double val2 = (1.0 / MACOEFF);
  if (areaS > 0.0 && xmms > 0.0) valTmp = (X.FOUR_RGASLATM_T * aerVol * HSTAR_EPOX * kPart) / (areaS * xmms);
  double val3 = 0.0;
  if (valTmp > 0.0) val3 = 1.0 / valTmp;
  double gamma = 0.0;
  if (kPart >= 1.e-8) gamma = 1.0 / (val1 + val2 + val3);
  if (gamma < 0.0) gamma = 0.0;
  return gamma;
}

__device__ __forceinline__ double IEPOXuptk1stOrd(const HetCell& X, double srMw, bool doScale) {
  double k = 0.0;
  if (X.RELHUM >= CRITRH) {
    double gamma = EpoxUptkGamma(X, srMw);
    if (doScale && (X.h(HET_H_plus) > 8.0e-5)) gamma = gamma / 30.0;
    k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), gamma, srMw);
  }
  return k;
}

__device__ __forceinline__ double MGLYuptk1stOrd(const HetCell& X, double srMw) {
  double k = 0.0;
  if (X.RELHUM >= CRITRH) k = k + Ars_L1k(X, X.xArea(SUL), X.xRadi(SUL), 3.6e-7, srMw);
  return k;
}

__device__ __forceinline__ double VOCuptk1stOrd(const HetCell& X, double srMw, double gamma) {
  double k = 0.0;
  if (X.RELHUM >= CRITRH) {
    const int types[7] = {SUL, BKC, ORC, SSA, SSC, SLA, IIC};
    for (int i = 0; i < 7; ++i) k = k + Ars_L1k(X, X.xArea(types[i]), X.xRadi(types[i]), gamma, srMw);
  }
  return k;
}

// Heterogeneous rate law `id` (gcchem.rates_program HET_LAWS order) with its
// numeric arguments a[] (the HetState argument H is implicit).
static __device__ __noinline__ double het_law(int id, const double* a, const HetCell& X) {
  switch (id) {
    case 0: return BrNO3uptkByH2O(X);  // BrNO3uptkByH2O
    case 1: return BrNO3uptkByHCl(X);  // BrNO3uptkByHCl
    case 2: return ClNO2uptkByBrSALA(X);  // ClNO2uptkByBrSALA
    case 3: return ClNO2uptkByBrSALC(X);  // ClNO2uptkByBrSALC
    case 4: return ClNO2uptkByHBr(X);  // ClNO2uptkByHBr
    case 5: return ClNO2uptkBySALACL(X);  // ClNO2uptkBySALACL
    case 6: return ClNO2uptkBySALCCL(X);  // ClNO2uptkBySALCCL
    case 7: return ClNO2uptkByHCl(X);  // ClNO2uptkByHCl
    case 8: return ClNO3uptkByH2O(X);  // ClNO3uptkByH2O
    case 9: return ClNO3uptkByHCl(X);  // ClNO3uptkByHCl
    case 10: return ClNO3uptkByHBr(X);  // ClNO3uptkByHBr
    case 11: return ClNO3uptkByBrSALA(X);  // ClNO3uptkByBrSALA
    case 12: return ClNO3uptkByBrSALC(X);  // ClNO3uptkByBrSALC
    case 13: return ClNO3uptkBySALACL(X);  // ClNO3uptkBySALACL
    case 14: return ClNO3uptkBySALCCL(X);  // ClNO3uptkBySALCCL
    case 15: return HBrUptkBySALA(X);  // HBrUptkBySALA
    case 16: return HBrUptkBySALC(X);  // HBrUptkBySALC
    case 17: return HO2uptk1stOrd(X);  // HO2uptk1stOrd
    case 18: return HOBrUptkByHBr(X);  // HOBrUptkByHBr
    case 19: return HOBrUptkByHCl(X);  // HOBrUptkByHCl
    case 20: return HOBrUptkByBrSALA(X);  // HOBrUptkByBrSALA
    case 21: return HOBrUptkByBrSALC(X);  // HOBrUptkByBrSALC
    case 22: return HOBrUptkBySALACL(X);  // HOBrUptkBySALACL
    case 23: return HOBrUptkBySALCCL(X);  // HOBrUptkBySALCCL
    case 24: return HOBrUptkByHSO3m(X);  // HOBrUptkByHSO3m
    case 25: return HOBrUptkBySO3mm(X);  // HOBrUptkBySO3mm
    case 26: return HOClUptkByHCl(X);  // HOClUptkByHCl
    case 27: return HOClUptkByHBr(X);  // HOClUptkByHBr
    case 28: return HOClUptkBySALACL(X);  // HOClUptkBySALACL
    case 29: return HOClUptkBySALCCL(X);  // HOClUptkBySALCCL
    case 30: return HOClUptkByHSO3m(X);  // HOClUptkByHSO3m
    case 31: return HOClUptkBySO3mm(X);  // HOClUptkBySO3mm
    case 32: return IuptkBySulf1stOrd(X, a[0], a[1]);  // IuptkBySulf1stOrd
    case 33: return IuptkBySALA1stOrd(X, a[0], a[1]);  // IuptkBySALA1stOrd
    case 34: return IuptkByAlkSALA1stOrd(X, a[0], a[1]);  // IuptkByAlkSALA1stOrd
    case 35: return IuptkBySALC1stOrd(X, a[0], a[1]);  // IuptkBySALC1stOrd
    case 36: return IuptkByAlkSALC1stOrd(X, a[0], a[1]);  // IuptkByAlkSALC1stOrd
    case 37: return ibrkdn(X, a[0], a[1], a[2], true, 0.15, HS_BrSALA);  // IbrkdnByAcidBrSALA
    case 38: return ibrkdn(X, a[0], a[1], a[2], false, 0.15, HS_BrSALC);  // IbrkdnByAcidBrSALC
    case 39: return ibrkdn(X, a[0], a[1], a[2], true, 0.85, HS_SALACL);  // IbrkdnByAcidSALACl
    case 40: return ibrkdn(X, a[0], a[1], a[2], false, 0.85, HS_SALCCL);  // IbrkdnByAcidSALCCl
    case 41: return IONO2uptkByH2O(X);  // IONO2uptkByH2O
    case 42: return N2O5uptkByH2O(X);  // N2O5uptkByH2O
    case 43: return N2O5uptkBySALACl(X);  // N2O5uptkBySALACl
    case 44: return N2O5uptkBySALCCl(X);  // N2O5uptkBySALCCl
    case 45: return N2O5uptkByCloud(X);  // N2O5uptkByCloud
    case 46: return N2O5uptkByStratHCl(X);  // N2O5uptkByStratHCl
    case 47: return NO2uptk1stOrdAndCloud(X);  // NO2uptk1stOrdAndCloud
    case 48: return NO3uptk1stOrdAndCloud(X);  // NO3uptk1stOrdAndCloud
    case 49: return no3_hydrolysis(X, true);  // NO3hypsisClonSALA
    case 50: return no3_hydrolysis(X, false);  // NO3hypsisClonSALC
    case 51: return O3uptkByHBr(X);  // O3uptkByHBr
    case 52: return o3_seasalt(X, true);  // O3uptkByBrSALA
    case 53: return o3_seasalt(X, false);  // O3uptkByBrSALC
    case 54: return oh_seasalt(X, true);  // OHuptkBySALACl
    case 55: return oh_seasalt(X, false);  // OHuptkBySALCCl
    case 56: return GLYXuptk1stOrd(X, a[0]);  // GLYXuptk1stOrd
    case 57: return IEPOXuptk1stOrd(X, a[0], a[1] != 0.0);  // IEPOXuptk1stOrd
    case 58: return MGLYuptk1stOrd(X, a[0]);  // MGLYuptk1stOrd
    case 59: return VOCuptk1stOrd(X, a[0], a[1]);  // VOCuptk1stOrd
    default: return __longlong_as_double(0x7ff8000000000000LL);
  }
}
}  // namespace gcrates
