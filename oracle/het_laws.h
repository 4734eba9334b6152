/* Heterogeneous rate laws of the fullchem Update_RCONST, restated in C for
 * the CPU oracle -- TEST INFRASTRUCTURE (checks the GPU rate kernel).
 *
 * Sources (GEOS-Chem tree), one C function per Fortran routine, statement by
 * statement:
 *   SafeDiv, Is_SafeDiv, Ars_L1k, kIIR1Ltd, CloudHet, coth, ReactoDiff_Corr
 *                         KPP/fullchem/rateLawUtilFuncs.F90:77-522
 *   het rate functions    KPP/fullchem/fullchem_RateLawFuncs.F90:795-3460
 *   TEMP terms, RELHUM    GeosCore/fullchem_mod.F90:2147-2165
 *
 * The HetState is a struct (het_state_t) filled from the row array of the
 * batch interface (oracle_het_layout.h, written by gen_oracle.py from the
 * HetState field list).  The generated kpp_rates_oracle.c defines the
 * species indices OHS_* (-1 when absent) and the MW/SR_MW/HENRY arrays of the
 * species database before including this file.
 */
#ifndef ORACLE_HET_LAWS_H
#define ORACLE_HET_LAWS_H
#include <math.h>
#include <stdbool.h>

#include "oracle_het_layout.h"
#include "rate_laws.h"

typedef struct {
  double AVO, PI, aClArea, aClRadi, aClVol, aIce, aLiq, aWater[3];
  bool natSurface, stratBox, SSA_is_Alk, SSA_is_Acid, SSC_is_Alk, SSC_is_Acid, TurnOffHetRates;
  double Br_conc_Cld, Br_conc_SSA, Br_conc_SSC, Br_over_Cl_Cld, Br_over_Cl_SSA, Br_over_Cl_SSC;
  double Cl_conc_Cld, Cl_conc_SSA, Cl_conc_SSC, CldFr, ClearFr;
  double frac_Br_CldA, frac_Br_CldC, frac_Br_CldG, frac_Cl_CldA, frac_Cl_CldC, frac_Cl_CldG;
  double frac_HSO3_aq, frac_SALACL, frac_SO3_aq, gamma_HO2, HBr_theta, HCl_theta;
  double H_conc_LCl, H_conc_SSA, H_conc_SSC, HNO3_theta, HSO3_aq, SO3_aq, HSO3m, SO3mm, TSO3_aq, H_PLUS;
  double KHETI_SLA[12], HSO4_molal, NO3_molal, SO4_molal, pHCloud, pHSSA[3], OMOC_POA, OMOC_OPOA;
  double rIce, rLiq, f_Acid_SSA, f_Acid_SSC, f_Alk_SSA, f_Alk_SSC;
  double xArea[15], xRadi[15], xVol[15], xH2O[15]; /* 1-based as in Fortran */
} het_state_t;

typedef struct {
  het_state_t H;
  const double* C;  /* the cell's concentrations C(1:NSPEC), 0-based */
  double TEMP, NUMDEN, INV_TEMP, SR_TEMP, FOUR_R_T, FOUR_RGASLATM_T, EIGHT_RSTARG_T, RELHUM, SUNCOS;
} het_cell_t;

enum { O_DU1 = 1, O_DU2, O_DU3, O_DU4, O_DU5, O_DU6, O_DU7, O_SUL, O_BKC, O_ORC, O_SSA, O_SSC, O_SLA, O_IIC };
enum {
  O_N2O5_plus_H2O = 1, O_N2O5_plus_HCl, O_ClNO3_plus_H2O, O_ClNO3_plus_HCl, O_ClNO3_plus_HBr, O_BrNO3_plus_H2O,
  O_BrNO3_plus_HCl, O_HOCl_plus_HCl, O_HOCl_plus_HBr, O_HOBr_plus_HCl, O_HOBr_plus_HBr
};
#define O_CON_R 0.083144598
#define O_RSTARG 8.3144598
#define O_RGASLATM 8.2057e-2
#define O_BOLTZ 1.38064852e-23
#define O_CRITRH 35.0
#define O_CON_ATM_BAR (1.0 / 1.01325)
#define O_INV_T298 (1.0 / 298.15)
#define O_HET_MIN_LIFE 1.e-3
#define O_HET_MIN_RATE (1.0 / O_HET_MIN_LIFE)

static inline double oC(const het_cell_t* X, int ind) { return ind >= 0 ? X->C[ind] : 0.0; }

/* row array -> struct (one cell) */
static inline void het_cell_load(het_cell_t* X, const rate_env_t* E, const double* het, long long ldh,
                                 const double* C) {
  het_state_t* H = &X->H;
#define R(f) het[(long long)(f) * ldh]
  H->AVO = R(OHET_AVO);
  H->PI = R(OHET_PI);
  H->natSurface = R(OHET_natSurface) != 0.0;
  H->stratBox = R(OHET_stratBox) != 0.0;
  H->aClArea = R(OHET_aClArea);
  H->aClRadi = R(OHET_aClRadi);
  H->aClVol = R(OHET_aClVol);
  H->aIce = R(OHET_aIce);
  H->aLiq = R(OHET_aLiq);
  H->aWater[1] = R(OHET_aWater);
  H->aWater[2] = R(OHET_aWater + 1);
  H->Br_conc_Cld = R(OHET_Br_conc_Cld);
  H->Br_conc_SSA = R(OHET_Br_conc_SSA);
  H->Br_conc_SSC = R(OHET_Br_conc_SSC);
  H->Br_over_Cl_Cld = R(OHET_Br_over_Cl_Cld);
  H->Br_over_Cl_SSA = R(OHET_Br_over_Cl_SSA);
  H->Br_over_Cl_SSC = R(OHET_Br_over_Cl_SSC);
  H->Cl_conc_Cld = R(OHET_Cl_conc_Cld);
  H->Cl_conc_SSA = R(OHET_Cl_conc_SSA);
  H->Cl_conc_SSC = R(OHET_Cl_conc_SSC);
  H->CldFr = R(OHET_cldFr);
  H->ClearFr = R(OHET_clearFr);
  H->frac_Br_CldA = R(OHET_frac_Br_CldA);
  H->frac_Br_CldC = R(OHET_frac_Br_CldC);
  H->frac_Br_CldG = R(OHET_frac_Br_CldG);
  H->frac_Cl_CldA = R(OHET_frac_Cl_CldA);
  H->frac_Cl_CldC = R(OHET_frac_Cl_CldC);
  H->frac_Cl_CldG = R(OHET_frac_Cl_CldG);
  H->frac_HSO3_aq = R(OHET_frac_HSO3_aq);
  H->frac_SALACL = R(OHET_frac_SALACL);
  H->frac_SO3_aq = R(OHET_frac_SO3_aq);
  H->gamma_HO2 = R(OHET_gamma_HO2);
  H->HBr_theta = R(OHET_HBr_theta);
  H->HCl_theta = R(OHET_HCl_theta);
  H->H_conc_LCl = R(OHET_H_conc_LCl);
  H->H_conc_SSA = R(OHET_H_conc_SSA);
  H->H_conc_SSC = R(OHET_H_conc_SSC);
  H->HNO3_theta = R(OHET_HNO3_theta);
  H->HSO3_aq = R(OHET_HSO3_aq);
  H->SO3_aq = R(OHET_SO3_aq);
  H->HSO3m = R(OHET_HSO3m);
  H->SO3mm = R(OHET_SO3mm);
  H->TSO3_aq = R(OHET_TSO3_aq);
  H->H_PLUS = R(OHET_H_plus);
  for (int i = 1; i <= 11; ++i) H->KHETI_SLA[i] = R(OHET_KHETI_SLA + i - 1);
  H->HSO4_molal = R(OHET_HSO4_molal);
  H->NO3_molal = R(OHET_NO3_molal);
  H->SO4_molal = R(OHET_SO4_molal);
  H->pHCloud = R(OHET_pHCloud);
  H->pHSSA[1] = R(OHET_pHSSA);
  H->pHSSA[2] = R(OHET_pHSSA + 1);
  H->OMOC_POA = R(OHET_OMOC_POA);
  H->OMOC_OPOA = R(OHET_OMOC_OPOA);
  H->rIce = R(OHET_rIce);
  H->rLiq = R(OHET_rLiq);
  H->f_Acid_SSA = R(OHET_f_Acid_SSA);
  H->f_Acid_SSC = R(OHET_f_Acid_SSC);
  H->f_Alk_SSA = R(OHET_f_Alk_SSA);
  H->f_Alk_SSC = R(OHET_f_Alk_SSC);
  H->SSA_is_Alk = R(OHET_SSA_is_Alk) != 0.0;
  H->SSA_is_Acid = R(OHET_SSA_is_Acid) != 0.0;
  H->SSC_is_Alk = R(OHET_SSC_is_Alk) != 0.0;
  H->SSC_is_Acid = R(OHET_SSC_is_Acid) != 0.0;
  H->TurnOffHetRates = R(OHET_TurnOffHetRates) != 0.0;
  for (int t = 1; t <= 14; ++t) {
    H->xArea[t] = R(OHET_xArea + t - 1);
    H->xRadi[t] = R(OHET_xRadi + t - 1);
    H->xVol[t] = R(OHET_xVol + t - 1);
    H->xH2O[t] = R(OHET_xH2O + t - 1);
  }
  X->SUNCOS = R(OHET_SUNCOS);
#undef R
  X->C = C;
  /* Set_Kpp_GridBox_Values (GeosCore/fullchem_mod.F90:2147-2165) */
  X->TEMP = E->TEMP;
  X->NUMDEN = E->NUMDEN;
  X->INV_TEMP = E->INV_TEMP;
  X->SR_TEMP = E->SR_TEMP;
  X->FOUR_R_T = 4.0 * O_CON_R * E->TEMP;
  X->FOUR_RGASLATM_T = 4.0 * O_RGASLATM * E->TEMP;
  X->EIGHT_RSTARG_T = 8.0 * O_RSTARG * E->TEMP;
  {
    const double CONSVAP = 6.1078e+03 / (O_BOLTZ * 1e+7);
    const double CONSEXP = 17.2693882 * (E->TEMP - 273.16) / (E->TEMP - 35.86);
    const double VPRESH2O = CONSVAP * exp(CONSEXP) / E->TEMP;
    X->RELHUM = (E->H2O / VPRESH2O) * 100.0;
  }
}

/* ---- rateLawUtilFuncs.F90 --------------------------------------------- */
static inline int o_exponent(double x) {
  int e = 0;
  if (x != 0.0) frexp(x, &e);
  return e;
}

static inline double o_SafeDiv(double num, double denom, double alt) {
  int ediff = o_exponent(num) - o_exponent(denom);
  if (ediff > 1023 || denom == 0.0) return alt;
  if (ediff < -1020) return 0.0;
  return num / denom;
}

static inline bool o_Is_SafeDiv(double num, double denom) {
  int ediff = o_exponent(num) - o_exponent(denom);
  bool safe = true;
  if (ediff < -1020 || ediff > 1023 || denom == 0.0) safe = false;
  return safe;
}

static inline double o_Ars_L1k(const het_cell_t* X, double area, double radius, double gamma, double srMw) {
  double k, dfkg;
  if (gamma < 1.0e-30 || radius < 1.0e-30) {
    k = 0.0;
    return k;
  }
  dfkg = (9.45E+17 / X->NUMDEN) * X->SR_TEMP * sqrt(3.472E-2 + 1.0 / (srMw * srMw));
  k = area / ((radius / dfkg) + 2.749064E-4 * srMw / (gamma * X->SR_TEMP));
  return k;
}

static inline double o_kIIR1Ltd(double concGas, double concEduct, double kISource) {
  double kIGas = 0.0, kIEduct = 0.0, kII = 0.0, lifeA, lifeB;
  if (concEduct < 1.0) return kII;
  if (!o_Is_SafeDiv(concGas * kISource, concEduct)) return kII;
  kIGas = kISource;
  kIEduct = kIGas * concGas / concEduct;
  kII = kIGas / concEduct;
  if (kIGas > 0.0) {
    lifeA = o_SafeDiv(1.0, kIGas, 0.0);
    lifeB = o_SafeDiv(1.0, kIEduct, 0.0);
    if ((lifeA < lifeB) && (lifeA < O_HET_MIN_LIFE)) {
      kII = o_SafeDiv(O_HET_MIN_RATE, concEduct, 0.0);
    } else if (lifeB < O_HET_MIN_LIFE) {
      kII = o_SafeDiv(O_HET_MIN_RATE, concGas, 0.0);
    }
  }
  return kII;
}

static inline double o_CloudHet(const het_cell_t* X, double srMw, double gamLiq, double gamIce, double brLiq,
                                double brIce) {
  const het_state_t* H = &X->H;
  const double tauc = 3600.0;
  double kI, kIb, ktmp, kHet, area, branch, kk, ff, xx;
  if ((H->CldFr < 0.0001) || (H->aLiq + H->aIce <= 0.0)) return 0.0;
  kI = 0.0;
  kIb = 0.0;
  ktmp = 0.0;
  kHet = 0.0;
  if (brLiq > 0.0) {
    area = o_SafeDiv(H->aLiq, H->CldFr, 0.0);
    if (area > 0.0) {
      ktmp = o_Ars_L1k(X, area, H->rLiq, gamLiq, srMw);
      kI = kI + ktmp;
      kIb = kIb + (ktmp * brLiq);
    }
  }
  if (brIce > 0.0) {
    area = o_SafeDiv(H->aIce, H->CldFr, 0.0);
    if (area > 0.0) {
      ktmp = o_Ars_L1k(X, area, H->rIce, gamIce, srMw);
      kI = kI + ktmp;
      kIb = kIb + (ktmp * brIce);
    }
  }
  branch = o_SafeDiv(kIb, kI, 0.0);
  if (!(branch > 0.0)) return 0.0;
  kk = kI * tauc;
  ff = o_SafeDiv(H->CldFr, H->ClearFr, 1.0e+30);
  ff = fmin(ff, 1.0e+30);
  xx = (ff - kk - 1.0) / 2.0 + sqrt(1.0 + ff * ff + kk * kk + 2.0 * ff + 2.0 * kk - 2.0 * ff * kk) / 2.0;
  xx = fmax(xx, 0.0);
  kHet = kI / (1.0 + o_SafeDiv(1.0, xx, 1.0e+30));
  kHet = kHet * branch;
  return kHet;
}

static inline double o_coth(double x) {
  double y = exp(-2.0 * x);
  return (1.0 + y) / (1.0 - y);
}

static inline double o_ReactoDiff_Corr(double radius, double l) {
  double x = radius / l;
  if (x > 1000.0) return 1.0;
  if (x < 0.1) return x / 3.0;
  return o_coth(x) - (1.0 / x);
}


#define SRMW(s) O_SRMW[OHSI_##s]
#define MWX(s) O_MW[OHSI_##s]
#define CC(s) oC(X, OHS_##s)

/* ---- BrNO3 (fullchem_RateLawFuncs.F90:803-866) ---------------------- */
static double o_BrNO3uptkByH2O(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k, gamma, gamLiq, gamIce, srMw;
  k = 0.0;
  gamLiq = 0.0021 * X->TEMP - 0.561;
  gamIce = 5.3e-4 * exp(1100.0 / X->TEMP);
  srMw = SRMW(BrNO3);
  gamma = gamLiq;
  k = k + o_Ars_L1k(X, H->ClearFr * H->xArea[O_SUL], H->xRadi[O_SUL], gamma, srMw);
  k = k + o_Ars_L1k(X, H->ClearFr * H->xArea[O_SSA], H->xRadi[O_SSA], gamma, srMw);
  k = k + o_Ars_L1k(X, H->ClearFr * H->xArea[O_SSC], H->xRadi[O_SSC], gamma, srMw);
  k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_BrNO3_plus_H2O];
  gamma = 0.3;
  if (H->natSurface) gamma = 0.001;
  k = k + o_Ars_L1k(X, H->ClearFr * H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  k = k + o_CloudHet(X, srMw, gamLiq, gamIce, 1.0, 1.0);
  k = o_kIIR1Ltd(CC(BrNO3), CC(H2O), k);
  return k;
}

static double o_BrNO3uptkByHCl(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, srMw = SRMW(BrNO3);
  if (H->stratBox) {
    k = k + o_Ars_L1k(X, H->xArea[O_SUL], H->xRadi[O_SUL], 0.9, srMw);
    k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_BrNO3_plus_HCl];
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], 0.3, srMw);
  }
  k = o_kIIR1Ltd(CC(BrNO3), CC(HCl), k);
  if (H->TurnOffHetRates) k = 0.0;
  return k;
}

/* ---- ClNO2 (fullchem_RateLawFuncs.F90:872-1108) --------------------- */
static void o_Gam_ClNO2(const het_cell_t* X, double radius, double pH, double C_Cl, double C_Br, double* gamma,
                        double* branchCl, double* branchBr) {
  const double INV_AB = 1.0 / 0.01, D_l = 1.0e-5;
  double cavg, gb_tot, H_X, k_Cl, k_Br, k_tot, l_r, M_X;
  M_X = MWX(ClNO2) * 1.0e-3;
  cavg = sqrt(X->EIGHT_RSTARG_T / (X->H.PI * M_X)) * 100.0;
  H_X = 4.5e-2 * O_CON_ATM_BAR;
  k_Cl = 1.0e+7 * C_Cl;
  if (pH >= 2.0) k_Cl = 0.0;
  k_Br = (1.01e-1 / (H_X * H_X * D_l)) * C_Br;
  k_tot = k_Cl + k_Br;
  *gamma = 0.0;
  *branchCl = 0.0;
  *branchBr = 0.0;
  if (k_tot > 0.0) {
    l_r = sqrt(D_l / k_tot);
    gb_tot = X->FOUR_R_T * H_X * l_r * k_tot / cavg;
    gb_tot = gb_tot * o_ReactoDiff_Corr(radius, l_r);
    *gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
    *branchCl = k_Cl / k_tot;
    *branchBr = k_Br / k_tot;
  }
}

static double o_ClNO2uptkByBrSALA(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, gamma, branch, branchBr, dummy, srMw, k = 0.0;
  srMw = SRMW(ClNO2);
  if (!H->stratBox) {
    o_Gam_ClNO2(X, H->rLiq, H->pHCloud, H->Cl_conc_Cld, H->Br_conc_Cld, &gamma, &dummy, &branchBr);
    branch = branchBr * H->frac_Br_CldA;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  o_Gam_ClNO2(X, H->aClRadi, H->pHSSA[1], H->Cl_conc_SSA, H->Br_conc_SSA, &gamma, &dummy, &branchBr);
  area = H->ClearFr * H->aClArea;
  k = k + o_Ars_L1k(X, area, H->aClRadi, gamma, srMw) * branchBr;
  k = o_kIIR1Ltd(CC(ClNO2), CC(BrSALA), k);
  return k;
}

static double o_ClNO2uptkByBrSALC(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, gamma, branch, branchBr, dummy, srMw, k = 0.0;
  srMw = SRMW(ClNO2);
  if (!H->stratBox) {
    o_Gam_ClNO2(X, H->rLiq, H->pHCloud, H->Cl_conc_Cld, H->Br_conc_Cld, &gamma, &dummy, &branchBr);
    branch = branchBr * H->frac_Br_CldC;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  o_Gam_ClNO2(X, H->xRadi[O_SSC], H->pHSSA[2], H->Cl_conc_SSC, H->Br_conc_SSC, &gamma, &dummy, &branchBr);
  area = H->ClearFr * H->xArea[O_SSC];
  k = k + o_Ars_L1k(X, area, H->xRadi[O_SSC], gamma, srMw) * branchBr;
  k = o_kIIR1Ltd(CC(ClNO2), CC(BrSALC), k);
  return k;
}

static double o_ClNO2uptkByHBr(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double gamma, branch, branchBr, dummy, srMw, k = 0.0;
  srMw = SRMW(ClNO2);
  if (!H->stratBox) {
    o_Gam_ClNO2(X, H->rLiq, H->pHCloud, H->Cl_conc_Cld, H->Br_conc_Cld, &gamma, &dummy, &branchBr);
    branch = branchBr * H->frac_Br_CldG;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  k = o_kIIR1Ltd(CC(ClNO2), CC(HBr), k);
  return k;
}

static double o_ClNO2uptkBySALACL(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, gamma, branch, branchCl, dummy, srMw, k = 0.0;
  srMw = SRMW(ClNO2);
  if (!H->stratBox) {
    o_Gam_ClNO2(X, H->rLiq, H->pHCloud, H->Cl_conc_Cld, H->Br_conc_Cld, &gamma, &branchCl, &dummy);
    branch = branchCl * H->frac_Cl_CldA;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  o_Gam_ClNO2(X, H->aClRadi, H->pHSSA[1], H->Cl_conc_SSA, H->Br_conc_SSA, &gamma, &branchCl, &dummy);
  area = H->ClearFr * H->aClArea;
  k = k + o_Ars_L1k(X, area, H->aClRadi, gamma, srMw) * branchCl;
  k = o_kIIR1Ltd(CC(ClNO2), CC(SALACL), k);
  return k;
}

static double o_ClNO2uptkBySALCCL(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double gamma, branch, branchCl, dummy, srMw, k = 0.0;
  srMw = SRMW(ClNO2);
  if (!H->stratBox) {
    o_Gam_ClNO2(X, H->rLiq, H->pHCloud, H->Cl_conc_Cld, H->Br_conc_Cld, &gamma, &branchCl, &dummy);
    branch = branchCl * H->frac_Cl_CldC;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  k = o_kIIR1Ltd(CC(ClNO2), CC(SALCCL), k);
  return k;
}

static double o_ClNO2uptkByHCl(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double gamma, branch, branchCl, dummy, srMw, k = 0.0;
  srMw = SRMW(ClNO2);
  if (!H->stratBox) {
    o_Gam_ClNO2(X, H->rLiq, H->pHCloud, H->Cl_conc_Cld, H->Br_conc_Cld, &gamma, &branchCl, &dummy);
    branch = branchCl * H->frac_Cl_CldG;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  k = o_kIIR1Ltd(CC(ClNO2), CC(HCl), k);
  return k;
}

/* ---- ClNO3 (fullchem_RateLawFuncs.F90:1114-1420) -------------------- */
static void o_Gam_ClNO3_Aer(const het_cell_t* X, double C_Br, double* gamma, double* branchBr) {
  const double INV_AB = 1.0 / 0.108, K_0 = pow(1.2e+5, 2.0), D_l = 5.0e-6;
  double M_X, cavg, k_Br, k_tot, gb_tot;
  M_X = MWX(ClNO3) * 1.0e-3;
  cavg = sqrt(X->EIGHT_RSTARG_T / (X->H.PI * M_X)) * 100.0;
  k_Br = 1.0e+12 * C_Br;
  k_tot = K_0 + k_Br;
  gb_tot = X->FOUR_R_T * sqrt(k_tot * D_l) / cavg;
  *gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
  *branchBr = k_Br / k_tot;
}

static void o_Gam_ClNO3_Ice(const het_cell_t* X, double* gamma, double* brHCl, double* brHBr, double* brH2O) {
  const double twenty = 1.0 / 0.5;
  double cavg, g1, g2, g3, H2Os, kks, M_X;
  g1 = 0.24 * X->H.HCl_theta;
  g2 = 0.56 * X->H.HBr_theta;
  M_X = MWX(ClNO3) * 1.0e-3;
  cavg = sqrt(X->EIGHT_RSTARG_T / (X->H.PI * M_X)) * 100.0;
  H2Os = 1e+15 - (3.0 * 2.7e+14 * X->H.HNO3_theta);
  kks = 4.0 * 5.2e-17 * exp(2032.0 / X->TEMP);
  g3 = 1.0 / (twenty + cavg / (kks * H2Os));
  *gamma = g1 + g2 + g3;
  *brHCl = g1 / *gamma;
  *brHBr = g2 / *gamma;
  *brH2O = g3 / *gamma;
}

static double o_ClNO3uptkByH2O(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, branchBr, branchLiq, branchIce, dum1, dum2, gamma, gammaIce, srMw, k = 0.0;
  srMw = SRMW(ClNO3);
  o_Gam_ClNO3_Aer(X, H->Br_conc_SSA, &gamma, &branchBr);
  area = H->ClearFr * H->aClArea;
  branchLiq = (1.0 - branchBr) * (1.0 - H->frac_SALACL);
  k = k + o_Ars_L1k(X, area, H->aClRadi, gamma, srMw) * branchLiq;
  k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_ClNO3_plus_H2O];
  gamma = 0.3;
  if (H->natSurface) gamma = 0.004;
  k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  if (!H->stratBox) {
    o_Gam_ClNO3_Aer(X, H->Br_conc_Cld, &gamma, &branchBr);
    branchLiq = 1.0 - branchBr;
    o_Gam_ClNO3_Ice(X, &gammaIce, &dum1, &dum2, &branchIce);
    k = k + o_CloudHet(X, srMw, gamma, gammaIce, branchLiq, branchIce);
  }
  k = o_kIIR1Ltd(CC(ClNO3), CC(H2O), k);
  return k;
}

static double o_ClNO3uptkByHCl(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double branchIce, dum1, dum2, gamma, gammaIce, srMw, k = 0.0;
  srMw = SRMW(ClNO3);
  if (H->stratBox) {
    gamma = 0.1e-4;
    k = k + o_Ars_L1k(X, H->xArea[O_SUL], H->xRadi[O_SUL], gamma, srMw);
    k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_ClNO3_plus_HCl];
    gamma = 0.3;
    if (H->natSurface) gamma = 0.2;
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  } else {
    o_Gam_ClNO3_Ice(X, &gammaIce, &branchIce, &dum1, &dum2);
    k = k + o_CloudHet(X, srMw, 0.0, gammaIce, 0.0, branchIce);
  }
  k = o_kIIR1Ltd(CC(ClNO3), CC(HCl), k);
  return k;
}

static double o_ClNO3uptkByHBr(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double branchBr, branchLiq, branchIce, dum1, dum2, gamma, gammaIce, srMw, k = 0.0;
  srMw = SRMW(ClNO3);
  if (H->stratBox) {
    k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_ClNO3_plus_HBr];
    gamma = 0.3;
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  } else {
    o_Gam_ClNO3_Aer(X, H->Br_conc_Cld, &gamma, &branchBr);
    branchLiq = branchBr * H->frac_Br_CldG;
    o_Gam_ClNO3_Ice(X, &gammaIce, &dum1, &branchIce, &dum2);
    k = o_CloudHet(X, srMw, gamma, gammaIce, branchLiq, branchIce);
  }
  k = o_kIIR1Ltd(CC(ClNO3), CC(HBr), k);
  if (H->TurnOffHetRates) k = 0.0;
  return k;
}

static double o_ClNO3uptkByBrSALA(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, branch, branchBr, gamma, srMw, k = 0.0;
  srMw = SRMW(ClNO3);
  if (!H->stratBox) {
    o_Gam_ClNO3_Aer(X, H->Br_conc_Cld, &gamma, &branchBr);
    branch = branchBr * H->frac_Br_CldA;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  o_Gam_ClNO3_Aer(X, H->Br_conc_SSA, &gamma, &branchBr);
  area = H->ClearFr * H->aClArea;
  k = k + o_Ars_L1k(X, area, H->aClRadi, gamma, srMw) * branchBr;
  k = o_kIIR1Ltd(CC(ClNO3), CC(BrSALA), k);
  if (H->TurnOffHetRates) k = 0.0;
  return k;
}

static double o_ClNO3uptkByBrSALC(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, branch, branchBr, gamma, srMw, k = 0.0;
  srMw = SRMW(ClNO3);
  if (!H->stratBox) {
    o_Gam_ClNO3_Aer(X, H->Br_conc_Cld, &gamma, &branchBr);
    branch = branchBr * H->frac_Br_CldC;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  o_Gam_ClNO3_Aer(X, H->Br_conc_SSC, &gamma, &branchBr);
  area = H->ClearFr * H->xArea[O_SSC];
  k = k + o_Ars_L1k(X, area, H->xRadi[O_SSC], gamma, srMw) * branchBr;
  k = o_kIIR1Ltd(CC(ClNO3), CC(BrSALC), k);
  if (H->TurnOffHetRates) k = 0.0;
  return k;
}

static double o_ClNO3uptkBySALACL(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, branch, branchBr, gamma, srMw, k = 0.0;
  if (H->stratBox) return k;
  o_Gam_ClNO3_Aer(X, H->Br_conc_SSA, &gamma, &branchBr);
  srMw = SRMW(ClNO3);
  area = H->ClearFr * H->aClArea;
  branch = (1.0 - branchBr) * H->frac_SALACL;
  k = k + o_Ars_L1k(X, area, H->aClRadi, gamma, srMw) * branch;
  k = o_kIIR1Ltd(CC(ClNO3), CC(SALACL), k);
  return k;
}

static double o_ClNO3uptkBySALCCL(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, branch, branchBr, gamma, srMw, k = 0.0;
  if (H->stratBox) return k;
  o_Gam_ClNO3_Aer(X, H->Br_conc_SSC, &gamma, &branchBr);
  srMw = SRMW(ClNO3);
  area = H->ClearFr * H->xArea[O_SSC];
  branch = 1.0 - branchBr;
  k = k + o_Ars_L1k(X, area, H->xRadi[O_SSC], gamma, srMw) * branch;
  k = o_kIIR1Ltd(CC(ClNO3), CC(SALCCL), k);
  return k;
}

/* ---- HBr, HO2 (fullchem_RateLawFuncs.F90:1423-1488) ----------------- */
static double o_HBrUptkBySALA(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, gamma, k = 0.0;
  if (H->stratBox) return k;
  area = H->ClearFr * H->aClArea;
  gamma = 1.3e-8 * exp(4290.0 / X->TEMP);
  k = o_Ars_L1k(X, area, H->aClRadi, gamma, SRMW(HBr));
  return k;
}

static double o_HBrUptkBySALC(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double area, gamma, k = 0.0;
  if (H->stratBox) return k;
  area = H->ClearFr * H->xArea[O_SSC];
  gamma = 1.3e-8 * exp(4290.0 / X->TEMP);
  k = o_Ars_L1k(X, area, H->xRadi[O_SSC], gamma, SRMW(HBr));
  return k;
}

static double o_HO2uptk1stOrd(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, srMw = SRMW(HO2);
  const int types[12] = {O_DU1, O_DU2, O_DU3, O_DU4, O_DU5, O_DU6, O_DU7, O_SUL, O_BKC, O_ORC, O_SSA, O_SSC};
  for (int i = 0; i < 12; ++i) k = k + o_Ars_L1k(X, H->xArea[types[i]], H->xRadi[types[i]], H->gamma_HO2, srMw);
  return k;
}

/* ---- HOBr (fullchem_RateLawFuncs.F90:1490-2050) --------------------- */
static double o_Br2_Yield(double Br_over_Cl) {
  double Y_Br2 = 0.0;
  if (Br_over_Cl > 0.0) {
    Y_Br2 = 0.41 * log10(Br_over_Cl) + 2.25;
    Y_Br2 = fmax(fmin(Y_Br2, 0.9), 0.0);
  }
  return Y_Br2;
}

static void o_Gam_HOBr_Aer(const het_cell_t* X, double radius, double C_Hp, double C_Clm, double C_Brm,
                           double* gamma) {
  const double INV_AB = 1.0 / 0.6, D_l = 1.4e-5;
  double H_X, M_X, cavg, C_Hp1, C_Hp2, k_HOBr_Cl, k_HOBr_Br, k_tot, l_r, gb_tot;
  H_X = (O_HK0[OHSI_HOBr] * O_CON_ATM_BAR) * exp(O_HCR[OHSI_HOBr] * (1.0 / X->TEMP - O_INV_T298));
  M_X = MWX(HOBr) * 1.0e-3;
  cavg = sqrt(X->EIGHT_RSTARG_T / (X->H.PI * M_X)) * 100.0;
  C_Hp1 = fmax(fmin(C_Hp, 1.0e-6), 1.0e-9);
  C_Hp2 = fmax(fmin(C_Hp, 1.0e-2), 1.0e-6);
  k_HOBr_Cl = 2.3e+10 * C_Clm * C_Hp1;
  k_HOBr_Br = 1.6e+10 * C_Brm * C_Hp2;
  k_tot = k_HOBr_Cl + k_HOBr_Br;
  *gamma = 0.0;
  if (k_tot > 0.0) {
    l_r = sqrt(D_l / k_tot);
    gb_tot = X->FOUR_R_T * H_X * l_r * k_tot / cavg;
    gb_tot = gb_tot * o_ReactoDiff_Corr(radius, l_r);
    *gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
  }
}

static void o_Gam_HOBr_Cld(const het_cell_t* X, double* gamma, double* k_tot, double* k_HOBr_Cl, double* k_HOBr_Br,
                           double* k_HOBr_HSO3, double* k_HOBr_HSO3_2) {
  const double INV_AB = 1.0 / 0.6, D_l = 1.4e-5;
  const het_state_t* H = &X->H;
  double H_X, M_X, cavg, C_Hp1, C_Hp2, l_r, gb_tot;
  H_X = (O_HK0[OHSI_HOBr] * O_CON_ATM_BAR) * exp(O_HCR[OHSI_HOBr] * (1.0 / X->TEMP - O_INV_T298));
  M_X = MWX(HOBr) * 1.0e-3;
  cavg = sqrt(X->EIGHT_RSTARG_T / (H->PI * M_X)) * 100.0;
  C_Hp1 = fmin(H->H_conc_LCl, 1.0e-6);
  C_Hp2 = fmin(H->H_conc_LCl, 1.0e-2);
  C_Hp1 = fmax(C_Hp1, 1.0e-9);
  C_Hp2 = fmax(C_Hp2, 1.0e-6);
  *k_HOBr_Cl = 2.3e+10 * H->Cl_conc_Cld * C_Hp1;
  *k_HOBr_Br = 1.6e+10 * H->Br_conc_Cld * C_Hp2;
  *k_HOBr_HSO3 = 2.6e+7 * H->HSO3_aq;
  *k_HOBr_HSO3_2 = 5.0e+9 * H->SO3_aq;
  *k_tot = *k_HOBr_Cl + *k_HOBr_Br + *k_HOBr_HSO3 + *k_HOBr_HSO3_2;
  *gamma = 0.0;
  if (*k_tot > 0.0) {
    l_r = sqrt(D_l / *k_tot);
    gb_tot = X->FOUR_R_T * H_X * l_r * *k_tot / cavg;
    gb_tot = gb_tot * o_ReactoDiff_Corr(H->rLiq, l_r);
    *gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
  }
}

static void o_Gam_HOBr_Ice(const het_cell_t* X, double* gamma, double* branch_HCl, double* branch_HBr) {
  double gamma_HCl, gamma_HBr;
  gamma_HCl = X->H.HCl_theta * 0.25;
  gamma_HBr = X->H.HBr_theta * 4.8e-4 * exp(1240.0 / X->TEMP);
  *gamma = gamma_HCl + gamma_HBr;
  *branch_HCl = 0.0;
  *branch_HBr = 0.0;
  if (*gamma > 0.0) {
    *branch_HCl = gamma_HCl / *gamma;
    *branch_HBr = gamma_HBr / *gamma;
  }
}

static double o_HOBrUptkByHBr(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, brIce = 0.0, brLiq = 0.0, gammaIce = 0.0, gammaLiq = 0.0, srMw, branch, branch_0, dummy;
  double k_tot, kCl, kBr, kHSO3, kSO3;
  srMw = SRMW(HOBr);
  if (H->stratBox) {
    gammaLiq = 0.25;
    k = k + o_Ars_L1k(X, H->xArea[O_SUL], H->xRadi[O_SUL], gammaLiq, srMw);
    k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_HOBr_plus_HBr];
    gammaIce = 0.3;
    if (H->natSurface) gammaIce = 0.001;
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gammaIce, srMw);
  } else {
    o_Gam_HOBr_Cld(X, &gammaLiq, &k_tot, &kCl, &kBr, &kHSO3, &kSO3);
    branch_0 = (kCl + kBr) / k_tot;
    branch = branch_0 * 0.9;
    if (H->Br_over_Cl_Cld <= 5.0e-4) branch = branch_0 * o_Br2_Yield(H->Br_over_Cl_Cld);
    brLiq = branch * H->frac_Br_CldG;
    o_Gam_HOBr_Ice(X, &gammaIce, &dummy, &brIce);
    k = k + o_CloudHet(X, srMw, gammaLiq, gammaIce, brLiq, brIce);
  }
  k = o_kIIR1Ltd(CC(HOBr), CC(HBr), k);
  return k;
}

static double o_HOBrUptkByHCl(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, brIce = 0.0, brLiq = 0.0, gammaIce = 0.0, gammaLiq = 0.0, srMw, branch, branch_0, dummy;
  double k_tot, kCl, kBr, kHSO3, kSO3;
  srMw = SRMW(HOBr);
  if (H->stratBox) {
    gammaLiq = 0.2;
    k = k + o_Ars_L1k(X, H->xArea[O_SUL], H->xRadi[O_SUL], gammaLiq, srMw);
    k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_HOBr_plus_HCl];
    gammaIce = 0.3;
    if (H->natSurface) gammaIce = 0.1;
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gammaIce, srMw);
  } else {
    o_Gam_HOBr_Cld(X, &gammaLiq, &k_tot, &kCl, &kBr, &kHSO3, &kSO3);
    branch_0 = (kCl + kBr) / k_tot;
    branch = branch_0 * 0.1;
    if (H->Br_over_Cl_Cld <= 5.0e-4) branch = branch_0 * (1.0 - o_Br2_Yield(H->Br_over_Cl_Cld));
    brLiq = branch * H->frac_Cl_CldG;
    o_Gam_HOBr_Ice(X, &gammaIce, &brIce, &dummy);
    k = k + o_CloudHet(X, srMw, gammaLiq, gammaIce, brLiq, brIce);
  }
  k = o_kIIR1Ltd(CC(HOBr), CC(HCl), k);
  return k;
}

/* HOBrUptkByBrSALA/BrSALC/SALACL/SALCCL (fullchem_RateLawFuncs.F90:1759-1997)
 * share one shape; br selects the Br- (0.9, Br2 yield) or Cl- branch, fine
 * the fine (aCl*) or coarse (SSC) sea salt. */
static double o_hobr_ss(const het_cell_t* X, int br, int fine, double fracCld, int educt) {
  const het_state_t* H = &X->H;
  double k = 0.0, brLiq = 0.0, gammaAer = 0.0, gammaLiq = 0.0, srMw, branch, branch_0, area;
  double k_tot, kCl, kBr, kHSO3, kSO3;
  srMw = SRMW(HOBr);
  if (!H->stratBox) {
    o_Gam_HOBr_Cld(X, &gammaLiq, &k_tot, &kCl, &kBr, &kHSO3, &kSO3);
    branch_0 = (kCl + kBr) / k_tot;
    branch = branch_0 * (br ? 0.9 : 0.1);
    if (H->Br_over_Cl_Cld <= 5.0e-4)
      branch = br ? branch_0 * o_Br2_Yield(H->Br_over_Cl_Cld) : branch_0 * (1.0 - o_Br2_Yield(H->Br_over_Cl_Cld));
    brLiq = branch * fracCld;
    k = k + o_CloudHet(X, srMw, gammaLiq, 0.0, brLiq, 0.0);
  }
  if (fine ? H->SSA_is_Acid : H->SSC_is_Acid) {
    if (fine)
      o_Gam_HOBr_Aer(X, H->aClRadi, H->H_conc_SSA, H->Cl_conc_SSA, H->Br_conc_SSA, &gammaAer);
    else
      o_Gam_HOBr_Aer(X, H->xRadi[O_SSC], H->H_conc_SSC, H->Cl_conc_SSC, H->Br_conc_SSC, &gammaAer);
    branch = br ? 0.9 : 0.1;
    double ratio = fine ? H->Br_over_Cl_SSA : H->Br_over_Cl_SSC;
    if (ratio <= 5.0e-4) branch = br ? o_Br2_Yield(ratio) : 1.0 - o_Br2_Yield(ratio);
    if (fine) {
      area = H->ClearFr * H->aClArea * H->f_Acid_SSA;
      k = k + o_Ars_L1k(X, area, H->aClRadi, gammaAer, srMw) * branch;
    } else {
      area = H->ClearFr * H->xArea[O_SSC] * H->f_Acid_SSC;
      k = k + o_Ars_L1k(X, area, H->xRadi[O_SSC], gammaAer, srMw) * branch;
    }
  }
  k = o_kIIR1Ltd(CC(HOBr), oC(X, educt), k);
  return k;
}
static double o_HOBrUptkByBrSALA(const het_cell_t* X) { return o_hobr_ss(X, 1, 1, X->H.frac_Br_CldA, OHS_BrSALA); }
static double o_HOBrUptkByBrSALC(const het_cell_t* X) { return o_hobr_ss(X, 1, 0, X->H.frac_Br_CldC, OHS_BrSALC); }
static double o_HOBrUptkBySALACL(const het_cell_t* X) { return o_hobr_ss(X, 0, 1, X->H.frac_Cl_CldA, OHS_SALACL); }
static double o_HOBrUptkBySALCCL(const het_cell_t* X) { return o_hobr_ss(X, 0, 0, X->H.frac_Cl_CldC, OHS_SALCCL); }

static double o_HOBrUptkByHSO3m(const het_cell_t* X) {
  double k = 0.0, brLiq = 0.0, gammaLiq = 0.0, k_tot, kCl, kBr, kHSO3, kSO3;
  if (!X->H.stratBox) {
    o_Gam_HOBr_Cld(X, &gammaLiq, &k_tot, &kCl, &kBr, &kHSO3, &kSO3);
    brLiq = kHSO3 / k_tot;
    k = k + o_CloudHet(X, SRMW(HOBr), gammaLiq, 0.0, brLiq, 0.0);
  }
  k = o_kIIR1Ltd(CC(HOBr), CC(SO2), k);
  return k;
}

static double o_HOBrUptkBySO3mm(const het_cell_t* X) {
  double k = 0.0, brLiq, gammaLiq, k_tot, kCl, kBr, kHSO3, kSO3;
  if (!X->H.stratBox) {
    o_Gam_HOBr_Cld(X, &gammaLiq, &k_tot, &kCl, &kBr, &kHSO3, &kSO3);
    brLiq = kSO3 / k_tot;
    k = k + o_CloudHet(X, SRMW(HOBr), gammaLiq, 0.0, brLiq, 0.0);
  }
  k = o_kIIR1Ltd(CC(HOBr), CC(SO2), k);
  return k;
}

/* ---- HOCl (fullchem_RateLawFuncs.F90:2075-2364) --------------------- */
static void o_Gam_HOCl_Cld(const het_cell_t* X, double* gamma, double* branchCl, double* branchSO3) {
  const double INV_AB = 1.0 / 0.8, D_l = 2.0e-5;
  const het_state_t* H = &X->H;
  double k_Cl, k_SO3, k_tot, M_X, cavg, H_X, l_r, gb_tot;
  k_Cl = 1.5e+4 * H->H_conc_LCl * H->Cl_conc_Cld;
  k_SO3 = 2.8e+5 * H->TSO3_aq;
  k_tot = k_Cl + k_SO3;
  *gamma = 0.0;
  *branchCl = 0.0;
  *branchSO3 = 0.0;
  if (k_tot > 0.0) {
    M_X = MWX(HOCl) * 1.0e-3;
    cavg = sqrt(X->EIGHT_RSTARG_T / (H->PI * M_X)) * 100.0;
    H_X = (O_HK0[OHSI_HOCl] * O_CON_ATM_BAR) * exp(O_HCR[OHSI_HOCl] * (X->INV_TEMP - O_INV_T298));
    l_r = sqrt(D_l / k_tot);
    gb_tot = X->FOUR_R_T * H_X * l_r * k_tot / cavg;
    gb_tot = gb_tot * o_ReactoDiff_Corr(H->rLiq, l_r);
    *gamma = 1.0 / (INV_AB + 1.0 / gb_tot);
    *branchCl = k_Cl / k_tot;
    *branchSO3 = k_SO3 / k_tot;
  }
}

static void o_Gam_HOCl_Aer(const het_cell_t* X, double radius, double C_Hp, double C_Cl, double* gamma) {
  const double INV_AB = 1.0 / 0.8, D_l = 2.0e-5, K_TER = 1.5e+4;
  double M_X, cavg, H_X, l_r, gb;
  *gamma = 0.0;
  if (!(C_Cl > 0.0)) return;
  M_X = MWX(HOCl) * 1.0e-3;
  cavg = sqrt(X->EIGHT_RSTARG_T / (X->H.PI * M_X)) * 100.0;
  H_X = (O_HK0[OHSI_HOCl] * O_CON_ATM_BAR) * exp(O_HCR[OHSI_HOCl] * (X->INV_TEMP - O_INV_T298));
  l_r = sqrt(D_l / (K_TER * C_Hp * C_Cl));
  gb = X->FOUR_R_T * H_X * l_r * K_TER * C_Hp * C_Cl / cavg;
  gb = gb * o_ReactoDiff_Corr(radius, l_r);
  *gamma = 1.0 / (INV_AB + 1.0 / gb);
}

static double o_HOClUptkByHCl(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, branch, branchCl, dummy, gammaIce, brIce, srMw = SRMW(HOCl);
  if (H->stratBox) {
    gamma = 0.8;
    k = k + o_Ars_L1k(X, H->xArea[O_SUL], H->xRadi[O_SUL], gamma, srMw);
    k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_HOCl_plus_HCl];
    gamma = 0.2;
    if (H->natSurface) gamma = 0.1;
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
    k = o_kIIR1Ltd(CC(HOCl), CC(HCl), k);
    return k;
  }
  o_Gam_HOCl_Cld(X, &gamma, &branchCl, &dummy);
  branch = branchCl * H->frac_Cl_CldG;
  gammaIce = 0.22 * H->HCl_theta;
  brIce = 1.0;
  k = k + o_CloudHet(X, srMw, gamma, gammaIce, branch, brIce);
  k = o_kIIR1Ltd(CC(HOCl), CC(HCl), k);
  return k;
}

static double o_HOClUptkByHBr(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, srMw = SRMW(HOCl);
  if (H->stratBox) {
    gamma = 0.8;
    k = k + o_Ars_L1k(X, H->xArea[O_SUL], H->xRadi[O_SUL], gamma, srMw);
    k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_HOCl_plus_HBr];
    gamma = 0.3;
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  }
  k = o_kIIR1Ltd(CC(HOCl), CC(HBr), k);
  if (H->TurnOffHetRates) k = 0.0;
  return k;
}

static double o_HOClUptkBySALACL(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, branch, branchCl, dummy, area, srMw = SRMW(HOCl);
  if (!H->stratBox) {
    o_Gam_HOCl_Cld(X, &gamma, &branchCl, &dummy);
    branch = branchCl * H->frac_Cl_CldA;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  if (H->SSA_is_Acid) {
    o_Gam_HOCl_Aer(X, H->aClRadi, H->H_conc_SSA, H->Cl_conc_SSA, &gamma);
    area = H->ClearFr * H->aClArea * H->f_Acid_SSA;
    k = k + o_Ars_L1k(X, area, H->aClRadi, gamma, srMw);
  }
  k = o_kIIR1Ltd(CC(HOCl), CC(SALACL), k);
  return k;
}

static double o_HOClUptkBySALCCL(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, branch, branchCl, dummy, area, srMw = SRMW(HOCl);
  if (!H->stratBox) {
    o_Gam_HOCl_Cld(X, &gamma, &branchCl, &dummy);
    branch = branchCl * H->frac_Cl_CldC;
    k = k + o_CloudHet(X, srMw, gamma, 0.0, branch, 0.0);
  }
  if (H->SSC_is_Acid) {
    o_Gam_HOCl_Aer(X, H->xRadi[O_SSC], H->H_conc_SSC, H->Cl_conc_SSC, &gamma);
    area = H->ClearFr * H->xArea[O_SSC] * H->f_Acid_SSC;
    k = k + o_Ars_L1k(X, area, H->xRadi[O_SSC], gamma, srMw);
  }
  k = o_kIIR1Ltd(CC(HOCl), CC(SALCCL), k);
  return k;
}

static double o_HOClUptkByHSO3m(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, branch, branchSO3, dummy;
  if (!H->stratBox) {
    o_Gam_HOCl_Cld(X, &gamma, &dummy, &branchSO3);
    branch = branchSO3 * H->frac_HSO3_aq;
    k = k + o_CloudHet(X, SRMW(HOCl), gamma, 0.0, branch, 0.0);
  }
  k = o_kIIR1Ltd(CC(HOCl), CC(SO2), k) * H->HSO3m;
  return k;
}

static double o_HOClUptkBySO3mm(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, branch, branchSO3, dummy;
  if (!H->stratBox) {
    o_Gam_HOCl_Cld(X, &gamma, &dummy, &branchSO3);
    branch = branchSO3 * H->frac_SO3_aq;
    k = k + o_CloudHet(X, SRMW(HOCl), gamma, 0.0, branch, 0.0);
  }
  k = o_kIIR1Ltd(CC(HOCl), CC(SO2), k) * H->SO3mm;
  return k;
}

/* ---- iodine (fullchem_RateLawFuncs.F90:2371-2541) ------------------- */
static double o_IuptkBySulf1stOrd(const het_cell_t* X, double srMw, double gamma) {
  double k = o_Ars_L1k(X, X->H.xArea[O_SUL], X->H.xRadi[O_SUL], gamma, srMw);
  k = k + o_Ars_L1k(X, X->H.xArea[O_SLA], X->H.xRadi[O_SLA], gamma, srMw);
  return k;
}
static double o_IuptkBySALA1stOrd(const het_cell_t* X, double srMw, double gamma) {
  if (X->H.stratBox) return 0.0;
  return o_Ars_L1k(X, X->H.xArea[O_SSA], X->H.xRadi[O_SSA], gamma, srMw);
}
static double o_IuptkByAlkSALA1stOrd(const het_cell_t* X, double srMw, double gamma) {
  double k = 0.0, ssarea;
  if (X->H.stratBox) return k;
  if (X->H.SSA_is_Alk) {
    ssarea = X->H.f_Alk_SSA * X->H.xArea[O_SSA];
    k = o_Ars_L1k(X, ssarea, X->H.xRadi[O_SSA], gamma, srMw);
  }
  return k;
}
static double o_IuptkBySALC1stOrd(const het_cell_t* X, double srMw, double gamma) {
  if (X->H.stratBox) return 0.0;
  return o_Ars_L1k(X, X->H.xArea[O_SSC], X->H.xRadi[O_SSC], gamma, srMw);
}
static double o_IuptkByAlkSALC1stOrd(const het_cell_t* X, double srMw, double gamma) {
  double k = 0.0, ssarea;
  if (X->H.stratBox) return k;
  if (X->H.SSC_is_Alk) {
    ssarea = X->H.f_Alk_SSC * X->H.xArea[O_SSC];
    k = o_Ars_L1k(X, ssarea, X->H.xRadi[O_SSC], gamma, srMw);
  }
  return k;
}
static double o_IbrkdnByAcidBrSALA(const het_cell_t* X, double srMw, double conc, double gamma) {
  double k = 0.0, ssarea;
  if (X->H.stratBox) return k;
  if (X->H.SSA_is_Acid) {
    ssarea = X->H.f_Acid_SSA * X->H.xArea[O_SSA];
    k = 0.15 * o_Ars_L1k(X, ssarea, X->H.xRadi[O_SSA], gamma, srMw);
    k = o_kIIR1Ltd(conc, CC(BrSALA), k);
  }
  return k;
}
static double o_IbrkdnByAcidBrSALC(const het_cell_t* X, double srMw, double conc, double gamma) {
  double k = 0.0, ssarea;
  if (X->H.stratBox) return k;
  if (X->H.SSC_is_Acid) {
    ssarea = X->H.f_Acid_SSC * X->H.xArea[O_SSC];
    k = 0.15 * o_Ars_L1k(X, ssarea, X->H.xRadi[O_SSC], gamma, srMw);
    k = o_kIIR1Ltd(conc, CC(BrSALC), k);
  }
  return k;
}
static double o_IbrkdnByAcidSALACl(const het_cell_t* X, double srMw, double conc, double gamma) {
  double k = 0.0, ssarea;
  if (X->H.stratBox) return k;
  if (X->H.SSA_is_Acid) {
    ssarea = X->H.f_Acid_SSA * X->H.xArea[O_SSA];
    k = 0.85 * o_Ars_L1k(X, ssarea, X->H.xRadi[O_SSA], gamma, srMw);
    k = o_kIIR1Ltd(conc, CC(SALACL), k);
  }
  return k;
}
static double o_IbrkdnByAcidSALCCl(const het_cell_t* X, double srMw, double conc, double gamma) {
  double k = 0.0, ssarea;
  if (X->H.stratBox) return k;
  if (X->H.SSC_is_Acid) {
    ssarea = X->H.f_Acid_SSC * X->H.xArea[O_SSC];
    k = 0.85 * o_Ars_L1k(X, ssarea, X->H.xRadi[O_SSC], gamma, srMw);
    k = o_kIIR1Ltd(conc, CC(SALCCL), k);
  }
  return k;
}

/* ---- IONO2, N2O5 (fullchem_RateLawFuncs.F90:2544-2926) -------------- */
static double o_IONO2uptkByH2O(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, area, gamma, srMw = SRMW(IONO2);
  area = H->ClearFr * H->xArea[O_SUL];
  gamma = fmax((0.0021 * X->TEMP - 0.561), 0.0);
  k = k + o_Ars_L1k(X, area, H->xRadi[O_SUL], gamma, srMw);
  k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_BrNO3_plus_H2O];
  area = H->ClearFr * H->xArea[O_IIC];
  gamma = 0.3;
  if (H->natSurface) gamma = 0.001;
  k = k + o_Ars_L1k(X, area, H->xRadi[O_IIC], gamma, srMw);
  k = k + o_CloudHet(X, srMw, 0.01, 0.01, 1.0, 1.0);
  k = o_kIIR1Ltd(CC(IONO2), CC(H2O), k);
  return k;
}

static double o_ClNO2_BT(double Cl, double H2O) {
  const double k2k3 = 1.0 / 4.5e+2;
  double phi;
  if (H2O < 0.1) {
    phi = 0.0;
    if (Cl > 1e-3) phi = 1.0;
    return phi;
  }
  phi = 1.0 / (1.0 + k2k3 * o_SafeDiv(H2O, Cl, 1.0e+30));
  return phi;
}

static void o_N2O5_InorgOrg(const het_cell_t* X, double volInorg, double volOrg, double H2Oinorg, double H2Oorg,
                            double Rcore, double NIT, double Cl, double* gamma, double* Y_ClNO2, double* rp,
                            double* areaTotal) {
  const double KH = 5.1e+1, k3k2b = 4.0e-2, beta = 1.15e+6, delta = 1.3e-1, Haq = 5e+3, Daq = 1e-9;
  const double ONE_THIRD = 1.0 / 3.0;
  const het_state_t* H = &X->H;
  double volTotal, H2Ototal, volRatioDry, Rp, l, M_N2O5, speed, M_H2O, M_NIT, M_Cl, OCratio, eps;
  double gamma_coat, gamma_core, A, k2f;
  volTotal = volInorg + volOrg;
  H2Ototal = H2Oinorg + H2Oorg;
  volRatioDry = o_SafeDiv(fmax(volInorg - H2Oinorg, 0.0), fmax(volTotal - H2Ototal, 0.0), 0.0);
  Rp = o_SafeDiv(Rcore, pow(volRatioDry, ONE_THIRD), Rcore);
  l = Rp - Rcore;
  M_N2O5 = MWX(N2O5) * 1.0e-3;
  speed = sqrt(X->EIGHT_RSTARG_T / (H->PI * M_N2O5));
  M_H2O = H2Ototal / 18e+0 / volTotal * 1000.0;
  M_NIT = NIT / volTotal / H->AVO * 1000.0;
  M_Cl = Cl / volTotal / H->AVO * 1000.0;
  OCratio = (((H->OMOC_POA + H->OMOC_OPOA) / 2.0) - 1.17) / 1.29;
  eps = 1.5e-1 * OCratio + 1.6e-3 * X->RELHUM;
  if (l <= 0.0e+0) {
    gamma_coat = 0.0;
  } else {
    gamma_coat = (X->FOUR_RGASLATM_T * 1.0e-3 * eps * Haq * Daq * Rcore / 100.0) / (speed * l / 100.0 * Rp / 100.0);
  }
  *areaTotal = 3.0 * volTotal / Rp;
  if (M_H2O < 0.1) {
    gamma_core = 0.005;
  } else {
    speed = speed * 1e+2;
    A = ((4.0 * volTotal) / (speed * *areaTotal)) * KH;
    A = fmin(A, 3.2e-8);
    if (delta * M_H2O < 1e-2) {
      k2f = beta * (delta * M_H2O);
    } else {
      k2f = beta * (1e+0 - exp(-delta * M_H2O));
    }
    gamma_core = A * k2f * (1.0 - 1.0 / (1.0 + o_SafeDiv(k3k2b * M_H2O, M_NIT, 1.0e+30)));
  }
  if (gamma_coat <= 0.0) {
    *gamma = gamma_core;
  } else if (gamma_core <= 0.0) {
    *gamma = 0.0;
  } else {
    *gamma = 1.0 / ((1.0 / gamma_core) + (1.0 / gamma_coat));
  }
  *Y_ClNO2 = o_ClNO2_BT(M_Cl, M_H2O);
  *rp = Rp;
}

static double o_N2O5uptkByH2O(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, Y_ClNO2, Rp, SA, ktmp, srMw = SRMW(N2O5);
  gamma = 0.02;
  for (int t = O_DU1; t <= O_DU7; ++t) k = k + o_Ars_L1k(X, H->ClearFr * H->xArea[t], H->xRadi[t], gamma, srMw);
  o_N2O5_InorgOrg(X, H->aClVol, H->xVol[O_ORC], H->xH2O[O_SUL], H->xH2O[O_ORC], H->aClRadi, CC(NIT), CC(SALACL),
                  &gamma, &Y_ClNO2, &Rp, &SA);
  ktmp = o_Ars_L1k(X, H->ClearFr * SA, Rp, gamma, srMw);
  k = k + ktmp - (ktmp * Y_ClNO2 * 0.25);
  gamma = 0.005;
  k = k + o_Ars_L1k(X, H->ClearFr * H->xArea[O_BKC], H->xRadi[O_BKC], gamma, srMw);
  o_N2O5_InorgOrg(X, H->xVol[O_SSC], 0.0, H->xH2O[O_SSC], 0.0, H->xRadi[O_SSC], CC(NITs), CC(SALCCL), &gamma,
                  &Y_ClNO2, &Rp, &SA);
  ktmp = o_Ars_L1k(X, H->ClearFr * SA, Rp, gamma, srMw);
  k = k + ktmp - (ktmp * Y_ClNO2);
  k = k + H->xArea[O_SLA] * H->KHETI_SLA[O_N2O5_plus_H2O];
  gamma = 0.02;
  if (H->natSurface) gamma = 4.0e-4;
  k = k + o_Ars_L1k(X, H->ClearFr * H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  k = o_kIIR1Ltd(CC(N2O5), CC(H2O), k);
  return k;
}

static double o_N2O5uptkBySALACl(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, Y_ClNO2, Rp, SA;
  if (H->stratBox) return k;
  o_N2O5_InorgOrg(X, H->aClVol, H->xVol[O_ORC], H->xH2O[O_SUL], H->xH2O[O_ORC], H->aClRadi, CC(NIT), CC(SALACL),
                  &gamma, &Y_ClNO2, &Rp, &SA);
  k = o_Ars_L1k(X, H->ClearFr * SA, Rp, gamma, SRMW(N2O5));
  k = k * Y_ClNO2 * 0.25;
  k = o_kIIR1Ltd(CC(N2O5), CC(SALACL), k);
  return k;
}

static double o_N2O5uptkBySALCCl(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, Y_ClNO2, Rp, SA;
  if (H->stratBox) return k;
  o_N2O5_InorgOrg(X, H->xVol[O_SSC], 0.0, H->xH2O[O_SSC], 0.0, H->xRadi[O_SSC], CC(NITs), CC(SALCCL), &gamma,
                  &Y_ClNO2, &Rp, &SA);
  k = o_Ars_L1k(X, H->ClearFr * SA, Rp, gamma, SRMW(N2O5));
  k = k * Y_ClNO2;
  k = o_kIIR1Ltd(CC(N2O5), CC(SALCCL), k);
  return k;
}

static double o_N2O5uptkByCloud(const het_cell_t* X) {
  const double cnst = 0.03 / 0.019;
  double gamma = cnst * exp(-25.5265 + 9283.76 / X->TEMP - 851801.0 / (X->TEMP * X->TEMP));
  return o_CloudHet(X, SRMW(N2O5), gamma, 0.02, 1.0, 1.0);
}

static double o_N2O5uptkByStratHCl(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma;
  if (H->stratBox) {
    k = k + (H->xArea[O_SLA] * H->KHETI_SLA[O_N2O5_plus_HCl]);
    gamma = 0.03;
    if (H->natSurface) gamma = 0.003;
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, SRMW(N2O5));
  }
  k = o_kIIR1Ltd(CC(N2O5), CC(HCl), k);
  return k;
}

/* ---- NO2, NO3 (fullchem_RateLawFuncs.F90:2928-3104) ----------------- */
static double o_NO2uptk1stOrdAndCloud(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, srMw = SRMW(NO2);
  gamma = 1.0e-8;
  for (int t = O_DU1; t <= O_DU7; ++t) k = k + o_Ars_L1k(X, H->xArea[t], H->xRadi[t], gamma, srMw);
  gamma = 5e-6;
  k = k + o_Ars_L1k(X, H->xArea[O_SUL], H->xRadi[O_SUL], gamma, srMw);
  gamma = 1e-4;
  k = k + o_Ars_L1k(X, H->xArea[O_BKC], H->xRadi[O_BKC], gamma, srMw);
  gamma = 1e-6;
  k = k + o_Ars_L1k(X, H->xArea[O_ORC], H->xRadi[O_ORC], gamma, srMw);
  if (X->RELHUM < 40.0) {
    gamma = 1.0e-8;
  } else if (X->RELHUM > 70.0) {
    gamma = 1.0e-4;
  } else {
    gamma = 1.0e-8 + (1e-4 - 1e-8) * (X->RELHUM - 40.0) / 30.0;
  }
  k = k + o_Ars_L1k(X, H->xArea[O_SSA], H->xRadi[O_SSA], gamma, srMw);
  k = k + o_Ars_L1k(X, H->xArea[O_SSC], H->xRadi[O_SSC], gamma, srMw);
  gamma = 1.0e-4;
  k = k + o_Ars_L1k(X, H->xArea[O_SLA], H->xRadi[O_SLA], gamma, srMw);
  k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  k = k + o_CloudHet(X, SRMW(NO2), 1.0e-8, 0.0, 1.0, 0.0);
  return k;
}

static double o_Gam_NO3(const het_cell_t* X, double aArea, double aRadi, double aWater, double C_X) {
  const double INV_AB = 1.0 / 1.3e-2;
  double Vol, WaterC, M_X, cavg, k_tot, gamma, H_X, l_r, gb, corr;
  Vol = aArea * aRadi * 1.0e-3 / 3.0;
  WaterC = aWater / 18.0e+12 / Vol;
  M_X = MWX(NO3) * 1.0e-3;
  cavg = sqrt(X->EIGHT_RSTARG_T / (X->H.PI * M_X)) * 1.0e2;
  k_tot = (2.76e+6 * C_X) + (23.0 * WaterC);
  gamma = 0.0;
  if (k_tot > 0.0) {
    H_X = 0.6 * O_CON_ATM_BAR;
    l_r = sqrt(1.0e-5 / k_tot);
    gb = X->FOUR_R_T * H_X * l_r * k_tot / cavg;
    corr = o_ReactoDiff_Corr(aRadi, l_r);
    gb = gb * corr;
    gamma = 1.0 / (INV_AB + 1.0 / gb);
  }
  return gamma;
}

static double o_NO3uptk1stOrdAndCloud(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, gamma, srMw = SRMW(NO3);
  gamma = 0.01;
  for (int t = O_DU1; t <= O_DU7; ++t) k = k + o_Ars_L1k(X, H->xArea[t], H->xRadi[t], gamma, srMw);
  if (X->RELHUM < 50.0) {
    gamma = 2.0e-4;
  } else {
    gamma = 1.0e-3;
  }
  k = k + o_Ars_L1k(X, H->xArea[O_BKC], H->xRadi[O_BKC], gamma, srMw);
  gamma = 0.005;
  k = k + o_Ars_L1k(X, H->xArea[O_ORC], H->xRadi[O_ORC], gamma, srMw);
  gamma = 0.1;
  k = k + o_Ars_L1k(X, H->xArea[O_SLA], H->xRadi[O_SLA], gamma, srMw);
  k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  k = k + o_CloudHet(X, SRMW(NO3), 0.002, 0.001, 1.0, 1.0);
  return k;
}

static double o_NO3hypsisClonSALA(const het_cell_t* X) {
  double area = X->H.aClArea, radi = X->H.aClRadi, water = X->H.aWater[1], conc = X->H.Cl_conc_SSA, gamma;
  gamma = o_Gam_NO3(X, area, radi, water, conc) * 0.01;
  area = X->H.ClearFr * area;
  return o_Ars_L1k(X, area, radi, gamma, SRMW(NO3));
}

static double o_NO3hypsisClonSALC(const het_cell_t* X) {
  double area = X->H.xArea[O_SSC], radi = X->H.xRadi[O_SSC], water = X->H.aWater[2], conc = X->H.Cl_conc_SSC;
  double gamma = o_Gam_NO3(X, area, radi, water, conc) * 0.01;
  area = X->H.ClearFr * area;
  return o_Ars_L1k(X, area, radi, gamma, SRMW(NO3));
}

/* ---- O3, OH, organics (fullchem_RateLawFuncs.F90:3106-3458) --------- */
static double o_Gamma_O3_Br(const het_cell_t* X, double Radius, double C_Br) {
  const double K0_O3 = 1.1e-2 * O_CON_ATM_BAR;
  double H_X, M_X, cavg, Nmax, KLangC, k_s, C_Br_surf, gs, k_b, D_l, l_r, gb, gamma = 0.0;
  if (!(C_Br > 0.0)) return gamma;
  H_X = K0_O3 * exp(2300.0 * (X->INV_TEMP - O_INV_T298));
  M_X = MWX(O3) * 1.0e-3;
  cavg = sqrt(X->EIGHT_RSTARG_T / (X->H.PI * M_X)) * 100.0;
  Nmax = 3.0e+14;
  KLangC = 1.0e-13;
  k_s = 1.0e-16;
  C_Br_surf = fmin(3.41e+14 * C_Br, Nmax);
  gs = (4.0 * k_s * C_Br_surf * KLangC * Nmax) / (cavg * (1.0 + KLangC * CC(O3)));
  k_b = 6.3e+8 * exp(-4.45e+3 / X->TEMP);
  D_l = 8.9e-6;
  l_r = sqrt(D_l / (k_b * C_Br));
  gb = X->FOUR_R_T * H_X * l_r * k_b * C_Br / cavg;
  gb = gb * o_ReactoDiff_Corr(Radius, l_r);
  gamma = gb + gs;
  return gamma;
}

static double o_O3uptkByBrInTropCloud(const het_cell_t* X, double Br_branch) {
  double gamma;
  if (X->H.stratBox) return 0.0;
  gamma = o_Gamma_O3_Br(X, X->H.rLiq, X->H.Br_conc_Cld);
  return o_CloudHet(X, SRMW(O3), gamma, 0.0, Br_branch, 0.0);
}

static double o_O3uptkByHBr(const het_cell_t* X) {
  double k = o_O3uptkByBrInTropCloud(X, X->H.frac_Br_CldG);
  return o_kIIR1Ltd(CC(O3), CC(HBr), k);
}

static double o_O3uptkByBrSALA(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, area, gamma;
  if (H->stratBox) return k;
  k = k + o_O3uptkByBrInTropCloud(X, H->frac_Br_CldA);
  if (H->SSA_is_Acid) {
    area = H->ClearFr * H->aClArea * H->f_Acid_SSA;
    gamma = o_Gamma_O3_Br(X, H->aClRadi, H->Br_conc_SSA);
    k = k + o_Ars_L1k(X, area, H->aClRadi, gamma, SRMW(O3));
  }
  k = o_kIIR1Ltd(CC(O3), CC(BrSALA), k);
  return k;
}

static double o_O3uptkByBrSALC(const het_cell_t* X) {
  const het_state_t* H = &X->H;
  double k = 0.0, area, gamma;
  if (H->stratBox) return k;
  k = k + o_O3uptkByBrInTropCloud(X, H->frac_Br_CldC);
  if (H->SSC_is_Acid) {
    area = H->ClearFr * H->xArea[O_SSC] * H->f_Acid_SSC;
    gamma = o_Gamma_O3_Br(X, H->xRadi[O_SSC], H->Br_conc_SSC);
    k = k + o_Ars_L1k(X, area, H->xRadi[O_SSC], gamma, SRMW(O3));
  }
  k = o_kIIR1Ltd(CC(O3), CC(BrSALC), k);
  return k;
}

static double o_OHuptkBySALACl(const het_cell_t* X) {
  double k = 0.0, gamma;
  if (X->H.stratBox) return k;
  gamma = 0.04 * X->H.Cl_conc_SSA;
  k = o_Ars_L1k(X, X->H.aClArea, X->H.aClRadi, gamma, SRMW(OH));
  return o_kIIR1Ltd(CC(OH), CC(SALACL), k);
}

static double o_OHuptkBySALCCl(const het_cell_t* X) {
  double k = 0.0, gamma;
  if (X->H.stratBox) return k;
  gamma = 0.04 * X->H.Cl_conc_SSC;
  k = o_Ars_L1k(X, X->H.xArea[O_SSC], X->H.xRadi[O_SSC], gamma, SRMW(OH));
  return o_kIIR1Ltd(CC(OH), CC(SALCCL), k);
}

static double o_GLYXuptk1stOrd(const het_cell_t* X, double srMw) {
  double k = 0.0, gamma = 0.0;
  if (X->RELHUM >= O_CRITRH) {
    if (X->SUNCOS > 0.0) {
      gamma = 4.4e-3;
    } else {
      gamma = 8.0e-6;
    }
    k = k + o_Ars_L1k(X, X->H.xArea[O_SUL], X->H.xRadi[O_SUL], gamma, srMw);
  }
  return k;
}

static double o_EpoxUptkGamma(const het_cell_t* X, double srMw) {
  const double DIFF_N2O5_STD = 1.0e-1, MACOEFF = 1.0e-1, K_HPLUS = 3.6e-2, K_NUC = 2.0e-4, K_HSO4 = 7.3e-4,
               K_HYDRO = 0.0e+0, HSTAR_EPOX = 1.7e+7;
  const het_state_t* H = &X->H;
  double gamma = 0.0, valTmp = 0.0, aerVol, xmms, kPart, val1, val2, val3;
  aerVol = (H->xArea[O_SUL] * H->xRadi[O_SUL]) / 3.0;
  xmms = sqrt((2.117e+8 * X->TEMP) / (srMw * srMw));
  kPart = (K_HPLUS * H->H_PLUS) + (K_NUC * H->H_PLUS * (H->NO3_molal + H->SO4_molal)) + (K_HSO4 * H->HSO4_molal) +
          (K_HYDRO);
  val1 = (H->xRadi[O_SUL] * xmms) / (4.0 * DIFF_N2O5_STD);
  val2 = (1.0 / MACOEFF);
  if (H->xArea[O_SUL] > 0.0 && xmms > 0.0)
    valTmp = (X->FOUR_RGASLATM_T * aerVol * HSTAR_EPOX * kPart) / (H->xArea[O_SUL] * xmms);
  val3 = 0.0;
  if (valTmp > 0.0) val3 = 1.0 / valTmp;
  gamma = 0.0;
  if (kPart >= 1.e-8) gamma = 1.0 / (val1 + val2 + val3);
  if (gamma < 0.0) gamma = 0.0;
  return gamma;
}

static double o_IEPOXuptk1stOrd(const het_cell_t* X, double srMw, bool doScale) {
  double k = 0.0, gamma = 0.0;
  if (X->RELHUM >= O_CRITRH) {
    gamma = o_EpoxUptkGamma(X, srMw);
    if (doScale && (X->H.H_PLUS > 8.0e-5)) gamma = gamma / 30.0;
    k = k + o_Ars_L1k(X, X->H.xArea[O_SUL], X->H.xRadi[O_SUL], gamma, srMw);
  }
  return k;
}

static double o_MGLYuptk1stOrd(const het_cell_t* X, double srMw) {
  double k = 0.0, gamma = 0.0;
  if (X->RELHUM >= O_CRITRH) {
    gamma = 3.6e-7;
    k = k + o_Ars_L1k(X, X->H.xArea[O_SUL], X->H.xRadi[O_SUL], gamma, srMw);
  }
  return k;
}

static double o_VOCuptk1stOrd(const het_cell_t* X, double srMw, double gamma) {
  const het_state_t* H = &X->H;
  double k = 0.0;
  if (X->RELHUM >= O_CRITRH) {
    k = k + o_Ars_L1k(X, H->xArea[O_SUL], H->xRadi[O_SUL], gamma, srMw);
    k = k + o_Ars_L1k(X, H->xArea[O_BKC], H->xRadi[O_BKC], gamma, srMw);
    k = k + o_Ars_L1k(X, H->xArea[O_ORC], H->xRadi[O_ORC], gamma, srMw);
    k = k + o_Ars_L1k(X, H->xArea[O_SSA], H->xRadi[O_SSA], gamma, srMw);
    k = k + o_Ars_L1k(X, H->xArea[O_SSC], H->xRadi[O_SSC], gamma, srMw);
    k = k + o_Ars_L1k(X, H->xArea[O_SLA], H->xRadi[O_SLA], gamma, srMw);
    k = k + o_Ars_L1k(X, H->xArea[O_IIC], H->xRadi[O_IIC], gamma, srMw);
  }
  return k;
}

#undef SRMW
#undef MWX
#undef CC
#endif
