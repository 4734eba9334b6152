/* fullchem_SetStateHet restated in C for the CPU oracle -- TEST
 * INFRASTRUCTURE (checks the GPU producer of the HetState rows).
 *
 * Sources (GEOS-Chem tree), statement by statement:
 *   fullChem_SetStateHet     KPP/fullchem/fullchem_HetStateFuncs.F90:48-244
 *   Get_Theta_Ice            :268-310
 *   Halide_Conc              :325-468
 *   Get_Halide_CldConc       :483-560
 *   Get_Halide_SsaConc       :575-600
 *   Compute_L2G_Local        :615-650
 *   Cld_Params               KPP/fullchem/rateLawUtilFuncs.F90:281-417
 *   CALC_KH, CALC_HEFF       GeosUtil/henry_mod.F90:74-204
 *   fullchem_SulfurAqChem    KPP/fullchem/fullchem_SulfurChemFuncs.F90:120-305
 *   Ars_L1K, kIIR1Ltd        KPP/fullchem/rateLawUtilFuncs.F90:77-160
 *   AVO, PI                  Headers/physconstants.F90:32, 40
 *
 * Input rows OHIN_* and output rows OHET_* come from oracle_het_layout.h
 * (written by gen_oracle.py from the field lists of the batch interface);
 * the KPP indices of the species read are OSS_* there (-1 when absent).
 * The HetState is built in a struct first, field by field as the Fortran
 * assigns them, then written out as rows.
 */
#include <math.h>
#include <stdbool.h>
#include <string.h>

#include "kpp_dims.h"
#include "oracle_het_layout.h"

#define S_AVO 6.022140857e+23
#define S_PI 3.14159265358979323
#define S_TREF 298.15
#define S_R 8.3144598
#define S_ATM 101.325

typedef struct {
  double AVO, PI, CldFr, ClearFr, QICE, QLIQ, vAir;
  int nAeroType;
  double aClArea, aClRadi, aClVol, AWATER[2], xArea[15], xRadi[15], xVol[15], wetArea[15], xH2O[15];
  double OMOC_POA, OMOC_OPOA, HSO3_aq, SO3_aq, TSO3_aq, frac_HSO3_aq, frac_SO3_aq;
  double HSO4_molal, NO3_molal, SO4_molal, H_plus, pHCloud, pHSSA[2];
  double H_conc_Sul, H_conc_LCl, H_conc_ICl, H_conc_SSA, H_conc_SSC;
  double f_Alk_SSA, f_Acid_SSA, f_Alk_SSC, f_Acid_SSC;
  bool SSA_is_Alk, SSA_is_Acid, SSC_is_Alk, SSC_is_Acid;
  double gamma_HO2, fupdateHOBr, fupdateHOCl, HSO3m, SO3mm;
  double rLiq, rIce, ALiq, VLiq, AIce, VIce;
  double HNO3_theta, HCl_theta, HBr_theta;
  double Br_conc_CldG, Br_conc_CldA, Br_conc_CldC, Br_conc_Cld, Br_over_Cl_Cld, Br_over_Cl_SSA, Br_over_Cl_SSC;
  double Cl_conc_CldG, Cl_conc_CldA, Cl_conc_CldC, Cl_conc_Cld;
  double frac_Br_CldA, frac_Br_CldC, frac_Br_CldG, frac_Cl_CldA, frac_Cl_CldC, frac_Cl_CldG;
  double Br_conc_SSA, Br_conc_SSC, Cl_conc_SSA, Cl_conc_SSC, NIT_conc_SSA, NIT_conc_SSC, frac_SALACL;
  double KHETI_SLA[12];
  bool stratBox, pscBox, natSurface, TurnOffHetRates;
} ss_het_t;

/* Fortran EXPONENT and rateLawUtilFuncs SafeDiv (:118-160) */
static int ss_exponent(double x) {
  int e;
  if (x == 0.0) return 0;
  frexp(x, &e);
  return e;
}

static double ss_SafeDiv(double num, double denom, double alt) {
  int ediff = ss_exponent(num) - ss_exponent(denom);
  if (ediff > 1023 || denom == 0.0) return alt;
  if (ediff < -1020) return 0.0;
  return num / denom;
}

static double ss_C(const double* C, long long ldc, int ind) { return ind >= 0 ? C[(long long)ind * ldc] : 0.0; }

/* CALC_KH */
static double calc_kh(double k0, double cr, double tk) {
  return k0 * exp(cr * (1.0 / tk - 1.0 / S_TREF)) * S_R * tk / S_ATM;
}

/* CALC_HEFF */
static double calc_heff(double pka, double ph, double kh) {
  double heff = kh;
  if (ph > 0.0 && pka > -100.0) heff = heff * (1.0 + pow(10.0, ph - pka));
  return heff;
}

/* Compute_L2G_Local */
static double compute_l2g_local(double k0, double cr, double pka, double tk, double h2oliq, double ph) {
  double kh = calc_kh(k0, cr, tk);
  double heff = calc_heff(pka, ph, kh);
  return heff * h2oliq;
}

/* Cld_Params */
static void cld_params(double AD, double CLDF, double FRLAND, double FROCEAN, double QI, double QL, double T,
                       ss_het_t* H) {
  const double CLDR_CONT = 6.0e-4, CLDR_MARI = 10.0e-4, CLDR_ICE = 38.5e-4, DENS_LIQ = 0.001, DENS_ICE = 0.91e-3;
  double alpha, beta;
  if ((QL + QI <= 0.0) || (CLDF <= 0.0)) {
    H->rLiq = CLDR_CONT;
    H->rIce = CLDR_ICE;
    H->ALiq = 0.0;
    H->VLiq = 0.0;
    H->AIce = 0.0;
    H->VIce = 0.0;
    return;
  }
  if (FRLAND > FROCEAN)
    H->rLiq = CLDR_CONT;
  else
    H->rLiq = CLDR_MARI;
  H->VLiq = QL * AD / DENS_LIQ / H->vAir;
  H->VIce = QI * AD / DENS_ICE / H->vAir;
  H->ALiq = 3.0 * H->VLiq / H->rLiq;
  if (T < 202.0) {
    alpha = 83.3;
    beta = 0.0184;
  } else if (T < 217.0) {
    alpha = 9.1744e+4;
    beta = 0.117;
  } else {
    alpha = 308.4;
    beta = 0.0152;
  }
  H->rIce = 0.5 * alpha * exp(beta * (T - 273.15)) / 1e+4;
  H->AIce = 3.0 * H->VIce / H->rIce * 2.25;
}

/* Get_Theta_Ice */
static void get_theta_ice(double HNO3, double HCl, double HBr, double TEMP, ss_het_t* H) {
  double KLangC1, KLangC2, KlinC, denom;
  KlinC = 7.5e-5 * exp(4585.0 / TEMP);
  KLangC1 = KlinC / 2.7e+14;
  KlinC = 1.3e-5 * exp(4600.0 / TEMP);
  KLangC2 = KlinC / 3.0e+14;
  denom = 1.0 + KLangC1 * HNO3 + KLangC2 * HCl;
  H->HNO3_theta = KLangC1 * HNO3 / denom;
  H->HCl_theta = KLangC2 * HCl / denom;
  H->HBr_theta = 4.14e-10 * pow(HBr, 0.88);
  H->HBr_theta = fmin(H->HBr_theta, 1.0);
}

/* Get_Halide_CldConc */
static void get_halide_cldconc(const ss_het_t* H, double HBr, double HCl, double TEMP, double* Br_conc,
                               double* Cl_conc) {
  double V_tot, F_L, L2G;
  V_tot = H->VLiq;
  V_tot = ss_SafeDiv(V_tot, H->CldFr, 0.0);
  if (V_tot < 1.0e-20) {
    *Br_conc = 0.0;
    *Cl_conc = 0.0;
    return;
  }
  L2G = compute_l2g_local(1.0, 9000.0, -6.3, TEMP, V_tot, H->pHCloud);
  F_L = L2G / (1.0 + L2G);
  *Cl_conc = F_L * HCl / (V_tot * H->AVO * 1.0e-3);
  L2G = compute_l2g_local(7.5e-1, 10200.0, -9.0, TEMP, V_tot, H->pHCloud);
  F_L = L2G / (1.0 + L2G);
  *Br_conc = F_L * HBr / (V_tot * H->AVO * 1.0e-3);
}

/* Get_Halide_SsaConc */
static double get_halide_ssaconc(double n_x, double surf_area, double r_w) {
  double V_tot = (surf_area * r_w / 3.0) * 1e-3;
  double conc_x;
  if (V_tot <= 1.0e-20) return 0.0;
  conc_x = (n_x / S_AVO) / V_tot;
  return fmax(conc_x, 0.0);
}

/* Halide_Conc */
static void halide_conc(const double* C, long long ldc, double TEMP, ss_het_t* H) {
  double Br_conc, Cl_conc, denom, HBr, HCl;
  const double cHBr = ss_C(C, ldc, OSS_HBr), cBrSALA = ss_C(C, ldc, OSS_BrSALA), cBrSALC = ss_C(C, ldc, OSS_BrSALC);
  const double cHCl = ss_C(C, ldc, OSS_HCl), cSALACL = ss_C(C, ldc, OSS_SALACL), cSALCCL = ss_C(C, ldc, OSS_SALCCL);
  const double cNIT = ss_C(C, ldc, OSS_NIT), cNITs = ss_C(C, ldc, OSS_NITs), cSO4 = ss_C(C, ldc, OSS_SO4);
  H->Br_conc_CldG = H->Br_conc_CldA = H->Br_conc_CldC = 0.0;
  H->Br_over_Cl_Cld = H->Br_over_Cl_SSA = H->Br_over_Cl_SSC = 0.0;
  H->Cl_conc_CldG = H->Cl_conc_CldA = H->Cl_conc_CldC = 0.0;
  H->frac_Br_CldA = H->frac_Br_CldC = H->frac_Br_CldG = 0.0;
  H->frac_Cl_CldA = H->frac_Cl_CldC = H->frac_Cl_CldG = 0.0;

  HBr = cHBr + (cBrSALA * 0.7) + cBrSALC;
  HCl = cHCl + (cSALACL * 0.7) + cSALCCL;
  get_halide_cldconc(H, HBr, HCl, TEMP, &Br_conc, &Cl_conc);

  denom = cHBr + (cBrSALA * 0.7) + cBrSALC;
  if (denom > 0.0) {
    H->Br_conc_CldG = (Br_conc * cHBr) / denom;
    H->Br_conc_CldA = (Br_conc * cBrSALA * 0.7) / denom;
    H->Br_conc_CldC = (Br_conc * cBrSALC) / denom;
  }
  denom = cHCl + (cSALACL * 0.7) + cSALCCL;
  if (denom > 0.0) {
    H->Cl_conc_CldG = (Cl_conc * cHCl) / denom;
    H->Cl_conc_CldA = (Cl_conc * cSALACL * 0.7) / denom;
    H->Cl_conc_CldC = (Cl_conc * cSALCCL) / denom;
  }
  H->Br_conc_Cld = H->Br_conc_CldA + H->Br_conc_CldC + H->Br_conc_CldG;
  H->Cl_conc_Cld = H->Cl_conc_CldA + H->Cl_conc_CldC + H->Cl_conc_CldG;
  if (H->Br_conc_Cld > 0.0) {
    H->frac_Br_CldA = H->Br_conc_CldA / H->Br_conc_Cld;
    H->frac_Br_CldC = H->Br_conc_CldC / H->Br_conc_Cld;
    H->frac_Br_CldG = H->Br_conc_CldG / H->Br_conc_Cld;
  }
  if (H->Cl_conc_Cld > 0.0) {
    H->frac_Cl_CldA = H->Cl_conc_CldA / H->Cl_conc_Cld;
    H->frac_Cl_CldC = H->Cl_conc_CldC / H->Cl_conc_Cld;
    H->frac_Cl_CldG = H->Cl_conc_CldG / H->Cl_conc_Cld;
  }
  H->Br_conc_SSA = get_halide_ssaconc(cBrSALA, H->aClArea, H->aClRadi);
  H->Br_conc_SSC = get_halide_ssaconc(cBrSALC, H->xArea[12], H->xRadi[12]);
  H->Cl_conc_SSA = get_halide_ssaconc(cSALACL, H->aClArea, H->aClRadi);
  H->Cl_conc_SSC = get_halide_ssaconc(cSALCCL, H->xArea[12], H->xRadi[12]);
  H->NIT_conc_SSA = get_halide_ssaconc(cNIT, H->aClArea, H->aClRadi);
  H->NIT_conc_SSC = get_halide_ssaconc(cNITs, H->xArea[12], H->xRadi[12]);
  if (H->Cl_conc_Cld > 0.0) H->Br_over_Cl_Cld = H->Br_conc_Cld / H->Cl_conc_Cld;
  if (H->Cl_conc_SSA > 0.0) H->Br_over_Cl_SSA = H->Br_conc_SSA / H->Cl_conc_SSA;
  if (H->Cl_conc_SSC > 0.0) H->Br_over_Cl_SSC = H->Br_conc_SSC / H->Cl_conc_SSC;
  if ((cSALACL + cNIT + cSO4) > 0.0)
    H->frac_SALACL = cSALACL / (cSALACL + cNIT + cSO4);
  else
    H->frac_SALACL = 0.0;
}

/* fullChem_SetStateHet for one cell: in/C/het point at the cell's column,
 * rows ldi/ldc/ldh apart. */
static void set_state_het_cell(const double* in, long long ldi, const double* C, long long ldc, double gamma_HO2,
                               int LPSCCHEM, int TurnOffHetRates, double* het, long long ldh) {
  ss_het_t H;
  int t;
#define IN(f) in[(long long)(f) * ldi]
  memset(&H, 0, sizeof(H));
  const int NA = 14;
  const double CLDF = IN(OHIN_CLDF), QI = IN(OHIN_QI), QL = IN(OHIN_QL), TEMP = IN(OHIN_T);
  H.AVO = S_AVO;
  H.PI = S_PI;
  H.CldFr = fmin(fmax(CLDF, 0.0), 1.0);
  H.ClearFr = 1.0 - H.CldFr;
  H.QICE = QI;
  H.QLIQ = QL;
  H.vAir = IN(OHIN_AIRVOL) * 1.0e6;
  H.nAeroType = NA;
  H.aClArea = IN(OHIN_aClArea);
  H.aClRadi = IN(OHIN_aClRadi);
  H.aClVol = H.aClArea * H.aClRadi / 3.0;
  H.AWATER[0] = IN(OHIN_IsorropAeroH2O);
  H.AWATER[1] = IN(OHIN_IsorropAeroH2O + 1);
  for (t = 1; t <= NA; ++t) {
    H.xArea[t] = IN(OHIN_AeroArea + t - 1);
    H.xRadi[t] = IN(OHIN_AeroRadi + t - 1);
    H.xVol[t] = H.xArea[t] * H.xRadi[t] / 3.0;
    H.wetArea[t] = IN(OHIN_WetAeroArea + t - 1);
    H.xH2O[t] = IN(OHIN_AeroH2O + t - 1) * 1.0e-6;
  }
  H.OMOC_POA = IN(OHIN_OMOC_POA);
  H.OMOC_OPOA = IN(OHIN_OMOC_OPOA);
  H.HSO3_aq = IN(OHIN_HSO3_aq);
  H.SO3_aq = IN(OHIN_SO3_aq);
  H.TSO3_aq = H.HSO3_aq + H.SO3_aq;
  H.frac_HSO3_aq = ss_SafeDiv(H.HSO3_aq, H.TSO3_aq, 0.0);
  H.frac_SO3_aq = ss_SafeDiv(H.SO3_aq, H.TSO3_aq, 0.0);
  H.HSO4_molal = IN(OHIN_IsorropBisulfate);
  H.NO3_molal = IN(OHIN_IsorropNitrate);
  H.SO4_molal = IN(OHIN_IsorropSulfate);
  H.H_plus = IN(OHIN_IsorropHplus);
  H.pHCloud = IN(OHIN_pHCloud);
  H.pHSSA[0] = IN(OHIN_IsorropAeropH);
  H.pHSSA[1] = IN(OHIN_IsorropAeropH + 1);
  H.H_conc_Sul = pow(10.0, -1.0 * H.pHSSA[0]);
  H.H_conc_LCl = pow(10.0, -1.0 * H.pHCloud);
  H.H_conc_ICl = pow(10.0, -4.5);
  H.H_conc_SSA = H.H_conc_Sul;
  H.H_conc_SSC = pow(10.0, -5.0);
  H.f_Alk_SSA = ss_SafeDiv(IN(OHIN_SALAAL), IN(OHIN_SALA), 0.0);
  H.f_Alk_SSA = fmax(fmin(H.f_Alk_SSA, 1.0), 0.0);
  H.f_Acid_SSA = 1.0 - H.f_Alk_SSA;
  H.f_Alk_SSC = ss_SafeDiv(IN(OHIN_SALCAL), IN(OHIN_SALC), 0.0);
  H.f_Alk_SSC = fmax(fmin(H.f_Alk_SSC, 1.0), 0.0);
  H.f_Acid_SSC = 1.0 - H.f_Alk_SSC;
  H.SSA_is_Alk = fabs(H.f_Alk_SSA) > 0.01;
  H.SSA_is_Acid = !H.SSA_is_Alk;
  H.SSC_is_Alk = fabs(H.f_Alk_SSC) > 0.01;
  H.SSC_is_Acid = !H.SSC_is_Alk;
  H.gamma_HO2 = gamma_HO2;
  H.fupdateHOBr = IN(OHIN_fupdateHOBr);
  H.fupdateHOCl = IN(OHIN_fupdateHOCl);
  H.HSO3m = ss_SafeDiv(IN(OHIN_HSO3_aq) * 1.0e-3 * H.AVO * QL * IN(OHIN_AIRDEN) * 1.0e-3, CLDF, 0.0);
  H.HSO3m = ss_SafeDiv(H.HSO3m, ss_C(C, ldc, OSS_SO2), 0.0);
  H.SO3mm = ss_SafeDiv(IN(OHIN_SO3_aq) * 1.0e-3 * H.AVO * QL * IN(OHIN_AIRDEN) * 1.0e-3, CLDF, 0.0);
  H.SO3mm = ss_SafeDiv(H.SO3mm, ss_C(C, ldc, OSS_SO2), 0.0);
  cld_params(IN(OHIN_AD), CLDF, IN(OHIN_FRLAND), IN(OHIN_FROCEAN), QI, QL, TEMP, &H);
  get_theta_ice(ss_C(C, ldc, OSS_HNO3), ss_C(C, ldc, OSS_HCl), ss_C(C, ldc, OSS_HBr), TEMP, &H);
  halide_conc(C, ldc, TEMP, &H);
  for (t = 1; t <= 11; ++t) H.KHETI_SLA[t] = IN(OHIN_KHETI_SLA + t - 1);
  H.stratBox = IN(OHIN_InStratosphere) != 0.0;
  H.pscBox = (LPSCCHEM != 0) && (IN(OHIN_STATE_PSC) >= 2.0) && H.stratBox;
  H.natSurface = H.pscBox && (ss_C(C, ldc, OSS_NIT) > 0.0);
  H.TurnOffHetRates = TurnOffHetRates != 0;

  /* the struct as rows of the HetState array */
#define OUT(f, v) het[(long long)(f) * ldh] = (v)
  OUT(OHET_AVO, H.AVO);
  OUT(OHET_natSurface, H.natSurface ? 1.0 : 0.0);
  OUT(OHET_pscBox, H.pscBox ? 1.0 : 0.0);
  OUT(OHET_stratBox, H.stratBox ? 1.0 : 0.0);
  OUT(OHET_NAEROTYPE, (double)H.nAeroType);
  OUT(OHET_aClArea, H.aClArea);
  OUT(OHET_aClRadi, H.aClRadi);
  OUT(OHET_aClVol, H.aClVol);
  OUT(OHET_aIce, H.AIce);
  OUT(OHET_aLiq, H.ALiq);
  OUT(OHET_aWater, H.AWATER[0]);
  OUT(OHET_aWater + 1, H.AWATER[1]);
  OUT(OHET_Br_conc_CldA, H.Br_conc_CldA);
  OUT(OHET_Br_conc_CldC, H.Br_conc_CldC);
  OUT(OHET_Br_conc_CldG, H.Br_conc_CldG);
  OUT(OHET_Br_conc_Cld, H.Br_conc_Cld);
  OUT(OHET_Br_conc_SSA, H.Br_conc_SSA);
  OUT(OHET_Br_conc_SSC, H.Br_conc_SSC);
  OUT(OHET_Br_over_Cl_Cld, H.Br_over_Cl_Cld);
  OUT(OHET_Br_over_Cl_SSA, H.Br_over_Cl_SSA);
  OUT(OHET_Br_over_Cl_SSC, H.Br_over_Cl_SSC);
  OUT(OHET_Cl_conc_CldA, H.Cl_conc_CldA);
  OUT(OHET_Cl_conc_CldC, H.Cl_conc_CldC);
  OUT(OHET_Cl_conc_CldG, H.Cl_conc_CldG);
  OUT(OHET_Cl_conc_Cld, H.Cl_conc_Cld);
  OUT(OHET_Cl_conc_SSA, H.Cl_conc_SSA);
  OUT(OHET_Cl_conc_SSC, H.Cl_conc_SSC);
  OUT(OHET_cldFr, H.CldFr);
  OUT(OHET_clearFr, H.ClearFr);
  OUT(OHET_frac_Br_CldA, H.frac_Br_CldA);
  OUT(OHET_frac_Br_CldC, H.frac_Br_CldC);
  OUT(OHET_frac_Br_CldG, H.frac_Br_CldG);
  OUT(OHET_frac_Cl_CldA, H.frac_Cl_CldA);
  OUT(OHET_frac_Cl_CldC, H.frac_Cl_CldC);
  OUT(OHET_frac_Cl_CldG, H.frac_Cl_CldG);
  OUT(OHET_frac_HSO3_aq, H.frac_HSO3_aq);
  OUT(OHET_frac_SALACL, H.frac_SALACL);
  OUT(OHET_frac_SO3_aq, H.frac_SO3_aq);
  OUT(OHET_fupdateHOBr, H.fupdateHOBr);
  OUT(OHET_fupdateHOCl, H.fupdateHOCl);
  OUT(OHET_gamma_HO2, H.gamma_HO2);
  OUT(OHET_H2O, 0.0);
  OUT(OHET_HBr_theta, H.HBr_theta);
  OUT(OHET_HCl_theta, H.HCl_theta);
  OUT(OHET_H_conc_ICl, H.H_conc_ICl);
  OUT(OHET_H_conc_LCl, H.H_conc_LCl);
  OUT(OHET_H_conc_SSA, H.H_conc_SSA);
  OUT(OHET_H_conc_SSC, H.H_conc_SSC);
  OUT(OHET_H_conc_Sul, H.H_conc_Sul);
  OUT(OHET_HNO3_theta, H.HNO3_theta);
  OUT(OHET_HSO3_aq, H.HSO3_aq);
  OUT(OHET_SO3_aq, H.SO3_aq);
  OUT(OHET_HSO3m, H.HSO3m);
  OUT(OHET_SO3mm, H.SO3mm);
  OUT(OHET_TSO3_aq, H.TSO3_aq);
  OUT(OHET_H_plus, H.H_plus);
  for (t = 1; t <= 11; ++t) OUT(OHET_KHETI_SLA + t - 1, H.KHETI_SLA[t]);
  OUT(OHET_HSO4_molal, H.HSO4_molal);
  OUT(OHET_NO3_molal, H.NO3_molal);
  OUT(OHET_SO4_molal, H.SO4_molal);
  OUT(OHET_NIT_conc_SSA, H.NIT_conc_SSA);
  OUT(OHET_NIT_conc_SSC, H.NIT_conc_SSC);
  OUT(OHET_PI, H.PI);
  OUT(OHET_pHCloud, H.pHCloud);
  OUT(OHET_pHSSA, H.pHSSA[0]);
  OUT(OHET_pHSSA + 1, H.pHSSA[1]);
  OUT(OHET_OMOC_POA, H.OMOC_POA);
  OUT(OHET_OMOC_OPOA, H.OMOC_OPOA);
  OUT(OHET_qIce, H.QICE);
  OUT(OHET_qLiq, H.QLIQ);
  OUT(OHET_rIce, H.rIce);
  OUT(OHET_rLiq, H.rLiq);
  OUT(OHET_f_Acid_SSA, H.f_Acid_SSA);
  OUT(OHET_f_Acid_SSC, H.f_Acid_SSC);
  OUT(OHET_f_Alk_SSA, H.f_Alk_SSA);
  OUT(OHET_f_Alk_SSC, H.f_Alk_SSC);
  OUT(OHET_SSA_is_Alk, H.SSA_is_Alk ? 1.0 : 0.0);
  OUT(OHET_SSA_is_Acid, H.SSA_is_Acid ? 1.0 : 0.0);
  OUT(OHET_SSC_is_Alk, H.SSC_is_Alk ? 1.0 : 0.0);
  OUT(OHET_SSC_is_Acid, H.SSC_is_Acid ? 1.0 : 0.0);
  OUT(OHET_vAir, H.vAir);
  OUT(OHET_vIce, H.VIce);
  OUT(OHET_vLiq, H.VLiq);
  for (t = 1; t <= 14; ++t) {
    OUT(OHET_wetArea + t - 1, H.wetArea[t]);
    OUT(OHET_xArea + t - 1, H.xArea[t]);
    OUT(OHET_xH2O + t - 1, H.xH2O[t]);
    OUT(OHET_xRadi + t - 1, H.xRadi[t]);
    OUT(OHET_xVol + t - 1, H.xVol[t]);
  }
  OUT(OHET_cloudBox, 0.0);
  OUT(OHET_fracOrgAer, 0.0);
  OUT(OHET_fracInorgAer, 0.0);
  OUT(OHET_TurnOffHetRates, H.TurnOffHetRates ? 1.0 : 0.0);
  OUT(OHET_SUNCOS, IN(OHIN_SUNCOS));
#undef OUT
#undef IN
}

void oracle_set_state_het_batch(int ncell, const double* in, long long ldi, const double* C, long long ldc,
                                double gamma_HO2, int LPSCCHEM, int TurnOffHetRates, double* het, long long ldh) {
  for (int cell = 0; cell < ncell; ++cell)
    set_state_het_cell(in + cell, ldi, C + cell, ldc, gamma_HO2, LPSCCHEM, TurnOffHetRates, het + cell, ldh);
}

/* Ars_L1K at NUMDEN and SR_TEMP */
static double ss_ars_l1k(double NUMDEN, double SR_TEMP, double area, double radius, double gamma, double srMw) {
  double dfkg;
  if (gamma < 1.0e-30 || radius < 1.0e-30) return 0.0;
  dfkg = (9.45E+17 / NUMDEN) * SR_TEMP * sqrt(3.472E-2 + 1.0 / (srMw * srMw));
  return area / ((radius / dfkg) + 2.749064E-4 * srMw / (gamma * SR_TEMP));
}

static int ss_is_safediv(double num, double denom) {
  int ediff = ss_exponent(num) - ss_exponent(denom);
  return !(ediff < -1020 || ediff > 1023 || denom == 0.0);
}

/* kIIR1Ltd */
static double ss_kiir1ltd(double concGas, double concEduct, double kISource) {
  const double HET_MIN_LIFE = 1.e-3, HET_MIN_RATE = 1.0 / 1.e-3;
  double kIGas, kIEduct, kII = 0.0, lifeA, lifeB;
  if (concEduct < 1.0) return kII;
  if (!ss_is_safediv(concGas * kISource, concEduct)) return kII;
  kIGas = kISource;
  kIEduct = kIGas * concGas / concEduct;
  kII = kIGas / concEduct;
  if (kIGas > 0.0) {
    lifeA = ss_SafeDiv(1.0, kIGas, 0.0);
    lifeB = ss_SafeDiv(1.0, kIEduct, 0.0);
    if ((lifeA < lifeB) && (lifeA < HET_MIN_LIFE))
      kII = ss_SafeDiv(HET_MIN_RATE, concEduct, 0.0);
    else if (lifeB < HET_MIN_LIFE)
      kII = ss_SafeDiv(HET_MIN_RATE, concGas, 0.0);
  }
  return kII;
}

/* fullchem_SulfurAqChem for one cell: K_MT(1:6) into kmt[0..5] */
static void sulfur_aq_cell(const double* in, long long ldi, const double* C, long long ldc, double TEMP,
                           double NUMDEN, double* kmt) {
#define IN(f) in[(long long)(f) * ldi]
  const double SR_TEMP = sqrt(TEMP);
  double k_ex = 0.0;
  int SALAAL_gt_0_1, SALCAL_gt_0_1, O3_gt_1e10;
  for (int k = 0; k < 6; ++k) kmt[k] = 0.0;
  SALAAL_gt_0_1 = ss_C(C, ldc, OSS_SALAAL) > 0.1;
  SALCAL_gt_0_1 = ss_C(C, ldc, OSS_SALCAL) > 0.1;
  O3_gt_1e10 = ss_C(C, ldc, OSS_O3) > 1.0e+10;
  if (SALAAL_gt_0_1 && O3_gt_1e10) {
    k_ex = ss_ars_l1k(NUMDEN, SR_TEMP, IN(OHIN_WetAeroArea + 10), IN(OHIN_AeroRadi + 10), 0.11, OSS_SRMW_SO2);
    kmt[0] = ss_kiir1ltd(ss_C(C, ldc, OSS_SO2), ss_C(C, ldc, OSS_SALAAL), k_ex) / ss_C(C, ldc, OSS_O3);
  }
  if (SALAAL_gt_0_1) {
    k_ex = ss_ars_l1k(NUMDEN, SR_TEMP, IN(OHIN_WetAeroArea + 10), IN(OHIN_AeroRadi + 10), 0.07, OSS_SRMW_HCl);
    kmt[1] = ss_kiir1ltd(ss_C(C, ldc, OSS_HCl), ss_C(C, ldc, OSS_SALAAL), k_ex);
  }
  if (SALAAL_gt_0_1) {
    k_ex = ss_ars_l1k(NUMDEN, SR_TEMP, IN(OHIN_WetAeroArea + 10), IN(OHIN_AeroRadi + 10), 0.5, OSS_SRMW_HNO3);
    kmt[2] = ss_kiir1ltd(ss_C(C, ldc, OSS_HNO3), ss_C(C, ldc, OSS_SALAAL), k_ex);
  }
  if (SALCAL_gt_0_1 && O3_gt_1e10) {
    k_ex = ss_ars_l1k(NUMDEN, SR_TEMP, IN(OHIN_WetAeroArea + 11), IN(OHIN_AeroRadi + 11), 0.11, OSS_SRMW_SO2);
    kmt[3] = ss_kiir1ltd(ss_C(C, ldc, OSS_SO2), ss_C(C, ldc, OSS_SALCAL), k_ex) / ss_C(C, ldc, OSS_O3);
  }
  if (SALCAL_gt_0_1) {
    k_ex = ss_ars_l1k(NUMDEN, SR_TEMP, IN(OHIN_WetAeroArea + 11), IN(OHIN_AeroRadi + 11), 0.07, OSS_SRMW_HCl);
    kmt[4] = ss_kiir1ltd(ss_C(C, ldc, OSS_HCl), ss_C(C, ldc, OSS_SALCAL), k_ex);
  }
  if (SALCAL_gt_0_1) {
    k_ex = ss_ars_l1k(NUMDEN, SR_TEMP, IN(OHIN_WetAeroArea + 11), IN(OHIN_AeroRadi + 11), 0.5, OSS_SRMW_HNO3);
    kmt[5] = ss_kiir1ltd(ss_C(C, ldc, OSS_HNO3), ss_C(C, ldc, OSS_SALCAL), k_ex);
  }
#undef IN
}

/* K_MT of every cell: temp/numden [n], kmt out [6][ldk] */
void oracle_sulfur_aq_rates_batch(int ncell, const double* in, long long ldi, const double* C, long long ldc,
                                  const double* temp, const double* numden, double* kmt, long long ldk) {
  for (int cell = 0; cell < ncell; ++cell) {
    double k[6];
    sulfur_aq_cell(in + cell, ldi, C + cell, ldc, temp[cell], numden[cell], k);
    for (int r = 0; r < 6; ++r) kmt[(long long)r * ldk + cell] = k[r];
  }
}

/* ------------------------------------------------------------------------
 * fullchem_SulfurCldChem -> SET_SO2, restated statement by statement:
 *   SET_SO2 (in-cloud branch)  KPP/fullchem/fullchem_SulfurChemFuncs.F90:865-1620
 *   GET_HPLUS                  :1635-1853
 *   kCO21 .. dkAA              :1867-3091 (one function each)
 *   CaCO3_PRECIP               :3106-3156
 *   AQCHEM_SO2                 :3171-3549
 *   AIRMW, AVO, ATM            Headers/physconstants.F90:26, 32, 70
 * Literals written without a kind suffix in the Fortran (e.g. Kc1 = 4.3e-7)
 * are default REAL: their value is the single-precision rounding, written
 * here as (double)<literal>f.
 */
#define S_AIRMW 28.9644
#define S_ATMPA 1.01325e+5

/* the temperature factor exp(D * (1/T - 1/298)) of the Henry and
 * dissociation constants of GET_HPLUS's functions */
static double so2_tf(double D, double T) { return exp(D * ((1.0 / T) - (1.0 / 298.0))); }

static double kCO21(double P, double T, double LWC, double HPLUS) {
  const double Kc1 = (double)4.3e-7f, Kc2 = (double)4.68e-11f, DhrKc1 = -1000.0, DhrKc2 = -1760.0;
  const double Hco2 = (double)3.4e-2f, Dhco2 = 2.44e+3, CO2 = 390.0e-6;
  double Hco2_T = Hco2 * so2_tf(Dhco2, T);
  double Kc1_T = Kc1 * so2_tf(DhrKc1, T);
  double Kc2_T = Kc2 * so2_tf(DhrKc2, T);
  double Hco2eff = Hco2_T * (1.0 + (Kc1_T / HPLUS) + ((Kc1_T * Kc2_T) / (HPLUS * HPLUS)));
  double xCO2 = 1.0 / (1.0 + (Hco2eff * 0.08205 * T * LWC));
  double pCO2 = CO2 * P * xCO2;
  return Hco2_T / HPLUS * Kc1_T * pCO2;
}

static double sq(double x) { return x * x; }

static double dkCO21(double P, double T, double LWC, double HPLUS) {
  const double Kc1 = (double)4.3e-7f, Kc2 = (double)4.68e-11f, DhrKc1 = -1000.0, DhrKc2 = -1760.0;
  const double Hco2 = (double)3.4e-2f, Dhco2 = 2.44e+3, CO2 = 390.0e-6;
  double Hco2_T = Hco2 * so2_tf(Dhco2, T);
  double Kc1_T = Kc1 * so2_tf(DhrKc1, T);
  double Kc2_T = Kc2 * so2_tf(DhrKc2, T);
  return Kc1_T * Hco2_T * CO2 * P *
         (Kc1_T * Kc2_T * Hco2_T * 0.08205 * T * LWC - Hco2_T * 0.08205 * T * LWC * HPLUS * HPLUS - HPLUS * HPLUS) /
         sq(Kc1_T * Kc2_T * Hco2_T * 0.08205 * T * LWC + Kc1_T * Hco2_T * 0.08205 * T * LWC * HPLUS +
            Hco2_T * 0.08205 * T * LWC * HPLUS * HPLUS + HPLUS * HPLUS);
}

static double kCO22(double P, double T, double LWC, double HPLUS) {
  const double Kc1 = (double)4.3e-7f, Kc2 = (double)4.68e-11f, DhrKc1 = -1000.0, DhrKc2 = -1760.0;
  const double Hco2 = (double)3.4e-2f, Dhco2 = 2.44e+3, CO2 = 390.0e-6;
  double Hco2_T = Hco2 * so2_tf(Dhco2, T);
  double Kc1_T = Kc1 * so2_tf(DhrKc1, T);
  double Kc2_T = Kc2 * so2_tf(DhrKc2, T);
  double Hco2eff = Hco2_T * (1.0 + (Kc1_T / HPLUS) + ((Kc1_T * Kc2_T) / (HPLUS * HPLUS)));
  double xCO2 = 1.0 / (1.0 + (Hco2eff * 0.08205 * T * LWC));
  double pCO2 = CO2 * P * xCO2;
  return Kc1_T * Kc2_T * Hco2_T / HPLUS / HPLUS * pCO2;
}

static double dkCO22(double P, double T, double LWC, double HPLUS) {
  const double Kc1 = (double)4.3e-7f, Kc2 = (double)4.68e-11f, DhrKc1 = -1000.0, DhrKc2 = -1760.0;
  const double Hco2 = (double)3.4e-2f, Dhco2 = 2.44e+3, CO2 = 390.0e-6;
  double Hco2_T = Hco2 * so2_tf(Dhco2, T);
  double Kc1_T = Kc1 * so2_tf(DhrKc1, T);
  double Kc2_T = Kc2 * so2_tf(DhrKc2, T);
  return -1.0 * Kc1_T * Kc2_T * Hco2_T * CO2 * P *
         (Kc1_T * Hco2_T * 0.08205 * T * LWC + 2.0 * Hco2_T * 0.08205 * T * LWC * HPLUS + 2.0 * HPLUS) /
         sq(Kc1_T * Kc2_T * Hco2_T * 0.08205 * T * LWC + Kc1_T * Hco2_T * 0.08205 * T * LWC * HPLUS +
            Hco2_T * 0.08205 * T * LWC * HPLUS * HPLUS + HPLUS * HPLUS);
}

static double kSO21(double P, double T, double LWC, double HPLUS, double SO2) {
  const double Ks1 = (double)1.3e-2f, Ks2 = (double)6.6e-8f, Hso2 = (double)1.23f, Dhso2 = 3.14e+3;
  const double DhrKso21 = 1960.0, DhrKso22 = 1500.0;
  double Hso2_T = Hso2 * so2_tf(Dhso2, T);
  double Ks1_T = Ks1 * so2_tf(DhrKso21, T);
  double Ks2_T = Ks2 * so2_tf(DhrKso22, T);
  double Hso2eff = Hso2_T * (1.0 + (Ks1_T / HPLUS) + ((Ks1_T * Ks2_T) / (HPLUS * HPLUS)));
  double xSO2 = 1.0 / (1.0 + (Hso2eff * 0.08205 * T * LWC));
  double pSO2 = SO2 * P * xSO2;
  return Hso2_T * Ks1_T * pSO2 / HPLUS;
}

static double dkSO21(double P, double T, double LWC, double HPLUS, double SO2) {
  const double Ks1 = (double)1.3e-2f, Ks2 = (double)6.6e-8f, Hso2 = (double)1.23f, Dhso2 = 3.14e+3;
  const double DhrKso21 = 1960.0, DhrKso22 = 1500.0;
  double Hso2_T = Hso2 * so2_tf(Dhso2, T);
  double Ks1_T = Ks1 * so2_tf(DhrKso21, T);
  double Ks2_T = Ks2 * so2_tf(DhrKso22, T);
  return Ks1_T * Hso2_T * SO2 * P *
         (Ks1_T * Ks2_T * Hso2_T * 0.08205 * T * LWC - Hso2_T * 0.08205 * T * LWC * HPLUS * HPLUS - HPLUS * HPLUS) /
         sq(Ks1_T * Ks2_T * Hso2_T * 0.08205 * T * LWC + Ks1_T * Hso2_T * 0.08205 * T * LWC * HPLUS +
            Hso2_T * 0.08205 * T * LWC * HPLUS * HPLUS + HPLUS * HPLUS);
}

static double kSO22(double P, double T, double LWC, double HPLUS, double SO2) {
  const double Ks1 = (double)1.3e-2f, Ks2 = (double)6.6e-8f, Hso2 = (double)1.23f, Dhso2 = 3.14e+3;
  const double DhrKso21 = 1960.0, DhrKso22 = 1500.0;
  double Hso2_T = Hso2 * so2_tf(Dhso2, T);
  double Ks1_T = Ks1 * so2_tf(DhrKso21, T);
  double Ks2_T = Ks2 * so2_tf(DhrKso22, T);
  double Hso2eff = Hso2_T * (1.0 + (Ks1_T / HPLUS) + ((Ks1_T * Ks2_T) / (HPLUS * HPLUS)));
  double xSO2 = 1.0 / (1.0 + (Hso2eff * 0.08205 * T * LWC));
  double pSO2 = SO2 * P * xSO2;
  return Ks1_T * Ks2_T * Hso2_T / HPLUS / HPLUS * pSO2;
}

static double dkSO22(double P, double T, double LWC, double HPLUS, double SO2) {
  const double Ks1 = (double)1.3e-2f, Ks2 = (double)6.6e-8f, Hso2 = (double)1.23f, Dhso2 = 3.14e+3;
  const double DhrKso21 = 1960.0, DhrKso22 = 1500.0;
  double Hso2_T = Hso2 * so2_tf(Dhso2, T);
  double Ks1_T = Ks1 * so2_tf(DhrKso21, T);
  double Ks2_T = Ks2 * so2_tf(DhrKso22, T);
  return -1.0 * Ks1_T * Ks2_T * Hso2_T * SO2 * P *
         (Ks1_T * Hso2_T * 0.08205 * T * LWC + 2.0 * Hso2_T * 0.08205 * T * LWC * HPLUS + 2.0 * HPLUS) /
         sq(Ks1_T * Ks2_T * Hso2_T * 0.08205 * T * LWC + Ks1_T * Hso2_T * 0.08205 * T * LWC * HPLUS +
            Hso2_T * 0.08205 * T * LWC * HPLUS * HPLUS + HPLUS * HPLUS);
}

static double kHNO3(double P, double T, double LWC, double HPLUS, double HNO3) {
  const double Kn1 = (double)15.4f, Hhno3 = (double)2.1e5f, Dhhno3 = 0.0, DhrKn1 = 8700.0;
  double Hhno3_T = Hhno3 * so2_tf(Dhhno3, T);
  double Kn1_T = Kn1 * so2_tf(DhrKn1, T);
  double Hhno3eff = Hhno3_T * (1.0 + (Kn1_T / HPLUS));
  double xHNO3 = 1.0 / (1.0 + (Hhno3eff * 0.08205 * T * LWC));
  double pHNO3 = HNO3 * P * xHNO3;
  return Hhno3_T * Kn1_T * pHNO3 / HPLUS;
}

static double dkHNO3(double P, double T, double LWC, double HPLUS, double HNO3) {
  const double Kn1 = (double)15.4f, Hhno3 = (double)2.1e5f, Dhhno3 = 0.0, DhrKn1 = 8700.0;
  double Hhno3_T = Hhno3 * so2_tf(Dhhno3, T);
  double Kn1_T = Kn1 * so2_tf(DhrKn1, T);
  return -1.0 * Kn1_T * Hhno3_T * HNO3 * P * (1.0 + Hhno3_T * 0.08205 * T * LWC) /
         sq(Kn1_T * Hhno3_T * 0.08205 * T * LWC + Hhno3_T * 0.08205 * T * LWC * HPLUS + HPLUS);
}

static double kHCl(double P, double T, double LWC, double HPLUS, double Cl) {
  const double Kcl = 1.74e+6, Hcl = 1.5e+3, Dhcl = 2.3e+3, DhrKcl = 6900.0;
  double Hcl_T = Hcl * so2_tf(Dhcl, T);
  double Kcl_T = Kcl * so2_tf(DhrKcl, T);
  double Hcleff = Hcl_T * (1.0 + (Kcl_T / HPLUS));
  double xCl = 1.0 / (1.0 + (Hcleff * 0.08205 * T * LWC));
  double pHCl = Cl * P * xCl;
  return Hcl_T * Kcl_T * pHCl / HPLUS;
}

static double dkHCl(double P, double T, double LWC, double HPLUS, double Cl) {
  const double Kcl = 1.74e+6, Hcl = 1.5e+3, Dhcl = 2.3e+3, DhrKcl = 6900.0;
  double Hcl_T = Hcl * so2_tf(Dhcl, T);
  double Kcl_T = Kcl * so2_tf(DhrKcl, T);
  return -1.0 * Kcl_T * Hcl_T * Cl * P * (1.0 + Hcl_T * 0.08205 * T * LWC) /
         sq(Kcl_T * Hcl_T * 0.08205 * T * LWC + Hcl_T * 0.08205 * T * LWC * HPLUS + HPLUS);
}

static double kNH3(double P, double T, double LWC, double HPLUS, double NH3, double Kw) {
  const double Ka1 = (double)1.7e-5f, Hnh3 = 60.0, Dhnh3 = 4200.0, DhrKa1 = -450.0;
  double Hnh3_T = Hnh3 * so2_tf(Dhnh3, T);
  double Ka1_T = Ka1 * so2_tf(DhrKa1, T);
  double Hnh3eff = Hnh3_T * (1.0 + ((Ka1_T * HPLUS) / Kw));
  double xNH3 = 1.0 / (1.0 + (Hnh3eff * 0.08205 * T * LWC));
  double pNH3 = NH3 * P * xNH3;
  return HPLUS * Hnh3_T * Ka1_T * pNH3 / Kw;
}

static double dkNH3(double P, double T, double LWC, double HPLUS, double NH3, double Kw) {
  const double Ka1 = (double)1.7e-5f, Hnh3 = 60.0, Dhnh3 = 4200.0, DhrKa1 = -450.0;
  double Hnh3_T = Hnh3 * so2_tf(Dhnh3, T);
  double Ka1_T = Ka1 * so2_tf(DhrKa1, T);
  return Ka1_T * Hnh3_T * NH3 * Kw * P * (1.0 + Hnh3_T * 0.08205 * T * LWC) /
         sq(Hnh3_T * 0.08205 * T * LWC * (Kw + Ka1_T * HPLUS) + Kw);
}

static double kFA(double P, double T, double LWC, double HPLUS, double FA) {
  const double Kformate = 1.8e-4, Hfa = 8800.0, Dhfa = 6100.0, DhrKfa = 151.0;
  double Hfa_T = Hfa * so2_tf(Dhfa, T);
  double Kfa_T = Kformate * so2_tf(DhrKfa, T);
  double Hfaeff = Hfa_T * (1.0 + (Kfa_T / HPLUS));
  double xFA = 1.0 / (1.0 + (Hfaeff * 0.08205 * T * LWC));
  double pFA = FA * P * xFA;
  return Hfa_T * Kfa_T * pFA / HPLUS;
}

static double dkFA(double P, double T, double LWC, double HPLUS, double FA) {
  const double Kformate = 1.8e-4, Hfa = 8800.0, Dhfa = 6100.0, DhrKfa = 151.0;
  double Hfa_T = Hfa * so2_tf(Dhfa, T);
  double Kfa_T = Kformate * so2_tf(DhrKfa, T);
  return -1.0 * Kfa_T * Hfa_T * FA * P * (1.0 + Hfa_T * 0.08205 * T * LWC) /
         sq(Kfa_T * Hfa_T * 0.08205 * T * LWC + Hfa_T * 0.08205 * T * LWC * HPLUS + HPLUS);
}

static double kAA(double P, double T, double LWC, double HPLUS, double AA) {
  const double Kacetate = 1.75e-5, Haa = 4100.0, Dhaa = 6200.0, DhrKaa = 50.0;
  double Haa_T = Haa * so2_tf(Dhaa, T);
  double Kaa_T = Kacetate * so2_tf(DhrKaa, T);
  double Haaeff = Haa_T * (1.0 + (Kaa_T / HPLUS));
  double xAA = 1.0 / (1.0 + (Haaeff * 0.08205 * T * LWC));
  double pAA = AA * P * xAA;
  return Haa_T * Kaa_T * pAA / HPLUS;
}

static double dkAA(double P, double T, double LWC, double HPLUS, double AA) {
  const double Kacetate = 1.75e-5, Haa = 4100.0, Dhaa = 6200.0, DhrKaa = 50.0;
  double Haa_T = Haa * so2_tf(Dhaa, T);
  double Kaa_T = Kacetate * so2_tf(DhrKaa, T);
  return -1.0 * Kaa_T * Haa_T * AA * P * (1.0 + Haa_T * 0.08205 * T * LWC) /
         sq(Kaa_T * Haa_T * 0.08205 * T * LWC + Haa_T * 0.08205 * T * LWC * HPLUS + HPLUS);
}

static void CaCO3_PRECIP(double P, double T, double HPLUS, double* fCa, double* dCa) {
  const double Kc1 = 4.3e-7, Kc2 = 4.68e-11, DhrKc1 = -1000.0, DhrKc2 = -1760.0;
  const double Hco2 = 3.4e-2, Dhco2 = 2.44e+3, CO2 = 390.0e-6, Ksp = 3.3e-9, DHrKsp = -1200.0;
  double Hco2_T = Hco2 * so2_tf(Dhco2, T);
  double Kc1_T = Kc1 * so2_tf(DhrKc1, T);
  double Kc2_T = Kc2 * so2_tf(DhrKc2, T);
  double Ksp_T = Ksp * so2_tf(DHrKsp, T);
  *fCa = Ksp_T * HPLUS * HPLUS / (Kc1_T * Kc2_T * Hco2_T * CO2 * P);
  *dCa = 2.0 * Ksp_T * HPLUS / (Kc1_T * Kc2_T * Hco2_T * CO2 * P);
}

/* Newton iteration on the cloud water's electroneutrality; returns [H+] */
static double GET_HPLUS(double SO4nss, double HMSc, double TNH3, double TNO3, double SO2, double CL, double TNA,
                        double TDCA, double TFA, double TAA, double T, double PRES, double LWC, double iHPLUS,
                        int* niter) {
  const double Kw = 1.0e-14, DhrKw = -6710.0, MINVAL_ = (double)0.01f;
  double D, Kw_T, ipH, newpH, nHPLUS;
  double fHCO3, fCO3, fHSO3, fSO3, fHNO3, fNH4, fHCl, fFA, fAA;
  double dHCO3, dCO3, dHSO3, dSO3, dHNO3, dNH4, dHCl, dFA, dAA;
  double f, df, nnHPLUS, fCa, dCa;
  int count;
  ipH = -log10(iHPLUS);
  D = (2.0 * SO4nss) - TNA - (2.0 * TDCA) + (1.0 * HMSc);
  (void)D;
  Kw_T = Kw * exp(DhrKw * ((1.0 / T) - (1.0 / 298.0)));
  newpH = 0.0;
  count = 0;
  while (fabs(ipH - newpH) > MINVAL_) {
    count = count + 1;
    if (count != 1) ipH = newpH;
    nHPLUS = pow(10.0, -ipH);
    fHCO3 = kCO21(PRES, T, LWC, nHPLUS);
    fCO3 = kCO22(PRES, T, LWC, nHPLUS);
    fHSO3 = kSO21(PRES, T, LWC, nHPLUS, SO2);
    fSO3 = kSO22(PRES, T, LWC, nHPLUS, SO2);
    fHNO3 = kHNO3(PRES, T, LWC, nHPLUS, TNO3);
    fNH4 = kNH3(PRES, T, LWC, nHPLUS, TNH3, Kw_T);
    fHCl = kHCl(PRES, T, LWC, nHPLUS, CL);
    fFA = kFA(PRES, T, LWC, nHPLUS, TFA);
    fAA = kAA(PRES, T, LWC, nHPLUS, TAA);
    dHCO3 = dkCO21(PRES, T, LWC, nHPLUS);
    dCO3 = dkCO22(PRES, T, LWC, nHPLUS);
    dHSO3 = dkSO21(PRES, T, LWC, nHPLUS, SO2);
    dSO3 = dkSO22(PRES, T, LWC, nHPLUS, SO2);
    dHNO3 = dkHNO3(PRES, T, LWC, nHPLUS, TNO3);
    dNH4 = dkNH3(PRES, T, LWC, nHPLUS, TNH3, Kw_T);
    dHCl = dkHCl(PRES, T, LWC, nHPLUS, CL);
    dFA = dkFA(PRES, T, LWC, nHPLUS, TFA);
    dAA = dkAA(PRES, T, LWC, nHPLUS, TAA);
    CaCO3_PRECIP(PRES, T, nHPLUS, &fCa, &dCa);
    if (fCa >= TDCA) {
      D = (2.0 * SO4nss) - (TNA + 2.0 * TDCA);
      f = D - nHPLUS + Kw / nHPLUS + fHCO3 + 2.0 * fCO3 + fHSO3 + 2.0 * fSO3 + fHNO3 - fNH4 + fHCl + fFA + fAA;
      df = -1.0 - Kw / nHPLUS / nHPLUS + dHCO3 + 2.0 * dCO3 + dHSO3 + 2.0 * dSO3 + dHNO3 - dNH4 + dHCl + dFA + dAA;
    } else {
      D = (2.0 * SO4nss) - TNA;
      f = D - nHPLUS + Kw / nHPLUS + fHCO3 + 2.0 * fCO3 + fHSO3 + 2.0 * fSO3 + fHNO3 - fNH4 + fHCl + fFA + fAA -
          2.0 * fCa;
      df = -1.0 - Kw / nHPLUS / nHPLUS + dHCO3 + 2.0 * dCO3 + dHSO3 + 2.0 * dSO3 + dHNO3 - dNH4 + dHCl + dFA + dAA -
           2.0 * dCa;
    }
    nnHPLUS = nHPLUS - f / df;
    nnHPLUS = fmax(nnHPLUS, 1.0e-14);
    nnHPLUS = fmin(nnHPLUS, 1.0e-1);
    if (count > 50) {
      newpH = ((-log10(nnHPLUS)) + (-log10(nHPLUS))) / 2.0;
      break; /* the reference stops the model when newpH is NaN */
    } else {
      newpH = -log10(nnHPLUS);
      if (isnan(newpH)) break;
    }
  }
  *niter = count;
  return pow(10.0, -newpH);
}

typedef struct {
  double KaqH2O2, KaqO3, KaqO3_1, KaqO2, HSO3aq, SO3aq, KaqHCHO, KaqHMS, KaqHMS2;
} so2_aq_t;

static void AQCHEM_SO2(double LWC, double T, double P, double SO2, double H2O2, double O3, double HCHO,
                       double Hplus, double MnII, double FeIII, so2_aq_t* o) {
  const double R = 0.08205, dOH = 1.0e-19;
  double KH2O2, Ks1, Ks2, HCSO2, FHCSO2, XSO2g, SIV, XSO2aq, XHSO3, XSO3, Kh1, HCH2O2, FHCH2O2, XH2O2g;
  double KO0, KO1, KO2, HCO3, XO3g, XHCHOg, HCHCHO, FHCHCHO, KHCHO1, KHCHO2, KHMS, Kw1, Khc1, KHMS2;
  (void)O3;
  (void)H2O2;
  (void)HCHO;
  KH2O2 = 6.31e+14 * exp(-4.76e+3 / T);
  Ks1 = 1.30e-2 * exp(6.75 * (298.15 / T - 1.0));
  Ks2 = 6.31e-8 * exp(5.05 * (298.15 / T - 1.0));
  XSO2aq = 1.0 / (1.0 + Ks1 / Hplus + Ks1 * Ks2 / (Hplus * Hplus));
  XHSO3 = 1.0 / (1.0 + Hplus / Ks1 + Ks2 / Hplus);
  XSO3 = 1.0 / (1.0 + Hplus / Ks2 + Hplus * Hplus / (Ks1 * Ks2));
  HCSO2 = 1.22 * exp(10.55 * (298.15 / T - 1.0));
  FHCSO2 = HCSO2 * (1.0 + (Ks1 / Hplus) + (Ks1 * Ks2 / (Hplus * Hplus)));
  XSO2g = 1.0 / (1.0 + (FHCSO2 * R * T * LWC));
  SIV = FHCSO2 * XSO2g * SO2 * P;
  o->HSO3aq = SIV * XHSO3;
  o->SO3aq = SIV * XSO3;
  Kh1 = 2.20e-12 * exp(-12.52 * (298.15 / T - 1.0));
  HCH2O2 = 7.45e+4 * exp(22.21 * (298.15 / T - 1.0));
  FHCH2O2 = HCH2O2 * (1.0 + (Kh1 / Hplus));
  XH2O2g = 1.0 / (1.0 + (FHCH2O2 * R * T * LWC));
  o->KaqH2O2 = KH2O2 * Ks1 * FHCH2O2 * HCSO2 * XH2O2g * XSO2g * P * LWC * R * T;
  KO0 = 2.40e+4;
  KO1 = 3.49e+12 * exp(-4.83e+3 / T);
  KO2 = 7.32e+14 * exp(-4.03e+3 / T);
  HCO3 = 1.13e-2 * exp(8.51 * (298.15 / T - 1.0));
  XO3g = 1.0 / (1.0 + (HCO3 * R * T * LWC));
  o->KaqO3 = (KO0 * XSO2aq + KO1 * XHSO3 + KO2 * XSO3) * FHCSO2 * XSO2g * P * HCO3 * XO3g * LWC * R * T;
  o->KaqO3_1 = KO2 * XSO3 * FHCSO2 * XSO2g * P * HCO3 * XO3g * LWC * R * T;
  o->KaqO2 = FHCSO2 * XSO2g * ((750.0 * MnII) + (2600.0 * FeIII) + (1e+10 * MnII * FeIII)) * LWC * R * T;
  KHCHO1 = 7.9e+2 * exp(-16.44 * (298.15 / T - 1.0));
  KHCHO2 = 2.5e+7 * exp(-6.04 * (298.15 / T - 1.0));
  KHMS = 3.6e+3 * exp(-15.09 * (298.15 / T - 1.0));
  KHMS2 = 2.65e+8 * exp(-5.03 * (298.15 / T - 1.0));
  Khc1 = 2.53e+3 * exp(13.48 * (298.15 / T - 1.0));
  Kw1 = 1e-14 * exp(-22.51 * (298.15 / T - 1.0));
  HCHCHO = 2.5 * exp(21.6 * (298.15 / T - 1.0));
  FHCHCHO = HCHCHO * (1.0 + Khc1);
  XHCHOg = 1.0 / (1.0 + (FHCHCHO * R * T * LWC));
  o->KaqHCHO = (KHCHO1 * XHSO3 + KHCHO2 * XSO3) * FHCSO2 * XSO2g * P * HCHCHO * XHCHOg * LWC * R * T;
  o->KaqHMS = KHMS * (Kw1 / Hplus) * 0.7;
  o->KaqHMS2 = KHMS2 * dOH * 0.7;
}

/* SET_SO2 for one cell: K_CLD(1:6) into kcld[6]; HSO3_aq, SO3_aq, pHCloud
 * into *hso3, *so3, *phcloud; size_res and the GET_HPLUS iteration count
 * (0 outside the cloud branch) into *size_res, *niter. */
static void set_so2_cell(const double* in, long long ldi, const double* C, long long ldc, int lmetalcatso2,
                         double* kcld, double* hso3, double* so3, double* phcloud, int* size_res, int* niter) {
#define IN(f) in[(long long)(f) * ldi]
  const double HPLUS_45 = 3.16227766016837953e-5, MINDAT = 1.e-20;
  double RHO, CNVFAC, SO20, SO2_AfterSS, H2O20, PATM, TK, FC, LWC;
  double SO4nss, HMSc, TNH3, CL, TFA, TAA, TNA, DUST, TDCA, TNO3, GNO3, HPLUS;
  double FeIII, MnII, Fe_nat, Mn_nat, Fe_ant, Mn_ant, Mn_tot, Mn_d, Fe_d_ant, Fe_d_nat, Fe_d;
  double ALKdst, ALKss, ALKds, NH3;
  so2_aq_t aq;
  int sr = 0;
  *hso3 = 1.0e-32;
  *so3 = 1.0e-32;
  *phcloud = 0.0;
  *niter = 0;
  for (int k = 0; k < 6; ++k) kcld[k] = 0.0;
  RHO = IN(OHIN_AIRDEN);
  CNVFAC = 1.E3 * S_AIRMW / (RHO * S_AVO);
  SO20 = ss_C(C, ldc, OSS_SO2) * CNVFAC;
  SO2_AfterSS = ss_C(C, ldc, OSS_SO2) * CNVFAC;
  H2O20 = ss_C(C, ldc, OSS_H2O2) * CNVFAC;
  PATM = IN(OHIN_PMID_DRY) / (S_ATMPA * 1.e-2);
  TK = IN(OHIN_T);
  FC = IN(OHIN_CLDF);
  LWC = IN(OHIN_QL) * IN(OHIN_AIRDEN) * 1e-3;
  LWC = fmax(0.0, LWC);
  LWC = ss_SafeDiv(LWC, FC, 0.0);
  if ((FC > 1.0e-4) && (SO2_AfterSS > MINDAT) && (TK > 258.0) && (LWC > 1.0e-20)) {
    SO4nss = 1.e+3 * (ss_C(C, ldc, OSS_SO4) * 0.7 + ss_C(C, ldc, OSS_SO4s)) / (LWC * S_AVO);
    HMSc = 1.e+3 * ss_C(C, ldc, OSS_HMS) * 0.7 / (LWC * S_AVO);
    TNH3 = ((IN(OHIN_NH4) * 0.7) + IN(OHIN_NH3)) * CNVFAC;
    CL = (ss_C(C, ldc, OSS_SALACL) * 0.7) + ss_C(C, ldc, OSS_SALCCL);
    CL = (CL + ss_C(C, ldc, OSS_HCl)) * CNVFAC;
    TFA = ss_C(C, ldc, OSS_HCOOH) * CNVFAC;
    TAA = ss_C(C, ldc, OSS_ACTA) * CNVFAC;
    TNA = 1.e3 * (IN(OHIN_SALA) * 0.7 + IN(OHIN_SALC)) * (31.6 * 0.359 / 23.0) / (LWC * S_AVO);
    DUST = (IN(OHIN_DSTbin) + IN(OHIN_DSTbin + 1) + IN(OHIN_DSTbin + 2) + IN(OHIN_DSTbin + 3) +
            IN(OHIN_DSTbin + 4) + IN(OHIN_DSTbin + 5) + IN(OHIN_DSTbin + 6)) *
           1.e+15 * OSS_MW_DSTbin1 / S_AVO;
    TDCA = DUST * 2.22e-15 / LWC;
    TNO3 = (ss_C(C, ldc, OSS_HNO3) + (ss_C(C, ldc, OSS_NIT) * 0.7) + ss_C(C, ldc, OSS_NITs)) * CNVFAC;
    GNO3 = ss_C(C, ldc, OSS_HNO3) * CNVFAC;
    HPLUS = GET_HPLUS(SO4nss, HMSc, TNH3, TNO3, SO2_AfterSS, CL, TNA, TDCA, TFA, TAA, TK, PATM, LWC, HPLUS_45,
                      niter);
    *phcloud = -1.0 * log10(HPLUS);
    FeIII = 0.0;
    MnII = 0.0;
    if (lmetalcatso2) {
      Fe_nat = DUST * 35e-3;
      Mn_nat = Fe_nat / 50.0;
      Fe_ant = IN(OHIN_pFe) * CNVFAC * 1.e+12 * IN(OHIN_AD) / (S_AIRMW / OSS_MW_pFe) / IN(OHIN_AIRVOL);
      Mn_ant = Fe_ant / 10.0;
      Mn_tot = Mn_ant + Mn_nat;
      if (LWC > 0.0) {
        Mn_d = Mn_tot * 1e-9 / 54.94 / LWC * 1e-3;
        Mn_d = Mn_d * 0.5;
      } else {
        Mn_d = 0.0;
      }
      if (LWC > 0.0) {
        Fe_d_ant = Fe_ant * 1e-9 / OSS_MW_pFe / LWC * 1e-3;
        Fe_d_nat = Fe_nat * 1e-9 / OSS_MW_pFe / LWC * 1e-3;
        Fe_d = Fe_d_ant * 0.1 + Fe_d_nat * 0.01;
      } else {
        Fe_d = 0.0;
      }
      if (IN(OHIN_SUNCOS) > 0.0)
        FeIII = Fe_d * 0.1;
      else
        FeIII = Fe_d * 0.9;
      MnII = Mn_d;
    }
    AQCHEM_SO2(LWC, TK, PATM, SO2_AfterSS, ss_C(C, ldc, OSS_H2O2) * CNVFAC, ss_C(C, ldc, OSS_O3) * CNVFAC,
               ss_C(C, ldc, OSS_CH2O) * CNVFAC, HPLUS, MnII, FeIII, &aq);
    kcld[0] = aq.KaqH2O2 * FC * CNVFAC;
    kcld[1] = aq.KaqO3 * FC * CNVFAC;
    kcld[2] = aq.KaqO2 * FC;
    kcld[3] = aq.KaqHCHO * FC * CNVFAC;
    kcld[4] = aq.KaqHMS * FC;
    kcld[5] = aq.KaqHMS2 * FC / ss_C(C, ldc, OSS_SO2);
    ALKdst = (IN(OHIN_DSTbin) + IN(OHIN_DSTbin + 1) + IN(OHIN_DSTbin + 2) + IN(OHIN_DSTbin + 3) +
              IN(OHIN_DSTbin + 4) + IN(OHIN_DSTbin + 5) + IN(OHIN_DSTbin + 6)) *
             CNVFAC * 1.e+9 * IN(OHIN_AD) / (S_AIRMW / OSS_MW_DSTbin1) / IN(OHIN_AIRVOL);
    ALKss = (IN(OHIN_SALA) + IN(OHIN_SALC)) * CNVFAC * 1.e+9 * IN(OHIN_AD) / (S_AIRMW / OSS_MW_SALA) /
            IN(OHIN_AIRVOL);
    ALKds = ALKdst + ALKss;
    NH3 = IN(OHIN_NH3) * CNVFAC;
    sr = 0;
    if (H2O20 > SO2_AfterSS + 1e-9) {
      sr = 0;
    } else if (LWC < 0.1e-6) {
      sr = 1;
    } else if (GNO3 > NH3) {
      if (SO2_AfterSS >= 5.e-9 && H2O20 >= SO20) sr = 0;
      if (LWC >= 0.3e-6 && SO2_AfterSS >= 3.e-9 && H2O20 >= SO2_AfterSS) sr = 0;
      if (ALKds >= 5.0 && LWC >= 0.5e-6 && H2O20 >= SO2_AfterSS) sr = 0;
      if (LWC >= 0.1e-6 && GNO3 <= (NH3 + 2.e-9)) sr = 0;
    } else if (LWC >= 0.5e-6) {
      if (H2O20 >= (0.9 * SO2_AfterSS)) sr = 0;
      if (NH3 <= 1.e-9 && ALKds >= 5.0 && SO2_AfterSS <= 10.e-9) sr = 0;
    } else if (LWC >= 0.3e-6) {
      if (NH3 >= (GNO3 + 5.e-9) && SO2_AfterSS <= 10.e-9) sr = 0;
      if (GNO3 <= 1.e-9 && NH3 >= (GNO3 + 2.e-9)) sr = 0;
      if (GNO3 <= 7.e-9 && NH3 >= (GNO3 + 3.e-9)) sr = 0;
      if (ALKds >= 3.0 && NH3 <= 10e-9 && SO2_AfterSS <= 5e-9) sr = 0;
      if (ALKds >= 5.0 && NH3 <= 10.e-9 && SO2_AfterSS <= 5.e-9) sr = 0;
      if (SO2_AfterSS >= 1.5e-9 && H2O20 >= SO2_AfterSS) sr = 0;
      if (NH3 <= 12.e-9 && ALKds >= 10.0) sr = 0;
      if (NH3 <= 1.e-9 && ALKds >= 4.0 && SO2_AfterSS <= 10.e-9) sr = 0;
      if (NH3 <= 5.e-9 && ALKds >= 6.0 && SO2_AfterSS <= 10.e-9) sr = 0;
      if (NH3 <= 7.e-9 && ALKds > -8.0 && SO2_AfterSS <= 10.e-9) sr = 0;
    } else if (LWC >= 0.1e-6) {
      if (NH3 <= 1.e-9 && ALKds >= 5.0) sr = 0;
      if (NH3 <= 5.e-9 && ALKds >= 10.0) sr = 0;
      if (GNO3 <= 1.e-9 && NH3 >= (GNO3 + 2.e-9) && SO2_AfterSS <= 7.e-9) sr = 0;
      if (GNO3 <= 1.e-9 && NH3 >= (GNO3 + 2.e-9) && ALKds >= 2.0) sr = 0;
      if (GNO3 <= 3.e-9 && NH3 >= (GNO3 + 4.e-9)) sr = 0;
      if (GNO3 <= 7.e-9 && NH3 >= (GNO3 + 3.e-9) && SO2_AfterSS <= 5.e-9) sr = 0;
      if (GNO3 <= 7.e-9 && NH3 >= (GNO3 + 3.e-9) && ALKds >= 4.0 && SO2_AfterSS <= 9.e-9) sr = 0;
      if (ALKds >= 3.0 && NH3 <= 3.e-9 && SO2_AfterSS <= 4.e-9) sr = 0;
      if (ALKds >= 5.0 && SO2_AfterSS <= 5.e-9 && NH3 <= 7.e-9) sr = 0;
      if (NH3 >= (GNO3 + 2.e-9) && SO2_AfterSS <= 5.e-9) sr = 0;
      if (NH3 >= (GNO3 + 4.e-9) && SO2_AfterSS <= 10.e-9) sr = 0;
      if (ALKds >= 2.0 && NH3 <= 10.e-9 && H2O20 >= SO2_AfterSS) sr = 0;
      if (NH3 <= 1.e-9 && SO2_AfterSS >= 3.e-9 && H2O20 >= SO2_AfterSS) sr = 0;
    } else {
      sr = 1;
    }
    *hso3 = aq.HSO3aq;
    *so3 = aq.SO3aq;
  }
  *size_res = sr;
#undef IN
}

/* SET_SO2 for every cell (with Set_Sulfur_Chem_Rates' fupdateHOBr/HOCl = 1):
 * in/out hetin rows HSO3_aq, SO3_aq, pHCloud, fupdateHOBr, fupdateHOCl;
 * kcld [6][ldk] out; size_res/niter [n] out (either may be NULL). */
void oracle_sulfur_cld_rates_batch(int ncell, double* in, long long ldi, const double* C, long long ldc,
                                   int lmetalcatso2, double* kcld, long long ldk, int* size_res, int* niter) {
  for (int cell = 0; cell < ncell; ++cell) {
    double k[6], hso3, so3, ph;
    int sr, it;
    set_so2_cell(in + cell, ldi, C + cell, ldc, lmetalcatso2, k, &hso3, &so3, &ph, &sr, &it);
    for (int r = 0; r < 6; ++r) kcld[(long long)r * ldk + cell] = k[r];
    in[(long long)OHIN_HSO3_aq * ldi + cell] = hso3;
    in[(long long)OHIN_SO3_aq * ldi + cell] = so3;
    in[(long long)OHIN_pHCloud * ldi + cell] = ph;
    in[(long long)OHIN_fupdateHOBr * ldi + cell] = 1.0;
    in[(long long)OHIN_fupdateHOCl * ldi + cell] = 1.0;
    if (size_res) size_res[cell] = sr;
    if (niter) niter[cell] = it;
  }
}

/* ------------------------------------------------------------------------
 * fullchem_HetDropChem (KPP/fullchem/fullchem_SulfurChemFuncs.F90:414-790)
 * with WhenExpCantBeDone (:808-849), IsSafeExp / SafeExp (KPP/fullchem/
 * rateLawUtilFuncs.F90:497-523), called from Do_FullChem where
 * (GeosCore/fullchem_mod.F90:913-934) the box is cloudy (CLDF > 1e-4),
 * SET_SO2 set size_res, the surface is water, TEMP > 268.15 K and the
 * in-cloud liquid water content exceeds 1e-20; elsewhere SRHOCl = SRHOBr =
 * 0 (fullchem_mod.F90:575-577).  The four sulfite uptake laws come from the
 * oracle's rate laws (oracle_sulfite_uptakes, generated with Update_RCONST).
 * RG_S**3 and NINE_HALVES * LOG(SIG_S)**2 are constant expressions of
 * PARAMETERs, which the Fortran compiler folds with correct rounding of each
 * operation; their values are written out as such.
 */
void oracle_sulfite_uptakes(const double* met, const double* C, const double* het, long long ldh, double* out);

#define S_G0 9.80665
#define S_PI_PHYS 3.14159265358979323

static double when_exp_cant(double R1, double R2, double K, double DT) {
  double DIFF = R1 - R2;
  if (DIFF < 0.0) return R1;
  if (DIFF > 0.0) return R2;
  return R1 - 1.0 / (K * DT + (1.0 / R1));
}

static int is_safe_exp(double x) { return fabs(x) < 709.0; }

/* the second-order loss of R1 and R2 over DT at rate K (the XX1/XX2/XX4/XX5
 * blocks of the Fortran) */
static double loss2(double R1, double R2, double K, double DT) {
  double Arg = (R1 - R2) * (K * DT);
  if (is_safe_exp(Arg) && fabs(Arg) > 0.0) {
    double XX = exp(Arg);
    return (R1 * R2) * (XX - 1.0) / ((R1 * XX) - R2);
  }
  return when_exp_cant(R1, R2, K, DT);
}

static void het_drop_cell(const double* in, long long ldi, const double* c, long long ldc, const double* met,
                          long long ldm, const double* het, long long ldh, double DT, int size_res, double* srhocl,
                          double* srhobr) {
#define IN(f) in[(long long)(f) * ldi]
#define CC(s) ss_C(c, ldc, s)
  const double SS_DEN = 2200.0, RG_S3 = 0x1.2e3b40a0e9b4fp-64 /* (0.4e-6)**3 */;
  const double THREE_FOURTHS = 3.0 / 4.0, ARG_SS = 0x1.8e02146ec938fp+0 /* 9/2 * LOG(1.8)**2 */;
  double M[18], Cc[ORACLE_NSPEC], up[4];
  double CVF, DTCHEM, FC, R1, R2, K, Arg, XX, XX1, XX2, XX3, XX4, XX5, LST;
  double NH3, SO2, H2O2, HNO3, SO4, B, CNss, NDss, CN, W, APV, H, sum_gas, DSVI, SR, DENOM, LWC;
  double aB, aNH3, aSO2, aH2O2, aHNO3, aW, aCN, aSO4;
  double TEMP = met[0];
  *srhocl = 0.0;
  *srhobr = 0.0;
  if (!(IN(OHIN_CLDF) > 1.0e-4)) return;
  LWC = (IN(OHIN_QL) * IN(OHIN_AIRDEN) * 1.0e-3 / IN(OHIN_CLDF));
  if (!(size_res && IN(OHIN_IsWater) != 0.0 && TEMP > 268.15 && LWC > 1.0e-20)) return;
  for (int k = 0; k < 18; ++k) M[k] = met[(long long)k * ldm];
  for (int k = 0; k < ORACLE_NSPEC; ++k) Cc[k] = c[(long long)k * ldc];
  oracle_sulfite_uptakes(M, Cc, het, ldh, up);
  CVF = 1.0e3 * S_AIRMW / (IN(OHIN_AIRDEN) * S_AVO);
  DTCHEM = DT;
  FC = IN(OHIN_CLDF);
  R1 = CC(OSS_SO2) * CVF;
  R2 = CC(OSS_H2O2) * CVF;
  K = M[12] / CVF / FC;
  XX1 = loss2(R1, R2, K, DTCHEM);
  R2 = CC(OSS_O3) * CVF;
  K = M[13] / CVF / FC;
  XX2 = loss2(R1, R2, K, DTCHEM);
  K = -M[14] / FC;
  Arg = K * DTCHEM;
  XX3 = 0.0;
  if (is_safe_exp(Arg)) {
    XX = exp(Arg);
    XX3 = R1 * (1.0 - XX);
  }
  R1 = CC(OSS_SO2) * CVF * IN(OHIN_HSO3_aq);
  R2 = CC(OSS_HOCl) * CVF;
  K = up[0] / CVF;
  XX4 = loss2(R1, R2, K, DTCHEM);
  R1 = CC(OSS_SO2) * CVF * IN(OHIN_SO3_aq);
  K = up[1] / CVF;
  XX4 = XX4 + loss2(R1, R2, K, DTCHEM);
  R1 = CC(OSS_SO2) * CVF * IN(OHIN_HSO3_aq);
  R2 = CC(OSS_HOBr) * CVF;
  K = up[2] / CVF;
  XX5 = loss2(R1, R2, K, DTCHEM);
  R1 = CC(OSS_SO2) * CVF * IN(OHIN_SO3_aq);
  K = up[3] / CVF;
  XX5 = XX5 + loss2(R1, R2, K, DTCHEM);
  LST = XX1 + XX2 + XX3 + XX4 + XX5;
  if (LST > R1) {
    XX1 = (R1 * XX1) / LST;
    XX2 = (R1 * XX2) / LST;
    XX3 = (R1 * XX3) / LST;
    XX4 = (R1 * XX4) / LST;
    XX5 = (R1 * XX5) / LST;
    LST = XX1 + XX2 + XX3 + XX4 + XX5;
  }
  NH3 = IN(OHIN_NH3) * CVF * 1.0e+12;
  SO2 = fmax(CC(OSS_SO2) * CVF - (LST * FC), 1.0e-20) * 1.0e+12;
  H2O2 = CC(OSS_H2O2) * CVF * 1.0e12;
  HNO3 = CC(OSS_HNO3) * CVF * 1.0e12;
  SO4 = (CC(OSS_SO4) * CVF * IN(OHIN_AD) * 1.0e+9) / ((S_AIRMW / OSS_MW_SO4) * IN(OHIN_AIRVOL));
  B = (LST * IN(OHIN_AD) * 1.0e+9) / ((S_AIRMW / OSS_MW_SO4) * IN(OHIN_AIRVOL));
  CNss = IN(OHIN_SALC) * CVF * IN(OHIN_AD) / ((S_AIRMW / OSS_MW_SALC) * IN(OHIN_AIRVOL));
  NDss = (THREE_FOURTHS * CNss) / (S_PI_PHYS * SS_DEN * RG_S3 * (is_safe_exp(ARG_SS) ? exp(ARG_SS) : 0.0)) * 1.e-6;
  CN = NDss;
  if (SO2 <= 200.00) {
    aB = 0.5318; aNH3 = -1.67e-7; aSO2 = 2.59e-6; aH2O2 = -1.77e-7; aHNO3 = -1.72e-7; aW = 1.22e-6; aCN = 4.58e-6;
    aSO4 = -1.00e-5;
  } else if (SO2 > 200.00 && SO2 <= 500.0) {
    aB = 0.5591; aNH3 = 3.62e-6; aSO2 = 1.66e-6; aH2O2 = 1.06e-7; aHNO3 = -5.45e-7; aW = -5.79e-7; aCN = 1.63e-5;
    aSO4 = -7.40e-6;
  } else if (SO2 > 500.0 && SO2 < 1000.0) {
    aB = 1.1547; aNH3 = -4.28e-8; aSO2 = -1.23e-7; aH2O2 = -9.05e-7; aHNO3 = 1.73e-7; aW = 7.22e-6; aCN = 2.44e-5;
    aSO4 = 3.25e-5;
  } else {
    aB = 1.1795; aNH3 = 2.57e-7; aSO2 = -5.54e-7; aH2O2 = -1.08e-6; aHNO3 = 1.95e-6; aW = 6.14e-6; aCN = 1.64e-5;
    aSO4 = 2.48e-6;
  }
  W = -IN(OHIN_OMEGA) / (IN(OHIN_AIRDEN) * S_G0) * 100.0;
  APV = sqrt(IN(OHIN_U) * IN(OHIN_U) + IN(OHIN_V) * IN(OHIN_V)) + (W * W * 1.0e-4);
  H = DTCHEM * APV;
  sum_gas = (aNH3 * NH3) + (aSO2 * SO2) + (aH2O2 * H2O2) + (aHNO3 * HNO3);
  DSVI = (aB * B) + (((aCN * CN) + (aW * W) + (aSO4 * SO4) + sum_gas) * H);
  SR = 0.0;
  if (W > 0.0 && CC(OSS_SO2) > 0.0) {
    SR = fmax((DSVI - B), 0.0);
    if (SR > 0.0) {
      SR = SR * (S_AIRMW / OSS_MW_SO4) * 1.e-9 / IN(OHIN_AIRDEN);
      SR = fmin(SR, SO2 / 1.0e12);
    }
  }
  SR = SR / CVF / DT;
  DENOM = XX2 + XX4 + XX5;
  *srhocl = SR * ss_SafeDiv(XX4, DENOM, 0.0);
  *srhobr = SR * ss_SafeDiv(XX5, DENOM, 0.0);
  *srhocl = ss_SafeDiv(*srhocl, (CC(OSS_SO2) * CC(OSS_HOCl)), 0.0);
  *srhobr = ss_SafeDiv(*srhobr, (CC(OSS_SO2) * CC(OSS_HOBr)), 0.0);
#undef IN
#undef CC
}

/* fullchem_HetDropChem for every cell: SRHOCl, SRHOBr into met rows 4, 5
 * (0 where Do_FullChem does not call it); met [18][ldm] in/out (TEMP and
 * K_CLD read), het the HetState rows of fullchem_SetStateHet. */
void oracle_het_drop_chem_batch(int ncell, double dt, const double* in, long long ldi, const double* C,
                                long long ldc, const double* het, long long ldh, const int* size_res, double* met,
                                long long ldm) {
  for (int cell = 0; cell < ncell; ++cell) {
    double a, b;
    het_drop_cell(in + cell, ldi, C + cell, ldc, met + cell, ldm, het + cell, ldh, dt, size_res[cell], &a, &b);
    met[4 * ldm + cell] = a;
    met[5 * ldm + cell] = b;
  }
}
