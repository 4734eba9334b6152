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
