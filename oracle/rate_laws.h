/* Gas-phase rate-law functions of the fullchem mechanism, restated in C for
 * the CPU oracle -- TEST INFRASTRUCTURE.
 *
 * Sources (GEOS-Chem tree):
 *   GCARR_ab/_ac/_abc          KPP/fullchem/rateLawUtilFuncs.F90:41-75
 *   ARRPLUS_*, TUNPLUS_*, GC_*, GCJPL*
 *                              KPP/fullchem/fullchem_RateLawFuncs.F90:107-800
 *   per-cell temperature terms  GeosCore/fullchem_mod.F90:2147-2160
 * Fortran integer powers (x**3, x**(-8), y**2) are written as the repeated
 * products gfortran emits for them; real powers call pow().
 */
#ifndef ORACLE_RATE_LAWS_H
#define ORACLE_RATE_LAWS_H
#include <math.h>

typedef struct {
  double TEMP, NUMDEN, H2O, PRESS, SRHOCl, SRHOBr;
  double INV_TEMP, TEMP_OVER_K300, K300_OVER_TEMP, SR_TEMP;
} rate_env_t;

static inline void rate_env_init(rate_env_t* E, double temp, double numden, double h2o, double press, double srhocl,
                                 double srhobr) {
  E->TEMP = temp;
  E->NUMDEN = numden;
  E->H2O = h2o;
  E->PRESS = press;
  E->SRHOCl = srhocl;
  E->SRHOBr = srhobr;
  E->INV_TEMP = 1.0 / temp;
  E->TEMP_OVER_K300 = temp / 300.0;
  E->K300_OVER_TEMP = 300.0 / temp;
  E->SR_TEMP = sqrt(temp);
}

static inline double ipow3(double x) { return x * x * x; }
static inline double ipow_m8(double x) {
  double t = x * x;
  t = t * t;
  t = t * t;
  return 1.0 / t;
}
static inline double sq(double x) { return x * x; }

static inline double GCARR_ab(const rate_env_t* E, double a0, double b0) { return a0 * pow(E->K300_OVER_TEMP, b0); }
static inline double GCARR_ac(const rate_env_t* E, double a0, double c0) { return a0 * exp(c0 / E->TEMP); }
static inline double GCARR_abc(const rate_env_t* E, double a0, double b0, double c0) {
  return a0 * exp(c0 / E->TEMP) * pow(E->K300_OVER_TEMP, b0);
}
static inline double ARRPLUS_ade(const rate_env_t* E, double a0, double d0, double e0) {
  double k = a0 * (d0 + (E->TEMP * e0));
  return fmax(k, 0.0);
}
static inline double ARRPLUS_abde(const rate_env_t* E, double a0, double b0, double d0, double e0) {
  double k = a0 * (d0 + (E->TEMP * e0)) * exp(-b0 / E->TEMP);
  return fmax(k, 0.0);
}
static inline double TUNPLUS_abcde(const rate_env_t* E, double a0, double b0, double c0, double d0, double e0) {
  double k = a0 * (d0 + (E->TEMP * e0));
  k = k * exp(b0 / E->TEMP) * exp(c0 / ipow3(E->TEMP));
  return fmax(k, 0.0);
}
static inline double GC_ISO1(const rate_env_t* E, double a0, double b0, double c0, double d0, double e0, double f0,
                             double g0) {
  double k0 = d0 * exp(e0 / E->TEMP) * exp(1.0E8 / ipow3(E->TEMP));
  double k1 = f0 * exp(g0 / E->TEMP);
  double k2 = c0 * k0 / (k0 + k1);
  return a0 * exp(b0 / E->TEMP) * (1.0 - k2);
}
static inline double GC_ISO2(const rate_env_t* E, double a0, double b0, double c0, double d0, double e0, double f0,
                             double g0) {
  double k0 = d0 * exp(e0 / E->TEMP) * exp(1.0E8 / ipow3(E->TEMP));
  double k1 = f0 * exp(g0 / E->TEMP);
  double k2 = c0 * k0 / (k0 + k1);
  return a0 * exp(b0 / E->TEMP) * k2;
}
static inline double GC_EPO_a(const rate_env_t* E, double a1, double e1, double m1) {
  double k1 = 1.0 / (m1 * E->NUMDEN + 1.0);
  return a1 * exp(e1 / E->TEMP) * k1;
}
static inline double GC_PAN_abab(const rate_env_t* E, double a0, double b0, double a1, double b1, double cf) {
  double k0 = a0 * exp(b0 / E->TEMP);
  double k1 = a1 * exp(b1 / E->TEMP);
  k0 = k0 * E->NUMDEN;
  double kr = k0 / k1;
  double nc = 0.75 - 1.27 * (log10(cf));
  double f = pow(10.0, log10(cf) / (1.0 + sq(log10(kr) / nc)));
  return k0 * k1 * f / (k0 + k1);
}
static inline double GC_PAN_acac(const rate_env_t* E, double a0, double c0, double a1, double c1, double cf) {
  double k0 = a0 * pow(E->TEMP_OVER_K300, c0);
  double k1 = a1 * pow(E->TEMP_OVER_K300, c1);
  k0 = k0 * E->NUMDEN;
  double kr = k0 / k1;
  double nc = 0.75 - 1.27 * (log10(cf));
  double f = pow(10.0, log10(cf) / (1.0 + sq(log10(kr) / nc)));
  return k0 * k1 * f / (k0 + k1);
}
static inline double GC_NIT(const rate_env_t* E, double a0, double b0, double c0, double n, double x0, double y0) {
  double k0 = 2.0E-22 * exp(n);
  double k1 = 4.3E-1 * ipow_m8(E->TEMP / 298.0);
  k0 = k0 * E->NUMDEN;
  k1 = k0 / k1;
  double k2 = (k0 / (1.0 + k1)) * pow(4.1E-1, 1.0 / (1.0 + sq(log10(k1))));
  double k3 = k2 / (k2 + c0);
  double k4 = a0 * (x0 - E->TEMP * y0);
  double k = k4 * exp(b0 / E->TEMP) * k3;
  return fmax(k, 0.0);
}
static inline double GC_ALK(const rate_env_t* E, double a0, double b0, double c0, double n, double x0, double y0) {
  double k0 = 2.0E-22 * exp(n);
  double k1 = 4.3E-1 * ipow_m8(E->TEMP / 298.0);
  k0 = k0 * E->NUMDEN;
  k1 = k0 / k1;
  double k2 = (k0 / (1.0 + k1)) * pow(4.1E-1, 1.0 / (1.0 + sq(log10(k1))));
  double k3 = c0 / (k2 + c0);
  double k4 = a0 * (x0 - E->TEMP * y0);
  double k = k4 * exp(b0 / E->TEMP) * k3;
  return fmax(k, 0.0);
}
static inline double GC_HO2HO2_acac(const rate_env_t* E, double a0, double c0, double a1, double c1) {
  double k0 = a0 * exp(c0 / E->TEMP);
  double k1 = a1 * exp(c1 / E->TEMP);
  return (k0 + k1 * E->NUMDEN) * (1.0 + 1.4E-21 * E->H2O * exp(2200.0 / E->TEMP));
}
static inline double GC_TBRANCH_1_acac(const rate_env_t* E, double a0, double c0, double a1, double c1) {
  double k0 = a0 * exp(c0 / E->TEMP);
  double k1 = a1 * exp(c1 / E->TEMP);
  return k0 / (1.0 + k1);
}
static inline double GC_RO2HO2_aca(const rate_env_t* E, double a0, double c0, double a1) {
  double k = a0 * exp(c0 / E->TEMP);
  return k * (1.0 - exp(-0.245 * a1));
}
static inline double GC_DMSOH_acac(const rate_env_t* E, double a0, double c0, double a1, double c1) {
  double k0 = a0 * exp(c0 / E->TEMP);
  double k1 = a1 * exp(c1 / E->TEMP);
  return (k0 * E->NUMDEN * 0.2095e0) / (1.0 + k1 * 0.2095e0);
}
static inline double GC_GLYXNO3_ac(const rate_env_t* E, double a0, double c0) {
  double O2 = E->NUMDEN * 0.2095;
  double k = a0 * exp(c0 / E->TEMP);
  return k * (O2 + 3.5E+18) / (2.0 * O2 + 3.5E+18);
}
static inline double GC_GLYCOH_A_a(const rate_env_t* E, double a0) {
  const double exp_arg = -1.0 / 73.0;
  double f = 1.0 - 11.0729 * exp(exp_arg * E->TEMP);
  f = fmax(f, 0.0);
  return a0 * f;
}
static inline double GC_GLYCOH_B_a(const rate_env_t* E, double a0) {
  const double exp_arg = -1.0 / 73.0;
  double f = 1.0 - 11.0729 * exp(exp_arg * E->TEMP);
  f = fmax(f, 0.0);
  return a0 * (1.0 - f);
}
static inline double GC_HACOH_A_ac(const rate_env_t* E, double a0, double c0) {
  const double exp_arg = -1.0 / 60.0;
  double k0 = a0 * exp(c0 / E->TEMP);
  double f = 1.0 - 23.7 * exp(exp_arg * E->TEMP);
  f = fmax(f, 0.0);
  return k0 * f;
}
static inline double GC_HACOH_B_ac(const rate_env_t* E, double a0, double c0) {
  const double exp_arg = -1.0 / 60.0;
  double k0 = a0 * exp(c0 / E->TEMP);
  double f = 1.0 - 23.7 * exp(exp_arg * E->TEMP);
  f = fmax(f, 0.0);
  return k0 * (1.0 - f);
}
static inline double GC_RO2NO_A1_ac(const rate_env_t* E, double a0, double c0) {
  return a0 * exp(c0 / E->TEMP) * 3.0e-4;
}
static inline double GC_RO2NO_B1_ac(const rate_env_t* E, double a0, double c0) {
  const double one_minus_fyrno3 = 1.0 - 3.0e-4;
  return a0 * exp(c0 / E->TEMP) * one_minus_fyrno3;
}
static inline double ro2no_fyrno3(const rate_env_t* E, double a1, int b_form) {
  double xxyn = 1.94e-22 * exp(0.97 * a1) * E->NUMDEN;
  double yyyn = b_form ? 0.826 * (pow(E->K300_OVER_TEMP, 8.1)) : 0.826 * (pow(300.0 / E->TEMP, 8.1));
  double aaa = log10(xxyn / yyyn);
  double zzyn = (1.0 / (1.0 + (aaa * aaa)));
  double rarb = (xxyn / (1.0 + (xxyn / yyyn))) * (pow(0.411, zzyn));
  return (rarb / (1.0 + rarb));
}
static inline double GC_RO2NO_A2_aca(const rate_env_t* E, double a0, double c0, double a1) {
  double k0 = a0 * exp(c0 / E->TEMP);
  return k0 * ro2no_fyrno3(E, a1, 0);
}
static inline double GC_RO2NO_B2_aca(const rate_env_t* E, double a0, double c0, double a1) {
  double k0 = a0 * exp(c0 / E->TEMP);
  return k0 * (1.0 - ro2no_fyrno3(E, a1, 1));
}
static inline double jpl_falloff(double rlow, double rhigh, double fv) {
  double xyrat = rlow / rhigh;
  double blog = log10(xyrat);
  double fexp = 1.0 / (1.0 + (blog * blog));
  return rlow * (pow(fv, fexp)) / (1.0 + xyrat);
}
static inline double GCJPLPR_aa(const rate_env_t* E, double a1, double a2, double fv) {
  return jpl_falloff(a1 * E->NUMDEN, a2, fv);
}
static inline double GCJPLPR_aba(const rate_env_t* E, double a1, double b1, double a2, double fv) {
  return jpl_falloff(a1 * (pow(E->K300_OVER_TEMP, b1)) * E->NUMDEN, a2, fv);
}
static inline double GCJPLPR_abab(const rate_env_t* E, double a1, double b1, double a2, double b2, double fv) {
  return jpl_falloff(a1 * (pow(E->K300_OVER_TEMP, b1)) * E->NUMDEN, a2 * (pow(E->K300_OVER_TEMP, b2)), fv);
}
static inline double GCJPLPR_abcabc(const rate_env_t* E, double a1, double b1, double c1, double a2, double b2,
                                    double c2, double fv) {
  double rlow = a1 * (pow(E->K300_OVER_TEMP, b1)) * exp(c1 / E->TEMP) * E->NUMDEN;
  double rhigh = a2 * (pow(E->K300_OVER_TEMP, b2)) * exp(c2 / E->TEMP);
  return jpl_falloff(rlow, rhigh, fv);
}
static inline double GCJPLEQ_acabab(const rate_env_t* E, double a0, double c0, double a1, double b1, double a2,
                                    double b2, double fv) {
  double k0 = a0 * exp(c0 / E->TEMP);
  double k1 = GCJPLPR_abab(E, a1, b1, a2, b2, fv);
  return k1 / k0;
}
static inline double GCJPLAC_ababac(const rate_env_t* E, double a1, double b1, double a2, double b2, double a3,
                                    double c3, double fv) {
  double rlow = a1 * (pow(E->K300_OVER_TEMP, b1)) * E->NUMDEN;
  double rhigh = a2 * (pow(E->K300_OVER_TEMP, b2));
  double k1 = jpl_falloff(rlow, rhigh, fv);
  double k2 = a3 * exp(c3 / E->TEMP);
  return k2 * (1.0 - (k1 / rhigh));
}
#endif
