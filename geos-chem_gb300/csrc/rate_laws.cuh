// Gas-phase rate laws of the fullchem mechanism (device code).
//
//   GCARR_ab/_ac/_abc        KPP/fullchem/rateLawUtilFuncs.F90:41-75
//   ARRPLUS_*, TUNPLUS_*, GC_*, GCJPL*
//                            KPP/fullchem/fullchem_RateLawFuncs.F90:107-800
//   temperature terms        GeosCore/fullchem_mod.F90:2147-2160
// Integer powers of the Fortran (x**3, x**(-8), y**2) are repeated products;
// real powers use pow().  exp/log10/pow are CUDA's own.
#pragma once
#include <cuda_runtime.h>

namespace gcrates {

struct Env {
  double TEMP, NUMDEN, H2O, PRESS, SRHOCl, SRHOBr;
  double INV_TEMP, TEMP_OVER_K300, K300_OVER_TEMP, SR_TEMP;
};

__device__ __forceinline__ void env_init(Env& E, double t, double nd, double h2o, double p, double shocl,
                                         double shobr) {
  E.TEMP = t;
  E.NUMDEN = nd;
  E.H2O = h2o;
  E.PRESS = p;
  E.SRHOCl = shocl;
  E.SRHOBr = shobr;
  E.INV_TEMP = 1.0 / t;
  E.TEMP_OVER_K300 = t / 300.0;
  E.K300_OVER_TEMP = 300.0 / t;
  E.SR_TEMP = sqrt(t);
}

__device__ __forceinline__ double cube(double x) { return x * x * x; }
__device__ __forceinline__ double inv8(double x) {
  double t = x * x;
  t = t * t;
  t = t * t;
  return 1.0 / t;
}
__device__ __forceinline__ double sqr(double x) { return x * x; }

__device__ __forceinline__ double jpl_fall(double rlow, double rhigh, double fv) {
  const double xyrat = rlow / rhigh;
  const double blog = log10(xyrat);
  const double fexp = 1.0 / (1.0 + (blog * blog));
  return rlow * (pow(fv, fexp)) / (1.0 + xyrat);
}

__device__ __forceinline__ double fyrno3(const Env& E, double a1, bool b_form) {
  const double xxyn = 1.94e-22 * exp(0.97 * a1) * E.NUMDEN;
  const double yyyn = b_form ? 0.826 * pow(E.K300_OVER_TEMP, 8.1) : 0.826 * pow(300.0 / E.TEMP, 8.1);
  const double aaa = log10(xxyn / yyyn);
  const double zzyn = (1.0 / (1.0 + (aaa * aaa)));
  const double rarb = (xxyn / (1.0 + (xxyn / yyyn))) * (pow(0.411, zzyn));
  return rarb / (1.0 + rarb);
}

__device__ __forceinline__ double nit_k2(const Env& E, double n) {
  double k0 = 2.0E-22 * exp(n);
  double k1 = 4.3E-1 * inv8(E.TEMP / 298.0);
  k0 = k0 * E.NUMDEN;
  k1 = k0 / k1;
  return (k0 / (1.0 + k1)) * pow(4.1E-1, 1.0 / (1.0 + sqr(log10(k1))));
}

__device__ __forceinline__ double pan(double k0, double k1, const Env& E, double cf) {
  k0 = k0 * E.NUMDEN;
  const double kr = k0 / k1;
  const double nc = 0.75 - 1.27 * (log10(cf));
  const double f = pow(10.0, log10(cf) / (1.0 + sqr(log10(kr) / nc)));
  return k0 * k1 * f / (k0 + k1);
}

// Evaluate law `id` (index into the law list of gcchem.rates_program) on
// arguments a[0..nargs).
__device__ __forceinline__ double law(int id, const double* a, const Env& E) {
  const double T = E.TEMP;
  switch (id) {
    case 0: return a[0] * pow(E.K300_OVER_TEMP, a[1]);                                   // GCARR_ab
    case 1: return a[0] * exp(a[1] / T);                                                  // GCARR_ac
    case 2: return a[0] * exp(a[2] / T) * pow(E.K300_OVER_TEMP, a[1]);                    // GCARR_abc
    case 3: return fmax(a[0] * (a[1] + (T * a[2])), 0.0);                                 // ARRPLUS_ade
    case 4: return fmax(a[0] * (a[2] + (T * a[3])) * exp(-a[1] / T), 0.0);                // ARRPLUS_abde
    case 5: {                                                                             // TUNPLUS_abcde
      double k = a[0] * (a[3] + (T * a[4]));
      k = k * exp(a[1] / T) * exp(a[2] / cube(T));
      return fmax(k, 0.0);
    }
    case 6:
    case 7: {  // GC_ISO1 / GC_ISO2
      const double k0 = a[3] * exp(a[4] / T) * exp(1.0E8 / cube(T));
      const double k1 = a[5] * exp(a[6] / T);
      const double k2 = a[2] * k0 / (k0 + k1);
      return id == 6 ? a[0] * exp(a[1] / T) * (1.0 - k2) : a[0] * exp(a[1] / T) * k2;
    }
    case 8: {  // GC_EPO_a
      const double k1 = 1.0 / (a[2] * E.NUMDEN + 1.0);
      return a[0] * exp(a[1] / T) * k1;
    }
    case 9: return pan(a[0] * exp(a[1] / T), a[2] * exp(a[3] / T), E, a[4]);                    // GC_PAN_abab
    case 10: return pan(a[0] * pow(E.TEMP_OVER_K300, a[1]), a[2] * pow(E.TEMP_OVER_K300, a[3]), E, a[4]);  // GC_PAN_acac
    case 11:
    case 12: {  // GC_NIT / GC_ALK
      const double k2 = nit_k2(E, a[3]);
      const double k3 = id == 11 ? k2 / (k2 + a[2]) : a[2] / (k2 + a[2]);
      const double k4 = a[0] * (a[4] - T * a[5]);
      return fmax(k4 * exp(a[1] / T) * k3, 0.0);
    }
    case 13: {  // GC_HO2HO2_acac
      const double k0 = a[0] * exp(a[1] / T);
      const double k1 = a[2] * exp(a[3] / T);
      return (k0 + k1 * E.NUMDEN) * (1.0 + 1.4E-21 * E.H2O * exp(2200.0 / T));
    }
    case 14: {  // GC_TBRANCH_1_acac
      const double k0 = a[0] * exp(a[1] / T);
      const double k1 = a[2] * exp(a[3] / T);
      return k0 / (1.0 + k1);
    }
    case 15: {  // GC_RO2HO2_aca
      const double k = a[0] * exp(a[1] / T);
      return k * (1.0 - exp(-0.245 * a[2]));
    }
    case 16: {  // GC_DMSOH_acac
      const double k0 = a[0] * exp(a[1] / T);
      const double k1 = a[2] * exp(a[3] / T);
      return (k0 * E.NUMDEN * 0.2095e0) / (1.0 + k1 * 0.2095e0);
    }
    case 17: {  // GC_GLYXNO3_ac
      const double O2 = E.NUMDEN * 0.2095;
      const double k = a[0] * exp(a[1] / T);
      return k * (O2 + 3.5E+18) / (2.0 * O2 + 3.5E+18);
    }
    case 18:
    case 19: {  // GC_GLYCOH_A_a / _B_a
      double f = 1.0 - 11.0729 * exp((-1.0 / 73.0) * T);
      f = fmax(f, 0.0);
      return id == 18 ? a[0] * f : a[0] * (1.0 - f);
    }
    case 20:
    case 21: {  // GC_HACOH_A_ac / _B_ac
      const double k0 = a[0] * exp(a[1] / T);
      double f = 1.0 - 23.7 * exp((-1.0 / 60.0) * T);
      f = fmax(f, 0.0);
      return id == 20 ? k0 * f : k0 * (1.0 - f);
    }
    case 22: return a[0] * exp(a[1] / T) * 3.0e-4;                  // GC_RO2NO_A1_ac
    case 23: return a[0] * exp(a[1] / T) * (1.0 - 3.0e-4);          // GC_RO2NO_B1_ac
    case 24: return a[0] * exp(a[1] / T) * fyrno3(E, a[2], false);  // GC_RO2NO_A2_aca
    case 25: return a[0] * exp(a[1] / T) * (1.0 - fyrno3(E, a[2], true));  // GC_RO2NO_B2_aca
    case 26: {  // GCJPLEQ_acabab
      const double k0 = a[0] * exp(a[1] / T);
      const double k1 = jpl_fall(a[2] * (pow(E.K300_OVER_TEMP, a[3])) * E.NUMDEN, a[4] * (pow(E.K300_OVER_TEMP, a[5])), a[6]);
      return k1 / k0;
    }
    case 27: return jpl_fall(a[0] * E.NUMDEN, a[1], a[2]);                                   // GCJPLPR_aa
    case 28: return jpl_fall(a[0] * (pow(E.K300_OVER_TEMP, a[1])) * E.NUMDEN, a[2], a[3]);     // GCJPLPR_aba
    case 29: return jpl_fall(a[0] * (pow(E.K300_OVER_TEMP, a[1])) * E.NUMDEN,
                             a[2] * (pow(E.K300_OVER_TEMP, a[3])), a[4]);                    // GCJPLPR_abab
    case 30: {  // GCJPLPR_abcabc
      const double rlow = a[0] * (pow(E.K300_OVER_TEMP, a[1])) * exp(a[2] / T) * E.NUMDEN;
      const double rhigh = a[3] * (pow(E.K300_OVER_TEMP, a[4])) * exp(a[5] / T);
      return jpl_fall(rlow, rhigh, a[6]);
    }
    case 31: {  // GCJPLAC_ababac
      const double rlow = a[0] * (pow(E.K300_OVER_TEMP, a[1])) * E.NUMDEN;
      const double rhigh = a[2] * (pow(E.K300_OVER_TEMP, a[3]));
      const double k1 = jpl_fall(rlow, rhigh, a[6]);
      const double k2 = a[4] * exp(a[5] / T);
      return k2 * (1.0 - (k1 / rhigh));
    }
    default: return __longlong_as_double(0x7ff8000000000000LL);  // unknown law: NaN
  }
}

}  // namespace gcrates
