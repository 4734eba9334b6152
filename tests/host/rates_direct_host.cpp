// Host build of the generated straight-line Update_RCONST (rates_direct.inc,
// the body of rates_direct_kernel in geos-chem_gb300/csrc/gckpp_capi.cu) with
// the GPU rate laws (rate_laws.cuh, het_rates.cuh), for tests/test_rates.py:
// the device qualifiers become plain C++, CUDA's math functions glibc's and
// the round-to-nearest intrinsics plain operations (built -ffp-contract=off),
// so the product's rates can be compared with the oracle's on the same libm.
// Inputs: met.bin [18][n], photol.bin [200][n], c.bin [nspec][n], optional
// het.bin [168][n], hs*.bin (species table of the heterogeneous laws).
// Output: out.bin [nreact][n].
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#define __device__
#define __global__
#define __forceinline__ inline
#define __noinline__
#define __launch_bounds__(...)
template <class T>
static inline T __ldg(const T* p) {
  return *p;
}
static inline double __longlong_as_double(long long v) {
  double d;
  memcpy(&d, &v, 8);
  return d;
}
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline double __dmul_rn(double a, double b) { return a * b; }
using std::exp;
using std::fmax;
using std::fmin;
using std::frexp;
using std::log10;
using std::pow;
using std::sqrt;
#include "het_rates.cuh"
#include "kpp_rates.h"
#include "rate_laws.cuh"

namespace gcrates {
template <typename... A>
inline double lawv(int id, const Env& E, A... v) {
  const double t[] = {double(v)...};
  return law(id, t, E);
}
template <typename... A>
inline double hetv(int id, bool has_het, const HetCell& X, A... v) {
  if (!has_het) return 0.0;
  const double t[] = {double(v)..., 0.0};
  return het_law(id, t, X);
}
static void rates_cell(const RatesDev& rp, const RatesArgs& a, int cell) {
#define M(f) a.met[(long long)(f) * a.ldm + cell]
#define PH(j) a.photol[(long long)(j) * a.ldp + cell]
#define CC(i) a.c[(long long)(i) * a.ldc + cell]
#define OUT(r) a.rconst[(long long)(r) * a.ldr + cell]
  Env E;
  env_init(E, M(0), M(1), M(2), M(3), M(4), M(5));
  const bool has_het = a.het != nullptr;
  HetCell X;
  X.H = a.het;
  X.ldh = a.ldh;
  X.C = a.c;
  X.ldc = a.ldc;
  X.cell = cell;
  X.sp = HetSpecies{rp.hs_ind, rp.hs_mw, rp.hs_srmw, rp.hs_hk0, rp.hs_hcr};
  if (has_het) het_cell_init(X, E);
#include "rates_direct.inc"
#undef M
#undef PH
#undef CC
#undef OUT
}
}  // namespace gcrates

static std::vector<double> rd(const char* f, size_t n) {
  std::vector<double> v(n);
  FILE* p = fopen(f, "rb");
  if (!p || fread(v.data(), 8, n, p) != n) {
    fprintf(stderr, "cannot read %s\n", f);
    exit(1);
  }
  fclose(p);
  return v;
}

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  const int n = atoi(argv[1]), nspec = atoi(argv[2]), nreact = atoi(argv[3]), with_het = atoi(argv[4]);
  auto met = rd("met.bin", 18 * (size_t)n), ph = rd("photol.bin", 200 * (size_t)n),
       c = rd("c.bin", (size_t)nspec * n);
  std::vector<double> het;
  if (with_het) het = rd("het.bin", (size_t)HET_NFIELD * n);
  auto spi = rd("hsind.bin", gcrates::HS_N), spm = rd("hsmw.bin", gcrates::HS_N),
       sps = rd("hssr.bin", gcrates::HS_N), sk = rd("hsk0.bin", gcrates::HS_N), sc = rd("hscr.bin", gcrates::HS_N);
  std::vector<int> ind(gcrates::HS_N);
  for (int i = 0; i < gcrates::HS_N; ++i) ind[i] = (int)spi[i];
  std::vector<double> out((size_t)nreact * n);
  gcrates::RatesDev rp{};
  rp.hs_ind = ind.data();
  rp.hs_mw = spm.data();
  rp.hs_srmw = sps.data();
  rp.hs_hk0 = sk.data();
  rp.hs_hcr = sc.data();
  gcrates::RatesArgs a{};
  a.ncell = n;
  a.met = met.data();
  a.ldm = n;
  a.photol = ph.data();
  a.ldp = n;
  a.c = c.data();
  a.ldc = n;
  a.rconst = out.data();
  a.ldr = n;
  a.het = with_het ? het.data() : nullptr;
  a.ldh = n;
  for (int cell = 0; cell < n; ++cell) gcrates::rates_cell(rp, a, cell);
  FILE* p = fopen("out.bin", "wb");
  fwrite(out.data(), 8, out.size(), p);
  fclose(p);
  return 0;
}
