// Host build of the GPU heterogeneous rate laws (geos-chem_gb300/csrc/het_rates.cuh)
// for tests/test_het_rates.py: the device qualifiers become plain C++, CUDA's
// math functions glibc's, so the laws can be compared with the oracle's
// restatement on the same libm.  Inputs: met.bin [18][n], c.bin [nspec][n],
// het.bin [168][n], calls.bin [ncall][4] (law id, up to three arguments; an
// argument -1-i stands for the concentration C(i)), hs*.bin (the species
// table of the laws).  Output: out.bin [ncall][n].
#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <vector>
#define __device__
#define __forceinline__ inline
#define __noinline__
template <class T> static inline T __ldg(const T* p) { return *p; }
static inline double __longlong_as_double(long long v) { double d; memcpy(&d, &v, 8); return d; }
using std::exp; using std::log10; using std::pow; using std::sqrt; using std::fmin; using std::fmax; using std::frexp;
#include "het_rates.cuh"
using namespace gcrates;
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
  int n = atoi(argv[1]), nspec = atoi(argv[2]), ncall = atoi(argv[3]);
  auto met = rd("met.bin", 18 * (size_t)n), c = rd("c.bin", (size_t)nspec * n), het = rd("het.bin", 168 * (size_t)n);
  auto calls = rd("calls.bin", (size_t)ncall * 4);  // id, a0, a1, a2 (a conc arg as -1 - index)
  auto spi = rd("hsind.bin", HS_N), spm = rd("hsmw.bin", HS_N), sps = rd("hssr.bin", HS_N), sk = rd("hsk0.bin", HS_N), sc = rd("hscr.bin", HS_N);
  std::vector<int> ind(HS_N); for (int i = 0; i < HS_N; ++i) ind[i] = (int)spi[i];
  std::vector<double> out((size_t)ncall * n);
  for (int cell = 0; cell < n; ++cell) {
    Env E; env_init(E, met[cell], met[n + cell], met[2 * n + cell], met[3 * n + cell], met[4 * n + cell], met[5 * n + cell]);
    HetCell X; X.H = het.data(); X.ldh = n; X.C = c.data(); X.ldc = n; X.cell = cell;
    X.sp = HetSpecies{ind.data(), spm.data(), sps.data(), sk.data(), sc.data()};
    het_cell_init(X, E);
    for (int k = 0; k < ncall; ++k) {
      double a[3];
      for (int j = 0; j < 3; ++j) { double v = calls[k * 4 + 1 + j]; a[j] = v <= -1.0 && v == (double)(long long)v && v > -1000 ? c[(size_t)(-1 - (long long)v) * n + cell] : v; }
      out[(size_t)k * n + cell] = het_law((int)calls[k * 4], a, X);
    }
  }
  FILE* p = fopen("out.bin", "wb"); fwrite(out.data(), 8, out.size(), p); fclose(p);
  return 0;
}
