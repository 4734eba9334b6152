// Update_RCONST on the GPU (KPP/fullchem/gckpp_Rates.F90:408-1503): one
// thread per cell runs the postfix program of all 1058 rate expressions
// (lowered by gcchem.rates_program); the opcode stream is warp-uniform.
// Heterogeneous laws (het_rates.cuh) read the cell's HetState rows; without
// a HetState array they are 0 (no aerosol surface, no cloud).
#include "het_rates.cuh"
#include "kpp_rates.h"
#include "rate_laws.cuh"

namespace gcrates {

enum : int { OP_END = 0, OP_CONST, OP_VAR, OP_PHOTOL, OP_CONC, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG, OP_EXP,
             OP_LOG10, OP_CALL, OP_HETZERO, OP_HET };

constexpr int NMET_MAX = 32;
constexpr int STACK = 24;

__global__ void __launch_bounds__(128) rates_kernel(RatesDev rp, RatesArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= a.ncell) return;
  double v[NMET_MAX];
  for (int f = 0; f < rp.nmet; ++f) v[f] = a.met[(long long)f * a.ldm + cell];
  Env E;
  env_init(E, v[0], v[1], v[2], v[3], v[4], v[5]);
  HetCell X;
  X.H = a.het;
  X.ldh = a.ldh;
  X.C = a.c;
  X.ldc = a.ldc;
  X.cell = cell;
  X.sp = HetSpecies{rp.hs_ind, rp.hs_mw, rp.hs_srmw, rp.hs_hk0, rp.hs_hcr};
  if (a.het) het_cell_init(X, E);
  double st[STACK];
  for (int r = 0; r < rp.nreact; ++r) {
    int pc = __ldg(rp.start + r);
    int sp = 0;
    bool bad = false;
    while (true) {
      const int op = __ldg(rp.code + pc++);
      if (op == OP_END) break;
      switch (op) {
        case OP_CONST: st[sp++] = __ldg(rp.consts + __ldg(rp.code + pc++)); break;
        case OP_VAR: st[sp++] = v[__ldg(rp.code + pc++)]; break;
        case OP_PHOTOL: st[sp++] = a.photol[(long long)__ldg(rp.code + pc++) * a.ldp + cell]; break;
        case OP_CONC: st[sp++] = a.c[(long long)__ldg(rp.code + pc++) * a.ldc + cell]; break;
        case OP_ADD: --sp; st[sp - 1] = st[sp - 1] + st[sp]; break;
        case OP_SUB: --sp; st[sp - 1] = st[sp - 1] - st[sp]; break;
        case OP_MUL: --sp; st[sp - 1] = st[sp - 1] * st[sp]; break;
        case OP_DIV: --sp; st[sp - 1] = st[sp - 1] / st[sp]; break;
        case OP_NEG: st[sp - 1] = -st[sp - 1]; break;
        case OP_EXP: st[sp - 1] = exp(st[sp - 1]); break;
        case OP_LOG10: st[sp - 1] = log10(st[sp - 1]); break;
        case OP_CALL: {
          const int id = __ldg(rp.code + pc++);
          const int n = __ldg(rp.law_nargs + id);
          sp -= n;
          st[sp] = law(id, st + sp, E);
          ++sp;
          break;
        }
        case OP_HETZERO: st[sp++] = 0.0; break;
        case OP_HET: {
          const int id = __ldg(rp.code + pc++);
          const int n = __ldg(rp.het_nargs + id);
          sp -= n;
          st[sp] = a.het ? het_law(id, st + sp, X) : 0.0;
          ++sp;
          break;
        }
        default: bad = true; break;
      }
      if (bad || sp > STACK - 8 || sp < 0) {
        bad = true;
        break;
      }
    }
    a.rconst[(long long)r * a.ldr + cell] = bad ? __longlong_as_double(0x7ff8000000000000LL) : st[0];
  }
}

cudaError_t launch_rates(const RatesDev& rp, const RatesArgs& a, cudaStream_t s) {
  const int block = 128;
  const int grid = (a.ncell + block - 1) / block;
  if (grid > 0) rates_kernel<<<grid, block, 0, s>>>(rp, a);
  return cudaGetLastError();
}

}  // namespace gcrates
