// common.cuh -- shared definitions of libpog.so (GB300 / sm_103a D3Q19 LBM + particles).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pog.h"

namespace pog {

// D3Q19 in the reference's config/core.py:36-47 ordering; OPP from legacy/lbm_solver.py:431-439.
__host__ __device__ constexpr int cx(int q) {
  return q == 1 || q == 7 || q == 9 || q == 11 || q == 13 ? 1
         : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1
                                                               : 0;
}
__host__ __device__ constexpr int cy(int q) {
  return q == 3 || q == 7 || q == 8 || q == 15 || q == 17 ? 1
         : (q == 4 || q == 9 || q == 10 || q == 16 || q == 18) ? -1
                                                               : 0;
}
__host__ __device__ constexpr int cz(int q) {
  return q == 5 || q == 11 || q == 12 || q == 15 || q == 16 ? 1
         : (q == 6 || q == 13 || q == 14 || q == 17 || q == 18) ? -1
                                                                : 0;
}
__host__ __device__ constexpr int opp(int q) {
  return q == 0 ? 0 : (q <= 6 ? (q % 2 == 1 ? q + 1 : q - 1) : (q == 7 ? 10 : q == 8 ? 9 : q == 9 ? 8 : q == 10 ? 7 : q == 11 ? 14 : q == 12 ? 13 : q == 13 ? 12 : q == 14 ? 11 : q == 15 ? 18 : q == 16 ? 17 : q == 17 ? 16 : 15));
}
__host__ __device__ constexpr double wd(int q) {
  return q == 0 ? 1.0 / 3.0 : (q <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
}
static_assert(opp(7) == 10 && opp(8) == 9 && opp(11) == 14 && opp(12) == 13 && opp(15) == 18 &&
                  opp(16) == 17 && opp(1) == 2 && opp(6) == 5,
              "opposite table");

constexpr float F16_SCALE = 4096.0f;       // FP16S stores (f - w rho0) * 2^12
constexpr float F16_INV_SCALE = 1.0f / 4096.0f;

// Parameters as the kernels consume them (derived on the host once per call).
struct KParams {
  uint32_t nx, ny, nz, n;  // n = nx*ny*nz
  uint32_t nxny;
  // cells whose 18 neighbours are all inside the grid: guard_lo <= c <= guard_hi.  Kernels
  // that read neighbours skip cells outside this range whatever the flags say, so a caller's
  // malformed flags (a fluid cell on the outer shell) cannot drive an access out of bounds.
  uint32_t guard_lo, guard_hi;
  int32_t off[19];         // neighbour offset of direction q in cells
  // Element offsets relative to a cell's own element c (all non-negative, < 19 n < 2^32):
  //   pl[q] = q n              slot (c, q)
  //   rd[q] = opp(q) n - off[q] odd-step streaming read (c - e_q, opp q)
  //   wr[q] = q n + off[q]      odd-step streaming write (c + e_q, q)
  uint32_t pl[19], rd[19], wr[19];
  int32_t les_mode, drag_mode, forcing_mode, clamp_tau, storage;
  float tau, rho0, gx, gy, gz;
  float cs2, strain_floor, nu_max, tau_min, tau_max, nu0;
  float K0, CF0, eps0, g0;  // porous: uniform K/C_F and Kozeny-Carman normaliser g(eps0)
  float drag_cap;
  float u_inlet, inlet_R, cxf, cyf, rho_out;
  float coef[POG_INLET_NCOEF];
  const float* inlet_ctl;  // device [u_inlet, a_0..a_15] or null
  const float* pour;       // device pour-nozzle block (POG_POUR_*) or null
  const float* blockage;   // device filter-paper blockage b [n] or null
  const float* phase;      // device phase indicator [n] (0 air, 1 water) or null
  float tau_air;
  const uint32_t* dmask;   // device bit mask of the cells with a particle deposit, or null
  __half* dref;            // FP16S per-cell reference density deviations [n], or null
};

KParams make_kparams(const pog_params* p);

// A copy of a register the compiler cannot see through (so it neither merges two computations
// of the same value nor keeps the first alive until the second): a kernel recomputes an address
// or a conversion instead of holding it in a register across the collision.
__device__ __forceinline__ uint32_t opaque(uint32_t v) {
  uint32_t r;
  asm volatile("mov.b32 %0, %1;" : "=r"(r) : "r"(v));
  return r;
}

// Error plumbing (thread-local message, no exceptions across the ABI).
int set_error(int code, const char* fmt, ...);
int check_cuda(cudaError_t e, const char* what);
void count_launch(int n = 1);
// Persistent grid size for a kernel: SMs x resident blocks per SM.
int persistent_blocks(const void* kernel, int block, size_t smem = 0);

}  // namespace pog

#define POG_TRY_CUDA(expr)                                            \
  do {                                                                \
    cudaError_t _e = (expr);                                          \
    if (_e != cudaSuccess) return ::pog::check_cuda(_e, #expr);       \
  } while (0)
