// diag.cu -- field statistics for the diagnostics (LBMDiagnostics, src/visualization/
// lbm_diagnostics.py:151-460) reduced on the device in one pass over rho and u, so a check moves
// POG_STAT_COUNT doubles to the host instead of two full fields.
#include "common.cuh"

namespace pog {

constexpr int DIAG_BLOCK = 256;

// Warp + block sum of `v` into out[slot] (one atomic per block).
__device__ __forceinline__ void block_add(double v, double* out, double* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double x = lane < (DIAG_BLOCK / 32) ? sm[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0 && x != 0.0) atomicAdd(out, x);
  }
}

// Block max of a non-negative value into out (IEEE order of non-negative doubles = bit order).
__device__ __forceinline__ void block_max(double v, double* out, double* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double x = lane < (DIAG_BLOCK / 32) ? sm[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
    if (lane == 0 && x > 0.0)
      atomicMax(reinterpret_cast<unsigned long long*>(out), (unsigned long long)__double_as_longlong(x));
  }
}

__global__ void __launch_bounds__(DIAG_BLOCK) field_stats_kernel(
    const KParams kp, const float* __restrict__ rho, const float* __restrict__ u,
    const float* __restrict__ rho_prev, const float* __restrict__ u_prev, double* __restrict__ st) {
  __shared__ double sm[DIAG_BLOCK / 32];
  const uint32_t n = kp.n;
  const uint32_t z30 = (uint32_t)(0.3 * kp.nz) * kp.nxny, z80 = (uint32_t)(0.8 * kp.nz) * kp.nxny;
  double a[POG_STAT_COUNT];
#pragma unroll
  for (int s = 0; s < POG_STAT_COUNT; ++s) a[s] = 0.0;
  const double cs01 = 0.1 / sqrt(3.0);
  for (uint32_t c = blockIdx.x * DIAG_BLOCK + threadIdx.x; c < n; c += gridDim.x * DIAG_BLOCK) {
    const double r = rho[c], ux = u[c], uy = u[n + c], uz = u[2u * n + c];
    const double u2 = ux * ux + uy * uy + uz * uz, um = sqrt(u2);
    a[POG_STAT_MASS] += r;
    a[POG_STAT_RHO2] += r * r;
    a[POG_STAT_MOMX] += r * ux;
    a[POG_STAT_MOMX + 1] += r * uy;
    a[POG_STAT_MOMX + 2] += r * uz;
    a[POG_STAT_UMAX] = fmax(a[POG_STAT_UMAX], um);
    if (um > 1e-10) {
      a[POG_STAT_UACT_SUM] += um;
      a[POG_STAT_UACT_N] += 1.0;
    }
    a[POG_STAT_U2] += u2;
    a[POG_STAT_UABS] += um;
    if (um > cs01) a[POG_STAT_MACH_N] += 1.0;
    a[POG_STAT_DRHO_MAX] = fmax(a[POG_STAT_DRHO_MAX], fabs(r - (double)kp.rho0));
    if (rho_prev) {
      const double d = r - (double)rho_prev[c];
      a[POG_STAT_DRHO2] += d * d;
    }
    if (u_prev) {
      const double dx = ux - u_prev[c], dy = uy - u_prev[n + c], dz = uz - u_prev[2u * n + c];
      a[POG_STAT_DU2] += dx * dx + dy * dy + dz * dz;
    }
    a[POG_STAT_USUM] += ux;
    a[POG_STAT_USUM + 1] += uy;
    a[POG_STAT_USUM + 2] += uz;
    a[POG_STAT_USQ] += ux * ux;
    a[POG_STAT_USQ + 1] += uy * uy;
    a[POG_STAT_USQ + 2] += uz * uz;
    a[POG_STAT_UREG + (c < z30 ? 0 : (c < z80 ? 1 : 2))] += um;
  }
#pragma unroll
  for (int s = 0; s < POG_STAT_COUNT; ++s) {
    if (s == POG_STAT_UMAX || s == POG_STAT_DRHO_MAX)
      block_max(a[s], st + s, sm);
    else
      block_add(a[s], st + s, sm);
  }
}

// Per-plane sum of rho: one block per plane.
__global__ void __launch_bounds__(DIAG_BLOCK) zprofile_kernel(const KParams kp, const float* __restrict__ rho,
                                                             double* __restrict__ zp) {
  __shared__ double sm[DIAG_BLOCK / 32];
  const uint32_t k = blockIdx.x, base = k * kp.nxny;
  double s = 0.0;
  for (uint32_t i = threadIdx.x; i < kp.nxny; i += DIAG_BLOCK) s += rho[base + i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) sm[warp] = s;
  __syncthreads();
  if (warp == 0) {
    double x = lane < (DIAG_BLOCK / 32) ? sm[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) zp[k] = x;
  }
}

}  // namespace pog

extern "C" int pog_field_stats(const pog_params* p, const float* rho, const float* u, const float* rho_prev,
                               const float* u_prev, double* stats, double* zprofile, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!rho || !u || !stats) return pog::set_error(POG_E_ARG, "rho/u/stats is NULL");
  pog::KParams kp = pog::make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  POG_TRY_CUDA(cudaMemsetAsync(stats, 0, POG_STAT_COUNT * sizeof(double), s));
  static thread_local int grid = 0;
  if (grid == 0) grid = pog::persistent_blocks((const void*)pog::field_stats_kernel, pog::DIAG_BLOCK);
  if (grid <= 0) return pog::set_error(POG_E_CUDA, "occupancy query failed");
  int want = (int)((kp.n + pog::DIAG_BLOCK - 1) / pog::DIAG_BLOCK);
  pog::field_stats_kernel<<<want < grid ? want : grid, pog::DIAG_BLOCK, 0, s>>>(kp, rho, u, rho_prev, u_prev, stats);
  pog::count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  if (zprofile) {
    pog::zprofile_kernel<<<kp.nz, pog::DIAG_BLOCK, 0, s>>>(kp, rho, zprofile);
    pog::count_launch();
    POG_TRY_CUDA(cudaGetLastError());
  }
  return POG_OK;
}
