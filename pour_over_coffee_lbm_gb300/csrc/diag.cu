// diag.cu -- field statistics for the diagnostics (LBMDiagnostics, src/visualization/
// lbm_diagnostics.py:151-460) reduced on the device in one pass over rho and u, so a check moves
// POG_STAT_COUNT doubles to the host instead of two full fields.
#include "common.cuh"

namespace pog {

constexpr int DIAG_BLOCK = 256;
constexpr int DIAG_WARPS = DIAG_BLOCK / 32;

// ---- compensated FP32 arithmetic ----------------------------------------------------------------
// FP64 runs at a small fraction of the FP32 rate on this GPU, so the per-cell sums are carried as
// FP32 pairs built from error-free transformations -- TwoSum (Knuth) and the FMA TwoProd -- in the
// form of Ogita, Rump & Oishi's Sum2/Dot2 (SIAM J. Sci. Comput. 26, 2005): a running sum s and an
// accumulated error term c, worth s + c.  Only the warps' totals are converted to FP64.
struct Acc2 {
  float s, c;
};
__device__ __forceinline__ void acc_add(Acc2& a, float x) {
  const float t = __fadd_rn(a.s, x);
  const float z = __fsub_rn(t, a.s);
  a.c = __fadd_rn(a.c, __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, z)), __fsub_rn(x, z)));
  a.s = t;
}
// x + lo, lo a low-order part (of an exact product or a root) far below x
__device__ __forceinline__ void acc_add(Acc2& a, float x, float lo) {
  acc_add(a, x);
  a.c = __fadd_rn(a.c, lo);
}
__device__ __forceinline__ void acc_prod(Acc2& a, float x, float y) {
  const float p = __fmul_rn(x, y);
  acc_add(a, p, __fmaf_rn(x, y, -p));
}
// (a.s + a.c) + (b.s + b.c) as a pair
__device__ __forceinline__ Acc2 acc_merge(Acc2 a, Acc2 b) {
  acc_add(a, b.s, b.c);
  return a;
}
__device__ __forceinline__ double acc_value(Acc2 a) { return (double)a.s + (double)a.c; }
// sign of (a.s + a.c) - (b.s + b.c) for pairs whose low parts are small
__device__ __forceinline__ bool pair_gt(float ah, float al, float bh, float bl) {
  return __fadd_rn(__fsub_rn(ah, bh), __fsub_rn(al, bl)) > 0.0f;
}
__device__ __forceinline__ Acc2 shfl_xor(Acc2 a, int o) {
  return {__shfl_xor_sync(0xffffffffu, a.s, o), __shfl_xor_sync(0xffffffffu, a.c, o)};
}

// The sixteen pair-summed statistics, in the order of the per-lane slots.
constexpr int NSLOT = 16;
enum Slot { S_RHO2, S_MOM, S_UACT = S_MOM + 3, S_DRHO2, S_DU2, S_USUM, S_USQ = S_USUM + 3, S_UREG = S_USQ + 3 };
static_assert(S_UREG + 3 == NSLOT, "slot table");

struct StatsArgs {
  const float* rho;
  const float* u;
  const float* rho_prev;
  const float* u_prev;
  double* st;
  double* zp;
  uint64_t cells_per_warp;  // a multiple of 32
  float act_h, act_l, mach_h, mach_l;  // the |u| thresholds as FP32 pairs
};

// One pass over rho, u (and rho_prev, u_prev): each warp takes a contiguous run of cells, 32 per
// step (coalesced), so a run crosses at most a few planes; the per-plane sum of rho is flushed to
// zp at each plane boundary and the |u| sum of the run's current plane into its region (planes
// [0,z30), [z30,z80), [z80,nz)).  The sums use the compensated pairs; the warp reduces its sixteen
// slots by recursive halving (lane L ends with slot L/2 summed over the warp), then the block's
// warps are added in FP64 and one atomic per statistic and block goes to st.
__global__ void __launch_bounds__(DIAG_BLOCK) field_stats_kernel(const KParams kp, const StatsArgs a) {
  __shared__ double sh_sum[NSLOT][DIAG_WARPS];
  __shared__ double sh_mass[DIAG_WARPS], sh_umax[DIAG_WARPS], sh_drho[DIAG_WARPS];
  __shared__ uint32_t sh_act[DIAG_WARPS], sh_mach[DIAG_WARPS];
  const uint32_t n = kp.n;
  const uint64_t plane = kp.nxny;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t)blockIdx.x * DIAG_WARPS + warp;
  const uint64_t b64 = gw * a.cells_per_warp, e64 = b64 + a.cells_per_warp;
  const uint32_t beg = b64 < n ? (uint32_t)b64 : n, end = e64 < n ? (uint32_t)e64 : n;
  const uint32_t z30 = (uint32_t)(0.3 * kp.nz), z80 = (uint32_t)(0.8 * kp.nz);
  const float rho0 = kp.rho0;
  const float *const ux_p = a.u, *const uy_p = a.u + n, *const uz_p = a.u + 2 * (size_t)n;
  const float *const px_p = a.u_prev, *const py_p = a.u_prev ? a.u_prev + n : nullptr,
              *const pz_p = a.u_prev ? a.u_prev + 2 * (size_t)n : nullptr;

  Acc2 v[NSLOT];
#pragma unroll
  for (int i = 0; i < NSLOT; ++i) v[i] = {0.0f, 0.0f};
  Acc2 rsum = {0.0f, 0.0f}, ut = {0.0f, 0.0f};  // rho and |u| of the current plane
  float umax_h = 0.0f, umax_l = 0.0f, rmin = INFINITY, rmax = -INFINITY;
  uint32_t n_act = 0u, n_mach = 0u;
  double mass = 0.0;  // lane 0: the flushed plane sums

  // hand the current plane's sums on: rho to zp[k] and the mass, |u| to the plane's region
  auto flush = [&](uint32_t k) {
    Acc2 r = rsum;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r = acc_merge(r, shfl_xor(r, o));
    if (lane == 0) {
      const double d = acc_value(r);
      if (a.zp) atomicAdd(a.zp + k, d);
      mass += d;
    }
    if (k < z30) v[S_UREG] = acc_merge(v[S_UREG], ut);
    else if (k < z80) v[S_UREG + 1] = acc_merge(v[S_UREG + 1], ut);
    else v[S_UREG + 2] = acc_merge(v[S_UREG + 2], ut);
    rsum = ut = {0.0f, 0.0f};
  };
  // the eight inputs of one cell (zeros past the run's end)
  struct In {
    float r, ux, uy, uz, rp, qx, qy, qz;
  };
  auto load = [&](uint32_t c, In& x) {
    x = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (c < end) {
      x.r = a.rho[c];
      x.ux = ux_p[c];
      x.uy = uy_p[c];
      x.uz = uz_p[c];
      if (a.rho_prev) x.rp = a.rho_prev[c];
      if (px_p) {
        x.qx = px_p[c];
        x.qy = py_p[c];
        x.qz = pz_p[c];
      }
    }
  };

  if (beg < end) {
    uint32_t k = beg / kp.nxny;
    uint64_t bnd = (uint64_t)(k + 1) * plane;
    In cur, nxt;
    load(beg + lane, cur);
    for (uint32_t c0 = beg; c0 < end; c0 += 32) {
      const uint32_t c = c0 + lane;
      load(c + 32, nxt);  // the next step's loads are in flight during this step's arithmetic
      float rv = 0.0f, mh = 0.0f, ml = 0.0f;
      if (c < end) {
        const float r = cur.r, ux = cur.ux, uy = cur.uy, uz = cur.uz;
        rv = r;
        rmin = fminf(rmin, r);
        rmax = fmaxf(rmax, r);
        acc_prod(v[S_RHO2], r, r);
        acc_prod(v[S_MOM], r, ux);
        acc_prod(v[S_MOM + 1], r, uy);
        acc_prod(v[S_MOM + 2], r, uz);
        acc_add(v[S_USUM], ux);
        acc_add(v[S_USUM + 1], uy);
        acc_add(v[S_USUM + 2], uz);
        const float px = __fmul_rn(ux, ux), py = __fmul_rn(uy, uy), pz = __fmul_rn(uz, uz);
        const float pxl = __fmaf_rn(ux, ux, -px), pyl = __fmaf_rn(uy, uy, -py), pzl = __fmaf_rn(uz, uz, -pz);
        acc_add(v[S_USQ], px, pxl);
        acc_add(v[S_USQ + 1], py, pyl);
        acc_add(v[S_USQ + 2], pz, pzl);
        // |u|^2 as a pair, then |u| = m + dm from the approximate root m and one correction step
        Acc2 q = {px, 0.0f};
        acc_add(q, py, pxl);
        acc_add(q, pz, __fadd_rn(pyl, pzl));
        if (q.s > 0.0f) {
          const float rs = rsqrtf(q.s);
          mh = __fmul_rn(q.s, rs);
          ml = __fmul_rn(__fmul_rn(__fadd_rn(__fmaf_rn(-mh, mh, q.s), q.c), rs), 0.5f);
        }
        if (pair_gt(mh, ml, umax_h, umax_l)) {
          umax_h = mh;
          umax_l = ml;
        }
        if (pair_gt(mh, ml, a.act_h, a.act_l)) {
          acc_add(v[S_UACT], mh, ml);
          ++n_act;
        }
        n_mach += pair_gt(mh, ml, a.mach_h, a.mach_l) ? 1u : 0u;
        if (a.rho_prev) {
          // (r - r')^2 from the exact difference d + e: d^2 exactly plus 2 d e
          Acc2 d = {r, 0.0f};
          acc_add(d, -cur.rp);
          const float p = __fmul_rn(d.s, d.s);
          acc_add(v[S_DRHO2], p, __fmaf_rn(2.0f * d.s, d.c, __fmaf_rn(d.s, d.s, -p)));
        }
        if (px_p) {
#pragma unroll
          for (int ax = 0; ax < 3; ++ax) {
            Acc2 d = {ax == 0 ? ux : (ax == 1 ? uy : uz), 0.0f};
            acc_add(d, -(ax == 0 ? cur.qx : (ax == 1 ? cur.qy : cur.qz)));
            const float p = __fmul_rn(d.s, d.s);
            acc_add(v[S_DU2], p, __fmaf_rn(2.0f * d.s, d.c, __fmaf_rn(d.s, d.s, -p)));
          }
        }
      }
      cur = nxt;
      // plane attribution (warp-uniform control): the step may reach into later planes
      const uint32_t step_end = end - c0 > 32u ? c0 + 32u : end;
      while (bnd < step_end) {
        const bool here = c < bnd;
        acc_add(rsum, here ? rv : 0.0f);
        acc_add(ut, here ? mh : 0.0f, here ? ml : 0.0f);
        if (here) rv = mh = ml = 0.0f;
        flush(k);
        ++k;
        bnd += plane;
      }
      acc_add(rsum, rv);
      acc_add(ut, mh, ml);
    }
    flush(k);
  }

  // warp: the sixteen slots by recursive halving, the rest by butterflies
#pragma unroll
  for (int o = 16, half = NSLOT / 2; o >= 2; o >>= 1, half >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const Acc2 send = up ? v[i] : v[i + half], keep = up ? v[i + half] : v[i];
      v[i] = acc_merge(keep, shfl_xor(send, o));
    }
  }
  v[0] = acc_merge(v[0], shfl_xor(v[0], 1));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, umax_h, o), l = __shfl_xor_sync(0xffffffffu, umax_l, o);
    if (pair_gt(h, l, umax_h, umax_l)) {
      umax_h = h;
      umax_l = l;
    }
    rmin = fminf(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
    rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
  }
  n_act = __reduce_add_sync(0xffffffffu, n_act);
  n_mach = __reduce_add_sync(0xffffffffu, n_mach);
  if (!(lane & 1)) sh_sum[lane >> 1][warp] = acc_value(v[0]);
  if (lane == 0) {
    sh_mass[warp] = mass;
    sh_umax[warp] = (double)umax_h + (double)umax_l;
    // max |rho - rho0| is reached at the smallest or the largest rho
    sh_drho[warp] = rmin <= rmax ? fmax(fabs((double)rmax - (double)rho0), fabs((double)rmin - (double)rho0)) : 0.0;
    sh_act[warp] = n_act;
    sh_mach[warp] = n_mach;
  }
  __syncthreads();
  if (threadIdx.x < POG_STAT_COUNT) {
    const int t = threadIdx.x;
    int slot = -1, nsum = 1;  // statistics that are one slot or the sum of three
    switch (t) {
      case POG_STAT_RHO2: slot = S_RHO2; break;
      case POG_STAT_MOMX: case POG_STAT_MOMX + 1: case POG_STAT_MOMX + 2: slot = S_MOM + t - POG_STAT_MOMX; break;
      case POG_STAT_UACT_SUM: slot = S_UACT; break;
      case POG_STAT_DRHO2: slot = S_DRHO2; break;
      case POG_STAT_DU2: slot = S_DU2; break;
      case POG_STAT_USUM: case POG_STAT_USUM + 1: case POG_STAT_USUM + 2: slot = S_USUM + t - POG_STAT_USUM; break;
      case POG_STAT_USQ: case POG_STAT_USQ + 1: case POG_STAT_USQ + 2: slot = S_USQ + t - POG_STAT_USQ; break;
      case POG_STAT_UREG: case POG_STAT_UREG + 1: case POG_STAT_UREG + 2: slot = S_UREG + t - POG_STAT_UREG; break;
      case POG_STAT_U2: slot = S_USQ; nsum = 3; break;    // sum |u|^2 = the three sums of u_a^2
      case POG_STAT_UABS: slot = S_UREG; nsum = 3; break; // sum |u| = the three regions
      default: break;
    }
    double x = 0.0;
    bool is_max = false;
    for (int w = 0; w < DIAG_WARPS; ++w) {
      if (slot >= 0) {
        for (int j = 0; j < nsum; ++j) x += sh_sum[slot + j][w];
      } else if (t == POG_STAT_MASS) {
        x += sh_mass[w];
      } else if (t == POG_STAT_UACT_N) {
        x += (double)sh_act[w];
      } else if (t == POG_STAT_MACH_N) {
        x += (double)sh_mach[w];
      } else {
        is_max = true;
        x = fmax(x, t == POG_STAT_UMAX ? sh_umax[w] : sh_drho[w]);
      }
    }
    if (is_max) {
      // non-negative doubles order like their bit patterns
      if (x > 0.0) atomicMax(reinterpret_cast<unsigned long long*>(a.st + t), (unsigned long long)__double_as_longlong(x));
    } else if (x != 0.0) {
      atomicAdd(a.st + t, x);
    }
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
  if (zprofile) POG_TRY_CUDA(cudaMemsetAsync(zprofile, 0, (size_t)p->nz * sizeof(double), s));
  static thread_local int grid = 0;
  if (grid == 0) grid = pog::persistent_blocks((const void*)pog::field_stats_kernel, pog::DIAG_BLOCK);
  if (grid <= 0) return pog::set_error(POG_E_CUDA, "occupancy query failed");
  // contiguous runs of a multiple of 32 cells per warp, as even as the grid allows
  const uint64_t warps = (uint64_t)grid * pog::DIAG_WARPS;
  const uint64_t per = ((kp.n + warps - 1) / warps + 31) / 32 * 32;
  const uint64_t used = (kp.n + per - 1) / per;
  pog::StatsArgs a;
  a.rho = rho;
  a.u = u;
  a.rho_prev = rho_prev;
  a.u_prev = u_prev;
  a.st = stats;
  a.zp = zprofile;
  a.cells_per_warp = per;
  // the thresholds of the counts as FP32 pairs: |u| > 1e-10 (active) and |u| > 0.1 c_s (Mach)
  const double thr[2] = {1e-10, 0.1 / sqrt(3.0)};
  float th[2], tl[2];
  for (int i = 0; i < 2; ++i) {
    th[i] = (float)thr[i];
    tl[i] = (float)(thr[i] - (double)th[i]);
  }
  a.act_h = th[0];
  a.act_l = tl[0];
  a.mach_h = th[1];
  a.mach_l = tl[1];
  pog::field_stats_kernel<<<(unsigned)((used + pog::DIAG_WARPS - 1) / pog::DIAG_WARPS), pog::DIAG_BLOCK, 0, s>>>(kp, a);
  pog::count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}
