// aa_cell.cuh -- one cell of the fused AA step, as the step kernels use it: the AA-pattern
// gather of its 19 populations, the collision with its macroscopic outputs, and the AA-pattern
// scatter of the result (lbm_aa.cu runs one cell per thread with it; lbm_pair.cu falls back to
// it for the cells its two-cell path does not take).
#pragma once
#include "collide.cuh"

namespace pog {

// The 19 incoming populations of cell c as stored values (AA read pattern of PARITY).  Every
// slot of cell c is element c + (a non-negative offset below 19 n) of the offset tables.  On the
// odd step, `open` (warp-uniform: no cell of the warp touches a solid neighbour) selects the plain
// streaming offsets; otherwise each direction chooses its streamed or bounced slot.
template <int S, int PARITY>
__device__ __forceinline__ void aa_load(const KParams& kp, const typename Store<S>::E* __restrict__ f,
                                        uint32_t c, uint32_t fl, bool open, typename Store<S>::E raw[19]) {
  // odd step: one 64-bit base per cell, each slot then one widening multiply-add of its 32-bit
  // offset (measured 4 % faster on the 16-bit odd step; the even step keeps 32-bit element
  // indices, which measured faster there)
  const typename Store<S>::E* __restrict__ fc = f + c;
  if (PARITY == 0) {
#pragma unroll
    for (int q = 0; q < 19; ++q) raw[q] = f[(uint32_t)q * kp.n + c];
  } else if (open) {
#pragma unroll
    for (int q = 0; q < 19; ++q) raw[q] = fc[kp.rd[q]];
  } else {
    // source c - e_q is the neighbour in direction opp(q); a solid one bounces f_q back
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const bool wall = q != 0 && ((fl >> (POG_LINK_SHIFT + opp(q))) & 1u);
      raw[q] = fc[wall ? kp.pl[q] : kp.rd[q]];
    }
  }
}

// Collision of cell c (populations fv in the storage's collision form), its macroscopic outputs
// and sums, and the AA stores of the post-collision populations (MACRO_ONLY: outputs only).
template <int S, int PARITY, bool REDUCE, bool MACRO_ONLY>
__device__ __forceinline__ void aa_update(const KParams& kp, typename Store<S>::E* __restrict__ f,
                                          uint32_t c, uint32_t fl, bool open, typename Store<S>::C fv[19],
                                          const float* __restrict__ force, const float* __restrict__ pdrag,
                                          const float* __restrict__ eps, const float* __restrict__ u_prev,
                                          float* __restrict__ u_next, float* __restrict__ rho_out,
                                          float* __restrict__ u_out, RedAcc<typename Store<S>::C>& acc) {
  using St = Store<S>;
  using C = typename St::C;
  const uint32_t n = kp.n;
  C nu_st = (C)0;
  if (!MACRO_ONLY && kp.les_mode == POG_LES_STENCIL && !(fl & POG_CELL_POROUS))
    nu_st = les_nu_stencil<C>(kp, c, u_prev);
  const C rs = (C)kp.rho0;  // shift density of the shifted storages
  const CellResult<C> r =
      collide_cell<C, St::SHIFTED>(kp, fl, c, fv, force, pdrag, eps, nu_st, (C)St::SCALE, rs);
  if (rho_out) rho_out[c] = (float)r.rho;
  if (u_out) {
    u_out[c] = (float)r.ux;
    u_out[n + c] = (float)r.uy;
    u_out[2u * n + c] = (float)r.uz;
  }
  if (!MACRO_ONLY && u_next) {
    u_next[c] = (float)r.ux;
    u_next[n + c] = (float)r.uy;
    u_next[2u * n + c] = (float)r.uz;
  }
  if (REDUCE) acc.add(r);
  if (MACRO_ONLY) return;
  if (PARITY == 0) {
#pragma unroll
    for (int q = 0; q < 19; ++q) f[(uint32_t)opp(q) * n + c] = St::ench(fv[q]);
    return;
  }
  typename St::E* __restrict__ fc = f + opaque(c);  // rebuilt, not held across the collision
  if (open) {
#pragma unroll
    for (int q = 0; q < 19; ++q) fc[kp.wr[q]] = St::ench(fv[q]);
  } else {
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const bool wall = q != 0 && ((fl >> (POG_LINK_SHIFT + q)) & 1u);
      fc[wall ? kp.pl[opp(q)] : kp.wr[q]] = St::ench(fv[q]);
    }
  }
}

__device__ __forceinline__ bool aa_live(const KParams& kp, uint32_t c, uint32_t fl) {
  return !(fl & POG_CELL_SOLID) && c >= kp.guard_lo && c <= kp.guard_hi;
}

// The even AA step of one cell of FP16S stored relative to per-cell reference densities
// (kp.dref): decode the cell's own slots with its reference, collide, set the reference to the new
// density (FP16-rounded) and store the outputs relative to it.  Shared by the per-cell reference
// kernel (lbm_ref.cu) and the two-cell even step (lbm_pair.cu) for the cells it does not pair.
template <bool REDUCE>
__device__ __forceinline__ void ref_even_cell(const KParams& kp, __half* __restrict__ f, uint32_t c, uint32_t fl,
                                              const float* __restrict__ force, const float* __restrict__ pdrag,
                                              const float* __restrict__ eps, const float* __restrict__ u_prev,
                                              float* __restrict__ u_next, float* __restrict__ rho_out,
                                              float* __restrict__ u_out, RedAcc<float>& acc) {
  using St = Store<POG_STORE_F16S>;
  const uint32_t n = kp.n;
  const float dc = __half2float(kp.dref[c]);
  float fv[19];
#pragma unroll
  for (int q = 0; q < 19; ++q) fv[q] = St::dech(f[(uint32_t)q * n + c]);
  float nu_st = 0.0f;
  if (kp.les_mode == POG_LES_STENCIL && !(fl & POG_CELL_POROUS)) nu_st = les_nu_stencil<float>(kp, c, u_prev);
  const CellResult<float> r =
      collide_cell<float, true>(kp, fl, c, fv, force, pdrag, eps, nu_st, St::SCALE, kp.rho0 + dc);
  if (rho_out) rho_out[c] = r.rho;
  if (u_out) {
    u_out[c] = r.ux;
    u_out[n + c] = r.uy;
    u_out[2u * n + c] = r.uz;
  }
  if (u_next) {
    u_next[c] = r.ux;
    u_next[n + c] = r.uy;
    u_next[2u * n + c] = r.uz;
  }
  if (REDUCE) acc.add(r);
  const __half dnew = __float2half_rn(r.rho - kp.rho0);
  const float shift = (__half2float(dnew) - dc) * F16_SCALE;
#pragma unroll
  for (int q = 0; q < 19; ++q) f[(uint32_t)opp(q) * n + c] = St::ench(__fmaf_rn(-(float)wd(q), shift, fv[q]));
  kp.dref[c] = dnew;
}

}  // namespace pog
