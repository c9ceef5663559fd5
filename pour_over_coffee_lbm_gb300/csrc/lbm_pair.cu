// lbm_pair.cu -- the even AA step of the 16-bit storages (FP16S, BF16S) with two x-adjacent
// cells per thread.
//
// Same update as aa_step_kernel (lbm_aa.cu; the reference's step: legacy/lbm_solver.py:488-654
// with les_turbulence.py:289-380 and filter_paper.py:471-536 fused in), arranged for the
// instruction budget of a step that moves only 2 x 38 bytes per cell: the 16-bit per-cell step
// issues more instructions per byte than the FP32 one and is bound by issue and latency, not by
// HBM.  A thread here owns the pair (c0, c0 + 1), c0 even.  On the even step a cell reads and
// writes only its own slots, so:
//   - each population pair (c0, q), (c0 + 1, q) is ONE aligned 32-bit load, and each pair
//     (c0, opp q), (c0 + 1, opp q) one 32-bit store;
//   - the populations stay packed (one 32-bit register per direction) and are converted per
//     direction where they are used;
//   - the moments, the LES stress and the BGK + Guo collision run in Blackwell's packed FP32x2
//     arithmetic (FADD2 / FMUL2 / FFMA2), one instruction for both cells; square roots,
//     reciprocals and the band's Darcy-Forchheimer solve run per cell;
//   - two floats go back to one packed 16-bit pair in one conversion.
// Band cells and cells next to a solid cell stay on this path (a warp with a solid cell in any of
// its pairs stores 16-bit halves); pairs with an inlet or outlet cell, a particle deposit, or a
// cell outside the guard range take the per-cell code of aa_cell.cuh for both cells.
//
// The odd step stays per-cell (aa_step_kernel): there the ten x-shifted directions straddle a
// 32-bit word and bounce-back picks the slot per cell and direction, and the same pairing
// measured slower than the per-cell kernel at 256^3 (516 against 393 us per odd step under ncu).
//
// Arithmetic: the moment sums are the per-cell kernel's operations in its order; the collision
// is the same algebra with FMA contraction chosen here, so the two kernels agree to FP32
// rounding before the 16-bit store (the stored values agree to one 16-bit ulp, not bit for bit).
#include "aa_cell.cuh"

namespace pog {

constexpr int PAIR_BLOCK = 128;
// Resident 128-thread blocks per SM: 8 (64 registers, 56 spilled bytes: 274 us per 256^3 even
// step against 276 at 72 registers and 282 at 80, which spills nothing) for the plain step, 6 (80)
// with the FP64 sums.
template <bool REDUCE>
constexpr int pair_min_blocks() {
  return REDUCE ? 6 : 8;
}

using F2 = float2;  // .x = cell c0, .y = cell c0 + 1
__device__ __forceinline__ F2 sp2(float a) { return make_float2(a, a); }
__device__ __forceinline__ F2 add2(F2 a, F2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ F2 sub2(F2 a, F2 b) { return __ffma2_rn(b, sp2(-1.0f), a); }  // a - b, one rounding
__device__ __forceinline__ F2 mul2(F2 a, F2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) { return __ffma2_rn(a, b, c); }

// Packed 16-bit pair <-> two floats (low half = the even cell).
template <int S>
struct Pair16;
template <>
struct Pair16<POG_STORE_F16S> {
  __device__ static __forceinline__ F2 unpack(uint32_t w) {
    __half2 h;
    memcpy(&h, &w, 4);
    return __half22float2(h);
  }
  __device__ static __forceinline__ uint32_t pack(F2 v) {
    const __half2 h = __float22half2_rn(v);
    uint32_t w;
    memcpy(&w, &h, 4);
    return w;
  }
};
template <>
struct Pair16<POG_STORE_BF16S> {
  __device__ static __forceinline__ F2 unpack(uint32_t w) {
    __nv_bfloat162 h;
    memcpy(&h, &w, 4);
    return __bfloat1622float2(h);
  }
  __device__ static __forceinline__ uint32_t pack(F2 v) {
    const __nv_bfloat162 h = __float22bfloat162_rn(v);
    uint32_t w;
    memcpy(&w, &h, 4);
    return w;
  }
};

// e.u for the representative Q of a direction pair, written with only its non-zero terms:
// pairs (1,2) (3,4) (5,6) on the axes, (7,10) (8,9) (11,14) (12,13) (15,18) (16,17) on edges.
template <int Q>
__device__ __forceinline__ F2 edot(F2 x, F2 y, F2 z) {
  if constexpr (Q == 1) return x;
  else if constexpr (Q == 3) return y;
  else if constexpr (Q == 5) return z;
  else if constexpr (Q == 7) return add2(x, y);
  else if constexpr (Q == 8) return sub2(y, x);
  else if constexpr (Q == 11) return add2(x, z);
  else if constexpr (Q == 12) return sub2(z, x);
  else if constexpr (Q == 15) return add2(y, z);
  else return sub2(z, y);  // Q == 16
}
// the signs above, checked against the velocity set
static_assert(cx(1) == 1 && cy(3) == 1 && cz(5) == 1, "axis representatives");
static_assert(cx(7) == 1 && cy(7) == 1 && cz(7) == 0 && cx(8) == -1 && cy(8) == 1 && cz(8) == 0, "xy edges");
static_assert(cx(11) == 1 && cy(11) == 0 && cz(11) == 1 && cx(12) == -1 && cy(12) == 0 && cz(12) == 1, "xz edges");
static_assert(cx(15) == 0 && cy(15) == 1 && cz(15) == 1 && cx(16) == 0 && cy(16) == -1 && cz(16) == 1, "yz edges");

// The collision coefficients of one weight class, per cell (see PairCoef in collide.cuh).
struct PairCoef2 {
  F2 A, B, Cc, D, b3;
};

template <int Q, int S>
__device__ __forceinline__ void collide_dir2(uint32_t w[19], F2 ux, F2 uy, F2 uz, F2 Fx, F2 Fy, F2 Fz, F2 keep,
                                             const PairCoef2& k) {
  constexpr int P = opp(Q);
  const F2 eu = edot<Q>(ux, uy, uz), eF = edot<Q>(Fx, Fy, Fz);
  const F2 sym = fma2(eu, fma2(k.Cc, eF, mul2(k.B, eu)), k.A);
  const F2 asym = fma2(k.D, eu, mul2(k.b3, eF));
  // converted again from the packed words (opaque copies), not kept from the moment pass: 19
  // registers instead of 38
  const F2 hq = Pair16<S>::unpack(opaque(w[Q])), hp = Pair16<S>::unpack(opaque(w[P]));
  w[Q] = Pair16<S>::pack(fma2(keep, hq, add2(sym, asym)));
  w[P] = Pair16<S>::pack(fma2(keep, hp, sub2(sym, asym)));
}

// REF: FP16S stored relative to per-cell reference densities (kp.dref, see lbm_ref.cu): each
// lane decodes with its cell's reference, sets it to the new density and shifts its outputs to it
// (folded into the collision's per-class constant terms).
template <int S, bool REDUCE, bool REF>
__global__ void __launch_bounds__(PAIR_BLOCK, (pair_min_blocks<REDUCE>())) aa_pair_even_kernel(
    const KParams kp, typename Store<S>::E* __restrict__ f, const uint32_t* __restrict__ flags,
    const float* __restrict__ force, const float* __restrict__ pdrag, const float* __restrict__ eps,
    float* __restrict__ rho_out, float* __restrict__ u_out, double* __restrict__ red) {
  using St = Store<S>;
  using Pk = Pair16<S>;
  RedAcc<float> acc;
  uint32_t* __restrict__ fw = reinterpret_cast<uint32_t*>(f);
  uint16_t* __restrict__ fh = reinterpret_cast<uint16_t*>(f);
  const uint32_t npair = kp.n >> 1;
  for (uint32_t p = blockIdx.x * PAIR_BLOCK + threadIdx.x; p < npair; p += gridDim.x * PAIR_BLOCK) {
    const uint32_t c0 = 2u * p, c1 = c0 + 1u;
    const uint2 fl = reinterpret_cast<const uint2*>(flags)[p];
    const bool in0 = c0 >= kp.guard_lo && c0 <= kp.guard_hi, in1 = c1 >= kp.guard_lo && c1 <= kp.guard_hi;
    const bool l0 = in0 && !(fl.x & POG_CELL_SOLID), l1 = in1 && !(fl.y & POG_CELL_SOLID);
    if (!(l0 || l1)) continue;
    const uint32_t fo = (l0 ? fl.x : 0u) | (l1 ? fl.y : 0u);  // flags of the live cells
    bool general = (fo & (POG_CELL_INLET | POG_CELL_OUTLET)) || !(in0 && in1);
    if (pdrag && (!kp.dmask || ((kp.dmask[c0 >> 5] >> (c0 & 31u)) & 3u))) general = true;
    if (general) {
#pragma unroll 1
      for (int lane = 0; lane < 2; ++lane) {
        const uint32_t c = c0 + (uint32_t)lane, flc = lane ? fl.y : fl.x;
        if (!(lane ? l1 : l0)) continue;
        if constexpr (REF) {
          ref_even_cell<REDUCE>(kp, f, c, flc, force, pdrag, eps, nullptr, nullptr, rho_out, u_out, acc);
        } else {
          typename St::E raw[19];
          aa_load<S, 0>(kp, f, c, flc, false, raw);
          float fv[19];
#pragma unroll
          for (int q = 0; q < 19; ++q) fv[q] = St::dech(raw[q]);
          aa_update<S, 0, REDUCE, false>(kp, f, c, flc, false, fv, force, pdrag, eps, nullptr, nullptr, rho_out,
                                         u_out, acc);
        }
      }
      continue;
    }
    // Warp-uniform store form: 32-bit pairs when every pair of the warp has two live cells,
    // else predicated 16-bit halves (a solid cell's slots are never written).
    const bool paired = __all_sync(__activemask(), l0 && l1);

    // ---- gather (c, q): adjacent and aligned for both cells; a dead cell's value is ignored --
    uint32_t w[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) w[q] = fw[(kp.pl[q] + c0) >> 1];

    // ---- moments: the per-cell kernel's sums, both cells per instruction -------------------
    F2 sxx, syy, szz, rsum, mxs, mys, mzs, pxy, pxz, pyz;
    {
      const F2 h0 = Pk::unpack(w[0]);
      const F2 h1 = Pk::unpack(w[1]), h2 = Pk::unpack(w[2]), h3 = Pk::unpack(w[3]), h4 = Pk::unpack(w[4]);
      const F2 h5 = Pk::unpack(w[5]), h6 = Pk::unpack(w[6]);
      const F2 sx = add2(h1, h2), sy = add2(h3, h4), sz = add2(h5, h6);
      const F2 d12 = sub2(h1, h2), d34 = sub2(h3, h4), d56 = sub2(h5, h6);
      const F2 h7 = Pk::unpack(w[7]), h8 = Pk::unpack(w[8]), h9 = Pk::unpack(w[9]), h10 = Pk::unpack(w[10]);
      const F2 a78 = add2(h7, h8), d78 = sub2(h7, h8), a910 = add2(h9, h10), d910 = sub2(h9, h10);
      const F2 h11 = Pk::unpack(w[11]), h12 = Pk::unpack(w[12]), h13 = Pk::unpack(w[13]), h14 = Pk::unpack(w[14]);
      const F2 a1112 = add2(h11, h12), d1112 = sub2(h11, h12), a1314 = add2(h13, h14), d1314 = sub2(h13, h14);
      const F2 h15 = Pk::unpack(w[15]), h16 = Pk::unpack(w[16]), h17 = Pk::unpack(w[17]), h18 = Pk::unpack(w[18]);
      const F2 a1516 = add2(h15, h16), d1516 = sub2(h15, h16), a1718 = add2(h17, h18), d1718 = sub2(h17, h18);
      const F2 sxy = add2(a78, a910), sxz = add2(a1112, a1314), syz = add2(a1516, a1718);
      rsum = add2(add2(add2(h0, add2(sx, sy)), add2(sz, sxy)), add2(sxz, syz));
      mxs = add2(add2(d12, add2(d78, d910)), add2(d1112, d1314));
      mys = add2(add2(d34, sub2(a78, a910)), add2(d1516, d1718));
      mzs = add2(add2(d56, sub2(a1112, a1314)), sub2(a1516, a1718));
      pxy = sub2(d78, d910);
      pxz = sub2(d1112, d1314);
      pyz = sub2(d1516, d1718);
      sxx = add2(add2(sx, sxy), sxz);
      syy = add2(add2(sy, sxy), syz);
      szz = add2(add2(sz, sxz), syz);
    }
    const float sc = St::SCALE, inv_sc = 1.0f / St::SCALE;  // powers of two: exact
    const F2 SC = sp2(sc);
    const F2 drho = mul2(SC, rsum);
    // the cells' shift densities: rho0, or their references rho0 + d_c
    F2 dd = sp2(0.0f);
    if constexpr (REF) {
      __half2 h;
      const uint32_t dw = reinterpret_cast<const uint32_t*>(kp.dref)[c0 >> 1];
      memcpy(&h, &dw, 4);
      dd = __half22float2(h);
    }
    const F2 rho = add2(add2(sp2(kp.rho0), dd), drho);
    // REF: the new references (this step's densities, FP16-rounded) and the shift of the outputs
    // to them, in stored units
    uint32_t dnew_w = 0u;
    F2 dshift = sp2(0.0f);
    if constexpr (REF) {
      const __half2 dn = __float22half2_rn(sub2(rho, sp2(kp.rho0)));
      memcpy(&dnew_w, &dn, 4);
      dshift = mul2(sub2(__half22float2(dn), dd), sp2(F16_SCALE));
    }
    const F2 mx = mul2(SC, mxs), my = mul2(SC, mys), mz = mul2(SC, mzs);
    F2 Gx = mul2(rho, sp2(kp.gx)), Gy = mul2(rho, sp2(kp.gy)), Gz = mul2(rho, sp2(kp.gz));
    if (force) {
      Gx = add2(Gx, reinterpret_cast<const F2*>(force)[p]);
      Gy = add2(Gy, reinterpret_cast<const F2*>(force + kp.n)[p]);
      Gz = add2(Gz, reinterpret_cast<const F2*>(force + 2u * kp.n)[p]);
    }
    if (kp.pour) {
      Gz.x -= pour_accel<float>(kp, c0);
      Gz.y -= pour_accel<float>(kp, c1);
    }
    const F2 inv_rho = make_float2(1.0f / rho.x, 1.0f / rho.y);
    const F2 half = sp2(0.5f);
    F2 ux = mul2(fma2(half, Gx, mx), inv_rho), uy = mul2(fma2(half, Gy, my), inv_rho),
       uz = mul2(fma2(half, Gz, mz), inv_rho);
    F2 Fx = Gx, Fy = Gy, Fz = Gz;
    const bool p0 = l0 && (fl.x & POG_CELL_POROUS), p1 = l1 && (fl.y & POG_CELL_POROUS);
    if (p0)
      porous_drag<float>(kp, c0, eps, rho.x, inv_rho.x, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, Gx.x, Gy.x, Gz.x, mx.x, my.x,
                         mz.x, ux.x, uy.x, uz.x, Fx.x, Fy.x, Fz.x);
    if (p1)
      porous_drag<float>(kp, c1, eps, rho.y, inv_rho.y, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, Gx.y, Gy.y, Gz.y, mx.y, my.y,
                         mz.y, ux.y, uy.y, uz.y, Fx.y, Fy.y, Fz.y);
    const F2 usq = fma2(ux, ux, fma2(uy, uy, mul2(uz, uz)));
    const float tau0 = kp.tau;
    F2 tau = sp2(tau0);
    if (kp.les_mode == POG_LES_LOCAL) {
      // Pi_neq = sum e e f - rho (u u + I/3), in the shifted form (collide.cuh)
      const F2 r3 = mul2(drho, sp2((float)(1.0 / 3.0)));
      const F2 rx = mul2(rho, ux), ry = mul2(rho, uy);
      const F2 Pxx = sub2(mul2(SC, sxx), fma2(rx, ux, r3));
      const F2 Pyy = sub2(mul2(SC, syy), fma2(ry, uy, r3));
      const F2 Pzz = sub2(mul2(SC, szz), fma2(mul2(rho, uz), uz, r3));
      const F2 Pxy = sub2(mul2(SC, pxy), mul2(rx, uy));
      const F2 Pxz = sub2(mul2(SC, pxz), mul2(rx, uz));
      const F2 Pyz = sub2(mul2(SC, pyz), mul2(ry, uz));
      const F2 off = fma2(Pxy, Pxy, fma2(Pxz, Pxz, mul2(Pyz, Pyz)));
      const F2 PP2 = fma2(sp2(4.0f), off, mul2(sp2(2.0f), fma2(Pxx, Pxx, fma2(Pyy, Pyy, mul2(Pzz, Pzz)))));
      const float t2 = tau0 * tau0, k18 = 18.0f * kp.cs2;
      const F2 Q = make_float2(sqrtf(PP2.x), sqrtf(PP2.y));
      const F2 Qr = mul2(Q, inv_rho);
      const F2 disc = fma2(sp2(k18), Qr, sp2(t2));
      const F2 tl = mul2(half, add2(sp2(tau0), make_float2(sqrtf(disc.x), sqrtf(disc.y))));
      // nu = (tl - tau0)/3, zero where |S| = 1.5 Q / (rho tl) is below the floor, capped at nu_max
      const F2 nu = mul2(sub2(tl, sp2(tau0)), sp2((float)(1.0 / 3.0)));
      const F2 smag_tl = mul2(sp2(1.5f), Qr);  // |S| tl
      const F2 floor_tl = mul2(sp2(kp.strain_floor), tl);
      float n0 = smag_tl.x < floor_tl.x || p0 ? 0.0f : fminf(nu.x, kp.nu_max);
      float n1 = smag_tl.y < floor_tl.y || p1 ? 0.0f : fminf(nu.y, kp.nu_max);
      tau = fma2(sp2(3.0f), make_float2(n0, n1), tau);
    }
    if (kp.clamp_tau) {
      tau.x = fminf(fmaxf(tau.x, kp.tau_min), kp.tau_max);
      tau.y = fminf(fmaxf(tau.y, kp.tau_min), kp.tau_max);
    }
    const F2 omega = make_float2(1.0f / tau.x, 1.0f / tau.y);
    const F2 keep = sub2(sp2(1.0f), omega);

    // ---- BGK + Guo collision, on the packed pairs ------------------------------------------
    {
      const F2 Ag = fma2(sp2(-0.5f), omega, sp2(1.0f));
      const F2 uF = fma2(ux, Fx, fma2(uy, Fy, mul2(uz, Fz)));
      const F2 base = fma2(sp2(-1.5f), usq, mul2(drho, inv_rho));
      const F2 or_ = mul2(mul2(omega, rho), sp2(inv_sc));
      const F2 As = mul2(Ag, sp2(inv_sc));
      const F2 a1_0 = mul2(or_, sp2((float)(1.0 / 3.0))), a1_1 = mul2(or_, sp2((float)(1.0 / 18.0))),
               a1_2 = mul2(or_, sp2((float)(1.0 / 36.0)));
      const F2 b3_1 = mul2(As, sp2((float)(3.0 / 18.0))), b3_2 = mul2(As, sp2((float)(3.0 / 36.0)));
      const F2 nuF = mul2(sp2(-1.0f), uF);
      const F2 h0 = Pk::unpack(opaque(w[0]));
      w[0] = Pk::pack(fma2(keep, h0, fma2(sp2(-(float)(1.0 / 3.0)), dshift, fma2(As, nuF, mul2(a1_0, base)))));
      PairCoef2 k1, k2;
      k1.A = fma2(sp2(-(float)(1.0 / 18.0)), dshift, fma2(b3_1, nuF, mul2(a1_1, base)));
      k1.B = mul2(sp2(4.5f), a1_1);
      k1.Cc = mul2(sp2(3.0f), b3_1);
      k1.D = mul2(sp2(3.0f), a1_1);
      k1.b3 = b3_1;
      k2.A = fma2(sp2(-(float)(1.0 / 36.0)), dshift, fma2(b3_2, nuF, mul2(a1_2, base)));
      k2.B = mul2(sp2(4.5f), a1_2);
      k2.Cc = mul2(sp2(3.0f), b3_2);
      k2.D = mul2(sp2(3.0f), a1_2);
      k2.b3 = b3_2;
      collide_dir2<1, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k1);
      collide_dir2<3, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k1);
      collide_dir2<5, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k1);
      collide_dir2<7, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_dir2<8, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_dir2<11, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_dir2<12, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_dir2<15, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_dir2<16, S>(w, ux, uy, uz, Fx, Fy, Fz, keep, k2);
    }

    // ---- macroscopic outputs and sums ------------------------------------------------------
    if (rho_out) {
      if (l0 && l1) {
        reinterpret_cast<F2*>(rho_out)[p] = rho;
      } else {
        if (l0) rho_out[c0] = rho.x;
        if (l1) rho_out[c1] = rho.y;
      }
    }
    if (u_out) {
      if (l0 && l1) {
        reinterpret_cast<F2*>(u_out)[p] = ux;
        reinterpret_cast<F2*>(u_out + kp.n)[p] = uy;
        reinterpret_cast<F2*>(u_out + 2u * kp.n)[p] = uz;
      } else {
#pragma unroll
        for (int lane = 0; lane < 2; ++lane) {
          if (!(lane ? l1 : l0)) continue;
          const uint32_t c = c0 + (uint32_t)lane;
          u_out[c] = lane ? ux.y : ux.x;
          u_out[kp.n + c] = lane ? uy.y : uy.x;
          u_out[2u * kp.n + c] = lane ? uz.y : uz.x;
        }
      }
    }
    if (REDUCE) {
      if (l0) acc.add(CellResult<float>{rho.x, ux.x, uy.x, uz.x, 0.0f});
      if (l1) acc.add(CellResult<float>{rho.y, ux.y, uy.y, uz.y, 0.0f});
    }

    // ---- scatter f*_q to slot (c, opp q) ------------------------------------------------
    // The store addresses repeat the gather's (slot (c, opp q) was gathered for opp q).
    // Rebuilding them from an opaque copy of c0 keeps the compiler from holding 19 64-bit
    // addresses across the collision: two integer instructions per store instead of 38 registers.
    const uint32_t cs = opaque(c0);
    if (paired) {
#pragma unroll
      for (int q = 0; q < 19; ++q) fw[(kp.pl[opp(q)] + cs) >> 1] = w[q];
      if constexpr (REF) reinterpret_cast<uint32_t*>(kp.dref)[cs >> 1] = dnew_w;
    } else {
#pragma unroll
      for (int q = 0; q < 19; ++q) {
        if (l0) fh[kp.pl[opp(q)] + cs] = (uint16_t)w[q];
        if (l1) fh[kp.pl[opp(q)] + cs + 1u] = (uint16_t)(w[q] >> 16);
      }
      if constexpr (REF) {
        uint16_t* dh = reinterpret_cast<uint16_t*>(kp.dref);
        if (l0) dh[cs] = (uint16_t)dnew_w;
        if (l1) dh[cs + 1u] = (uint16_t)(dnew_w >> 16);
      }
    }
  }
  if (REDUCE) reduce_add<float>(acc, red);
}

template <int S, bool REDUCE, bool REF = false>
static int launch_pair(const KParams& kp, void* f, const uint32_t* flags, const float* force, const float* pdrag,
                       const float* eps, float* rho_out, float* u_out, double* red, cudaStream_t s) {
  auto kern = aa_pair_even_kernel<S, REDUCE, REF>;
  static thread_local int grid = 0;
  if (grid == 0) grid = persistent_blocks((const void*)kern, PAIR_BLOCK);
  if (grid <= 0) return set_error(POG_E_CUDA, "occupancy query failed");
  const uint32_t npair = kp.n >> 1;
  const int want = (int)((npair + PAIR_BLOCK - 1) / PAIR_BLOCK);
  const int g = REDUCE ? (want < grid ? want : grid) : want;
  kern<<<g, PAIR_BLOCK, 0, s>>>(kp, (typename Store<S>::E*)f, flags, force, pdrag, eps, rho_out, u_out, red);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

static bool aligned(const void* p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) == 0; }

// The two-cell kernel for one even time step, or 1 when it does not apply (then the caller runs
// the per-cell kernel): an even step, 16-bit storage, even nx, Guo forcing, no phase field, LES
// off or local, and the buffers aligned for the paired accesses.
int launch_pair_step(const KParams& kp, int parity, bool reduce, void* f, const uint32_t* flags,
                     const float* force, const float* pdrag, const float* eps, float* rho_out, float* u_out,
                     double* red, cudaStream_t s) {
  if (parity != 0) return 1;
  if (kp.storage != POG_STORE_F16S && kp.storage != POG_STORE_BF16S) return 1;
  if ((kp.nx & 1u) || kp.les_mode == POG_LES_STENCIL || kp.forcing_mode != POG_FORCING_GUO || kp.phase) return 1;
  if (!aligned(f, 4) || !aligned(flags, 8) || !aligned(force, 8) || !aligned(rho_out, 8) || !aligned(u_out, 8))
    return 1;
  if (kp.dref) {  // FP16S relative to per-cell reference densities
    if (kp.storage != POG_STORE_F16S || !aligned(kp.dref, 4)) return 1;
    return reduce ? launch_pair<POG_STORE_F16S, true, true>(kp, f, flags, force, pdrag, eps, rho_out, u_out, red, s)
                  : launch_pair<POG_STORE_F16S, false, true>(kp, f, flags, force, pdrag, eps, rho_out, u_out, red, s);
  }
  if (kp.storage == POG_STORE_F16S)
    return reduce ? launch_pair<POG_STORE_F16S, true>(kp, f, flags, force, pdrag, eps, rho_out, u_out, red, s)
                  : launch_pair<POG_STORE_F16S, false>(kp, f, flags, force, pdrag, eps, rho_out, u_out, red, s);
  return reduce ? launch_pair<POG_STORE_BF16S, true>(kp, f, flags, force, pdrag, eps, rho_out, u_out, red, s)
                : launch_pair<POG_STORE_BF16S, false>(kp, f, flags, force, pdrag, eps, rho_out, u_out, red, s);
}

}  // namespace pog
