// collide.cuh -- per-cell physics shared by the AA kernels (lbm_aa.cu, lbm_tma.cu) and the push
// kernel (lbm_push.cu): moments, inlet/outlet equilibrium overwrite, Guo forcing with gravity and
// the external force, Darcy-Forchheimer drag in the filter band, LES relaxation, BGK collision.
//
// Reference structure restated (file:line in latteine1217/pour-over-coffee-lbm):
//   moments + Guo half-force velocity   src/core/legacy/lbm_solver.py:488-535
//   BGK + tau_eff = tau + 3 nu_sgs       src/core/legacy/lbm_solver.py:537-579
//   equilibrium                          src/core/lbm_algorithms.py:183-218
//   Guo forcing (standard form default)  docs/mathematical/mathematical_models.md:109-121,
//                                        legacy form legacy/lbm_solver.py:594-607,688-764
//   Smagorinsky nu_sgs + gates           src/physics/les_turbulence.py:318-380
//   Darcy-Forchheimer drag               src/physics/filter_paper.py:471-536
//   inlet/outlet overwrite               src/physics/boundary_conditions.py:194-324
//
// Arithmetic layout (same mathematics as the oracle, arranged for few instructions):
//   - all moments (rho, m, and the raw second moments for LES) come from one sweep of adds
//     over shared partial sums;
//   - the non-equilibrium stress is Pi_neq = sum e e f - rho (u u + I/3), exact for the D3Q19
//     second-order equilibrium, so no per-direction f_eq pass is needed before tau is known;
//   - the collision treats each direction q with its opposite together: f_eq and the Guo term
//     split into a part even in e (shared) and a part odd in e (sign flips), halving the work.
#pragma once
#include "common.cuh"

namespace pog {

template <typename C>
struct CellResult {
  C rho, ux, uy, uz;
  C outflow;  // -m_z on outlet cells, else 0
};

template <typename C>
__host__ __device__ __forceinline__ C inlet_uz(const KParams& kp, uint32_t c) {
  uint32_t i = c % kp.nx;
  uint32_t j = (c / kp.nx) % kp.ny;
  C dx = (C)i - (C)kp.cxf, dy = (C)j - (C)kp.cyf;
  C r = sqrt(dx * dx + dy * dy);
  C R = (C)kp.inlet_R;
  C s = R > (C)0 ? (C)2 * r / R - (C)1 : (C)0;
  const float* ctl = kp.inlet_ctl;
  const float* a = ctl ? ctl + 1 : kp.coef;
  C t0 = (C)1, t1 = s;
  C acc = (C)a[0] + (C)a[1] * t1;
#pragma unroll
  for (int k = 2; k < POG_INLET_NCOEF; ++k) {
    C t2 = (C)2 * s * t1 - t0;
    acc += (C)a[k] * t2;
    t0 = t1;
    t1 = t2;
  }
  return (C)(ctl ? ctl[0] : kp.u_inlet) * ((C)1 + acc);
}

template <typename C>
__host__ __device__ __forceinline__ C feq_q(int q, C rho, C ux, C uy, C uz, C usq15) {
  C eu = (C)cx(q) * ux + (C)cy(q) * uy + (C)cz(q) * uz;
  return (C)wd(q) * rho * ((C)1 + (C)3 * eu + (C)4.5 * eu * eu - usq15);
}

// Downward force density of the pour nozzle on cell c (POG_POUR_* block, precise_pouring.py:
// 100-160): 0 outside the stream cylinder, else min(velocity I flow / dt, cap) with the Gaussian
// radial and exponential vertical intensity I.  Cells outside the stream's planes leave after one
// index compare, so the term costs a full cell only inside the nozzle.  Out of line: its
// registers are not reserved in the step kernel's main path.
template <typename C>
__device__ __noinline__ C pour_accel(const KParams& kp, uint32_t c) {
  const float* b = kp.pour;
  if (b[POG_POUR_ACTIVE] == 0.0f) return (C)0;
  const float ztop = b[POG_POUR_ZTOP];
  const float klo = ceilf(ztop - b[POG_POUR_HEIGHT]), khi = floorf(ztop);
  if (!(khi >= 0.0f) || klo > (float)(kp.nz - 1) || khi < klo) return (C)0;
  const uint32_t c0 = (uint32_t)fmaxf(klo, 0.0f) * kp.nxny;
  const uint32_t c1 = ((uint32_t)fminf(khi, (float)(kp.nz - 1)) + 1u) * kp.nxny;
  if (c < c0 || c >= c1) return (C)0;
  const uint32_t k = c / kp.nxny, rem = c - k * kp.nxny, j = rem / kp.nx, i = rem - j * kp.nx;
  const C dx = (C)i - (C)b[POG_POUR_X], dy = (C)j - (C)b[POG_POUR_Y];
  const C R = (C)b[POG_POUR_RADIUS];
  const C d = sqrt(dx * dx + dy * dy);
  if (!(d <= R)) return (C)0;
  const C dr = d / R;
  const C I = exp((C)-0.5 * dr * dr) * exp(-((C)ztop - (C)k) / (C)2);
  const C dt = (C)b[POG_POUR_DT];
  C a = dt > (C)1e-8 ? (C)b[POG_POUR_VELOCITY] * I * (C)b[POG_POUR_FLOW] / dt : (C)0;
  const C cap = (C)b[POG_POUR_ACCEL_CAP];
  return a < cap ? a : cap;
}

// f_eq_q - w_q rs for a density rr = rs + dr, without forming f_eq_q: w_q (dr + rr (3 e.u +
// 4.5 (e.u)^2 - 1.5 u.u)).
template <typename C>
__host__ __device__ __forceinline__ C feq_dev_q(int q, C rr, C dr, C ux, C uy, C uz, C usq15) {
  C eu = (C)cx(q) * ux + (C)cy(q) * uy + (C)cz(q) * uz;
  return (C)wd(q) * (dr + rr * ((C)3 * eu + (C)4.5 * eu * eu - usq15));
}

// One direction pair (q, opp q) of the BGK + Guo collision, q with e = (ex, ey, ez), written as
// a chain of FMAs.  Per weight class w (a1 = omega w rho, b3 = 3 (1 - omega/2) w):
//   omega f_eq + S, even in e:  sym  = A + (e.u)(B e.u + Cc e.F),  A = a1 (1 - 1.5 u.u) - b3 u.F,
//                                                                  B = 4.5 a1, Cc = 3 b3
//   omega f_eq + S, odd in e:   asym = D e.u + b3 e.F,             D = 3 a1
//   f*_q = (1 - omega) f_q + sym + asym,  f*_opp = (1 - omega) f_opp + sym - asym.
template <typename C>
struct PairCoef {
  C A, B, Cc, D, b3;
};
template <typename C>
__host__ __device__ __forceinline__ PairCoef<C> pair_coef(C a1, C b3, C uF, C base) {
  PairCoef<C> k;
  k.A = a1 * base - b3 * uF;
  k.B = (C)4.5 * a1;
  k.Cc = (C)3 * b3;
  k.D = (C)3 * a1;
  k.b3 = b3;
  return k;
}
// e_q . v with only the non-zero components of e_q (signs folded at compile time).  Same value
// as cx v_x + cy v_y + cz v_z summed left to right: the zero terms add nothing, and IEEE
// arithmetic would not let the compiler drop 0 * v itself.
template <int Q, typename C>
__host__ __device__ __forceinline__ C edotq(C x, C y, C z) {
  constexpr int a = cx(Q), b = cy(Q), c = cz(Q);
  C r;
  if constexpr (a != 0) {
    r = a > 0 ? x : -x;
    if constexpr (b != 0) r = b > 0 ? r + y : r - y;
    if constexpr (c != 0) r = c > 0 ? r + z : r - z;
  } else if constexpr (b != 0) {
    r = b > 0 ? y : -y;
    if constexpr (c != 0) r = c > 0 ? r + z : r - z;
  } else {
    r = c > 0 ? z : -z;
  }
  return r;
}

template <int Q, typename C>
__host__ __device__ __forceinline__ void collide_pair(C f[19], C ux, C uy, C uz, C Fx, C Fy, C Fz, C keep,
                                                      const PairCoef<C>& k) {
  constexpr int P = opp(Q);
  const C eu = edotq<Q, C>(ux, uy, uz);
  const C eF = edotq<Q, C>(Fx, Fy, Fz);
  const C sym = fma(eu, fma(k.Cc, eF, k.B * eu), k.A);
  const C asym = fma(k.D, eu, k.b3 * eF);
  const C fq = f[Q], fp = f[P];
  f[Q] = fma(keep, fq, sym + asym);
  f[P] = fma(keep, fp, sym - asym);
}

// Two direction pairs (Q1, Q2) of one weight class at once, in Blackwell's packed FP32x2
// arithmetic (FFMA2/FADD2/FMUL2: two FP32 lanes per instruction, each lane rounded as its
// scalar counterpart).  Same update as collide_pair.
template <int Q1, int Q2, typename C>
__device__ __forceinline__ void collide_pair2(C f[19], C ux, C uy, C uz, C Fx, C Fy, C Fz, C keep,
                                              const PairCoef<C>& k) {
  static_assert(sizeof(C) == 4, "packed pairs are FP32");
  constexpr int P1 = opp(Q1), P2 = opp(Q2);
  const float2 EU = make_float2(edotq<Q1, C>(ux, uy, uz), edotq<Q2, C>(ux, uy, uz));
  const float2 EF = make_float2(edotq<Q1, C>(Fx, Fy, Fz), edotq<Q2, C>(Fx, Fy, Fz));
  const float2 A = make_float2(k.A, k.A), B = make_float2(k.B, k.B), Cc = make_float2(k.Cc, k.Cc);
  const float2 D = make_float2(k.D, k.D), b3 = make_float2(k.b3, k.b3), K = make_float2(keep, keep);
  const float2 sym = __ffma2_rn(EU, __ffma2_rn(Cc, EF, __fmul2_rn(B, EU)), A);
  const float2 asym = __ffma2_rn(D, EU, __fmul2_rn(b3, EF));
  const float2 FQ = __ffma2_rn(K, make_float2(f[Q1], f[Q2]), __fadd2_rn(sym, asym));
  const float2 FP = __ffma2_rn(K, make_float2(f[P1], f[P2]), __ffma2_rn(asym, make_float2(-1.0f, -1.0f), sym));
  f[Q1] = FQ.x;
  f[Q2] = FQ.y;
  f[P1] = FP.x;
  f[P2] = FP.y;
}

// Velocity and total force of a cell of the filter-paper band (filter_paper.py:471-536): the
// Darcy-Forchheimer drag rho (nu/K + C_F |u| / sqrt K) u, semi-implicit (Guo & Zhao 2002, solved
// in closed form) or explicit and capped (POG_DRAG_EXPLICIT_CAP), with the particle deposit
// (Kp, Kv) implicit.  On entry u = (m + (G + Kv)/2) / rho, the velocity with every explicit force
// and A = 1 + Kp/(2 rho) not yet divided out; on exit u and F are the cell's collision velocity
// and force density.
template <typename C>
__host__ __device__ __forceinline__ void porous_drag(const KParams& kp, uint32_t c, const float* __restrict__ eps,
                                                     C rho, C inv_rho, C A, C Kp, C Kvx, C Kvy, C Kvz, C Gx,
                                                     C Gy, C Gz, C mx, C my, C mz, C& ux, C& uy, C& uz, C& Fx,
                                                     C& Fy, C& Fz) {
  C K = (C)kp.K0, CF = (C)kp.CF0;
  if (eps) {
    C e = (C)eps[c];
    C g = e * e * e / (((C)1 - e) * ((C)1 - e));
    K = (C)kp.K0 * (g / (C)kp.g0);
    C r = (C)kp.eps0 / e;
    CF = (C)kp.CF0 * (r * sqrt(r));
  }
  // Darcy nu/K and Forchheimer C_F/sqrt(K) coefficients, both scaled by the filter
  // blockage factor 1 + b when a blockage field is given
  C dk = (C)kp.nu0 / K, fk = CF / sqrt(K);
  if (kp.blockage) {
    const C bf = (C)1 + (C)kp.blockage[c];
    dk *= bf;
    fk *= bf;
  }
  if (kp.drag_mode == POG_DRAG_SEMI_IMPLICIT) {
    // Guo & Zhao 2002: u (A + nu/(2K) + C_F|u|/(2 sqrt K)) = v, solved in closed form.
    C c0 = (C)0.5 * (A + (C)0.5 * dk);
    C c1 = (C)0.5 * fk;
    C vm = sqrt(ux * ux + uy * uy + uz * uz);
    C s = (C)1 / (c0 + sqrt(c0 * c0 + c1 * vm));
    ux *= s;
    uy *= s;
    uz *= s;
    C um = sqrt(ux * ux + uy * uy + uz * uz);
    C coef = rho * (dk + fk * um) + Kp;
    Fx = Gx + Kvx - coef * ux;
    Fy = Gy + Kvy - coef * uy;
    Fz = Gz + Kvz - coef * uz;
  } else {
    ux /= A;
    uy /= A;
    uz /= A;
    C vm = sqrt(ux * ux + uy * uy + uz * uz);
    C coef = rho * (dk + fk * vm);
    C dx = -coef * ux, dy = -coef * uy, dz = -coef * uz;
    C dm = sqrt(dx * dx + dy * dy + dz * dz);
    C cap = (C)kp.drag_cap;
    if (dm > cap) {
      C sc = cap / dm;
      dx *= sc;
      dy *= sc;
      dz *= sc;
    }
    // capped drag as an explicit force, particle drag implicit: u A = (m + (G + Kv + F_d)/2)/rho
    ux = (mx + (C)0.5 * (Gx + Kvx + dx)) * inv_rho / A;
    uy = (my + (C)0.5 * (Gy + Kvy + dy)) * inv_rho / A;
    uz = (mz + (C)0.5 * (Gz + Kvz + dz)) * inv_rho / A;
    Fx = Gx + dx + Kvx - Kp * ux;
    Fy = Gy + dy + Kvy - Kp * uy;
    Fz = Gz + dz + Kvz - Kp * uz;
  }
}

// f[19]: incoming populations on entry, post-collision populations on exit.
// SH (shifted): f holds h_q = (f_q - w_q rs) / sc instead of f_q, in and out -- the form the
// shifted storages keep, rs = the cell's shift density.  Moments, Pi_neq and the post-collision
// update are rewritten for h (the shift and scale fold into per-cell coefficients), so no
// population is ever converted back.
// nu_st: nu_sgs from the velocity stencil (LES_STENCIL mode), computed by the caller.
// pdrag: [4][n] particle drag deposit (Kp = sum w beta, Kv = sum w beta v_p) or null; the
// particle force on the fluid, Kv - Kp u, is taken implicitly in u (stable at any loading).
template <typename C, bool SH = false>
__host__ __device__ __forceinline__ CellResult<C> collide_cell(const KParams& kp, uint32_t fl, uint32_t c,
                                                               C f[19], const float* __restrict__ force,
                                                               const float* __restrict__ pdrag,
                                                               const float* __restrict__ eps, C nu_st,
                                                               C sc = (C)1, C rs = (C)0) {
  CellResult<C> res;
  const C rho0 = rs;  // shift density (SH only)
  // ---- moments from one sweep of adds (of h when SH: sum w = 1, sum w e = 0, sum w e e = I/3) --
  const C sx = f[1] + f[2], sy = f[3] + f[4], sz = f[5] + f[6];
  const C sxy = (f[7] + f[8]) + (f[9] + f[10]);
  const C sxz = (f[11] + f[12]) + (f[13] + f[14]);
  const C syz = (f[15] + f[16]) + (f[17] + f[18]);
  const C rsum = f[0] + (sx + sy) + (sz + sxy) + (sxz + syz);
  const C mxs = (f[1] - f[2]) + ((f[7] - f[8]) + (f[9] - f[10])) + ((f[11] - f[12]) + (f[13] - f[14]));
  const C mys = (f[3] - f[4]) + ((f[7] + f[8]) - (f[9] + f[10])) + ((f[15] - f[16]) + (f[17] - f[18]));
  const C mzs = (f[5] - f[6]) + ((f[11] + f[12]) - (f[13] + f[14])) + ((f[15] + f[16]) - (f[17] + f[18]));
  // SH: drho = rho - rs straight from the deviations (no cancellation against rs)
  const C drho = SH ? sc * rsum : (C)0;
  const C rho = SH ? rho0 + drho : rsum;
  const C mx = SH ? sc * mxs : mxs, my = SH ? sc * mys : mys, mz = SH ? sc * mzs : mzs;
  const C inv_sc = SH ? (C)1 / sc : (C)1;
  res.outflow = (C)0;
  if (fl & (POG_CELL_INLET | POG_CELL_OUTLET)) {
    C ux, uy, uz, rr;
    if (fl & POG_CELL_INLET) {
      ux = (C)0;
      uy = (C)0;
      uz = inlet_uz<C>(kp, c);
      rr = rho;
    } else {
      ux = mx / rho;
      uy = my / rho;
      uz = mz / rho;
      rr = (C)kp.rho_out;
      res.outflow = -mz;
    }
    C usq15 = (C)1.5 * (ux * ux + uy * uy + uz * uz);
    // SH: f_eq - w rs = w ((rr - rs) + rr (3 e.u + 4.5 (e.u)^2 - 1.5 u.u)), rr - rs exact
    const C dr = SH ? ((fl & POG_CELL_INLET) ? drho : rr - rho0) : (C)0;
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q] = SH ? feq_dev_q<C>(q, rr, dr, ux, uy, uz, usq15) * inv_sc
                                           : feq_q<C>(q, rr, ux, uy, uz, usq15);
    res.rho = rho;
    res.ux = ux;
    res.uy = uy;
    res.uz = uz;
    return res;
  }

  // Phase indicator (multiphase runs): gravity acts on the water fraction only, tau follows
  // the phase, LES is off in the interface and the air (legacy/lbm_solver.py:558-592).
  const C ph = kp.phase ? (C)kp.phase[c] : (C)1;
  // Total non-drag force density: gravity rho*g plus the external (particle/plugin) force.
  const C rg = kp.phase ? (ph > (C)0.001 ? rho * ph : (C)0) : rho;
  C Gx = rg * (C)kp.gx, Gy = rg * (C)kp.gy, Gz = rg * (C)kp.gz;
  if (force) {
    Gx += (C)force[c];
    Gy += (C)force[kp.n + c];
    Gz += (C)force[2u * kp.n + c];
  }
  if (kp.pour) Gz -= pour_accel<C>(kp, c);
  const C inv_rho = (C)1 / rho;
  // Particle drag deposit: F_p = Kv - Kp u with u implicit.  v is the velocity with every
  // explicit force, A the implicit factor (1 without particles).
  C Kp = (C)0, Kvx = (C)0, Kvy = (C)0, Kvz = (C)0;
  // with a deposit mask only the cells the particles deposited into are read (zero elsewhere)
  if (pdrag && kp.dmask && !((kp.dmask[c >> 5] >> (c & 31u)) & 1u)) pdrag = nullptr;
  if (pdrag) {
    Kp = (C)pdrag[c];
    Kvx = (C)pdrag[kp.n + c];
    Kvy = (C)pdrag[2u * kp.n + c];
    Kvz = (C)pdrag[3u * kp.n + c];
  }
  const C A = (C)1 + (C)0.5 * Kp * inv_rho;
  C ux = (mx + (C)0.5 * (Gx + Kvx)) * inv_rho, uy = (my + (C)0.5 * (Gy + Kvy)) * inv_rho,
    uz = (mz + (C)0.5 * (Gz + Kvz)) * inv_rho;
  C Fx = Gx, Fy = Gy, Fz = Gz;
  const bool porous = (fl & POG_CELL_POROUS) != 0;
  if (porous) {
    porous_drag<C>(kp, c, eps, rho, inv_rho, A, Kp, Kvx, Kvy, Kvz, Gx, Gy, Gz, mx, my, mz, ux, uy, uz, Fx, Fy,
                   Fz);
  } else if (pdrag) {
    ux /= A;
    uy /= A;
    uz /= A;
    Fx = Gx + Kvx - Kp * ux;
    Fy = Gy + Kvy - Kp * uy;
    Fz = Gz + Kvz - Kp * uz;
  }
  const C usq = ux * ux + uy * uy + uz * uz;
  const C tau0 = kp.phase ? (ph > (C)0.5 ? (C)kp.tau : (C)kp.tau_air) : (C)kp.tau;
  // the LES phase gate |phase| < 0.9 (les_turbulence.py:362-366)
  const bool les_on = !porous && !(kp.phase && ph < (C)0.9 && ph > (C)-0.9);
  C nu = (C)0;
  if (kp.les_mode == POG_LES_LOCAL && les_on) {
    // Pi_neq = sum e e f - rho (u u + I/3)
    // SH: sum e_a e_b f = rho0/3 delta_ab + sc sum e_a e_b h
    const C r3 = (SH ? drho : rho) * (C)(1.0 / 3.0);
    const C m2 = SH ? sc : (C)1;
    const C Pxx = m2 * (sx + sxy + sxz) - (rho * ux * ux + r3);
    const C Pyy = m2 * (sy + sxy + syz) - (rho * uy * uy + r3);
    const C Pzz = m2 * (sz + sxz + syz) - (rho * uz * uz + r3);
    const C Pxy = m2 * ((f[7] - f[8]) - (f[9] - f[10])) - rho * ux * uy;
    const C Pxz = m2 * ((f[11] - f[12]) - (f[13] - f[14])) - rho * ux * uz;
    const C Pyz = m2 * ((f[15] - f[16]) - (f[17] - f[18])) - rho * uy * uz;
    const C PP = Pxx * Pxx + Pyy * Pyy + Pzz * Pzz + (C)2 * (Pxy * Pxy + Pxz * Pxz + Pyz * Pyz);
    const C Q = sqrt((C)2 * PP);
    const C tl = (C)0.5 * (tau0 + sqrt(tau0 * tau0 + (C)18 * (C)kp.cs2 * Q * inv_rho));
    const C smag = (C)1.5 * Q * inv_rho / tl;
    nu = (tl - tau0) * (C)(1.0 / 3.0);
    if (smag < (C)kp.strain_floor) nu = (C)0;
    nu = nu < (C)kp.nu_max ? nu : (C)kp.nu_max;
  } else if (kp.les_mode == POG_LES_STENCIL && les_on) {
    nu = nu_st;
  }
  C tau = tau0 + (C)3 * nu;
  if (kp.clamp_tau) tau = tau < (C)kp.tau_min ? (C)kp.tau_min : (tau > (C)kp.tau_max ? (C)kp.tau_max : tau);
  const C omega = (C)1 / tau;
  const C keep = (C)1 - omega;

  if (kp.forcing_mode == POG_FORCING_GUO) {
    const C A = (C)1 - (C)0.5 * omega;
    const C uF = ux * Fx + uy * Fy + uz * Fz;
    // SH: h* = keep h + (omega f_eq + S - omega w rs) / sc.  The shift joins the even part as
    // base = (rho - rs)/rho - 1.5 u.u (omega w rho (1 - 1.5 u.u) - omega w rs), with rho - rs
    // taken from the deviation sum, and 1/sc scales the two per-cell factors omega rho and A, so
    // every coefficient below carries both.
    const C base = SH ? drho * inv_rho - (C)1.5 * usq : (C)1 - (C)1.5 * usq;
    const C or_ = SH ? omega * rho * inv_sc : omega * rho;
    const C As = SH ? A * inv_sc : A;
    // weight classes: w0 = 1/3 (rest), w1 = 1/18 (axes), w2 = 1/36 (edges)
    const C a1_0 = or_ * (C)(1.0 / 3.0), a1_1 = or_ * (C)(1.0 / 18.0), a1_2 = or_ * (C)(1.0 / 36.0);
    const C b3_0 = As, b3_1 = As * (C)(3.0 / 18.0), b3_2 = As * (C)(3.0 / 36.0);
    // rest population: f0* = keep f0 + omega w0 rho base - 3 A w0 uF
    f[0] = keep * f[0] + (a1_0 * base - b3_0 * uF);
    const PairCoef<C> k1 = pair_coef<C>(a1_1, b3_1, uF, base), k2 = pair_coef<C>(a1_2, b3_2, uF, base);
    if constexpr (sizeof(C) == 4) {
      // FP32: eight of the nine pairs two at a time in packed FP32x2 arithmetic
      collide_pair2<1, 3>(f, ux, uy, uz, Fx, Fy, Fz, keep, k1);
      collide_pair<5, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k1);
      collide_pair2<7, 8>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_pair2<11, 12>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_pair2<15, 16>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
    } else {
      collide_pair<1, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k1);
      collide_pair<3, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k1);
      collide_pair<5, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k1);
      collide_pair<7, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_pair<8, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_pair<11, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_pair<12, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_pair<15, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
      collide_pair<16, C>(f, ux, uy, uz, Fx, Fy, Fz, keep, k2);
    }
  } else {
    const C usq15 = (C)1.5 * usq;
    C taus = tau < (C)0.6 ? (C)0.6 : (tau > (C)1.5 ? (C)1.5 : tau);
    C fn = sqrt(Fx * Fx + Fy * Fy + Fz * Fz);
    C sf = fn > (C)10 ? (C)10 / fn : (C)1;
    C fx = Fx * sf, fy = Fy * sf, fz = Fz * sf;
    C un = sqrt(usq);
    C su = un <= (C)0.2 ? (C)1 : (C)0.2 / un;
    C sxv = ux * su, syv = uy * su, szv = uz * su;
    C uf = sxv * fx + syv * fy + szv * fz;
    C pref = (C)1 - (C)0.5 / taus;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      C S = (C)0;
      if (fn > (C)1e-15) {
        C eu = (C)cx(q) * sxv + (C)cy(q) * syv + (C)cz(q) * szv;
        C ef = (C)cx(q) * fx + (C)cy(q) * fy + (C)cz(q) * fz;
        S = (C)wd(q) * pref * ((C)3 * ef + (C)9 * eu * uf);
        S = S < (C)-0.5 ? (C)-0.5 : (S > (C)0.5 ? (C)0.5 : S);
      }
      const C fe = feq_q<C>(q, rho, ux, uy, uz, usq15);
      if (SH) {
        const C he = feq_dev_q<C>(q, rho, drho, ux, uy, uz, usq15) * inv_sc;
        f[q] = he + keep * (f[q] - he) + S * inv_sc;
      } else {
        f[q] = fe + keep * (f[q] - fe) + S;
      }
    }
  }
  res.rho = rho;
  res.ux = ux;
  res.uy = uy;
  res.uz = uz;
  return res;
}

// Central-difference velocity gradient of cell c from u[3][n]: g[3 a + b] = du_a/dx_b
// (les_turbulence.py:318-380).  Fluid cells are interior, so the 6 neighbours exist.
template <typename C>
__host__ __device__ __forceinline__ void les_stencil_grad(const KParams& kp, uint32_t c, const float* __restrict__ u,
                                                         C g[9]) {
  const uint32_t n = kp.n, st[3] = {1u, kp.nx, kp.nxny};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float* v = u + (uint32_t)a * n;
#pragma unroll
    for (int b = 0; b < 3; ++b) g[3 * a + b] = ((C)v[c + st[b]] - (C)v[c - st[b]]) * (C)0.5;
  }
}

// |S| = sqrt(2 S:S) of a gradient g (S the symmetric part).
template <typename C>
__host__ __device__ __forceinline__ C les_smag(const C g[9]) {
  const C S12 = (C)0.5 * (g[1] + g[3]), S13 = (C)0.5 * (g[2] + g[6]), S23 = (C)0.5 * (g[5] + g[7]);
  return sqrt((C)2 * (g[0] * g[0] + g[4] * g[4] + g[8] * g[8] + (C)2 * (S12 * S12 + S13 * S13 + S23 * S23)));
}

// LES nu_sgs from central differences of the previous step's velocity u[3][n]
// (les_turbulence.py:318-380): nu = min(cs^2 |S|, nu_max), zero below the strain floor.
template <typename C>
__host__ __device__ __forceinline__ C les_nu_stencil(const KParams& kp, uint32_t c,
                                                     const float* __restrict__ u) {
  C g[9];
  les_stencil_grad<C>(kp, c, u, g);
  const C smag = les_smag<C>(g);
  if (smag < (C)kp.strain_floor) return (C)0;
  C nu = (C)kp.cs2 * smag;
  return nu < (C)kp.nu_max ? nu : (C)kp.nu_max;
}

// ---- storage formats ------------------------------------------------------------------------
template <int S>
struct Store;
// dec/enc convert between a stored value and f_q (rs = the shift density of the slot's cell);
// dech/ench between a stored value and the form collide_cell<C, SHIFTED> works on (h_q =
// (f_q - w_q rs) / SCALE when SHIFTED, else f_q).  FP32 and FP64 store the shifted form (scale
// 1): f_q of a slow flow is w_q rs plus a small deviation, and keeping only the deviation keeps its
// digits (in FP64 it keeps the rounding noise of a trajectory ~100x below that of stored f, which
// is what finite-difference checks of the adjoint resolve).
template <>
struct Store<POG_STORE_F32> {
  using E = float;
  using C = float;
  static constexpr bool SHIFTED = true;
  static constexpr float SCALE = 1.0f;
  __device__ static __forceinline__ C dec(E v, int q, C rs) { return __fadd_rn(v, __fmul_rn((float)wd(q), rs)); }
  __device__ static __forceinline__ E enc(C v, int q, C rs) { return __fsub_rn(v, __fmul_rn((float)wd(q), rs)); }
  __device__ static __forceinline__ C dech(E v) { return v; }
  __device__ static __forceinline__ E ench(C v) { return v; }
  __device__ static __forceinline__ C ld(const E* p, uint32_t i, int q, C r) { return dec(p[i], q, r); }
  __device__ static __forceinline__ void st(E* p, uint32_t i, int q, C v, C r) { p[i] = enc(v, q, r); }
};
template <>
struct Store<POG_STORE_F64> {
  using E = double;
  using C = double;
  static constexpr bool SHIFTED = true;
  static constexpr float SCALE = 1.0f;
  __device__ static __forceinline__ C dec(E v, int q, C rs) { return v + wd(q) * rs; }
  __device__ static __forceinline__ E enc(C v, int q, C rs) { return v - wd(q) * rs; }
  __device__ static __forceinline__ C dech(E v) { return v; }
  __device__ static __forceinline__ E ench(C v) { return v; }
  __device__ static __forceinline__ C ld(const E* p, uint32_t i, int q, C r) { return dec(p[i], q, r); }
  __device__ static __forceinline__ void st(E* p, uint32_t i, int q, C v, C r) { p[i] = enc(v, q, r); }
};
// 16-bit storages hold the shifted form h = (f - w_q rs) / SCALE (FP16: SCALE = 2^-12 keeps
// small deviations normal; BF16: SCALE = 1).  dec is one rounding of w + h SCALE and enc rounds
// (f - w) / SCALE once before the 16-bit rounding, w = fl(w_q rs): the same roundings, in the
// same order, as the oracle's storage emulation.  The step kernel skips dec/enc altogether and
// collides h directly (dech/ench are the bare 16-bit conversions).
template <>
struct Store<POG_STORE_F16S> {
  using E = __half;
  using C = float;
  static constexpr bool SHIFTED = true;
  static constexpr float SCALE = F16_INV_SCALE;
  __device__ static __forceinline__ C dec(E v, int q, C rho0) {
    return __fmaf_rn(__half2float(v), F16_INV_SCALE, __fmul_rn((float)wd(q), rho0));
  }
  __device__ static __forceinline__ E enc(C v, int q, C rho0) {
    const float w = __fmul_rn((float)wd(q), rho0);
    return __float2half_rn(__fmaf_rn(v, F16_SCALE, -w * F16_SCALE));
  }
  __device__ static __forceinline__ C dech(E v) { return __half2float(v); }
  __device__ static __forceinline__ E ench(C v) { return __float2half_rn(v); }
  __device__ static __forceinline__ C ld(const E* p, uint32_t i, int q, C r) { return dec(p[i], q, r); }
  __device__ static __forceinline__ void st(E* p, uint32_t i, int q, C v, C r) { p[i] = enc(v, q, r); }
};
template <>
struct Store<POG_STORE_BF16S> {
  using E = __nv_bfloat16;
  using C = float;
  static constexpr bool SHIFTED = true;
  static constexpr float SCALE = 1.0f;
  __device__ static __forceinline__ C dec(E v, int q, C rho0) {
    return __fadd_rn(__bfloat162float(v), __fmul_rn((float)wd(q), rho0));
  }
  __device__ static __forceinline__ E enc(C v, int q, C rho0) {
    return __float2bfloat16_rn(__fsub_rn(v, __fmul_rn((float)wd(q), rho0)));
  }
  __device__ static __forceinline__ C dech(E v) { return __bfloat162float(v); }
  __device__ static __forceinline__ E ench(C v) { return __float2bfloat16_rn(v); }
  __device__ static __forceinline__ C ld(const E* p, uint32_t i, int q, C r) { return dec(p[i], q, r); }
  __device__ static __forceinline__ void st(E* p, uint32_t i, int q, C v, C r) { p[i] = enc(v, q, r); }
};

// Per-thread partial sums of the POG_RED_* slots (mass, momentum, outflow, non-finite count).
// GB300 issues FP64 arithmetic at a small fraction of the FP32 rate, so FP32 cells accumulate in
// double-float form: an unevaluated sum hi + lo of two floats, updated with error-free
// transformations (Knuth's TwoSum; the product rho*u split exactly by one FMA).  The partial
// carries ~48 significant bits; FP64 is used once per thread, when the partials enter the block
// reduction.  FP64 cells accumulate in FP64.
template <typename C>
struct RedAcc {
  double s[POG_RED_COUNT];
  __device__ __forceinline__ RedAcc() {
#pragma unroll
    for (int r = 0; r < POG_RED_COUNT; ++r) s[r] = 0.0;
  }
  __device__ __forceinline__ void add(const CellResult<C>& r) {
    s[POG_RED_MASS] += (double)r.rho;
    s[POG_RED_MOMX] += (double)r.rho * (double)r.ux;
    s[POG_RED_MOMY] += (double)r.rho * (double)r.uy;
    s[POG_RED_MOMZ] += (double)r.rho * (double)r.uz;
    s[POG_RED_OUTFLOW] += (double)r.outflow;
    const bool bad = !(isfinite((double)r.rho) && isfinite((double)r.ux) && isfinite((double)r.uy) &&
                       isfinite((double)r.uz));
    s[POG_RED_NONFINITE] += bad ? 1.0 : 0.0;
  }
  __device__ __forceinline__ void finish(double out[POG_RED_COUNT]) const {
#pragma unroll
    for (int r = 0; r < POG_RED_COUNT; ++r) out[r] = s[r];
  }
};

template <>
struct RedAcc<float> {
  float hi[POG_RED_COUNT - 1], lo[POG_RED_COUNT - 1];
  unsigned bad;
  __device__ __forceinline__ RedAcc() : bad(0u) {
#pragma unroll
    for (int r = 0; r < POG_RED_COUNT - 1; ++r) hi[r] = lo[r] = 0.0f;
  }
  // (hi, lo) += x without rounding loss: TwoSum gives s + e == hi + x exactly
  __device__ static __forceinline__ void two_sum(float& h, float& l, float x) {
    const float s = __fadd_rn(h, x);
    const float bv = __fsub_rn(s, h);
    const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bv)), __fsub_rn(x, bv));
    h = s;
    l = __fadd_rn(l, e);
  }
  __device__ static __forceinline__ void two_prod_sum(float& h, float& l, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);  // a*b == p + pe exactly
    two_sum(h, l, p);
    l = __fadd_rn(l, pe);
  }
  __device__ __forceinline__ void add(const CellResult<float>& r) {
    two_sum(hi[POG_RED_MASS], lo[POG_RED_MASS], r.rho);
    two_prod_sum(hi[POG_RED_MOMX], lo[POG_RED_MOMX], r.rho, r.ux);
    two_prod_sum(hi[POG_RED_MOMY], lo[POG_RED_MOMY], r.rho, r.uy);
    two_prod_sum(hi[POG_RED_MOMZ], lo[POG_RED_MOMZ], r.rho, r.uz);
    two_sum(hi[POG_RED_OUTFLOW], lo[POG_RED_OUTFLOW], r.outflow);
    bad += (isfinite(r.rho) && isfinite(r.ux) && isfinite(r.uy) && isfinite(r.uz)) ? 0u : 1u;
  }
  __device__ __forceinline__ void finish(double out[POG_RED_COUNT]) const {
#pragma unroll
    for (int r = 0; r < POG_RED_COUNT - 1; ++r) out[r] = (double)hi[r] + (double)lo[r];
    out[POG_RED_NONFINITE] = (double)bad;
  }
  // Sum the warp's 32 accumulators into lane 0, still in FP32 double-float form (FP64
  // arithmetic runs at a small fraction of the FP32 rate on this GPU, so it is left to one
  // lane per warp).
  __device__ __forceinline__ void warp_sum() {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int r = 0; r < POG_RED_COUNT - 1; ++r) {
        const float h2 = __shfl_down_sync(0xffffffffu, hi[r], o);
        const float l2 = __shfl_down_sync(0xffffffffu, lo[r], o);
        two_sum(hi[r], lo[r], h2);
        lo[r] = __fadd_rn(lo[r], l2);
      }
      bad += __shfl_down_sync(0xffffffffu, bad, o);
    }
  }
};
static_assert(POG_RED_NONFINITE == POG_RED_COUNT - 1, "the count slot is last");

// FP64 block reduction of the POG_RED_* slots: warp shuffles, shared memory, one atomic per
// block and slot.  All threads of the block must call it.
__device__ __forceinline__ void block_reduce_add(double v[POG_RED_COUNT], double* out) {
  __shared__ double sm[POG_RED_COUNT][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int r = 0; r < POG_RED_COUNT; ++r) {
    double x = v[r];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sm[r][warp] = x;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int r = 0; r < POG_RED_COUNT; ++r) {
      double x = lane < nw ? sm[r][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0 && x != 0.0) atomicAdd(out + r, x);
    }
  }
}

// Block reduction of a thread's accumulator into the POG_RED_* slots (one atomic per block and
// slot).  FP32 accumulators are summed across the warp in double-float form first and only the
// warps' totals are converted to FP64; FP64 accumulators take block_reduce_add.
template <typename C>
__device__ __forceinline__ void reduce_add(RedAcc<C>& acc, double* out) {
  if constexpr (sizeof(C) == 8) {
    double part[POG_RED_COUNT];
    acc.finish(part);
    block_reduce_add(part, out);
  } else {
    __shared__ double sm[POG_RED_COUNT][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    acc.warp_sum();
    if (lane == 0) {
      double part[POG_RED_COUNT];
      acc.finish(part);
#pragma unroll
      for (int r = 0; r < POG_RED_COUNT; ++r) sm[r][warp] = part[r];
    }
    __syncthreads();
    if (warp == 0 && lane < POG_RED_COUNT) {
      double x = 0.0;
      for (int w = 0; w < nw; ++w) x += sm[lane][w];
      if (x != 0.0) atomicAdd(out + lane, x);
    }
  }
}

}  // namespace pog
