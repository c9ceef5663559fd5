// adjoint.cu -- reverse of one natural-layout step (pog_step_push), hand-derived.
//
// The reference has no adjoint (no Taichi autodiff on this path); this is new work checked
// against central finite differences of the forward step and against the CPU restatement's
// FP64 adjoint.  Forward step: f^{t+1} = Stream(Collide(f^t; eps, a)) with the per-cell
// collision of collide.cuh.  Given lam^{t+1} = dJ/df^{t+1}, a cell x
//   1. pulls lam*_q(x) = lam^{t+1}_q(x + e_q), or lam^{t+1}_{opp q}(x) when x + e_q is solid
//      (the transpose of push streaming with half-way bounce-back, legacy/lbm_solver.py:
//      609-628);
//   2. recomputes its forward collision from f^t(x) and applies the transposed Jacobian
//      (reverse mode by hand): f* = f_eq + (1 - w)(f - f_eq) + S(u, F, w), through the LES
//      relaxation w = 1/tau(Pi_neq, rho) and the semi-implicit Darcy-Forchheimer velocity
//      u = s(|v|, K(eps), C_F(eps)) v;
//   3. adds dflux_t/df = -c_z on outlet cells (J = sum_t outflow flux);
//   4. accumulates dJ/deps (per cell) and dJ/da_k (inlet profile) in FP64.
// Supported forward configuration: LES off, LOCAL or STENCIL, drag SEMI_IMPLICIT, Guo forcing, no
// tau clamp, no external force field.  LES STENCIL: step t's nu_sgs reads the velocity u_{t-1} that
// step t-1 output, so the adjoint carries dJ/du across steps: reversing step t takes dJ/du_t (its
// own output velocity, read by step t+1) and returns dJ/du_{t-1} through the transposed central
// differences (les_grad_vjp_kernel, les_mu_kernel); a particle drag deposit (Kp, Kv) enters as a fixed input of
// the step (its force Kv - Kp u is differentiated through u, the deposit itself is held).  Gated LES cells (|S| below the floor, nu at its cap) and
// |u| = 0 points take the zero subgradient.
#include "collide.cuh"

namespace pog {

constexpr int ADJ_BLOCK = 256;
// The adjoint step kernel: 128-thread blocks, 4 resident per SM for FP32 (128 registers, no spill;
// at 96 registers and 5 blocks it spills 60 bytes and runs 3 % slower), FP64 at its register need.
constexpr int ADJ_STEP_BLOCK = 128;
template <int S>
constexpr int adj_min_blocks() {
  return S == POG_STORE_F64 ? 1 : 4;
}

// Weighted lattice moments of a direction vector a_q: m0 = sum w_q a_q, m1_a = sum w_q a_q e_qa,
// m2_ab = sum w_q a_q e_qa e_qb.  Every sum over q in the reverse step below is a polynomial of
// degree <= 2 in e_q times w_q a_q, so it is a contraction of these ten numbers (formed once per
// cell from the opposite-pair sums and differences) instead of a 19-term loop of its own.
template <typename C>
struct WMom {
  C m0, x, y, z, xx, yy, zz, xy, xz, yz;
};

template <typename C>
__device__ __forceinline__ WMom<C> wmoments(const C a[19]) {
  WMom<C> M;
  M.m0 = (C)wd(0) * a[0];
  M.x = M.y = M.z = M.xx = M.yy = M.zz = M.xy = M.xz = M.yz = (C)0;
#pragma unroll
  for (int q = 1; q < 19; ++q) {
    if (q > opp(q)) continue;  // each opposite pair once: e_opp = -e_q
    const C w = (C)wd(q);
    const C sp = a[q] + a[opp(q)], dm = a[q] - a[opp(q)];
    M.m0 += w * sp;
    if (cx(q)) M.x += (C)cx(q) * w * dm;
    if (cy(q)) M.y += (C)cy(q) * w * dm;
    if (cz(q)) M.z += (C)cz(q) * w * dm;
    if (cx(q)) M.xx += w * sp;
    if (cy(q)) M.yy += w * sp;
    if (cz(q)) M.zz += w * sp;
    if (cx(q) && cy(q)) M.xy += (C)(cx(q) * cy(q)) * w * sp;
    if (cx(q) && cz(q)) M.xz += (C)(cx(q) * cz(q)) * w * sp;
    if (cy(q) && cz(q)) M.yz += (C)(cy(q) * cz(q)) * w * sp;
  }
  return M;
}

// d(sum_q lam_q feq_q)/d(rho, u) for feq at (rho, u), from the weighted moments M of lam:
// sum_q w lam (1 + 3 e.u + 4.5 (e.u)^2 - 1.5 u.u) and rho sum_q w lam ((3 + 9 e.u) e - 3 u).
template <typename C>
__device__ __forceinline__ void eq_vjp(const WMom<C>& M, C rho, C ux, C uy, C uz, C& brho, C& bux, C& buy,
                                       C& buz) {
  const C usq = ux * ux + uy * uy + uz * uz;
  const C Mux = M.xx * ux + M.xy * uy + M.xz * uz;
  const C Muy = M.xy * ux + M.yy * uy + M.yz * uz;
  const C Muz = M.xz * ux + M.yz * uy + M.zz * uz;
  brho = M.m0 * ((C)1 - (C)1.5 * usq) + (C)3 * (ux * M.x + uy * M.y + uz * M.z) +
         (C)4.5 * (ux * Mux + uy * Muy + uz * Muz);
  bux = rho * ((C)3 * M.x + (C)9 * Mux - (C)3 * ux * M.m0);
  buy = rho * ((C)3 * M.y + (C)9 * Muy - (C)3 * uy * M.m0);
  buz = rho * ((C)3 * M.z + (C)9 * Muz - (C)3 * uz * M.m0);
}

// Inlet cell c (f* = feq(rho, (0, 0, u_z(a)))): bar f (all directions equal) from the pulled
// lam*, and the cell's contributions to dJ/da_k added into g[16].
template <typename C>
__device__ __forceinline__ C adj_inlet_cell(const KParams& kp, uint32_t c, const C ls[19], C rho, C mu_z, double g[16]) {
  const C uz = inlet_uz<C>(kp, c);
  C brho, bux, buy, buz;
  eq_vjp<C>(wmoments<C>(ls), rho, (C)0, (C)0, uz, brho, bux, buy, buz);
  buz += mu_z;  // the cell's output velocity (0, 0, u_z) read by the next step's LES stencil
  // uz = u_inlet (1 + sum a_k T_k(s)), s = 2 r / R - 1
  const uint32_t i = c % kp.nx, j = (c / kp.nx) % kp.ny;
  const C dx = (C)i - (C)kp.cxf, dy = (C)j - (C)kp.cyf;
  const C r = sqrt(dx * dx + dy * dy);
  const C R = (C)kp.inlet_R;
  const C s = R > (C)0 ? (C)2 * r / R - (C)1 : (C)0;
  C t0 = (C)1, t1 = s;
  const C ub = (C)(kp.inlet_ctl ? kp.inlet_ctl[0] : kp.u_inlet);
  g[0] += (double)(buz * ub);
  g[1] += (double)(buz * ub * t1);
#pragma unroll
  for (int k = 2; k < POG_INLET_NCOEF; ++k) {
    const C t2 = (C)2 * s * t1 - t0;
    g[k] += (double)(buz * ub * t2);
    t0 = t1;
    t1 = t2;
  }
  return brho;
}

// The pull of the transposed streaming at cell c: lam*_q = lam_{t+1} at slot (c + e_q, q), element
// c + wr[q], or lam_{t+1} at (c, opp q), element c + pl[opp q], when c + e_q is solid.  `open`
// (warp-uniform: no cell of the warp has a solid neighbour) skips the per-direction choice.
template <int S>
__device__ __forceinline__ void adj_pull(const KParams& kp, const typename Store<S>::E* __restrict__ lam_next,
                                         uint32_t c, uint32_t fl, bool open, typename Store<S>::C ls[19]) {
  using C = typename Store<S>::C;
  const typename Store<S>::E* __restrict__ lc = lam_next + c;
  if (open) {
#pragma unroll
    for (int q = 0; q < 19; ++q) ls[q] = (C)lc[kp.wr[q]];
  } else {
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const bool wall = q != 0 && ((fl >> (POG_LINK_SHIFT + q)) & 1u);
      ls[q] = (C)lc[wall ? kp.pl[opp(q)] : kp.wr[q]];
    }
  }
}

// The inlet disk's plane (k = nz - 2, where pog_build_flags puts the inlet).  Block b takes the
// cells [lo + b chunk, lo + (b + 1) chunk) and sums its cells' dJ/da_k in a fixed order (thread
// partials, warp shuffles, then the warps in order); with `part` it writes the block's 16 sums to
// part[b] for inlet_sum_kernel, without it (one block over the whole plane) it adds them to
// grad_inlet itself.  Either way the gradients repeat bit for bit.
template <int S>
__global__ void __launch_bounds__(ADJ_BLOCK) adjoint_inlet_kernel(
    const KParams kp, const typename Store<S>::E* __restrict__ ft,
    const typename Store<S>::E* __restrict__ lam_next, typename Store<S>::E* __restrict__ lam_t,
    const uint32_t* __restrict__ flags, uint32_t lo, uint32_t hi, uint32_t chunk,
    const typename Store<S>::E* __restrict__ mu_in, double* __restrict__ part, double* __restrict__ grad_inlet) {
  using St = Store<S>;
  using C = typename St::C;
  using E = typename St::E;
  const uint32_t n = kp.n;
  const uint32_t b0 = lo + blockIdx.x * chunk;
  const uint32_t b1 = hi - b0 < chunk ? hi : b0 + chunk;
  double g[POG_INLET_NCOEF];
#pragma unroll
  for (int k = 0; k < POG_INLET_NCOEF; ++k) g[k] = 0.0;
  for (uint32_t c = b0 + threadIdx.x; c < b1; c += ADJ_BLOCK) {
    const uint32_t fl = flags[c];
    if (!(fl & POG_CELL_INLET) || (fl & POG_CELL_SOLID) || c < kp.guard_lo || c > kp.guard_hi) continue;
    C ls[19];
    adj_pull<S>(kp, lam_next, c, fl, false, ls);
    C rho = 0;
#pragma unroll
    for (int q = 0; q < 19; ++q) rho += St::ld(ft, (uint32_t)q * n + c, q, (C)kp.rho0);
    const C brho = adj_inlet_cell<C>(kp, c, ls, rho, mu_in ? (C)mu_in[2u * n + c] : (C)0, g);
#pragma unroll
    for (int q = 0; q < 19; ++q) lam_t[(uint32_t)q * n + c] = (E)brho;
  }
  if (!part && !grad_inlet) return;
  __shared__ double sm[POG_INLET_NCOEF][ADJ_BLOCK / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < POG_INLET_NCOEF; ++k) {
    double x = g[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sm[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < POG_INLET_NCOEF) {
    double x = 0.0;
    for (int w = 0; w < ADJ_BLOCK / 32; ++w) x += sm[threadIdx.x][w];
    if (part)
      part[(size_t)blockIdx.x * POG_INLET_NCOEF + threadIdx.x] = x;
    else
      grad_inlet[threadIdx.x] += x;
  }
}

// grad_inlet[k] += sum over blocks b (in order) of part[b][k].
__global__ void inlet_sum_kernel(const double* __restrict__ part, uint32_t nblocks, double* __restrict__ grad_inlet) {
  const uint32_t k = threadIdx.x;
  if (k >= POG_INLET_NCOEF) return;
  double x = 0.0;
  for (uint32_t b = 0; b < nblocks; ++b) x += part[(size_t)b * POG_INLET_NCOEF + k];
  grad_inlet[k] += x;
}

// Cells of the inlet plane per block of the parallel inlet pass: four per thread.
constexpr uint32_t INLET_CHUNK = 4u * ADJ_BLOCK;

template <int S>
__global__ void __launch_bounds__(ADJ_STEP_BLOCK, (adj_min_blocks<S>())) adjoint_kernel(
    const KParams kp, const typename Store<S>::E* __restrict__ ft,
    const typename Store<S>::E* __restrict__ lam_next, typename Store<S>::E* __restrict__ lam_t,
    const uint32_t* __restrict__ flags, const float* __restrict__ eps, const float* __restrict__ pdrag,
    const float* __restrict__ u_prev, const typename Store<S>::E* __restrict__ mu_in,
    typename Store<S>::C* __restrict__ bar_nu, double* __restrict__ grad_eps, double* __restrict__ grad_inlet,
    uint32_t inlet_lo, uint32_t inlet_hi) {
  using St = Store<S>;
  using C = typename St::C;
  using E = typename St::E;
  const uint32_t n = kp.n;
  // inlet cells off the inlet plane (custom flags only): shared FP64 accumulators
  __shared__ double ginl[POG_INLET_NCOEF];
  if (threadIdx.x < POG_INLET_NCOEF) ginl[threadIdx.x] = 0.0;
  __syncthreads();
  for (uint32_t c = blockIdx.x * ADJ_STEP_BLOCK + threadIdx.x; c < n; c += gridDim.x * ADJ_STEP_BLOCK) {
    const uint32_t fl = flags[c];
    if (bar_nu) bar_nu[c] = (C)0;  // dJ/dnu of the cells whose stencil nu is live, below
    if ((fl & POG_CELL_SOLID) || c < kp.guard_lo || c > kp.guard_hi) {
#pragma unroll
      for (int q = 0; q < 19; ++q) lam_t[(uint32_t)q * n + c] = (E)0;
      continue;
    }
    // dJ/du of the velocity this step outputs (read by the next step's LES stencil)
    const C mux = mu_in ? (C)mu_in[c] : (C)0, muy = mu_in ? (C)mu_in[n + c] : (C)0,
            muz = mu_in ? (C)mu_in[2u * n + c] : (C)0;
    // the inlet plane's inlet cells are done by adjoint_inlet_kernel
    if ((fl & POG_CELL_INLET) && c >= inlet_lo && c < inlet_hi) continue;
    // 1. transpose of push streaming
    C ls[19];
    const bool open = __all_sync(__activemask(), (fl >> POG_LINK_SHIFT) == 0u);
    adj_pull<S>(kp, lam_next, c, fl, open, ls);
    // the stored deviations h_q = f_q - w_q rho0: density deviation, momentum, raw second moments
    // and sum_q lam*_q h_q in one pass (f itself is never formed; no O(1) terms cancel)
    C drho = 0, mx = 0, my = 0, mz = 0, Sxx = 0, Syy = 0, Szz = 0, Sxy = 0, Sxz = 0, Syz = 0, lh = 0;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const C h = St::dech(ft[(uint32_t)q * n + c]);
      drho += h;
      if (cx(q)) mx += (C)cx(q) * h;
      if (cy(q)) my += (C)cy(q) * h;
      if (cz(q)) mz += (C)cz(q) * h;
      if (cx(q)) Sxx += h;
      if (cy(q)) Syy += h;
      if (cz(q)) Szz += h;
      if (cx(q) && cy(q)) Sxy += (C)(cx(q) * cy(q)) * h;
      if (cx(q) && cz(q)) Sxz += (C)(cx(q) * cz(q)) * h;
      if (cy(q) && cz(q)) Syz += (C)(cy(q) * cz(q)) * h;
      lh += ls[q] * h;
    }
    const C rho = (C)kp.rho0 + drho;
    C brho = 0, bmx = 0, bmy = 0, bmz = 0;
    C bf[19];
    if (fl & POG_CELL_INLET) {
      double g[POG_INLET_NCOEF];
#pragma unroll
      for (int k = 0; k < POG_INLET_NCOEF; ++k) g[k] = 0.0;
      brho = adj_inlet_cell<C>(kp, c, ls, rho, muz, g);
#pragma unroll
      for (int k = 0; k < POG_INLET_NCOEF; ++k) atomicAdd(&ginl[k], g[k]);
#pragma unroll
      for (int q = 0; q < 19; ++q) bf[q] = brho;
    } else if (fl & POG_CELL_OUTLET) {
      const C ux = mx / rho, uy = my / rho, uz = mz / rho;
      C br_out, bux, buy, buz;
      eq_vjp<C>(wmoments<C>(ls), (C)kp.rho_out, ux, uy, uz, br_out, bux, buy, buz);
      (void)br_out;
      bux += mux;
      buy += muy;
      buz += muz;
      bmx = bux / rho;
      bmy = buy / rho;
      bmz = buz / rho;
      brho = -(bux * ux + buy * uy + buz * uz) / rho;
#pragma unroll
      for (int q = 0; q < 19; ++q)
        bf[q] = brho + (C)cx(q) * bmx + (C)cy(q) * bmy + (C)cz(q) * bmz - (C)cz(q);  // + dflux/df
    } else {
      // ---- forward recomputation ----
      // particle drag deposit (Kp, Kv) of this step, a fixed input: the fluid force Kv - Kp u
      // with u implicit (collide_cell), A = 1 + Kp / (2 rho)
      C Kp = 0, Kvx = 0, Kvy = 0, Kvz = 0;
      if (pdrag) {
        Kp = (C)pdrag[c];
        Kvx = (C)pdrag[n + c];
        Kvy = (C)pdrag[2u * n + c];
        Kvz = (C)pdrag[3u * n + c];
      }
      const C Ap = (C)1 + (C)0.5 * Kp / rho;
      const C Gx = rho * (C)kp.gx, Gy = rho * (C)kp.gy, Gz = rho * (C)kp.gz;
      const C vx = (mx + (C)0.5 * (Gx + Kvx)) / rho, vy = (my + (C)0.5 * (Gy + Kvy)) / rho,
              vz = (mz + (C)0.5 * (Gz + Kvz)) / rho;
      C ux = vx / Ap, uy = vy / Ap, uz = vz / Ap;
      C Fx = Gx + Kvx - Kp * ux, Fy = Gy + Kvy - Kp * uy, Fz = Gz + Kvz - Kp * uz;
      const bool porous = (fl & POG_CELL_POROUS) != 0;
      C K = (C)kp.K0, CF = (C)kp.CF0, e = (C)kp.eps0;
      C sK = 0, c0 = 0, c1 = 0, vm = 0, Ed = 0, D = 0, s = 0, um = 0, a = 0, b = 0, coef = 0;
      const C nu0 = (C)kp.nu0;
      if (porous) {
        if (eps) {
          e = (C)eps[c];
          C g = e * e * e / (((C)1 - e) * ((C)1 - e));
          K = (C)kp.K0 * (g / (C)kp.g0);
          C rr = (C)kp.eps0 / e;
          CF = (C)kp.CF0 * (rr * sqrt(rr));
        }
        sK = sqrt(K);
        c0 = (C)0.5 * (Ap + (C)0.5 * nu0 / K);
        c1 = (C)0.5 * CF / sK;
        vm = sqrt(vx * vx + vy * vy + vz * vz);
        Ed = sqrt(c0 * c0 + c1 * vm);
        D = c0 + Ed;
        s = (C)1 / D;
        ux = vx * s;
        uy = vy * s;
        uz = vz * s;
        um = sqrt(ux * ux + uy * uy + uz * uz);
        a = nu0 / K;
        b = CF / sK;
        coef = rho * (a + b * um);
        Fx = Gx + Kvx - (coef + Kp) * ux;
        Fy = Gy + Kvy - (coef + Kp) * uy;
        Fz = Gz + Kvz - (coef + Kp) * uz;
      }
      const C tau0 = (C)kp.tau;
      C tau = tau0;
      bool les_live = false;
      bool st_live = false;  // the stencil nu is in its linear range (not gated, not capped)
      if (kp.les_mode == POG_LES_STENCIL && !porous) {
        C gr[9];
        les_stencil_grad<C>(kp, c, u_prev, gr);
        const C smag = les_smag<C>(gr);
        if (!(smag < (C)kp.strain_floor)) {
          const C nu = (C)kp.cs2 * smag;
          st_live = nu < (C)kp.nu_max;
          tau = tau0 + (C)3 * (st_live ? nu : (C)kp.nu_max);
        }
      }
      C Pxx = 0, Pyy = 0, Pzz = 0, Pxy = 0, Pxz = 0, Pyz = 0, Q = 0, Rr = 0;
      if (kp.les_mode == POG_LES_LOCAL && !porous) {
        // Pi_neq = sum e e (f - f_eq) = S(h) - (drho / 3) I - rho u u (the D3Q19 equilibrium's
        // second moment is rho / 3 I + rho u u)
        const C d3 = drho * ((C)1 / (C)3);
        Pxx = Sxx - d3 - rho * ux * ux;
        Pyy = Syy - d3 - rho * uy * uy;
        Pzz = Szz - d3 - rho * uz * uz;
        Pxy = Sxy - rho * ux * uy;
        Pxz = Sxz - rho * ux * uz;
        Pyz = Syz - rho * uy * uz;
        const C PP = Pxx * Pxx + Pyy * Pyy + Pzz * Pzz + (C)2 * (Pxy * Pxy + Pxz * Pxz + Pyz * Pyz);
        Q = sqrt((C)2 * PP);
        Rr = sqrt(tau0 * tau0 + (C)18 * (C)kp.cs2 * Q / rho);
        const C tl = (C)0.5 * (tau0 + Rr);
        const C smag = (C)3 * Q / ((C)2 * rho * tl);
        C nu = (tl - tau0) / (C)3;
        les_live = true;
        if (smag < (C)kp.strain_floor) {
          nu = 0;
          les_live = false;
        }
        if (nu > (C)kp.nu_max) {
          nu = (C)kp.nu_max;
          les_live = false;
        }
        tau = tau0 + (C)3 * nu;
      }
      const C omega = (C)1 / tau;
      const C A = (C)1 - (C)0.5 * omega;
      const C uF = ux * Fx + uy * Fy + uz * Fz;
      // ---- reverse ----
      // f* = f_eq + (1 - omega) neq + A w_q B_q, neq = f - f_eq.  Every sum over q below is a
      // contraction of the weighted moments L of lam* (the sums of w lam* times 1, e_a, e_a e_b).
      const WMom<C> L = wmoments<C>(ls);
      const C L2ux = L.xx * ux + L.xy * uy + L.xz * uz, L2uy = L.xy * ux + L.yy * uy + L.yz * uz,
              L2uz = L.xz * ux + L.yz * uy + L.zz * uz;
      // bar omega = -sum lam* neq = -sum lam* h - rho0 L0 + sum lam* f_eq
      const C usq = ux * ux + uy * uy + uz * uz;
      C bomega = -lh + L.m0 * (drho - (C)1.5 * rho * usq) +
                 rho * ((C)3 * (ux * L.x + uy * L.y + uz * L.z) + (C)4.5 * (ux * L2ux + uy * L2uy + uz * L2uz));
      // the forcing term S_q = A w_q B_q, B_q = 3 (e.F - u.F) + 9 (e.u)(e.F)
      const C L2Fx = L.xx * Fx + L.xy * Fy + L.xz * Fz, L2Fy = L.xy * Fx + L.yy * Fy + L.yz * Fz,
              L2Fz = L.xz * Fx + L.yz * Fy + L.zz * Fz;
      const C bA = (C)3 * (Fx * L.x + Fy * L.y + Fz * L.z - uF * L.m0) +
                   (C)9 * (ux * L2Fx + uy * L2Fy + uz * L2Fz);
      const C bFx = A * ((C)3 * (L.x - ux * L.m0) + (C)9 * L2ux);
      const C bFy = A * ((C)3 * (L.y - uy * L.m0) + (C)9 * L2uy);
      const C bFz = A * ((C)3 * (L.z - uz * L.m0) + (C)9 * L2uz);
      C bux = A * ((C)-3 * Fx * L.m0 + (C)9 * L2Fx);
      C buy = A * ((C)-3 * Fy * L.m0 + (C)9 * L2Fy);
      C buz = A * ((C)-3 * Fz * L.m0 + (C)9 * L2Fz);
      bomega += (C)-0.5 * bA;
      const C btau = -bomega / (tau * tau);
      if (st_live && bar_nu) bar_nu[c] = (C)3 * btau;
      // this cell's output velocity is u: dJ/du from the next step's stencil joins here
      bux += mux;
      buy += muy;
      buz += muz;
      // bar neq_q = (1 - omega) lam*_q + e_q^T bP e_q (LES local: tau through Pi_neq)
      C bPxx = 0, bPyy = 0, bPzz = 0, bPxy = 0, bPxz = 0, bPyz = 0;
      if (les_live) {
        const C bnu = (C)3 * btau;
        const C btl = bnu / (C)3;
        const C bR = (C)0.5 * btl;
        const C cs2 = (C)kp.cs2;
        const C bQ = bR * (C)9 * cs2 / (rho * Rr);
        brho += bR * (-(C)9 * cs2 * Q / (rho * rho * Rr));
        const C bPP = Q > (C)0 ? bQ / Q : (C)0;
        bPxx = (C)2 * Pxx * bPP;
        bPyy = (C)2 * Pyy * bPP;
        bPzz = (C)2 * Pzz * bPP;
        bPxy = (C)4 * Pxy * bPP;
        bPxz = (C)4 * Pxz * bPP;
        bPyz = (C)4 * Pyz * bPP;
      }
      // bar f_eq = lam* - bar neq: its weighted moments D = omega L - moments of e^T bP e
      // (D3Q19: sum w e_a^4 = 1/3, sum w e_a^2 e_b^2 = 1/9 for a != b, odd moments 0)
      {
        WMom<C> D;
        const C third = (C)1 / (C)3, ninth = (C)1 / (C)9;
        D.m0 = omega * L.m0 - third * (bPxx + bPyy + bPzz);
        D.x = omega * L.x;
        D.y = omega * L.y;
        D.z = omega * L.z;
        D.xx = omega * L.xx - (third * bPxx + ninth * (bPyy + bPzz));
        D.yy = omega * L.yy - (third * bPyy + ninth * (bPxx + bPzz));
        D.zz = omega * L.zz - (third * bPzz + ninth * (bPxx + bPyy));
        D.xy = omega * L.xy - ninth * bPxy;
        D.xz = omega * L.xz - ninth * bPxz;
        D.yz = omega * L.yz - ninth * bPyz;
        C br, bx, by, bz;
        eq_vjp<C>(D, rho, ux, uy, uz, br, bx, by, bz);
        brho += br;
        bux += bx;
        buy += by;
        buz += bz;
      }
      C bvx, bvy, bvz, bGx, bGy, bGz, bAp = 0;
      if (porous) {
        bGx = bFx;
        bGy = bFy;
        bGz = bFz;
        const C bcoef = -(bFx * ux + bFy * uy + bFz * uz);
        bux += -(coef + Kp) * bFx;
        buy += -(coef + Kp) * bFy;
        buz += -(coef + Kp) * bFz;
        brho += bcoef * (a + b * um);
        const C bum = bcoef * rho * b;
        const C ba = bcoef * rho;
        const C bb = bcoef * rho * um;
        if (um > (C)0) {
          bux += bum * ux / um;
          buy += bum * uy / um;
          buz += bum * uz / um;
        }
        const C bs = bux * vx + buy * vy + buz * vz;
        bvx = s * bux;
        bvy = s * buy;
        bvz = s * buz;
        const C bD = -bs / (D * D);
        const C bc0 = bD * ((C)1 + c0 / Ed);
        bAp += (C)0.5 * bc0;
        const C bc1 = bD * vm / ((C)2 * Ed);
        const C bvm = bD * c1 / ((C)2 * Ed);
        if (vm > (C)0) {
          bvx += bvm * vx / vm;
          bvy += bvm * vy / vm;
          bvz += bvm * vz / vm;
        }
        if (eps && grad_eps) {
          C bK = bc0 * (-(C)0.25 * nu0 / (K * K)) + bc1 * (-(C)0.25 * CF / (K * sK)) +
                 ba * (-nu0 / (K * K)) + bb * (-(C)0.5 * CF / (K * sK));
          C bCF = bc1 * (C)0.5 / sK + bb / sK;
          C dK = K * ((C)3 / e + (C)2 / ((C)1 - e));
          C dCF = (C)-1.5 * CF / e;
          grad_eps[c] += (double)(bK * dK + bCF * dCF);
        }
      } else {
        // F = G + Kv - Kp u, u = v / Ap
        bux += -Kp * bFx;
        buy += -Kp * bFy;
        buz += -Kp * bFz;
        bvx = bux / Ap;
        bvy = buy / Ap;
        bvz = buz / Ap;
        bAp = -(bux * ux + buy * uy + buz * uz) / Ap;
        bGx = bFx;
        bGy = bFy;
        bGz = bFz;
      }
      // Ap = 1 + Kp / (2 rho)
      brho += bAp * ((C)-0.5 * Kp / (rho * rho));
      // v = (m + (G + Kv)/2)/rho, G = rho g
      bmx = bvx / rho;
      bmy = bvy / rho;
      bmz = bvz / rho;
      bGx += (C)0.5 * bvx / rho;
      bGy += (C)0.5 * bvy / rho;
      bGz += (C)0.5 * bvz / rho;
      brho += -(bvx * vx + bvy * vy + bvz * vz) / rho;
      brho += bGx * (C)kp.gx + bGy * (C)kp.gy + bGz * (C)kp.gz;
      const C keep = (C)1 - omega;
#pragma unroll
      for (int q = 0; q < 19; ++q)
        bf[q] = keep * ls[q] + (C)(cx(q) * cx(q)) * bPxx + (C)(cy(q) * cy(q)) * bPyy +
                (C)(cz(q) * cz(q)) * bPzz + (C)(cx(q) * cy(q)) * bPxy + (C)(cx(q) * cz(q)) * bPxz +
                (C)(cy(q) * cz(q)) * bPyz + brho + (C)cx(q) * bmx + (C)cy(q) * bmy + (C)cz(q) * bmz;
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) lam_t[(uint32_t)q * n + c] = (E)bf[q];
  }
  if (grad_inlet) {
    __syncthreads();
    if (threadIdx.x < POG_INLET_NCOEF && ginl[threadIdx.x] != 0.0)
      atomicAdd(grad_inlet + threadIdx.x, ginl[threadIdx.x]);
  }
}

// dJ/dnu -> dJ/d(grad u) of each cell's stencil (nu = cs^2 |S|, |S| = sqrt(2 P), P the strain
// invariant of the central-difference gradient): bar_g[3 a + b] = dJ/d(du_a/dx_b), 0 where the
// stencil is not live (bar_nu 0).
template <typename C>
__global__ void les_grad_vjp_kernel(const KParams kp, const float* __restrict__ u_prev, const C* __restrict__ bar_nu,
                                    C* __restrict__ bar_g) {
  const uint32_t n = kp.n;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    C out[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const C bn = bar_nu[c];
    if (bn != (C)0 && c >= kp.guard_lo && c <= kp.guard_hi) {
      C g[9];
      les_stencil_grad<C>(kp, c, u_prev, g);
      const C smag = les_smag<C>(g);
      const C bP = bn * (C)kp.cs2 / smag;  // d|S|/dP = 1/|S|
      const C s12 = (C)0.5 * (g[1] + g[3]), s13 = (C)0.5 * (g[2] + g[6]), s23 = (C)0.5 * (g[5] + g[7]);
      out[0] = bP * (C)2 * g[0];
      out[4] = bP * (C)2 * g[4];
      out[8] = bP * (C)2 * g[8];
      out[1] = out[3] = bP * (C)2 * s12;
      out[2] = out[6] = bP * (C)2 * s13;
      out[5] = out[7] = bP * (C)2 * s23;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) bar_g[(uint32_t)k * n + c] = out[k];
  }
}

// dJ/du_prev(x)_a = sum_b (bar_g_ab(x - e_b) - bar_g_ab(x + e_b)) / 2: the transpose of the
// central differences du_a/dx_b(y) = (u_a(y + e_b) - u_a(y - e_b)) / 2.
template <typename C, typename E>
__global__ void les_mu_kernel(const KParams kp, const C* __restrict__ bar_g, E* __restrict__ mu_out) {
  const uint32_t n = kp.n;
  const uint32_t st[3] = {1u, kp.nx, kp.nxny};
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const bool in = c >= kp.nxny && c + kp.nxny < n;  // both neighbours along every axis exist
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      C m = 0;
      if (in) {
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          const C* g = bar_g + (uint32_t)(3 * a + b) * n;
          m += (C)0.5 * (g[c - st[b]] - g[c + st[b]]);
        }
      }
      mu_out[(uint32_t)a * n + c] = (E)m;
    }
  }
}

// Bytes of the stencil mode's part of the adjoint scratch (bar_nu and bar_g, 10 values per cell),
// rounded up to 16 bytes; the inlet pass's per-block sums follow.
static inline size_t adj_stencil_bytes(size_t n, bool stencil, size_t elem) {
  return stencil ? (10 * n * elem + 15) / 16 * 16 : 0;
}

template <int S>
static int launch_adj(const KParams& kp, const void* ft, const void* ln, void* lt, const uint32_t* flags,
                      const float* eps, const float* pdrag, const float* u_prev, const void* mu_in, void* mu_out,
                      void* scratch, double* ge, double* gi, cudaStream_t s) {
  auto kern = adjoint_kernel<S>;
  static thread_local int grid = 0;
  if (grid == 0) grid = persistent_blocks((const void*)kern, ADJ_STEP_BLOCK);
  if (grid <= 0) return set_error(POG_E_CUDA, "occupancy query failed");
  int want = (int)((kp.n + ADJ_STEP_BLOCK - 1) / ADJ_STEP_BLOCK);
  int g = want < grid ? want : grid;
  using E = typename Store<S>::E;
  using C = typename Store<S>::C;
  const uint32_t lo = (kp.nz - 2u) * kp.nxny, hi = lo + kp.nxny;  // the inlet plane
  const bool stencil = kp.les_mode == POG_LES_STENCIL;
  // scratch: the stencil mode's bar_nu [n] and bar_g [9 n] (storage type), then the inlet pass's
  // per-block sums (pog_adjoint_scratch_bytes)
  C* bar_nu = (scratch && stencil) ? (C*)scratch : nullptr;
  double* part = scratch ? (double*)((char*)scratch + adj_stencil_bytes(kp.n, stencil, sizeof(C))) : nullptr;
  kern<<<g, ADJ_STEP_BLOCK, 0, s>>>(kp, (const E*)ft, (const E*)ln, (E*)lt, flags, eps, pdrag, u_prev, (const E*)mu_in,
                               bar_nu, ge, gi, lo, hi);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  if (part) {
    const uint32_t nb = (kp.nxny + INLET_CHUNK - 1) / INLET_CHUNK;
    adjoint_inlet_kernel<S><<<nb, ADJ_BLOCK, 0, s>>>(kp, (const E*)ft, (const E*)ln, (E*)lt, flags, lo, hi,
                                                     INLET_CHUNK, (const E*)mu_in, gi ? part : nullptr, nullptr);
    count_launch();
    POG_TRY_CUDA(cudaGetLastError());
    if (gi) {
      inlet_sum_kernel<<<1, 32, 0, s>>>(part, nb, gi);
      count_launch();
      POG_TRY_CUDA(cudaGetLastError());
    }
  } else {
    adjoint_inlet_kernel<S><<<1, ADJ_BLOCK, 0, s>>>(kp, (const E*)ft, (const E*)ln, (E*)lt, flags, lo, hi,
                                                    kp.nxny, (const E*)mu_in, nullptr, gi);
    count_launch();
    POG_TRY_CUDA(cudaGetLastError());
  }
  if (bar_nu && mu_out) {
    C* bar_g = bar_nu + kp.n;
    les_grad_vjp_kernel<C><<<g, ADJ_BLOCK, 0, s>>>(kp, u_prev, bar_nu, bar_g);
    les_mu_kernel<C, E><<<g, ADJ_BLOCK, 0, s>>>(kp, bar_g, (E*)mu_out);
    count_launch(2);
    POG_TRY_CUDA(cudaGetLastError());
  }
  return POG_OK;
}

// Outflow flux of a natural-layout state, -sum over outlet cells of sum_q c_qz f_q, added to an
// int64 accumulator in units of 2^-48 per cell: integer addition is associative, so the total does
// not depend on the order in which blocks arrive and repeated runs agree bit for bit.
constexpr double OUTFLOW_FIX_SCALE = 281474976710656.0;  // 2^48

// acc[0] += the flux in units of 2^-48 (rounded per cell), acc[1] += each cell's rounding remainder
// in units of 2^-96.  x 2^48 is exact (a power of two), the remainder xs - rint(xs) is exact
// (|xs - rint(xs)| <= 1/2 and Sterbenz), and so is its scaling by 2^48: the two words hold the
// exact sum of the per-cell FP64 fluxes down to 2^-96, in integers, whatever the order.
template <int S>
__global__ void outflow_fixed_kernel(const KParams kp, const typename Store<S>::E* __restrict__ f,
                                     const uint32_t* __restrict__ flags, unsigned long long* __restrict__ acc) {
  using St = Store<S>;
  using C = typename St::C;
  const uint32_t n = kp.n;
  long long hi = 0, lo = 0;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const uint32_t fl = flags[c];
    if (!(fl & POG_CELL_OUTLET) || (fl & POG_CELL_SOLID)) continue;
    C mz = 0;
#pragma unroll
    for (int q = 0; q < 19; ++q)
      if (cz(q) != 0) mz += (C)cz(q) * St::ld(f, (uint32_t)q * n + c, q, (C)kp.rho0);
    const double xs = -(double)mz * OUTFLOW_FIX_SCALE;
    const double r = rint(xs);
    hi += (long long)r;
    lo += __double2ll_rn((xs - r) * OUTFLOW_FIX_SCALE);
  }
  if (hi != 0) atomicAdd(acc, (unsigned long long)hi);
  if (lo != 0) atomicAdd(acc + 1, (unsigned long long)lo);
}

}  // namespace pog

using namespace pog;

extern "C" int pog_outflow_fixed(const pog_params* p, const void* f_nat, const uint32_t* flags,
                                 long long* acc, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!f_nat || !flags || !acc) return set_error(POG_E_ARG, "NULL pointer");
  KParams kp = make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  long long want = ((long long)kp.n + 255) / 256;
  const int grid = (int)(want < 152 * 8 ? want : 152 * 8);
  if (p->storage == POG_STORE_F32)
    outflow_fixed_kernel<POG_STORE_F32><<<grid, 256, 0, s>>>(kp, (const float*)f_nat, flags, (unsigned long long*)acc);
  else if (p->storage == POG_STORE_F64)
    outflow_fixed_kernel<POG_STORE_F64><<<grid, 256, 0, s>>>(kp, (const double*)f_nat, flags, (unsigned long long*)acc);
  else
    return set_error(POG_E_ARG, "pog_outflow_fixed reads F32 or F64 natural-layout states");
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

extern "C" size_t pog_adjoint_scratch_bytes(const pog_params* p) {
  if (!p || p->nx <= 0 || p->ny <= 0 || p->nz <= 0) return 0;
  const size_t n = (size_t)p->nx * p->ny * p->nz, nxny = (size_t)p->nx * p->ny;
  const size_t elem = p->storage == POG_STORE_F64 ? sizeof(double) : sizeof(float);
  const size_t nb = (nxny + INLET_CHUNK - 1) / INLET_CHUNK;
  return adj_stencil_bytes(n, p->les_mode == POG_LES_STENCIL, elem) + nb * POG_INLET_NCOEF * sizeof(double);
}

extern "C" int pog_adjoint_step(const pog_params* p, const void* f_t, const void* lam_next,
                                void* lam_t, const uint32_t* flags, const float* porosity, const float* pdrag,
                                const float* u_prev, const void* dJ_du, void* dJ_du_prev, void* scratch,
                                double* grad_porosity, double* grad_inlet, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!f_t || !lam_next || !lam_t || !flags) return set_error(POG_E_ARG, "NULL pointer");
  if (lam_next == lam_t) return set_error(POG_E_ARG, "lam_next and lam_t must differ");
  const bool stencil = p->les_mode == POG_LES_STENCIL;
  if (stencil && (!u_prev || !dJ_du_prev || !scratch))
    return set_error(POG_E_ARG, "LES stencil mode needs u_prev, dJ_du_prev and scratch");
  if (stencil && dJ_du == dJ_du_prev) return set_error(POG_E_ARG, "dJ_du and dJ_du_prev must differ");
  if (!stencil) {  // scratch stays: the inlet pass's per-block sums
    u_prev = nullptr;
    dJ_du = nullptr;
    dJ_du_prev = nullptr;
  }
  if (scratch && ((uintptr_t)scratch & 15u)) return set_error(POG_E_ARG, "scratch must be 16-byte aligned");
  if (p->drag_mode != POG_DRAG_SEMI_IMPLICIT || p->forcing_mode != POG_FORCING_GUO || p->clamp_tau)
    return set_error(POG_E_ARG, "adjoint supports semi-implicit drag, Guo forcing, no tau clamp");
  if (grad_porosity && !porosity) return set_error(POG_E_ARG, "grad_porosity needs porosity");
  if (p->pour_control || p->filter_blockage || p->phase)
    return set_error(POG_E_ARG, "adjoint does not differentiate the pour stream, filter blockage or phase field");
  KParams kp = make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  if (p->storage == POG_STORE_F32)
    return launch_adj<POG_STORE_F32>(kp, f_t, lam_next, lam_t, flags, porosity, pdrag, u_prev, dJ_du, dJ_du_prev,
                                     scratch, grad_porosity, grad_inlet, s);
  if (p->storage == POG_STORE_F64)
    return launch_adj<POG_STORE_F64>(kp, f_t, lam_next, lam_t, flags, porosity, pdrag, u_prev, dJ_du, dJ_du_prev,
                                     scratch, grad_porosity, grad_inlet, s);
  return set_error(POG_E_ARG, "adjoint storage must be F32 or F64");
}
