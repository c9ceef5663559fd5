// lbm_ref.cu -- FP16S storage with a per-cell reference density (pog_params.density_ref).
//
// FP16S stores h = (f_q - w_q rs) 2^12 in IEEE half.  With rs = rho0 for every cell, a stored
// deviation carries the cell's density deviation w_q (rho - rho0) next to its velocity part
// w_q rho (3 e.u + ...), and in a box crossed by pressure waves the density part is the larger
// (rho - 1 rms 1-2.5e-3 against rms |u| 1-8e-4 at 256^3), so FP16's 11-bit significand rounds
// away velocity information.  Here each cell c carries its own reference rs_c = rho0 + d_c, d_c an
// FP16 value in density_ref[c], and every slot of the AA buffer is stored relative to the
// reference of the cell that owns the slot (the AA pattern's slot (c, q) belongs to cell c):
//   even step  cell c reads and writes only its own slots: it decodes with d_c, collides, sets
//              d_c = fp16(rho_c - rho0) from the density it just computed and encodes its 19
//              outputs relative to the new reference (one shift per weight class);
//   odd step   cell c reads (c - e_q, opp q), owned by its neighbour c - e_q, and writes
//              (c + e_q, q), owned by c + e_q: each incoming deviation is moved to c's reference
//              and each outgoing one to the target's, w_q (d_neighbour - d_c) 2^12, with the 18
//              neighbours' d read from density_ref (bounced slots are c's own and need nothing).
// The reference changes only on even steps, between which every slot is written and read once
// under the same reference, so the stored state decodes exactly as before; only the rounding
// point moves.  Cost: 2 B read and write per cell on even steps, 18 neighbour reads (mostly L1
// hits) and two shifts per direction on odd steps.
//
// Same update as aa_step_kernel otherwise (the collision is collide_cell in the shifted form
// with rs = rs_c).
#include "aa_cell.cuh"

namespace pog {

constexpr int REF_BLOCK = 128;

// resident 128-thread blocks per SM: 9 (56 registers) for the even step, 8 (64, a few spilled
// bytes; 451 us per 256^3 odd step against 461 at 72 registers, which spills nothing) for the odd
// step with its neighbour shifts and for the variants with the FP64 sums
template <int PARITY, bool REDUCE>
constexpr int ref_min_blocks() {
  return REDUCE ? 8 : (PARITY == 1 ? 8 : 9);
}

// the representative Q of the k-th direction pair (Q, opp Q)
__host__ __device__ constexpr int pair_rep(int k) {
  return k == 0 ? 1 : k == 1 ? 3 : k == 2 ? 5 : k == 3 ? 7 : k == 4 ? 8 : k == 5 ? 11 : k == 6 ? 12 : k == 7 ? 15 : 16;
}

template <int PARITY, bool REDUCE, bool MACRO_ONLY>
__global__ void __launch_bounds__(REF_BLOCK, (ref_min_blocks<PARITY, REDUCE>())) aa_ref_kernel(
    const KParams kp, __half* __restrict__ f, const uint32_t* __restrict__ flags,
    const float* __restrict__ force, const float* __restrict__ pdrag, const float* __restrict__ eps,
    const float* __restrict__ u_prev, float* __restrict__ u_next, float* __restrict__ rho_out,
    float* __restrict__ u_out, double* __restrict__ red, __half* __restrict__ dref) {
  using St = Store<POG_STORE_F16S>;
  RedAcc<float> acc;
  const uint32_t n = kp.n;
  for (uint32_t c = blockIdx.x * REF_BLOCK + threadIdx.x; c < n; c += gridDim.x * REF_BLOCK) {
    const uint32_t fl = flags[c];
    if (!aa_live(kp, c, fl)) continue;
    if (PARITY == 0 && !MACRO_ONLY) {
      ref_even_cell<REDUCE>(kp, f, c, fl, force, pdrag, eps, u_prev, u_next, rho_out, u_out, acc);
      continue;
    }
    const bool open = PARITY == 1 && __all_sync(__activemask(), (fl >> POG_LINK_SHIFT) == 0u);
    __half raw[19];
    aa_load<POG_STORE_F16S, PARITY>(kp, f, c, fl, open, raw);
    const float dc = __half2float(dref[c]);
    float fv[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) fv[q] = St::dech(raw[q]);
    // odd step: the shift w_q (d_n - d_c) 2^12 of each neighbour n, kept packed as FP16 pairs for
    // the outgoing slots (the outgoing value is rounded to FP16 right after, so a shift rounded
    // to FP16 changes nothing the storage keeps).  dsh[k] holds, for the k-th direction pair (Q,
    // opp Q), the shifts of neighbours c - e_Q (low half) and c + e_Q (high half).
    uint32_t dsh[9];
    if (PARITY == 1) {
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const int Q = pair_rep(k), P = opp(Q);
        const float wq = F16_SCALE * (float)wd(Q);
        const float da = __half2float(dref[c - (uint32_t)kp.off[Q]]) - dc;  // neighbour c - e_Q
        const float db = __half2float(dref[c + (uint32_t)kp.off[Q]]) - dc;  // neighbour c + e_Q
        const bool wa = (fl >> (POG_LINK_SHIFT + P)) & 1u;  // c - e_Q solid: slot Q bounced
        const bool wb = (fl >> (POG_LINK_SHIFT + Q)) & 1u;  // c + e_Q solid: slot opp Q bounced
        const float sa = wa ? 0.0f : da * wq, sb = wb ? 0.0f : db * wq;
        fv[Q] += sa;  // incoming Q comes from c - e_Q
        fv[P] += sb;  // incoming opp Q comes from c + e_Q
        const __half2 h = __floats2half2_rn(sa, sb);
        memcpy(&dsh[k], &h, 4);
      }
    }
    float nu_st = 0.0f;
    if (!MACRO_ONLY && kp.les_mode == POG_LES_STENCIL && !(fl & POG_CELL_POROUS))
      nu_st = les_nu_stencil<float>(kp, c, u_prev);
    const float rs = kp.rho0 + dc;
    const CellResult<float> r =
        collide_cell<float, true>(kp, fl, c, fv, force, pdrag, eps, nu_st, St::SCALE, rs);
    if (rho_out) rho_out[c] = r.rho;
    if (u_out) {
      u_out[c] = r.ux;
      u_out[n + c] = r.uy;
      u_out[2u * n + c] = r.uz;
    }
    if (!MACRO_ONLY && u_next) {
      u_next[c] = r.ux;
      u_next[n + c] = r.uy;
      u_next[2u * n + c] = r.uz;
    }
    if (REDUCE) acc.add(r);
    if (MACRO_ONLY || PARITY == 0) continue;  // (the even step's update is ref_even_cell)
    // outgoing: slot q goes to c + e_q (shift of neighbour c + e_q), slot opp Q to c - e_Q; a
    // bounced slot is c's own (its shift is zero)
    const uint32_t c2 = opaque(c);
    f[c2 + kp.wr[0]] = St::ench(fv[0]);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int Q = pair_rep(k), P = opp(Q);
      __half2 h;
      memcpy(&h, &dsh[k], 4);
      const float2 sh = __half22float2(h);
      const bool wq = (fl >> (POG_LINK_SHIFT + Q)) & 1u, wp = (fl >> (POG_LINK_SHIFT + P)) & 1u;
      f[c2 + (wq ? kp.pl[P] : kp.wr[Q])] = St::ench(fv[Q] - sh.y);
      f[c2 + (wp ? kp.pl[Q] : kp.wr[P])] = St::ench(fv[P] - sh.x);
    }
  }
  if (REDUCE) reduce_add<float>(acc, red);
}

// Natural-layout copy of the state at parity PARITY (as aa_export_kernel, each slot decoded with
// the reference of the cell that owns it).
template <int PARITY, typename O>
__global__ void aa_ref_export_kernel(const KParams kp, const __half* __restrict__ f, const uint32_t* __restrict__ flags,
                                     const __half* __restrict__ dref, O* __restrict__ out) {
  using St = Store<POG_STORE_F16S>;
  const uint32_t n = kp.n;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const uint32_t fl = flags[c];
    if ((fl & POG_CELL_SOLID) || c < kp.guard_lo || c > kp.guard_hi) {
#pragma unroll
      for (int q = 0; q < 19; ++q) out[(size_t)q * n + c] = (O)0;
      continue;
    }
    const float rc = kp.rho0 + __half2float(dref[c]);
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      float v;
      if (PARITY == 0) {
        v = St::ld(f, (uint32_t)q * n + c, q, rc);
      } else {
        const bool wall = q != 0 && ((fl >> (POG_LINK_SHIFT + opp(q))) & 1u);
        const uint32_t s = c - (uint32_t)kp.off[q];
        v = wall ? St::ld(f, (uint32_t)q * n + c, q, rc)
                 : St::ld(f, (uint32_t)opp(q) * n + s, opp(q), kp.rho0 + __half2float(dref[s]));
      }
      out[(size_t)q * n + c] = (O)v;
    }
  }
}

// Even-parity state from natural f (as aa_import_kernel), each cell relative to its current
// reference.
template <typename I>
__global__ void aa_ref_import_kernel(const KParams kp, const I* __restrict__ in, const uint32_t* __restrict__ flags,
                                     const __half* __restrict__ dref, __half* __restrict__ f) {
  using St = Store<POG_STORE_F16S>;
  const uint32_t n = kp.n;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const bool solid = flags[c] & POG_CELL_SOLID;
    const float rc = kp.rho0 + __half2float(dref[c]);
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const float v = solid ? (float)wd(q) * rc : (float)in[(size_t)q * n + c];
      St::st(f, (uint32_t)q * n + c, q, v, rc);
    }
  }
}

// Equilibrium at (rho, u) everywhere, each cell's reference set to fp16(rho - rho0).
__global__ void aa_ref_init_kernel(const KParams kp, __half* __restrict__ f, const uint32_t* __restrict__ flags,
                                   __half* __restrict__ dref, float rho, float ux, float uy, float uz) {
  using St = Store<POG_STORE_F16S>;
  const uint32_t n = kp.n;
  const float usq15 = 1.5f * (ux * ux + uy * uy + uz * uz);
  const __half d = __float2half_rn(rho - kp.rho0);
  const float rc = kp.rho0 + __half2float(d);
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const bool solid = flags[c] & POG_CELL_SOLID;
    dref[c] = d;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const float v = solid ? (float)wd(q) * rc : feq_q<float>(q, rho, ux, uy, uz, usq15);
      St::st(f, (uint32_t)q * n + c, q, v, rc);
    }
  }
}

static int ref_grid(uint32_t n, int block) {
  long long want = ((long long)n + block - 1) / block;
  return (int)(want < 152 * 64 ? want : 152 * 64);
}

template <int PARITY, bool REDUCE, bool MACRO>
static int launch_ref(const KParams& kp, void* f, const uint32_t* flags, const float* force, const float* pdrag,
                      const float* eps, const float* u_prev, float* u_next, float* rho_out, float* u_out,
                      double* red, cudaStream_t s) {
  auto kern = aa_ref_kernel<PARITY, REDUCE, MACRO>;
  static thread_local int grid = 0;
  if (grid == 0) grid = persistent_blocks((const void*)kern, REF_BLOCK);
  if (grid <= 0) return set_error(POG_E_CUDA, "occupancy query failed");
  const int want = (int)((kp.n + REF_BLOCK - 1) / REF_BLOCK);
  const int g = REDUCE ? (want < grid ? want : grid) : want;
  kern<<<g, REF_BLOCK, 0, s>>>(kp, (__half*)f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red,
                               kp.dref);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int launch_ref_step(const KParams& kp, int parity, bool reduce, bool macro, void* f, const uint32_t* flags,
                    const float* force, const float* pdrag, const float* eps, const float* u_prev, float* u_next,
                    float* rho_out, float* u_out, double* red, cudaStream_t s) {
#define POG_REF_CASE(P, R, M) \
  if (parity == P && reduce == R && macro == M) return launch_ref<P, R, M>(kp, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
  POG_REF_CASE(0, false, false)
  POG_REF_CASE(1, false, false)
  POG_REF_CASE(0, true, false)
  POG_REF_CASE(1, true, false)
  POG_REF_CASE(0, false, true)
  POG_REF_CASE(1, false, true)
#undef POG_REF_CASE
  return set_error(POG_E_ARG, "unsupported step variant");
}

int ref_export(const KParams& kp, const void* f, const uint32_t* flags, int parity, void* f_nat, int out_storage,
               cudaStream_t s) {
  const int g = ref_grid(kp.n, 256);
  if (out_storage == POG_STORE_F32) {
    if (parity) aa_ref_export_kernel<1, float><<<g, 256, 0, s>>>(kp, (const __half*)f, flags, kp.dref, (float*)f_nat);
    else aa_ref_export_kernel<0, float><<<g, 256, 0, s>>>(kp, (const __half*)f, flags, kp.dref, (float*)f_nat);
  } else {
    if (parity) aa_ref_export_kernel<1, double><<<g, 256, 0, s>>>(kp, (const __half*)f, flags, kp.dref, (double*)f_nat);
    else aa_ref_export_kernel<0, double><<<g, 256, 0, s>>>(kp, (const __half*)f, flags, kp.dref, (double*)f_nat);
  }
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int ref_import(const KParams& kp, const void* f_nat, int in_storage, const uint32_t* flags, void* f, cudaStream_t s) {
  const int g = ref_grid(kp.n, 256);
  if (in_storage == POG_STORE_F32)
    aa_ref_import_kernel<float><<<g, 256, 0, s>>>(kp, (const float*)f_nat, flags, kp.dref, (__half*)f);
  else
    aa_ref_import_kernel<double><<<g, 256, 0, s>>>(kp, (const double*)f_nat, flags, kp.dref, (__half*)f);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int ref_init(const KParams& kp, void* f, const uint32_t* flags, float rho, float ux, float uy, float uz,
             cudaStream_t s) {
  aa_ref_init_kernel<<<ref_grid(kp.n, 256), 256, 0, s>>>(kp, (__half*)f, flags, kp.dref, rho, ux, uy, uz);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

}  // namespace pog
