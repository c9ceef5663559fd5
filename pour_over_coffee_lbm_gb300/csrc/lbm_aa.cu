// lbm_aa.cu -- the fused D3Q19 step on ONE distribution buffer (AA pattern, Bailey et al.
// 2009), plus init / export / import / macroscopic kernels over the same layout.
//
// Replaces, fused into one pass per time step: LBMSolver._compute_macroscopic_quantities
// (legacy/lbm_solver.py:488-535), _apply_collision_and_streaming (:537-628), swap_fields
// (:630-654, eliminated), the LES update (les_turbulence.py:289-380), the filter-band drag
// (filter_paper.py:471-536), add_particle_reaction_forces (:1478-1483) and the boundary
// manager's inlet/outlet overwrite (boundary_conditions.py:384-409).
//
// Layout: f[q*n + c], c = (k*ny + j)*nx + i, one thread per cell, consecutive threads on
// consecutive x, so every population plane is read and written with coalesced 32-bit (F32),
// 16-bit (F16S/BF16S) or 64-bit (F64) accesses.
//
// AA pattern.  At an even time t the slot (c, q) holds f_q(c).  Even step: read (c, q), write
// the post-collision f*_q to (c, opp q): no neighbour access at all.  Odd step: read f_q from
// (c - e_q, opp q) -- or from (c, q) when c - e_q is solid (half-way bounce-back) -- and write
// f*_q to (c + e_q, q) -- or to (c, opp q) when c + e_q is solid.  A cell reads and writes the
// same 19 slots, so the update is in place and race-free.  Which neighbours are solid comes from
// the 18 link bits of the cell's own flag word: a cell without any takes the odd step's plain
// streaming addresses (per-direction offset tables, no per-direction tests), the others choose
// per direction between the streamed and the bounced slot.
#include "aa_cell.cuh"

namespace pog {

constexpr int AA_BLOCK = 128;
// Resident 128-thread blocks per SM the step kernel is compiled for (it caps the registers per
// thread): 9 (56 registers, 36 warps per SM) for the plain FP32/16-bit step, 8 (64) for the
// variants with the FP64 sums, 3 (168) for FP64 storage -- each the most that compiles without
// spilling.  At 256^3 the 56-register step runs 40.3 GLUPS FP32 against 37.9 with 256-thread
// blocks at 64 registers (32 warps).
template <int S, bool REDUCE>
constexpr int aa_min_blocks() {
  return S == POG_STORE_F64 ? 3 : (REDUCE ? 8 : 9);
}
// Whether the non-reducing variants run one cell per thread (1) or a persistent grid-stride loop (0).
#ifndef POG_AA_ONE_CELL
#define POG_AA_ONE_CELL 1
#endif

// One cell per thread (grid-stride when the grid is smaller than the lattice).
template <int S, int PARITY, bool REDUCE, bool MACRO_ONLY>
__global__ void __launch_bounds__(AA_BLOCK, (aa_min_blocks<S, REDUCE>())) aa_step_kernel(
    const KParams kp, typename Store<S>::E* __restrict__ f, const uint32_t* __restrict__ flags,
    const float* __restrict__ force, const float* __restrict__ pdrag, const float* __restrict__ eps,
    const float* __restrict__ u_prev, float* __restrict__ u_next, float* __restrict__ rho_out,
    float* __restrict__ u_out, double* __restrict__ red) {
  using St = Store<S>;
  using C = typename St::C;
  RedAcc<C> acc;
  for (uint32_t c = blockIdx.x * AA_BLOCK + threadIdx.x; c < kp.n; c += gridDim.x * AA_BLOCK) {
    const uint32_t fl = flags[c];
    if (!aa_live(kp, c, fl)) continue;
    const bool open = PARITY == 1 && __all_sync(__activemask(), (fl >> POG_LINK_SHIFT) == 0u);
    typename St::E raw[19];
    aa_load<S, PARITY>(kp, f, c, fl, open, raw);
    C fv[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) fv[q] = St::dech(raw[q]);
    aa_update<S, PARITY, REDUCE, MACRO_ONLY>(kp, f, c, fl, open, fv, force, pdrag, eps, u_prev, u_next,
                                             rho_out, u_out, acc);
  }
  if (REDUCE) reduce_add<C>(acc, red);
}

// Natural-layout copy of the AA state at parity PARITY (odd = the odd-step read gather).
template <int S, int PARITY, typename O>
__global__ void aa_export_kernel(const KParams kp, const typename Store<S>::E* __restrict__ f,
                                 const uint32_t* __restrict__ flags, O* __restrict__ out) {
  using St = Store<S>;
  using C = typename St::C;
  const C rho0 = (C)kp.rho0;
  const uint32_t n = kp.n;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const uint32_t fl = flags[c];
    if ((fl & POG_CELL_SOLID) || c < kp.guard_lo || c > kp.guard_hi) {
#pragma unroll
      for (int q = 0; q < 19; ++q) out[(size_t)q * n + c] = (O)0;
      continue;
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      C v;
      if (PARITY == 0) {
        v = St::ld(f, (uint32_t)q * n + c, q, rho0);
      } else {
        const bool wall = q != 0 && ((fl >> (POG_LINK_SHIFT + opp(q))) & 1u);
        v = wall ? St::ld(f, (uint32_t)q * n + c, q, rho0)
                 : St::ld(f, (uint32_t)opp(q) * n + (c - (uint32_t)kp.off[q]), opp(q), rho0);
      }
      out[(size_t)q * n + c] = (O)v;
    }
  }
}

template <int S, typename I>
__global__ void aa_import_kernel(const KParams kp, const I* __restrict__ in,
                                 const uint32_t* __restrict__ flags, typename Store<S>::E* __restrict__ f) {
  using St = Store<S>;
  using C = typename St::C;
  const C rho0 = (C)kp.rho0;
  const uint32_t n = kp.n;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const bool solid = flags[c] & POG_CELL_SOLID;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      C v = solid ? (C)wd(q) * rho0 : (C)in[(size_t)q * n + c];
      St::st(f, (uint32_t)q * n + c, q, v, rho0);
    }
  }
}

template <int S>
__global__ void aa_init_kernel(const KParams kp, typename Store<S>::E* __restrict__ f,
                               const uint32_t* __restrict__ flags, float rho, float ux, float uy,
                               float uz) {
  using St = Store<S>;
  using C = typename St::C;
  const C rho0 = (C)kp.rho0;
  const uint32_t n = kp.n;
  const C usq15 = (C)1.5 * ((C)ux * (C)ux + (C)uy * (C)uy + (C)uz * (C)uz);
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const bool solid = flags[c] & POG_CELL_SOLID;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      C v = solid ? (C)wd(q) * rho0 : feq_q<C>(q, (C)rho, (C)ux, (C)uy, (C)uz, usq15);
      St::st(f, (uint32_t)q * n + c, q, v, rho0);
    }
  }
}

// ---- host dispatch ----------------------------------------------------------------------------
template <int S, int PARITY, bool REDUCE, bool MACRO>
static int launch_aa(const KParams& kp, void* f, const uint32_t* flags, const float* force,
                     const float* pdrag, const float* eps, const float* u_prev, float* u_next, float* rho_out,
                     float* u_out, double* red, cudaStream_t s) {
  auto kern = aa_step_kernel<S, PARITY, REDUCE, MACRO>;
  static thread_local int grid = 0;
  if (grid == 0) grid = persistent_blocks((const void*)kern, AA_BLOCK);
  if (grid <= 0) return set_error(POG_E_CUDA, "occupancy query failed");
  int want = (int)((kp.n + AA_BLOCK - 1) / AA_BLOCK);
  int g = (POG_AA_ONE_CELL && !REDUCE) ? want : (want < grid ? want : grid);
  kern<<<g, AA_BLOCK, 0, s>>>(kp, (typename Store<S>::E*)f, flags, force, pdrag, eps, u_prev, u_next,
                              rho_out, u_out, red);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

template <int S>
static int dispatch_aa(const KParams& kp, int parity, bool reduce, bool macro, void* f,
                       const uint32_t* flags, const float* force, const float* pdrag, const float* eps,
                       const float* u_prev, float* u_next, float* rho_out, float* u_out,
                       double* red, cudaStream_t s) {
#define POG_AA_CASE(P, R, M)                                                                    \
  if (parity == P && reduce == R && macro == M)                                                 \
    return launch_aa<S, P, R, M>(kp, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
  POG_AA_CASE(0, false, false)
  POG_AA_CASE(1, false, false)
  POG_AA_CASE(0, true, false)
  POG_AA_CASE(1, true, false)
  POG_AA_CASE(0, false, true)
  POG_AA_CASE(1, false, true)
#undef POG_AA_CASE
  return set_error(POG_E_ARG, "unsupported AA kernel variant");
}

static int dispatch_storage(const KParams& kp, int parity, bool reduce, bool macro, void* f,
                            const uint32_t* flags, const float* force, const float* pdrag, const float* eps,
                            const float* u_prev, float* u_next, float* rho_out, float* u_out,
                            double* red, cudaStream_t s) {
  switch (kp.storage) {
    case POG_STORE_F32:
      return dispatch_aa<POG_STORE_F32>(kp, parity, reduce, macro, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
    case POG_STORE_F16S:
      return dispatch_aa<POG_STORE_F16S>(kp, parity, reduce, macro, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
    case POG_STORE_BF16S:
      return dispatch_aa<POG_STORE_BF16S>(kp, parity, reduce, macro, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
    case POG_STORE_F64:
      return dispatch_aa<POG_STORE_F64>(kp, parity, reduce, macro, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
  }
  return set_error(POG_E_ARG, "storage %d unknown", kp.storage);
}

int launch_rows_step(const KParams& kp, int parity, bool reduce, void* f, const uint32_t* flags,
                     const int32_t* cells, int32_t ncells, const float* force, const float* pdrag, const float* eps,
                     const float* u_prev, float* u_next, float* rho_out, float* u_out, double* red,
                     cudaStream_t s);

int launch_pair_step(const KParams& kp, int parity, bool reduce, void* f, const uint32_t* flags,
                     const float* force, const float* pdrag, const float* eps, float* rho_out, float* u_out,
                     double* red, cudaStream_t s);
int launch_ref_step(const KParams& kp, int parity, bool reduce, bool macro, void* f, const uint32_t* flags,
                    const float* force, const float* pdrag, const float* eps, const float* u_prev, float* u_next,
                    float* rho_out, float* u_out, double* red, cudaStream_t s);
int ref_export(const KParams& kp, const void* f, const uint32_t* flags, int parity, void* f_nat, int out_storage,
               cudaStream_t s);
int ref_import(const KParams& kp, const void* f_nat, int in_storage, const uint32_t* flags, void* f, cudaStream_t s);
int ref_init(const KParams& kp, void* f, const uint32_t* flags, float rho, float ux, float uy, float uz,
             cudaStream_t s);

static int grid_for(uint32_t n, int block) {
  long long want = ((long long)n + block - 1) / block;
  return (int)(want < 152 * 64 ? want : 152 * 64);
}

// Host-side fault injection: POG_FAULT_INJECT_STEP=<t> makes pog_step fail with
// POG_E_INJECTED, before launching anything, when step t is part of the call.
static long long fault_step() {
  static long long v = -2;
  if (v == -2) {
    const char* e = getenv("POG_FAULT_INJECT_STEP");
    v = e ? atoll(e) : -1;
  }
  return v;
}

}  // namespace pog

using namespace pog;

extern "C" {

int pog_init_equilibrium(const pog_params* p, void* f, const uint32_t* flags, float rho0, float ux,
                         float uy, float uz, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!f || !flags) return set_error(POG_E_ARG, "f/flags is NULL");
  KParams kp = make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  if (kp.dref) return ref_init(kp, f, flags, rho0, ux, uy, uz, s);
  int g = grid_for(kp.n, 256);
  switch (p->storage) {
    case POG_STORE_F32: aa_init_kernel<POG_STORE_F32><<<g, 256, 0, s>>>(kp, (float*)f, flags, rho0, ux, uy, uz); break;
    case POG_STORE_F16S: aa_init_kernel<POG_STORE_F16S><<<g, 256, 0, s>>>(kp, (__half*)f, flags, rho0, ux, uy, uz); break;
    case POG_STORE_BF16S: aa_init_kernel<POG_STORE_BF16S><<<g, 256, 0, s>>>(kp, (__nv_bfloat16*)f, flags, rho0, ux, uy, uz); break;
    case POG_STORE_F64: aa_init_kernel<POG_STORE_F64><<<g, 256, 0, s>>>(kp, (double*)f, flags, rho0, ux, uy, uz); break;
  }
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_step(const pog_params* p, void* f, const uint32_t* flags, long long t, int nsteps,
             const float* force, const float* pdrag, const float* porosity, float* u_prev, float* u_next,
             float* rho_out, float* u_out, double* reductions, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!f || !flags) return set_error(POG_E_ARG, "f/flags is NULL");
  if (nsteps < 0 || t < 0) return set_error(POG_E_ARG, "nsteps=%d t=%lld invalid", nsteps, t);
  const bool stencil = p->les_mode == POG_LES_STENCIL;
  if (stencil && (!u_prev || !u_next || u_prev == u_next))
    return set_error(POG_E_ARG, "LES stencil mode needs two distinct u buffers");
  long long fs = fault_step();
  if (fs >= t && fs < t + nsteps)
    return set_error(POG_E_INJECTED, "fault injected at step %lld (POG_FAULT_INJECT_STEP)", fs);
  KParams kp = make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  float* up = u_prev;
  float* un = u_next;
  for (int i = 0; i < nsteps; ++i) {
    const bool last = i == nsteps - 1;
    const int parity = (int)((t + i) & 1);
    // the row-tiled kernel when the caller supplied the bounce-back cell list (and it applies)
    rc = 1;
    if (kp.dref) {
      if (p->step_kernel == POG_STEP_AUTO && !stencil)
        rc = launch_pair_step(kp, parity, reductions != nullptr, f, flags, force, pdrag, porosity,
                              last ? rho_out : nullptr, last ? u_out : nullptr, reductions, s);
      if (rc == 1)
        rc = launch_ref_step(kp, parity, reductions != nullptr, false, f, flags, force, pdrag, porosity,
                             stencil ? up : nullptr, stencil ? un : nullptr, last ? rho_out : nullptr,
                             last ? u_out : nullptr, reductions, s);
    } else if (p->wall_cells)
      rc = launch_rows_step(kp, parity, reductions != nullptr, f, flags, p->wall_cells, p->n_wall_cells, force,
                            pdrag, porosity, stencil ? up : nullptr, stencil ? un : nullptr,
                            last ? rho_out : nullptr, last ? u_out : nullptr, reductions, s);
    else if (p->step_kernel == POG_STEP_AUTO)
      rc = launch_pair_step(kp, parity, reductions != nullptr, f, flags, force, pdrag, porosity,
                            last ? rho_out : nullptr, last ? u_out : nullptr, reductions, s);
    if (rc == 1)
      rc = dispatch_storage(kp, parity, reductions != nullptr, false, f, flags, force, pdrag, porosity,
                            stencil ? up : nullptr, stencil ? un : nullptr,
                            last ? rho_out : nullptr, last ? u_out : nullptr,
                            reductions, s);
    if (rc) return rc;
    if (stencil) {
      float* tmp = up;
      up = un;
      un = tmp;
    }
  }
  return POG_OK;
}

int pog_macroscopic(const pog_params* p, const void* f, const uint32_t* flags, long long t,
                    const float* force, const float* pdrag, float* rho_out, float* u_out, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!f || !flags) return set_error(POG_E_ARG, "f/flags is NULL");
  KParams kp = make_kparams(p);
  if (kp.les_mode == POG_LES_STENCIL) kp.les_mode = POG_LES_OFF;  // u does not depend on tau
  if (kp.dref)
    return launch_ref_step(kp, (int)(t & 1), false, true, (void*)f, flags, force, pdrag, nullptr, nullptr, nullptr,
                           rho_out, u_out, nullptr, (cudaStream_t)stream);
  return dispatch_storage(kp, (int)(t & 1), false, true, (void*)f, flags, force, pdrag, nullptr, nullptr,
                          nullptr, rho_out, u_out, nullptr, (cudaStream_t)stream);
}

int pog_export_natural(const pog_params* p, const void* f, const uint32_t* flags, long long t,
                       void* f_nat, int out_storage, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!f || !flags || !f_nat) return set_error(POG_E_ARG, "NULL pointer");
  if (out_storage != POG_STORE_F32 && out_storage != POG_STORE_F64)
    return set_error(POG_E_ARG, "out_storage must be F32 or F64");
  KParams kp = make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  const int par = (int)(t & 1);
  if (kp.dref) return ref_export(kp, f, flags, par, f_nat, out_storage, s);
  int g = grid_for(kp.n, 256);
#define POG_EXP(SS, E)                                                                         \
  if (p->storage == SS) {                                                                      \
    if (out_storage == POG_STORE_F32) {                                                        \
      if (par) aa_export_kernel<SS, 1, float><<<g, 256, 0, s>>>(kp, (const E*)f, flags, (float*)f_nat); \
      else aa_export_kernel<SS, 0, float><<<g, 256, 0, s>>>(kp, (const E*)f, flags, (float*)f_nat);     \
    } else {                                                                                   \
      if (par) aa_export_kernel<SS, 1, double><<<g, 256, 0, s>>>(kp, (const E*)f, flags, (double*)f_nat); \
      else aa_export_kernel<SS, 0, double><<<g, 256, 0, s>>>(kp, (const E*)f, flags, (double*)f_nat);     \
    }                                                                                          \
  }
  POG_EXP(POG_STORE_F32, float)
  POG_EXP(POG_STORE_F16S, __half)
  POG_EXP(POG_STORE_BF16S, __nv_bfloat16)
  POG_EXP(POG_STORE_F64, double)
#undef POG_EXP
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_import_natural(const pog_params* p, const void* f_nat, int in_storage, const uint32_t* flags,
                       void* f, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!f || !flags || !f_nat) return set_error(POG_E_ARG, "NULL pointer");
  if (in_storage != POG_STORE_F32 && in_storage != POG_STORE_F64)
    return set_error(POG_E_ARG, "in_storage must be F32 or F64");
  KParams kp = make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  if (kp.dref) return ref_import(kp, f_nat, in_storage, flags, f, s);
  int g = grid_for(kp.n, 256);
#define POG_IMP(SS, E)                                                                          \
  if (p->storage == SS) {                                                                       \
    if (in_storage == POG_STORE_F32)                                                            \
      aa_import_kernel<SS, float><<<g, 256, 0, s>>>(kp, (const float*)f_nat, flags, (E*)f);     \
    else                                                                                        \
      aa_import_kernel<SS, double><<<g, 256, 0, s>>>(kp, (const double*)f_nat, flags, (E*)f);   \
  }
  POG_IMP(POG_STORE_F32, float)
  POG_IMP(POG_STORE_F16S, __half)
  POG_IMP(POG_STORE_BF16S, __nv_bfloat16)
  POG_IMP(POG_STORE_F64, double)
#undef POG_IMP
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

}  // extern "C"
