// lbm_push.cu -- the same step on natural layout with two buffers: each fluid cell collides
// and pushes f*_q to c + e_q, or into opp(q) of its own cell when c + e_q is solid
// (legacy/lbm_solver.py:609-628).  Used where every intermediate state must be kept in
// natural layout: checkpointed recomputation under the adjoint and FP64 reference runs.
#include "collide.cuh"

namespace pog {

constexpr int PUSH_BLOCK = 128;
// Resident 128-thread blocks per SM, as the AA step: 9 (56 registers), 8 with the FP64 sums, 3
// for FP64 storage.
template <int S, bool REDUCE>
constexpr int push_min_blocks() {
  return S == POG_STORE_F64 ? 3 : (REDUCE ? 8 : 9);
}

template <int S, bool REDUCE>
__global__ void __launch_bounds__(PUSH_BLOCK, (push_min_blocks<S, REDUCE>())) push_step_kernel(
    const KParams kp, const typename Store<S>::E* __restrict__ fin,
    typename Store<S>::E* __restrict__ fout, const uint32_t* __restrict__ flags,
    const float* __restrict__ force, const float* __restrict__ pdrag, const float* __restrict__ eps,
    const float* __restrict__ u_prev, float* __restrict__ rho_out, float* __restrict__ u_out,
    double* __restrict__ red) {
  using St = Store<S>;
  using C = typename St::C;
  const uint32_t n = kp.n;
  RedAcc<C> acc;
  for (uint32_t c = blockIdx.x * PUSH_BLOCK + threadIdx.x; c < n; c += gridDim.x * PUSH_BLOCK) {
    const uint32_t fl = flags[c];
    if ((fl & POG_CELL_SOLID) || c < kp.guard_lo || c > kp.guard_hi) continue;
    const C rs = (C)kp.rho0;  // shift density of the shifted storages
    // the stored form is collided directly (the deviations h of the shifted storages; the shift
    // and bounce-back commute: slots q and opp q carry the same weight)
    C fv[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) fv[q] = St::dech(fin[(uint32_t)q * n + c]);
    C nu_st = (C)0;
    if (kp.les_mode == POG_LES_STENCIL && u_prev && !(fl & POG_CELL_POROUS))
      nu_st = les_nu_stencil<C>(kp, c, u_prev);
    const CellResult<C> r =
        collide_cell<C, St::SHIFTED>(kp, fl, c, fv, force, pdrag, eps, nu_st, (C)St::SCALE, rs);
    if (rho_out) rho_out[c] = (float)r.rho;
    if (u_out) {
      u_out[c] = (float)r.ux;
      u_out[n + c] = (float)r.uy;
      u_out[2u * n + c] = (float)r.uz;
    }
    if (REDUCE) {
      acc.add(r);
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) {
      const uint32_t dst = c + (uint32_t)kp.off[q];
      const bool wall = q != 0 && ((fl >> (POG_LINK_SHIFT + q)) & 1u);
      if (wall)
        fout[(uint32_t)opp(q) * n + c] = St::ench(fv[q]);
      else
        fout[(uint32_t)q * n + dst] = St::ench(fv[q]);
    }
  }
  if (REDUCE) reduce_add<C>(acc, red);
}

template <int S, bool R>
static int launch_push(const KParams& kp, const void* fin, void* fout, const uint32_t* flags,
                       const float* force, const float* pdrag, const float* eps, const float* u_prev, float* rho_out,
                       float* u_out, double* red, cudaStream_t s) {
  auto kern = push_step_kernel<S, R>;
  static thread_local int grid = 0;
  if (grid == 0) grid = persistent_blocks((const void*)kern, PUSH_BLOCK);
  if (grid <= 0) return set_error(POG_E_CUDA, "occupancy query failed");
  int want = (int)((kp.n + PUSH_BLOCK - 1) / PUSH_BLOCK);
  int g = want < grid ? want : grid;
  using E = typename Store<S>::E;
  kern<<<g, PUSH_BLOCK, 0, s>>>(kp, (const E*)fin, (E*)fout, flags, force, pdrag, eps, u_prev, rho_out,
                                u_out, red);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

}  // namespace pog

using namespace pog;

extern "C" int pog_step_push(const pog_params* p, const void* f_in, void* f_out,
                             const uint32_t* flags, const float* force, const float* pdrag,
                             const float* porosity,
                             const float* u_prev, float* rho_out, float* u_out,
                             double* reductions, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!f_in || !f_out || !flags) return set_error(POG_E_ARG, "f_in/f_out/flags is NULL");
  if (f_in == f_out) return set_error(POG_E_ARG, "push step needs distinct f_in and f_out");
  if (p->density_ref) return set_error(POG_E_ARG, "the push step has no per-cell reference density form");
  if (p->les_mode == POG_LES_STENCIL && !u_prev)
    return set_error(POG_E_ARG, "LES stencil mode needs u_prev");
  KParams kp = make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  const bool R = reductions != nullptr;
#define POG_PUSH(SS)                                                                              \
  if (p->storage == SS)                                                                           \
    return R ? launch_push<SS, true>(kp, f_in, f_out, flags, force, pdrag, porosity, u_prev, rho_out, u_out, reductions, s) \
             : launch_push<SS, false>(kp, f_in, f_out, flags, force, pdrag, porosity, u_prev, rho_out, u_out, reductions, s);
  POG_PUSH(POG_STORE_F32)
  POG_PUSH(POG_STORE_F16S)
  POG_PUSH(POG_STORE_BF16S)
  POG_PUSH(POG_STORE_F64)
#undef POG_PUSH
  return set_error(POG_E_ARG, "storage %d unknown", p->storage);
}
