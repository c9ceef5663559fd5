// lbm_tma.cu -- the fused AA step with its distribution reads staged by bulk TMA copies.
//
// Same physics, layout and AA read/write pattern as aa_step_kernel (lbm_aa.cu); what changes is
// how the 19 populations reach the SMs.  A persistent CTA of TT threads walks tiles of TT
// consecutive cells.  One elected thread issues, per tile, 19 one-dimensional cp.async.bulk
// copies (one per population plane: the tile's own slots at an even step, the tile's slots
// shifted by -e_q in plane opp(q) at an odd step) into a STAGES-deep shared-memory ring, each
// stage completed on its own mbarrier.  Loads for tiles it+1 .. it+STAGES-1 are in flight while
// tile it is collided, so the bytes in flight per SM no longer depend on registers per thread
// or occupancy -- the limit of the register-staged kernel.  Stores stay coalesced global stores
// from registers (fire-and-forget).
//
// Alignment: a bulk copy needs 16-byte aligned addresses and sizes, so every plane copy starts
// at the 16-byte boundary at or below the first needed element and covers TT + 16/sizeof(E)
// elements; the thread reads its value at the remainder offset.  Copies are clipped to the last
// 16-byte boundary of the distribution array.  No element a computed cell needs is clipped: the
// largest index read is 18 n + guard_hi (even step) or p n + guard_hi + |off| <= 19 n - 2 with
// plane 18 only read through a positive offset at the odd step, all below the clip point.  All
// mbarrier waits are bounded (tma.cuh).
//
// Why the in-place AA update stays race-free with prefetching: every slot is owned by exactly
// one cell (the even step's (c, q) and the odd step's {(c - e_q, opp q)} = {(c + e_q, q)} are the
// same 19 slots of cell c), tiles are disjoint sets of cells, and padding elements outside a
// tile's own slots are never used.
#include "collide.cuh"
#include "tma.cuh"

namespace pog {

constexpr int TT = 256;                 // cells per tile == consumer threads per CTA
constexpr int NCW = TT / 32;            // consumer warps
constexpr int CTA_THREADS = TT + 32;    // + one producer warp

template <int S>
struct TmaCfg {
  using E = typename Store<S>::E;
  static constexpr int A = 16 / (int)sizeof(E);     // elements per 16 bytes
  static constexpr int PLANE = TT + A;              // smem elements per plane per stage
#ifndef POG_TMA_STAGES
#define POG_TMA_STAGES 4
#endif
  static constexpr int STAGES = sizeof(E) == 8 ? 3 : POG_TMA_STAGES;
  static constexpr size_t STAGE_BYTES = (size_t)19 * PLANE * sizeof(E);
  // ring | per-stage plane offsets (int[20]) | full mbarriers | empty mbarriers
  static constexpr size_t LEAD_OFF = STAGES * STAGE_BYTES;
  static constexpr size_t BAR_OFF = LEAD_OFF + STAGES * 20 * sizeof(int);
  static constexpr size_t SMEM = BAR_OFF + 2 * STAGES * sizeof(uint64_t);
#ifndef POG_TMA_MINB
#define POG_TMA_MINB 2
#endif
  static constexpr int MIN_BLOCKS = sizeof(E) == 8 ? 1 : POG_TMA_MINB;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// First element of plane copy q for the tile starting at cell c0.
template <int PARITY>
__device__ __forceinline__ long long plane_start(const KParams& kp, int q, uint32_t c0) {
  return PARITY == 0 ? (long long)q * kp.n + c0
                     : (long long)opp(q) * kp.n + (long long)c0 - kp.off[q];
}

// Issue the 19 plane copies of one tile into a stage: publish the per-plane offsets, arm the
// stage's full barrier with the byte count, start the copies.
template <int S, int PARITY>
__device__ __forceinline__ void issue_tile(const KParams& kp, const typename Store<S>::E* f,
                                           typename Store<S>::E* stage_buf, int* lead,
                                           uint64_t* bar, uint32_t tile) {
  using Cfg = TmaCfg<S>;
  using E = typename Store<S>::E;
  const long long total = ((long long)19 * kp.n) & ~(long long)(Cfg::A - 1);
  const uint32_t c0 = tile * TT;
  uint32_t bytes = 0;
  // plane offsets first: the arrive below releases them to the threads that wait on `bar`
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    long long st = plane_start<PARITY>(kp, q, c0);
    long long base = st & ~(long long)(Cfg::A - 1);
    long long end = (st + TT + Cfg::A - 1) & ~(long long)(Cfg::A - 1);
    if (end > total) end = total;
    lead[q] = (int)(st - base);
    if (end > base) bytes += (uint32_t)((end - base) * (long long)sizeof(E));
  }
  // order the consumers' earlier generic-proxy reads of this stage before the async writes
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_arrive_expect_tx(bar, bytes);
#pragma unroll
  for (int q = 0; q < 19; ++q) {
    long long st = plane_start<PARITY>(kp, q, c0);
    long long base = st & ~(long long)(Cfg::A - 1);
    long long end = (st + TT + Cfg::A - 1) & ~(long long)(Cfg::A - 1);
    if (end > total) end = total;
    if (end > base)
      tma_load_1d(stage_buf + q * Cfg::PLANE, f + base, (uint32_t)((end - base) * (long long)sizeof(E)), bar);
  }
}

// Warp-specialised persistent kernel.  Warp NCW (the producer) walks the CTA's tiles, waits for
// a stage to be released (empty barrier, one arrival per consumer warp) and refills it; the NCW
// consumer warps wait for a stage's copies (full barrier), collide one cell per thread, store,
// and release the stage.  No block-wide barrier inside the loop, so a slow warp only holds back
// the stage it is reading.
template <int S, int PARITY, bool REDUCE>
__global__ void __launch_bounds__(CTA_THREADS, TmaCfg<S>::MIN_BLOCKS) aa_tma_kernel(
    const KParams kp, typename Store<S>::E* __restrict__ f, const uint32_t* __restrict__ flags,
    const float* __restrict__ force, const float* __restrict__ pdrag, const float* __restrict__ eps,
    const float* __restrict__ u_prev, float* __restrict__ u_next, float* __restrict__ rho_out,
    float* __restrict__ u_out, double* __restrict__ red) {
  using Cfg = TmaCfg<S>;
  using St = Store<S>;
  using E = typename St::E;
  using C = typename St::C;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  E* ring = reinterpret_cast<E*>(smem_raw);
  int* leads = reinterpret_cast<int*>(smem_raw + Cfg::LEAD_OFF);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + Cfg::BAR_OFF);
  uint64_t* empty = full + Cfg::STAGES;
  __shared__ int s_abort;
  const uint32_t n = kp.n;
  const uint32_t ntiles = (n + TT - 1) / TT;
  const uint32_t tid = threadIdx.x;
  const uint32_t warp = tid >> 5, lane = tid & 31u;
  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < Cfg::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NCW);
    }
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();
  const uint32_t first = blockIdx.x, stride = gridDim.x;
  const uint32_t nit = first < ntiles ? (ntiles - first + stride - 1) / stride : 0;
  RedAcc<C> acc;

  if (warp == NCW) {
    // ---------------- producer ----------------
    if (lane == 0) {
      uint32_t it = 0;
      for (; it < nit; ++it) {
        const int st = (int)(it % Cfg::STAGES);
        const uint32_t use = it / Cfg::STAGES;
        if (use > 0 && !mbar_wait_bounded(&empty[st], (use - 1) & 1u)) {
          s_abort = 1;
          break;
        }
        if (s_abort) break;
        issue_tile<S, PARITY>(kp, f, ring + (size_t)st * 19 * Cfg::PLANE, leads + st * 20, &full[st],
                              first + it * stride);
      }
      if (s_abort) {
        // drain the copies that may still be in flight before shared memory is released
        const uint32_t lo_it = it > (uint32_t)Cfg::STAGES ? it - Cfg::STAGES : 0u;
        for (uint32_t k = lo_it; k < it; ++k) mbar_wait_bounded(&full[k % Cfg::STAGES], (k / Cfg::STAGES) & 1u);
      }
    }
  } else {
    // ---------------- consumers ----------------
    const uint32_t lo = kp.guard_lo, hi = kp.guard_hi;
    for (uint32_t it = 0; it < nit; ++it) {
      const int stage = (int)(it % Cfg::STAGES);
      if (!mbar_wait_bounded(&full[stage], (it / Cfg::STAGES) & 1u)) {
        s_abort = 1;
        break;
      }
      const uint32_t c = (first + it * stride) * TT + tid;
      const E* sb = ring + (size_t)stage * 19 * Cfg::PLANE;
      const int* sl = leads + stage * 20;
      const bool live = c <= hi && c >= lo;
      const uint32_t fl = live ? flags[c] : POG_CELL_SOLID;
      const C rs = (C)kp.rho0;  // shift density of the shifted storages
      C fv[19];
      if (!(fl & POG_CELL_SOLID)) {
#pragma unroll
        for (int q = 0; q < 19; ++q)
          fv[q] = St::ld(sb + q * Cfg::PLANE, (uint32_t)(sl[q] + (int)tid), q, rs);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[stage]);  // the stage's values are in registers
      if (fl & POG_CELL_SOLID) continue;
      if (PARITY == 1 && (fl & POG_CELL_NEAR_SOLID)) {
#pragma unroll
        for (int q = 1; q < 19; ++q)
          if ((fl >> (POG_LINK_SHIFT + opp(q))) & 1u) fv[q] = St::ld(f, (uint32_t)q * n + c, q, rs);
      }
      C nu_st = (C)0;
      if (kp.les_mode == POG_LES_STENCIL && !(fl & POG_CELL_POROUS)) nu_st = les_nu_stencil<C>(kp, c, u_prev);
      const CellResult<C> r = collide_cell<C>(kp, fl, c, fv, force, pdrag, eps, nu_st);
      if (rho_out) rho_out[c] = (float)r.rho;
      if (u_out) {
        u_out[c] = (float)r.ux;
        u_out[n + c] = (float)r.uy;
        u_out[2u * n + c] = (float)r.uz;
      }
      if (u_next) {
        u_next[c] = (float)r.ux;
        u_next[n + c] = (float)r.uy;
        u_next[2u * n + c] = (float)r.uz;
      }
      if (REDUCE) {
        acc.add(r);
      }
      if (PARITY == 0) {
#pragma unroll
        for (int q = 0; q < 19; ++q) St::st(f, (uint32_t)opp(q) * n + c, q, fv[q], rs);
      } else {
#pragma unroll
        for (int q = 0; q < 19; ++q) {
          const bool wall = q != 0 && ((fl >> (POG_LINK_SHIFT + q)) & 1u);
          const uint32_t idx = wall ? (uint32_t)opp(q) * n + c : (uint32_t)q * n + (c + (uint32_t)kp.off[q]);
          St::st(f, idx, q, fv[q], rs);
        }
      }
    }
  }
  if (REDUCE) {
    __syncthreads();
    if (!s_abort) {
      double part[POG_RED_COUNT];
      acc.finish(part);
      block_reduce_add(part, red);
    }
  }
}

template <int S, int PARITY, bool REDUCE>
static int launch_tma_one(const KParams& kp, void* f, const uint32_t* flags, const float* force,
                          const float* pdrag, const float* eps, const float* u_prev, float* u_next, float* rho_out,
                          float* u_out, double* red, cudaStream_t s) {
  using Cfg = TmaCfg<S>;
  auto kern = aa_tma_kernel<S, PARITY, REDUCE>;
  static thread_local int grid = 0;
  if (grid == 0) {
    POG_TRY_CUDA(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM));
    grid = persistent_blocks((const void*)kern, CTA_THREADS, Cfg::SMEM);
    if (grid <= 0) return set_error(POG_E_CUDA, "occupancy query failed");
  }
  const int ntiles = (int)((kp.n + TT - 1) / TT);
  const int g = ntiles < grid ? ntiles : grid;
  kern<<<g, CTA_THREADS, Cfg::SMEM, s>>>(kp, (typename Store<S>::E*)f, flags, force, pdrag, eps, u_prev, u_next, rho_out,
                                u_out, red);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

template <int S>
static int launch_tma_s(const KParams& kp, int parity, bool reduce, void* f, const uint32_t* flags,
                        const float* force, const float* pdrag, const float* eps, const float* u_prev, float* u_next,
                        float* rho_out, float* u_out, double* red, cudaStream_t s) {
  if (parity == 0)
    return reduce ? launch_tma_one<S, 0, true>(kp, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s)
                  : launch_tma_one<S, 0, false>(kp, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
  return reduce ? launch_tma_one<S, 1, true>(kp, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s)
                : launch_tma_one<S, 1, false>(kp, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
}

int launch_aa_tma(const KParams& kp, int parity, bool reduce, void* f, const uint32_t* flags,
                  const float* force, const float* pdrag, const float* eps, const float* u_prev, float* u_next,
                  float* rho_out, float* u_out, double* red, cudaStream_t s) {
  switch (kp.storage) {
    case POG_STORE_F32: return launch_tma_s<POG_STORE_F32>(kp, parity, reduce, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
    case POG_STORE_F16S: return launch_tma_s<POG_STORE_F16S>(kp, parity, reduce, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
    case POG_STORE_BF16S: return launch_tma_s<POG_STORE_BF16S>(kp, parity, reduce, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
    case POG_STORE_F64: return launch_tma_s<POG_STORE_F64>(kp, parity, reduce, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
  }
  return set_error(POG_E_ARG, "storage %d unknown", kp.storage);
}

}  // namespace pog

extern "C" int pog_device_status(int reset) {
  unsigned int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, pog::g_device_error, sizeof(v));
  if (e != cudaSuccess) return pog::check_cuda(e, "cudaMemcpyFromSymbol(g_device_error)");
  if (reset && v) {
    unsigned int z = 0;
    e = cudaMemcpyToSymbol(pog::g_device_error, &z, sizeof(z));
    if (e != cudaSuccess) return pog::check_cuda(e, "cudaMemcpyToSymbol(g_device_error)");
  }
  if (v & pog::DEV_ERR_WAIT_TIMEOUT)
    return pog::set_error(POG_E_STATE, "a bounded mbarrier wait gave up in a TMA-staged step kernel");
  return POG_OK;
}
