// lbm_tma.cu -- the fused AA step staged through shared memory by bulk TMA copies: the row-tiled
// step kernel, its bounce-back mailbox pass, and the wall-cell list both use.
//
// Same physics and the same AA read/write pattern as aa_step_kernel (lbm_aa.cu; reference:
// legacy/lbm_solver.py:488-654, les_turbulence.py:289-380, filter_paper.py:471-536); what changes is
// how the populations move between HBM and the SMs.
//
// Tiles of whole grid rows.  A tile is R consecutive rows (T = R nx cells, one thread per cell) of
// the planes 1 .. nz-2.  For each population plane p the tile's slots form one contiguous range
// of the distribution array:
//   even step  plane p, the tile's own cells                   (read (c, q), write (c, opp q))
//   odd step   plane p, the tile's cells shifted by the (y, z) part of e_p
// and -- the AA property -- each cell reads and writes the same 19 slots, so at both parities the
// range a tile loads for plane p is exactly the range it stores back.  One elected thread moves
// each range with one cp.async.bulk copy each way; every other thread touches shared memory only,
// at offsets fixed at compile time:
//   even  f_q  = tile[q][t]               f*_q -> tile[opp q][t]
//   odd   f_q  = tile[opp q][t - e_qx]    f*_q -> tile[q][t + e_qx]
// (the x part of e_q stays inside the row: cells i = 0 and nx-1 are never updated, the outer shell
// being solid).  A slot position no live cell writes is stored back with the value it was loaded
// with; tile ranges of one plane are disjoint, so no other block writes it meanwhile.
//
// Bounce-back through mailboxes.  The kernel streams every direction uniformly, walls included.
// For a fluid cell d whose neighbour s = d + e_p is solid, the odd step reads its f_{opp p} from
// the slot (s, p) -- the mailbox of link (d, p) -- and writes its f*_p there.  bb_mailbox_kernel
// runs over the list of such cells before an odd step (copy the even step's f*_p from (d, opp p)
// into the mailbox) and after it (copy the odd step's f*_p back to (d, opp p)).  Between steps the
// state is therefore exactly the one aa_step_kernel keeps, and the two kernels can be mixed.
//
// Pipeline: a persistent block walks its tiles with STAGES shared-memory stages; the loads of the
// next STAGES-1 tiles are in flight while a tile is collided, a tile's stores are issued as soon as
// its threads have written it, and a stage is reloaded once its stores have read it out.  Every
// mbarrier wait is bounded (tma.cuh): a wait that gives up raises the device error word, the block
// drains its copies in flight and returns.
#include "collide.cuh"
#include "tma.cuh"

namespace pog {

// Row-tile geometry of one launch (host-computed).
struct RowGeom {
  uint32_t R;       // rows per tile
  uint32_t T;       // cells per tile = R nx
  uint32_t row0;    // first row of plane 1 (row index r = k ny + j)
  uint32_t nrows;   // rows of the planes 1 .. nz-2
  uint32_t ntiles;  // ceil(nrows / R)
  int32_t sh[19];   // cell offset of plane p's range: odd step cy(p) nx + cz(p) nx ny, even step 0
};

// Tile capacity (cells per plane tile), pipeline depth and how many lanes issue the copies.
#ifndef POG_ROWS_PS
#define POG_ROWS_PS 512
#endif
#ifndef POG_ROWS_STAGES
#define POG_ROWS_STAGES 3
#endif
#ifndef POG_ROWS_LANES
#define POG_ROWS_LANES 19
#endif
#ifndef POG_ROWS_MINB
#define POG_ROWS_MINB 3
#endif
constexpr int ROWS_BLOCK = 256;  // threads per block; a thread updates PS / ROWS_BLOCK cells per tile

template <int S, int PS>
struct RowCfg {
  using E = typename Store<S>::E;
  static constexpr int STAGES = POG_ROWS_STAGES;
  static constexpr int CPT = PS / ROWS_BLOCK;
  static constexpr size_t STAGE_ELEMS = (size_t)19 * PS;
  static constexpr size_t BAR_OFF = STAGES * STAGE_ELEMS * sizeof(E);
  static constexpr size_t SMEM = BAR_OFF + STAGES * sizeof(uint64_t);
  static_assert(PS % ROWS_BLOCK == 0, "whole cells per thread");
  static_assert(BAR_OFF % 16 == 0, "stage size keeps 16-byte alignment");
  static_assert((PS * sizeof(E)) % 16 == 0, "plane tiles keep 16-byte alignment");
};

__device__ __forceinline__ void tma_store_1d(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// all but the newest bulk group of this thread have finished reading their shared-memory source
__device__ __forceinline__ void bulk_wait_read_all_but_one() {
  asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}
// every bulk group of this thread has completed (writes performed)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Rows of tile `tile` (the last tile may be short).
__device__ __forceinline__ uint32_t tile_rows(const RowGeom& g, uint32_t tile) {
  const uint32_t left = g.nrows - tile * g.R;
  return left < g.R ? left : g.R;
}

// First element of plane p's range for the tile starting at cell c0: p n + c0 + sh[p], which lies in
// [p n - nx, (p+1) n + nx) and, the shifts cancelling at the array ends, inside [0, 19 n).
__device__ __forceinline__ int64_t plane_range(const KParams& kp, const RowGeom& g, int p, uint32_t c0) {
  return (int64_t)p * kp.n + (int64_t)c0 + g.sh[p];
}

// The copies of one tile are issued by warp 0: with POG_ROWS_LANES == 19 lane p moves plane p
// (its own bulk-copy groups, so it alone waits for them), else lane 0 moves all 19.
__device__ __forceinline__ bool issuer(uint32_t tid) { return tid < (uint32_t)POG_ROWS_LANES; }

// Issue the plane loads of one tile into a stage (warp 0; every lane of warp 0 calls it).
template <int S, int PS>
__device__ __forceinline__ void rows_load(const KParams& kp, const RowGeom& g, const typename Store<S>::E* f,
                                          typename Store<S>::E* stage, uint64_t* bar, uint32_t tile,
                                          uint32_t lane) {
  using E = typename Store<S>::E;
  const uint32_t c0 = (g.row0 + tile * g.R) * kp.nx;
  const uint32_t bytes = tile_rows(g, tile) * kp.nx * (uint32_t)sizeof(E);
  if (lane == 0) mbar_arrive_expect_tx(bar, 19u * bytes);  // before any copy can complete
  __syncwarp();
  if (POG_ROWS_LANES == 19) {
    if (lane < 19u) tma_load_1d(stage + lane * PS, f + plane_range(kp, g, (int)lane, c0), bytes, bar);
  } else if (lane == 0) {
#pragma unroll
    for (int p = 0; p < 19; ++p) tma_load_1d(stage + p * PS, f + plane_range(kp, g, p, c0), bytes, bar);
  }
}

template <int S, int PS>
__device__ __forceinline__ void rows_store(const KParams& kp, const RowGeom& g, typename Store<S>::E* f,
                                           const typename Store<S>::E* stage, uint32_t tile, uint32_t lane) {
  const uint32_t c0 = (g.row0 + tile * g.R) * kp.nx;
  const uint32_t bytes = tile_rows(g, tile) * kp.nx * (uint32_t)sizeof(typename Store<S>::E);
  if (POG_ROWS_LANES == 19) {
    if (lane < 19u) {
      tma_store_1d(f + plane_range(kp, g, (int)lane, c0), stage + lane * PS, bytes);
      bulk_commit();
    }
  } else if (lane == 0) {
#pragma unroll
    for (int p = 0; p < 19; ++p) tma_store_1d(f + plane_range(kp, g, p, c0), stage + p * PS, bytes);
    bulk_commit();
  }
}

template <int S, int PS, int PARITY, bool REDUCE>
__global__ void __launch_bounds__(ROWS_BLOCK, POG_ROWS_MINB) rows_step_kernel(
    const KParams kp, const RowGeom g, typename Store<S>::E* __restrict__ f, const uint32_t* __restrict__ flags,
    const float* __restrict__ force, const float* __restrict__ pdrag, const float* __restrict__ eps,
    const float* __restrict__ u_prev, float* __restrict__ u_next, float* __restrict__ rho_out,
    float* __restrict__ u_out, double* __restrict__ red) {
  using Cfg = RowCfg<S, PS>;
  using St = Store<S>;
  using E = typename St::E;
  using C = typename St::C;
  constexpr int NST = Cfg::STAGES;
  constexpr int CPT = Cfg::CPT;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  E* ring = reinterpret_cast<E*>(smem_raw);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + Cfg::BAR_OFF);
  const uint32_t tid = threadIdx.x;
  const bool warp0 = tid < 32u;
  const uint32_t nit = blockIdx.x < g.ntiles ? (g.ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0u;
  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < NST; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (warp0)
    for (uint32_t s = 0; s < (uint32_t)NST && s < nit; ++s)
      rows_load<S, PS>(kp, g, f, ring + s * Cfg::STAGE_ELEMS, &bar[s], blockIdx.x + s * gridDim.x, tid);
  uint32_t issued = nit < (uint32_t)NST ? nit : (uint32_t)NST;  // tiles whose loads were issued (warp 0)
  // bit s: the cell tid + s*ROWS_BLOCK of a tile is updated by this kernel (tiles start on a row;
  // cells i = 0 and nx-1 of a row belong to the solid shell)
  uint32_t colmask = 0;
#pragma unroll
  for (int s = 0; s < CPT; ++s) {
    const uint32_t t = tid + (uint32_t)s * ROWS_BLOCK, i = t % kp.nx;
    if (t < g.T && i >= 1u && i + 1u < kp.nx) colmask |= 1u << s;
  }
  const C rs = (C)kp.rho0;
  RedAcc<C> acc;
  bool aborted = false;
  uint32_t it = 0;
  for (; it < nit; ++it) {
    const uint32_t stage = it % NST;
    const uint32_t tile = blockIdx.x + it * gridDim.x;
    const bool ok = mbar_wait_bounded(&bar[stage], (it / NST) & 1u);
    const uint32_t c0 = (g.row0 + tile * g.R) * kp.nx;
    const uint32_t ncells = tile_rows(g, tile) * kp.nx;
#pragma unroll 1
    for (int s = 0; s < CPT; ++s) {
      const uint32_t t = tid + (uint32_t)s * ROWS_BLOCK;
      const bool live = ok && ((colmask >> s) & 1u) && t < ncells;
      const uint32_t c = c0 + t;
      const uint32_t fl = live ? flags[c] : POG_CELL_SOLID;
      if (fl & POG_CELL_SOLID) continue;
      E* sp = ring + stage * Cfg::STAGE_ELEMS + t;  // this cell's column of the stage
      C fv[19];
      if (PARITY == 0) {
#pragma unroll
        for (int q = 0; q < 19; ++q) fv[q] = St::dech(sp[q * PS]);
      } else {
#pragma unroll
        for (int q = 0; q < 19; ++q) fv[q] = St::dech(sp[opp(q) * PS - cx(q)]);
      }
      C nu_st = (C)0;
      if (kp.les_mode == POG_LES_STENCIL && !(fl & POG_CELL_POROUS)) nu_st = les_nu_stencil<C>(kp, c, u_prev);
      const CellResult<C> r = collide_cell<C, St::SHIFTED>(kp, fl, c, fv, force, pdrag, eps, nu_st, (C)St::SCALE, rs);
      if (rho_out) rho_out[c] = (float)r.rho;
      if (u_out) {
        u_out[c] = (float)r.ux;
        u_out[kp.n + c] = (float)r.uy;
        u_out[2u * kp.n + c] = (float)r.uz;
      }
      if (u_next) {
        u_next[c] = (float)r.ux;
        u_next[kp.n + c] = (float)r.uy;
        u_next[2u * kp.n + c] = (float)r.uz;
      }
      if (REDUCE) acc.add(r);
      // each slot position is read and written by the same thread: no barrier between the two
      if (PARITY == 0) {
#pragma unroll
        for (int q = 0; q < 19; ++q) sp[opp(q) * PS] = St::ench(fv[q]);
      } else {
#pragma unroll
        for (int q = 0; q < 19; ++q) sp[q * PS + cx(q)] = St::ench(fv[q]);
      }
    }
    // the thread's generic shared-memory accesses are ordered before the async stores below
    fence_proxy_async();
    if (__syncthreads_or(ok ? 0 : 1)) {
      aborted = true;
      break;
    }
    if (warp0) {
      rows_store<S, PS>(kp, g, f, ring + stage * Cfg::STAGE_ELEMS, tile, tid);
      // reload the previous iteration's stage: its stores were issued one tile ago
      if (it >= 1 && issued < nit) {
        if (issuer(tid)) bulk_wait_read_all_but_one();
        const uint32_t ps = (it - 1) % NST;
        rows_load<S, PS>(kp, g, f, ring + ps * Cfg::STAGE_ELEMS, &bar[ps], blockIdx.x + issued * gridDim.x, tid);
        ++issued;
      }
    }
  }
  if (warp0) {
    if (aborted && tid == 0) {
      // drain the loads still in flight into this block's shared memory (bounded)
      for (uint32_t k = it; k < issued; ++k) mbar_wait_bounded(&bar[k % NST], (k / NST) & 1u);
    }
    if (issuer(tid)) bulk_wait_all();
  }
  if (REDUCE && !aborted) reduce_add<C>(acc, red);
}

// Mailbox copies of the bounce-back links of the listed cells (see the file comment):
// DIR 0 (before an odd step): (d + e_p, p) := (d, opp p); DIR 1 (after it): the reverse.
__device__ __forceinline__ int opp_rt(int q) {
  return q == 0 ? 0 : (q <= 6 ? ((q - 1) ^ 1) + 1 : 7 + (((q - 7) & ~3) | (3 - ((q - 7) & 3))));
}

template <typename E, int DIR>
__global__ void bb_mailbox_kernel(const KParams kp, E* __restrict__ f, const uint32_t* __restrict__ flags,
                                  const int32_t* __restrict__ cells, int32_t ncells) {
  for (int32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ncells; k += gridDim.x * blockDim.x) {
    const uint32_t d = (uint32_t)cells[k];
    if (d < kp.guard_lo || d > kp.guard_hi) continue;  // a malformed list cannot reach outside f
    uint32_t links = (flags[d] >> POG_LINK_SHIFT) & 0x7fffeu;  // bits q = 1..18
    while (links) {
      const int q = __ffs(links) - 1;
      links &= links - 1u;
      const uint32_t own = kp.pl[opp_rt(q)] + d;  // (d, opp q)
      const uint32_t mb = kp.wr[q] + d;           // (d + e_q, q)
      if (DIR == 0)
        f[mb] = f[own];
      else
        f[own] = f[mb];
    }
  }
}

// Cells the mailbox pass serves: fluid cells with a solid neighbour that the row-tiled step
// updates (planes 1 .. nz-2, 1 <= i <= nx-2).  Warp-aggregated append; `count` (device) receives
// the total, entries beyond `cap` are not written.
__global__ void wall_list_kernel(const KParams kp, const uint32_t* __restrict__ flags, int32_t* __restrict__ cells,
                                 int32_t cap, int32_t* __restrict__ count) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < kp.n; base += stride) {
    const uint32_t c = base + threadIdx.x;
    bool want = false;
    if (c < kp.n) {
      const uint32_t fl = flags[c];
      const uint32_t i = c % kp.nx, k = c / kp.nxny;
      want = !(fl & POG_CELL_SOLID) && ((fl >> POG_LINK_SHIFT) & 0x7fffeu) != 0u && k >= 1u && k + 1u < kp.nz &&
             i >= 1u && i + 1u < kp.nx;
    }
    const unsigned m = __ballot_sync(0xffffffffu, want);
    int32_t at = 0;
    if (lane == 0 && m) at = atomicAdd(count, (int32_t)__popc(m));
    at = __shfl_sync(0xffffffffu, at, 0);
    if (want) {
      const int32_t slot = at + (int32_t)__popc(m & ((1u << lane) - 1u));
      if (cells && slot < cap) cells[slot] = (int32_t)c;
    }
  }
}

// ---- host side --------------------------------------------------------------------------------
template <int S>
static constexpr uint32_t elem_bytes() {
  return (uint32_t)sizeof(typename Store<S>::E);
}

// Rows per tile for this lattice and plane-tile capacity ps (cells), or 0 when the row-tiled kernel
// does not apply (rows longer than a tile, rows not a multiple of 16 bytes, lattice too flat).
static uint32_t rows_per_tile(const KParams& kp, uint32_t esize, uint32_t ps) {
  if (kp.nx > ps || (kp.nx * esize) % 16u != 0u || kp.nz < 3 || kp.ny < 3) return 0;
  return ps / kp.nx;
}

template <int S, int PS, int PARITY, bool REDUCE>
static int launch_rows(const KParams& kp, const RowGeom& g, void* f, const uint32_t* flags, const float* force,
                       const float* pdrag, const float* eps, const float* u_prev, float* u_next, float* rho_out,
                       float* u_out, double* red, cudaStream_t s) {
  using Cfg = RowCfg<S, PS>;
  auto kern = rows_step_kernel<S, PS, PARITY, REDUCE>;
  static thread_local int grid = 0;
  static thread_local uint32_t grid_T = 0;
  if (grid == 0 || grid_T != g.T) {
    POG_TRY_CUDA(cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM));
    grid = persistent_blocks((const void*)kern, ROWS_BLOCK, Cfg::SMEM);
    grid_T = g.T;
    if (grid <= 0) return set_error(POG_E_CUDA, "occupancy query failed");
  }
  const int blocks = (int)g.ntiles < grid ? (int)g.ntiles : grid;
  kern<<<blocks, ROWS_BLOCK, Cfg::SMEM, s>>>(kp, g, (typename Store<S>::E*)f, flags, force, pdrag, eps, u_prev, u_next,
                                      rho_out, u_out, red);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

template <int S, int PS>
static int launch_rows_ps(const KParams& kp, const RowGeom& g, int parity, bool reduce, void* f, const uint32_t* flags,
                          const float* force, const float* pdrag, const float* eps, const float* u_prev,
                          float* u_next, float* rho_out, float* u_out, double* red, cudaStream_t s) {
  if (parity == 0)
    return reduce ? launch_rows<S, PS, 0, true>(kp, g, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s)
                  : launch_rows<S, PS, 0, false>(kp, g, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
  return reduce ? launch_rows<S, PS, 1, true>(kp, g, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s)
                : launch_rows<S, PS, 1, false>(kp, g, f, flags, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
}

template <typename E>
static int launch_mailbox(const KParams& kp, int dir, void* f, const uint32_t* flags, const int32_t* cells,
                          int32_t ncells, cudaStream_t s) {
  if (ncells <= 0) return POG_OK;
  const int block = 256;
  long long want = ((long long)ncells + block - 1) / block;
  const int grid = (int)(want < 152 * 16 ? want : 152 * 16);
  if (dir == 0)
    bb_mailbox_kernel<E, 0><<<grid, block, 0, s>>>(kp, (E*)f, flags, cells, ncells);
  else
    bb_mailbox_kernel<E, 1><<<grid, block, 0, s>>>(kp, (E*)f, flags, cells, ncells);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

template <int S>
static int rows_step_s(const KParams& kp, int parity, bool reduce, void* f, const uint32_t* flags,
                       const int32_t* cells, int32_t ncells, const float* force, const float* pdrag, const float* eps,
                       const float* u_prev, float* u_next, float* rho_out, float* u_out, double* red,
                       cudaStream_t s) {
  using E = typename Store<S>::E;
  RowGeom g;
  const uint32_t R = rows_per_tile(kp, elem_bytes<S>(), (uint32_t)POG_ROWS_PS);
  if (R == 0u) return 1;  // not applicable: the caller takes the register-staged kernel
  g.R = R;
  g.T = R * kp.nx;
  g.row0 = kp.ny;
  g.nrows = kp.ny * (kp.nz - 2u);
  g.ntiles = (g.nrows + R - 1u) / R;
  for (int p = 0; p < 19; ++p) g.sh[p] = parity ? cy(p) * (int32_t)kp.nx + cz(p) * (int32_t)kp.nxny : 0;
  int rc;
  if (parity == 1 && (rc = launch_mailbox<E>(kp, 0, f, flags, cells, ncells, s))) return rc;
  rc = launch_rows_ps<S, POG_ROWS_PS>(kp, g, parity, reduce, f, flags, force, pdrag, eps, u_prev, u_next, rho_out,
                                      u_out, red, s);
  if (rc) return rc;
  if (parity == 1 && (rc = launch_mailbox<E>(kp, 1, f, flags, cells, ncells, s))) return rc;
  return POG_OK;
}

// One step with the row-tiled kernel (and its mailbox passes at an odd step).  Returns 1, having
// launched nothing, when the kernel does not apply to this lattice or buffer; the caller then
// runs the register-staged step.
int launch_rows_step(const KParams& kp, int parity, bool reduce, void* f, const uint32_t* flags,
                     const int32_t* cells, int32_t ncells, const float* force, const float* pdrag, const float* eps,
                     const float* u_prev, float* u_next, float* rho_out, float* u_out, double* red,
                     cudaStream_t s) {
  if (((uintptr_t)f & 15u) != 0u || kp.dref) return 1;
  switch (kp.storage) {
    case POG_STORE_F32:
      return rows_step_s<POG_STORE_F32>(kp, parity, reduce, f, flags, cells, ncells, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
    case POG_STORE_F16S:
      return rows_step_s<POG_STORE_F16S>(kp, parity, reduce, f, flags, cells, ncells, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
    case POG_STORE_BF16S:
      return rows_step_s<POG_STORE_BF16S>(kp, parity, reduce, f, flags, cells, ncells, force, pdrag, eps, u_prev, u_next, rho_out, u_out, red, s);
  }
  return 1;  // FP64 reference runs keep the register-staged kernel
}

}  // namespace pog

using namespace pog;

extern "C" int pog_wall_list(const pog_params* p, const uint32_t* flags, int32_t* cells, int32_t capacity,
                             int32_t* count, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!flags || !count) return set_error(POG_E_ARG, "flags/count is NULL");
  if (cells && capacity < 0) return set_error(POG_E_ARG, "capacity %d < 0", capacity);
  KParams kp = make_kparams(p);
  cudaStream_t s = (cudaStream_t)stream;
  POG_TRY_CUDA(cudaMemsetAsync(count, 0, sizeof(int32_t), s));
  long long want = ((long long)kp.n + 255) / 256;
  const int grid = (int)(want < 152 * 32 ? want : 152 * 32);
  wall_list_kernel<<<grid, 256, 0, s>>>(kp, flags, cells, cells ? capacity : 0, count);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

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
    return pog::set_error(POG_E_STATE, "a bounded mbarrier wait gave up in the row-tiled step kernel");
  return POG_OK;
}
