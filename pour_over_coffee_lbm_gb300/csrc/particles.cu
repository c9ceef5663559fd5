// particles.cu -- Lagrangian coffee particles, two-way coupled to the lattice.
//
// Replaces CoffeeParticleSystem's coupling kernels (src/physics/coffee_particles.py):
// interpolate_fluid_velocity_from_field 1156-1198, distribute_force_to_grid 1048-1086,
// compute_drag_coefficient 1088-1099, compute_two_way_coupling_forces 1107-1154,
// apply_under_relaxation 1200-1212, update_particle_physics 641-720 (+ cone constraint
// 734-831), in the order of LBMSolver.step_with_two_way_coupling (legacy/lbm_solver.py:
// 1485-1509).  The fluid side: the reference spreads the explicit reaction -F onto the 8 nodes;
// here each particle deposits its drag coefficient beta = m_p/(tau_p + dt) and beta*v onto
// them (Kp, Kv) and the lattice step applies the particle force Kv - Kp u implicitly in u,
// which stays stable where the flow packs particles into a few cells (the explicit exchange
// diverges once a cell's particle mass exceeds its fluid mass).  Particles are processed in
// cell order (a stable LSD radix sort on the cell key) and lanes of a warp that hit the same
// node combine their contributions with a segmented warp reduction before one atomic per node
// ("warp-aggregated atomics").  A deterministic mode accumulates 2^32-scaled int64 fixed point
// instead, which is order-independent.
//
// This translation unit is compiled with -fmad=false: every float operation is a single
// IEEE operation in the written order, so per-particle results are bit-identical with the
// CPU restatement.
#include <math.h>

#include "common.cuh"

namespace pog {

constexpr int SORT_TILE = 512;  // elements (= threads) per sort block
constexpr int RADIX = 256;
constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_PER_THREAD = 4;
constexpr int SCAN_CHUNK = SCAN_BLOCK * SCAN_PER_THREAD;
constexpr int MAX_SORT_NP = 1 << 25;
constexpr double FIX_SCALE = 4294967296.0;  // 2^32

__device__ __forceinline__ int cell_axis(float x, int n) {
  float a = fminf((float)(n - 2), x);
  a = fmaxf(0.0f, a);
  return (int)a;
}

__global__ void bin_kernel(int nx, int ny, int nz, const float* __restrict__ pos,
                           const int32_t* __restrict__ active, int np, int32_t* __restrict__ keys) {
  const uint32_t ncell = (uint32_t)nx * ny * nz;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
    if (!active[q]) {
      keys[q] = (int32_t)ncell;
      continue;
    }
    int i = cell_axis(pos[q], nx), j = cell_axis(pos[np + q], ny), k = cell_axis(pos[2 * np + q], nz);
    keys[q] = (int32_t)((uint32_t)i + (uint32_t)nx * ((uint32_t)j + (uint32_t)ny * (uint32_t)k));
  }
}

// Per-tile digit histogram, digit-major: hist[d * ntiles + tile].
__global__ void __launch_bounds__(SORT_TILE) radix_hist_kernel(const uint32_t* __restrict__ keys,
                                                               int np, int shift, int ntiles,
                                                               uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[RADIX];
  for (int d = threadIdx.x; d < RADIX; d += blockDim.x) cnt[d] = 0;
  __syncthreads();
  int e = blockIdx.x * SORT_TILE + threadIdx.x;
  if (e < np) atomicAdd(&cnt[(keys[e] >> shift) & (RADIX - 1)], 1u);
  __syncthreads();
  for (int d = threadIdx.x; d < RADIX; d += blockDim.x) hist[(size_t)d * ntiles + blockIdx.x] = cnt[d];
}

// Exclusive scan in three launches: chunk sums, scan of the chunk sums, chunk-local scans.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[SCAN_BLOCK / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < (int)(blockDim.x / 32) ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    ws[lane] = w;
  }
  __syncthreads();
  uint32_t warp_prefix = warp > 0 ? ws[warp - 1] : 0;
  if (total) *total = ws[blockDim.x / 32 - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

__global__ void __launch_bounds__(SCAN_BLOCK) scan_reduce_kernel(const uint32_t* __restrict__ in,
                                                                 uint32_t m, uint32_t* __restrict__ sums) {
  uint32_t base = blockIdx.x * SCAN_CHUNK + threadIdx.x * SCAN_PER_THREAD;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i)
    if (base + i < m) s += in[base + i];
  uint32_t total;
  block_exclusive_scan(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_BLOCK) scan_sums_kernel(uint32_t* __restrict__ sums, uint32_t nb) {
  // nb <= SCAN_CHUNK (checked on the host)
  uint32_t base = threadIdx.x * SCAN_PER_THREAD;
  uint32_t v[SCAN_PER_THREAD], s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    v[i] = base + i < nb ? sums[base + i] : 0;
    s += v[i];
  }
  uint32_t pre = block_exclusive_scan(s, nullptr);
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    if (base + i < nb) sums[base + i] = pre;
    pre += v[i];
  }
}

__global__ void __launch_bounds__(SCAN_BLOCK) scan_down_kernel(uint32_t* __restrict__ data, uint32_t m,
                                                               const uint32_t* __restrict__ sums) {
  uint32_t base = blockIdx.x * SCAN_CHUNK + threadIdx.x * SCAN_PER_THREAD;
  uint32_t v[SCAN_PER_THREAD], s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    v[i] = base + i < m ? data[base + i] : 0;
    s += v[i];
  }
  uint32_t pre = block_exclusive_scan(s, nullptr) + sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < SCAN_PER_THREAD; ++i) {
    if (base + i < m) data[base + i] = pre;
    pre += v[i];
  }
}

// Stable scatter of one radix pass.  Rank within the tile = rank within the warp (match_any
// + popc of lower lanes) + count of the same digit in lower warps.
__global__ void __launch_bounds__(SORT_TILE) radix_scatter_kernel(
    const uint32_t* __restrict__ kin, const int32_t* __restrict__ vin, int np, int shift,
    int ntiles, const uint32_t* __restrict__ offsets, uint32_t* __restrict__ kout,
    int32_t* __restrict__ vout) {
  constexpr int NW = SORT_TILE / 32;
  __shared__ uint32_t wcnt[NW][RADIX];
  for (int i = threadIdx.x; i < NW * RADIX; i += blockDim.x) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int e = blockIdx.x * SORT_TILE + threadIdx.x;
  const bool valid = e < np;
  uint32_t key = valid ? kin[e] : 0u;
  int32_t val = valid ? (vin ? vin[e] : e) : 0;
  // invalid lanes get a private digit value (>= RADIX) so they never match a real digit
  uint32_t d = valid ? ((key >> shift) & (RADIX - 1)) : (uint32_t)(RADIX + lane);
  uint32_t peers = __match_any_sync(0xffffffffu, d);
  uint32_t lt = (1u << lane) - 1u;
  uint32_t rank = __popc(peers & lt);
  if (valid && (peers & lt) == 0) wcnt[warp][d] = __popc(peers);
  __syncthreads();
  // exclusive prefix over warps, per digit
  for (int dd = threadIdx.x; dd < RADIX; dd += blockDim.x) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      uint32_t c = wcnt[w][dd];
      wcnt[w][dd] = run;
      run += c;
    }
  }
  __syncthreads();
  if (valid) {
    uint32_t dst = offsets[(size_t)d * ntiles + blockIdx.x] + wcnt[warp][d] + rank;
    kout[dst] = key;
    vout[dst] = val;
  }
}

// ---- coupling -----------------------------------------------------------------------------------
struct PKParams {
  int nx, ny, nz;
  uint32_t n;
  float cxf, cyf, tanth, apex;
  float rho0, mu, rho_p, alpha, dt, gx, gy, gz;
  float zlo, zhi, margin, pullback, damping;
  int drag_model, deterministic;
  int reaction;       // enum pog_reaction
  const float* pour;  // device pour-nozzle block or null
  int32_t* dep_cells;  // device [np]: base cell of each particle's deposit (-1: none) or null
  uint32_t* dmask;     // device bit mask of the deposited cells or null
};

// Impact force of the pour stream on a particle at (x, y, z) (create_water_impact_force,
// precise_pouring.py:190-226): within 2R of the stream axis and above IMPACT_ZMIN, -S I e_z
// plus the radial push 0.3 S I (dx, dy)/r, I = exp(-(r/R)^2 / 2), |F| capped at IMPACT_MAX.
__device__ __forceinline__ bool pour_impact(const float* b, float x, float y, float z, float Fi[3]) {
  if (b[POG_POUR_ACTIVE] == 0.0f || !(b[POG_POUR_IMPACT] > 0.0f)) return false;
  const float dx = x - b[POG_POUR_X], dy = y - b[POG_POUR_Y];
  const float R = b[POG_POUR_RADIUS];
  const float r = sqrtf(dx * dx + dy * dy);
  if (!(r <= R * 2.0f) || !(z > b[POG_POUR_IMPACT_ZMIN])) return false;
  const float S = b[POG_POUR_IMPACT];
  const float rr = r / R;
  const float I = expf(-0.5f * (rr * rr));
  Fi[0] = 0.0f;
  Fi[1] = 0.0f;
  Fi[2] = -S * I;
  if (r > 0.1f) {
    const float rm = S * 0.3f * I;
    Fi[0] = rm * dx / r;
    Fi[1] = rm * dy / r;
  }
  const float fm = sqrtf(Fi[0] * Fi[0] + Fi[1] * Fi[1] + Fi[2] * Fi[2]);
  const float mx = b[POG_POUR_IMPACT_MAX];
  if (fm > mx) {
    const float sc = mx / fm;
    Fi[0] = Fi[0] * sc;
    Fi[1] = Fi[1] * sc;
    Fi[2] = Fi[2] * sc;
  }
  return true;
}

// Segmented warp sum over runs of consecutive lanes that share `node` (in cell order equal
// nodes are consecutive; in any other order a repeated node simply starts a new run).  Runs
// are numbered from the head-flag ballot, the suffix sum stays inside a run, and the head lane
// of each run adds the run's total with one atomic per component.  The four deposit components
// of a node share the runs and ride the same shuffles.
__device__ __forceinline__ void warp_aggregated_add4(float* base, uint32_t n, uint32_t node, bool ok, float v0,
                                                     float v1, float v2, float v3) {
  const int lane = threadIdx.x & 31;
  const uint32_t key = ok ? node : (0xffffffffu - (uint32_t)lane);
  const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
  const bool head = lane == 0 || prev != key;
  const uint32_t heads = __ballot_sync(0xffffffffu, head);
  const uint32_t upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
  const uint32_t seg = (uint32_t)__popc(heads & upto);
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t ss = __shfl_down_sync(0xffffffffu, seg, o);
    const float a0 = __shfl_down_sync(0xffffffffu, v0, o), a1 = __shfl_down_sync(0xffffffffu, v1, o);
    const float a2 = __shfl_down_sync(0xffffffffu, v2, o), a3 = __shfl_down_sync(0xffffffffu, v3, o);
    if (lane + o < 32 && ss == seg) {
      v0 += a0;
      v1 += a1;
      v2 += a2;
      v3 += a3;
    }
  }
  if (ok && head) {
    if (v0 != 0.0f) atomicAdd(base + node, v0);
    if (v1 != 0.0f) atomicAdd(base + n + node, v1);
    if (v2 != 0.0f) atomicAdd(base + 2u * n + node, v2);
    if (v3 != 0.0f) atomicAdd(base + 3u * n + node, v3);
  }
}

__device__ __forceinline__ void warp_aggregated_or(uint32_t* base, uint32_t word, bool ok, uint32_t v) {
  const int lane = threadIdx.x & 31;
  const uint32_t key = ok ? word : (0xffffffffu - (uint32_t)lane);
  const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
  const bool head = lane == 0 || prev != key;
  const uint32_t heads = __ballot_sync(0xffffffffu, head);
  const uint32_t upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
  const uint32_t seg = (uint32_t)__popc(heads & upto);
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t ss = __shfl_down_sync(0xffffffffu, seg, o);
    uint32_t vv = __shfl_down_sync(0xffffffffu, v, o);
    if (lane + o < 32 && ss == seg) v |= vv;
  }
  if (ok && head && v) atomicOr(base + word, v);
}

__global__ void couple_kernel(PKParams P, float* __restrict__ pos, float* __restrict__ vel,
                              const float* __restrict__ diam, float* __restrict__ drag_old,
                              int32_t* __restrict__ active, int np, const int32_t* __restrict__ order,
                              const float* __restrict__ u, float* __restrict__ pdrag,
                              unsigned long long* __restrict__ pdrag_fix,
                              float* __restrict__ u_at) {
  const float PI_F = 3.14159265358979f;
  const uint32_t n = P.n;
  // whole warps iterate together so the warp-level aggregation sees converged lanes
  const int stride = gridDim.x * blockDim.x;
  const int nloop = (np + stride - 1) / stride;
  for (int it = 0; it < nloop; ++it) {
    const int t = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    const int q = t < np ? (order ? order[t] : t) : -1;
    bool ok = q >= 0 && active[q] != 0;
    float x = 0, y = 0, z = 0;
    int i = 0, j = 0, k = 0;
    float w[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float F[3] = {0, 0, 0};
    float Fn[3] = {0, 0, 0};      // unrelaxed drag F_new
    float dep[4] = {0, 0, 0, 0};  // deposit (Kp, Kv): beta, beta * v_new; or 0, -F
    bool dep_ok = false;
    if (ok) {
      x = pos[q];
      y = pos[np + q];
      z = pos[2 * np + q];
      i = cell_axis(x, P.nx);
      j = cell_axis(y, P.ny);
      k = cell_axis(z, P.nz);
      float fx = fmaxf(0.0f, fminf(1.0f, x - (float)i));
      float fy = fmaxf(0.0f, fminf(1.0f, y - (float)j));
      float fz = fmaxf(0.0f, fminf(1.0f, z - (float)k));
      w[0] = (1 - fx) * (1 - fy) * (1 - fz);
      w[1] = (1 - fx) * (1 - fy) * fz;
      w[2] = (1 - fx) * fy * (1 - fz);
      w[3] = (1 - fx) * fy * fz;
      w[4] = fx * (1 - fy) * (1 - fz);
      w[5] = fx * (1 - fy) * fz;
      w[6] = fx * fy * (1 - fz);
      w[7] = fx * fy * fz;
    }
    const uint32_t sx = 1, sy = (uint32_t)P.nx, sz = (uint32_t)P.nx * (uint32_t)P.ny;
    const uint32_t c0 = (uint32_t)i + sy * (uint32_t)j + sz * (uint32_t)k;
    uint32_t nodes[8] = {c0, c0 + sz, c0 + sy, c0 + sy + sz, c0 + sx, c0 + sx + sz, c0 + sx + sy, c0 + sx + sy + sz};
    if (ok) {
      float uf[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float* v = u + (size_t)a * n;
        float s = w[0] * v[nodes[0]];
#pragma unroll
        for (int cc = 1; cc < 8; ++cc) s = s + w[cc] * v[nodes[cc]];
        uf[a] = s;
      }
      if (u_at) {
        u_at[q] = uf[0];
        u_at[np + q] = uf[1];
        u_at[2 * np + q] = uf[2];
      }
      float v0[3] = {vel[q], vel[np + q], vel[2 * np + q]};
      float ur[3] = {uf[0] - v0[0], uf[1] - v0[1], uf[2] - v0[2]};
      float d = diam[q];
      float vol = (PI_F / 6.0f) * (d * d * d);
      float mp = P.rho_p * vol;
      float mf = P.rho0 * vol;
      float taup = mp / (3.0f * PI_F * P.mu * d);
      if (P.drag_model == 1) {
        float urm = sqrtf(ur[0] * ur[0] + ur[1] * ur[1] + ur[2] * ur[2]);
        float re = P.rho0 * urm * d / P.mu;
        float fac = 1.0f;
        if (re >= 1000.0f)
          fac = 0.44f * re / 24.0f;
        else if (re >= 0.1f)
          fac = 1.0f + 0.15f * powf(re, 0.687f);
        taup = taup / fac;
      }
      const float gv[3] = {P.gx, P.gy, P.gz};
      const float beta = mp / (taup + P.dt);  // drag coefficient: F_new = beta (u_f - v)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        float fnew = mp * ur[a] / (taup + P.dt);
        Fn[a] = fnew;
        F[a] = P.alpha * fnew + (1.0f - P.alpha) * drag_old[a * np + q];
        drag_old[a * np + q] = F[a];
      }
      float nv[3], np3[3] = {x, y, z};
      float Fi[3];
      const bool impact = P.pour && pour_impact(P.pour, x, y, z, Fi);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        float acc = impact ? (F[a] + (mp - mf) * gv[a] + Fi[a]) / mp : (F[a] + (mp - mf) * gv[a]) / mp;
        nv[a] = v0[a] + acc * P.dt;
        np3[a] = np3[a] + nv[a] * P.dt;
      }
      bool hit = false;
      if (np3[2] < P.zlo) {
        np3[2] = P.zlo;
        hit = true;
      }
      if (np3[2] > P.zhi) {
        np3[2] = P.zhi;
        hit = true;
      }
      float rc = (np3[2] - P.apex) * P.tanth;
      float dx = np3[0] - P.cxf, dy = np3[1] - P.cyf;
      float r = sqrtf(dx * dx + dy * dy);
      if (r > P.margin * rc) {
        float s = r > 0.0f ? (P.pullback * rc) / r : 0.0f;
        np3[0] = P.cxf + dx * s;
        np3[1] = P.cyf + dy * s;
        hit = true;
      }
      if (hit) {
#pragma unroll
        for (int a = 0; a < 3; ++a) nv[a] = nv[a] * P.damping;
      }
      bool fin = true;
#pragma unroll
      for (int a = 0; a < 3; ++a) fin = fin && isfinite(np3[a]) && isfinite(nv[a]);
      if (!fin) {
        active[q] = 0;
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          pos[a * np + q] = np3[a];
          vel[a * np + q] = nv[a];
        }
        if (P.reaction == POG_REACTION_IMPLICIT) {
          dep[0] = beta;
#pragma unroll
          for (int a = 0; a < 3; ++a) dep[1 + a] = beta * nv[a];
        } else {
          // Newton's third law as an explicit body force (Kp stays 0)
#pragma unroll
          for (int a = 0; a < 3; ++a) dep[1 + a] = -(P.reaction == POG_REACTION_EXPLICIT ? F[a] : Fn[a]);
        }
        dep_ok = true;
      }
    }
    if (P.dep_cells && q >= 0) P.dep_cells[q] = dep_ok ? (int32_t)c0 : -1;
    if (P.dmask) {
      // the x-neighbour corners (c, c + 1) mostly share a 32-cell mask word: one OR for both,
      // aggregated over runs of lanes (cell-sorted neighbours) that hit the same word
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const uint32_t a = nodes[cc], b = a + 1u;
        const uint32_t wa = a >> 5, wb = b >> 5;
        warp_aggregated_or(P.dmask, wa, dep_ok, (1u << (a & 31u)) | (wa == wb ? (1u << (b & 31u)) : 0u));
        warp_aggregated_or(P.dmask, wb, dep_ok && wa != wb, 1u << (b & 31u));
      }
    }
    // Deposit the drag coefficient and its momentum weight (Kp += w beta, Kv += w beta v_new)
    // with the gather weights at the pre-update position; the lattice step applies the
    // particle force on the fluid, Kv - Kp u, implicitly in u.
    if (P.deterministic) {
#pragma unroll
      for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
          const float contrib = w[cc] * dep[a];
          if (dep_ok) {
            long long fixv = __double2ll_rn((double)contrib * FIX_SCALE);
            atomicAdd(pdrag_fix + (size_t)a * n + nodes[cc], (unsigned long long)fixv);
          }
        }
      }
    } else {
#pragma unroll
      for (int cc = 0; cc < 8; ++cc)
        warp_aggregated_add4(pdrag, n, nodes[cc], dep_ok, w[cc] * dep[0], w[cc] * dep[1], w[cc] * dep[2],
                             w[cc] * dep[3]);
    }
  }
}

// Zero the 8 deposit cells of each particle in all 4 components (several particles may share a
// cell: every write is the same zero).
__global__ void clear_deposit_kernel(uint32_t n, uint32_t sy, uint32_t sz, const int32_t* __restrict__ dep,
                                     const int32_t* __restrict__ order, int np, float* __restrict__ pdrag,
                                     uint32_t* __restrict__ dmask) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  // once the deposit is gone no cell holds one: the whole mask (n / 32 words) is cleared here too,
  // cheaper than clearing its bits one atomic at a time and without a separate memset
  if (dmask) {
    const uint32_t words = (n + 31u) / 32u;
    for (uint32_t w = (uint32_t)t; w < words; w += gridDim.x * blockDim.x) dmask[w] = 0u;
  }
  if (t >= np) return;
  // in cell order (the coupling pass's order) neighbouring threads zero neighbouring cells
  const int32_t c = dep[order ? order[t] : t];
  if (c < 0) return;
  const uint32_t c0 = (uint32_t)c;
  const uint32_t nodes[8] = {c0, c0 + sz, c0 + sy, c0 + sy + sz, c0 + 1, c0 + 1 + sz, c0 + 1 + sy, c0 + 1 + sy + sz};
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) pdrag[(size_t)a * n + nodes[cc]] = 0.0f;
}

// The deterministic deposit converted at the particles' cells only: each particle with a deposit
// takes the 4 fixed-point entries of its 8 corner cells, each by an atomic exchange with 0, so an
// entry shared by several particles is converted once (by whichever takes it first) and the
// fixed-point field is all zeros afterwards; the value added to pdrag is the one
// fixed_to_float_kernel computes.
__global__ void fixed_to_float_cells_kernel(uint32_t n, uint32_t sy, uint32_t sz, const int32_t* __restrict__ dep,
                                            const int32_t* __restrict__ order, int np,
                                            unsigned long long* __restrict__ fix, float* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const int32_t c = dep[order ? order[t] : t];
  if (c < 0) return;
  const uint32_t c0 = (uint32_t)c;
  const uint32_t nodes[8] = {c0, c0 + sz, c0 + sy, c0 + sy + sz, c0 + 1, c0 + 1 + sz, c0 + 1 + sy, c0 + 1 + sy + sz};
  const double inv = 1.0 / FIX_SCALE;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) {
      const size_t i = (size_t)a * n + nodes[cc];
      const unsigned long long v = atomicExch(fix + i, 0ull);
      if (v != 0ull) out[i] += (float)((double)(long long)v * inv);
    }
}

__global__ void fixed_to_float_kernel(uint32_t n3, const long long* __restrict__ fix,
                                      float* __restrict__ out) {
  const double inv = 1.0 / FIX_SCALE;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n3; c += gridDim.x * blockDim.x)
    out[c] = (float)((double)fix[c] * inv);
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct SortLayout {
  size_t k0, k1, v0, v1, hist, sums, total;
  int ntiles;
  uint32_t m, nchunks;
};
static SortLayout sort_layout(int np) {
  SortLayout L;
  L.ntiles = (np + SORT_TILE - 1) / SORT_TILE;
  L.m = (uint32_t)L.ntiles * RADIX;
  L.nchunks = (L.m + SCAN_CHUNK - 1) / SCAN_CHUNK;
  size_t a = align256((size_t)np * 4);
  L.k0 = 0;
  L.k1 = L.k0 + a;
  L.v0 = L.k1 + a;
  L.v1 = L.v0 + a;
  L.hist = L.v1 + a;
  L.sums = L.hist + align256((size_t)L.m * 4);
  L.total = L.sums + align256((size_t)L.nchunks * 4);
  return L;
}

}  // namespace pog

using namespace pog;

extern "C" {

size_t pog_particles_bin_scratch_bytes(int np) {
  if (np <= 0) return 256;
  return sort_layout(np).total;
}

int pog_particles_bin(const pog_params* p, const float* pos, const int32_t* active, int np,
                      int32_t* keys, int32_t* perm, void* scratch, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (np < 0) return set_error(POG_E_ARG, "np=%d < 0", np);
  if (np == 0) return POG_OK;
  if (np > MAX_SORT_NP) return set_error(POG_E_RANGE, "np=%d exceeds the sort limit %d", np, MAX_SORT_NP);
  if (!pos || !active || !keys) return set_error(POG_E_ARG, "pos/active/keys is NULL");
  if (perm && !scratch) return set_error(POG_E_ARG, "sorting needs scratch");
  cudaStream_t s = (cudaStream_t)stream;
  int grid = (np + 255) / 256;
  if (grid > 152 * 32) grid = 152 * 32;
  bin_kernel<<<grid, 256, 0, s>>>(p->nx, p->ny, p->nz, pos, active, np, keys);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  if (!perm) return POG_OK;
  SortLayout L = sort_layout(np);
  if (L.nchunks > (uint32_t)SCAN_CHUNK) return set_error(POG_E_RANGE, "too many sort tiles");
  char* base = (char*)scratch;
  uint32_t* K[2] = {(uint32_t*)(base + L.k0), (uint32_t*)(base + L.k1)};
  int32_t* V[2] = {(int32_t*)(base + L.v0), (int32_t*)(base + L.v1)};
  uint32_t* hist = (uint32_t*)(base + L.hist);
  uint32_t* sums = (uint32_t*)(base + L.sums);
  // keys are <= ncell: sort only the bits that can be set
  uint64_t maxkey = (uint64_t)p->nx * p->ny * p->nz;
  int bits = 1;
  while ((1ull << bits) <= maxkey) ++bits;
  const int passes = (bits + 7) / 8;
  const uint32_t* kin = (const uint32_t*)keys;
  const int32_t* vin = nullptr;
  for (int ps = 0; ps < passes; ++ps) {
    const int shift = 8 * ps;
    uint32_t* kout = K[ps & 1];
    int32_t* vout = ps == passes - 1 ? perm : V[ps & 1];
    radix_hist_kernel<<<L.ntiles, SORT_TILE, 0, s>>>(kin, np, shift, L.ntiles, hist);
    scan_reduce_kernel<<<L.nchunks, SCAN_BLOCK, 0, s>>>(hist, L.m, sums);
    scan_sums_kernel<<<1, SCAN_BLOCK, 0, s>>>(sums, L.nchunks);
    scan_down_kernel<<<L.nchunks, SCAN_BLOCK, 0, s>>>(hist, L.m, sums);
    radix_scatter_kernel<<<L.ntiles, SORT_TILE, 0, s>>>(kin, vin, np, shift, L.ntiles, hist, kout, vout);
    count_launch(5);
    POG_TRY_CUDA(cudaGetLastError());
    kin = kout;
    vin = vout;
  }
  return POG_OK;
}

int pog_particles_couple(const pog_params* p, const pog_particle_params* pp, float* pos, float* vel,
                         const float* diameter, float* drag_old, int32_t* active, int np,
                         const int32_t* order, const float* u, float* pdrag, long long* pdrag_fix,
                         float* u_at_particle, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!pp) return set_error(POG_E_ARG, "particle params NULL");
  if (np < 0) return set_error(POG_E_ARG, "np < 0");
  if (np == 0) return POG_OK;
  if (!pos || !vel || !diameter || !drag_old || !active || !u)
    return set_error(POG_E_ARG, "a particle array or u is NULL");
  if (pp->deterministic ? !pdrag_fix : !pdrag)
    return set_error(POG_E_ARG, "drag accumulator for the selected mode is NULL");
  if (pp->reaction < POG_REACTION_IMPLICIT || pp->reaction > POG_REACTION_EXPLICIT_NEW)
    return set_error(POG_E_ARG, "reaction %d unknown", pp->reaction);
  PKParams P;
  P.nx = p->nx;
  P.ny = p->ny;
  P.nz = p->nz;
  P.n = (uint32_t)p->nx * p->ny * p->nz;
  P.cxf = (float)(p->center_x < 0 ? 0.5 * p->nx : (double)p->center_x);
  P.cyf = (float)(p->center_y < 0 ? 0.5 * p->ny : (double)p->center_y);
  P.tanth = (float)tan((double)p->cone_half_angle_deg * M_PI / 180.0);
  P.apex = p->cone_apex_z;
  P.rho0 = p->rho0;
  float nu0 = (p->tau - 0.5f) / 3.0f;
  P.mu = p->rho0 * nu0;
  P.rho_p = pp->density_ratio * p->rho0;
  P.alpha = pp->relaxation;
  P.dt = pp->dt;
  P.gx = p->gx;
  P.gy = p->gy;
  P.gz = p->gz;
  P.zlo = p->cone_apex_z + pp->z_floor;
  P.zhi = (float)(p->nz - 3);
  P.margin = pp->wall_margin;
  P.pullback = pp->wall_pullback;
  P.damping = pp->wall_damping;
  P.drag_model = pp->drag_model;
  P.deterministic = pp->deterministic;
  P.reaction = pp->reaction;
  P.pour = p->pour_control;
  P.dep_cells = pp->deposit_cells;
  P.dmask = pp->deposit_mask;
  cudaStream_t s = (cudaStream_t)stream;
  // 64-thread blocks spread a small particle count over every SM (20,000 particles: 313 blocks
  // instead of 79; 20.0 -> 17.5 us per pass); the grid is capped at 4,096 threads per SM
  const int block = 64;
  const long long want = ((long long)np + block - 1) / block, cap = 152LL * 4096 / block;
  const int grid = (int)(want < cap ? want : cap);
  couple_kernel<<<grid, block, 0, s>>>(P, pos, vel, diameter, drag_old, active, np, order, u, pdrag,
                                       (unsigned long long*)pdrag_fix, u_at_particle);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_particles_clear_deposit(const pog_params* p, const int32_t* deposit_cells, int np, const int32_t* order,
                                float* pdrag, uint32_t* deposit_mask, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (np < 0) return set_error(POG_E_ARG, "np=%d", np);
  if (np == 0) return POG_OK;
  if (!deposit_cells || !pdrag) return set_error(POG_E_ARG, "NULL pointer");
  const uint32_t sy = (uint32_t)p->nx, sz = (uint32_t)p->nx * (uint32_t)p->ny;
  // a thread per particle, and at least one per 4 mask words (n / 32 words)
  const long long words = ((long long)sz * p->nz + 31) / 32;
  const long long pblocks = ((long long)np + 255) / 256;
  const long long mblocks = deposit_mask ? (words + 1023) / 1024 : 0;
  const long long want = pblocks > mblocks ? pblocks : mblocks;
  clear_deposit_kernel<<<(int)want, 256, 0, (cudaStream_t)stream>>>(sz * (uint32_t)p->nz, sy, sz, deposit_cells,
                                                                   order, np, pdrag, deposit_mask);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_drag_from_fixed_cells(const pog_params* p, long long* pdrag_fix, const int32_t* deposit_cells, int np,
                              const int32_t* order, float* pdrag, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (np < 0) return set_error(POG_E_ARG, "np=%d", np);
  if (np == 0) return POG_OK;
  if (!pdrag_fix || !deposit_cells || !pdrag) return set_error(POG_E_ARG, "NULL pointer");
  const uint32_t sy = (uint32_t)p->nx, sz = (uint32_t)p->nx * (uint32_t)p->ny;
  fixed_to_float_cells_kernel<<<(np + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      sz * (uint32_t)p->nz, sy, sz, deposit_cells, order, np, (unsigned long long*)pdrag_fix, pdrag);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_drag_from_fixed(const pog_params* p, const long long* pdrag_fix, float* pdrag, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!pdrag_fix || !pdrag) return set_error(POG_E_ARG, "NULL pointer");
  uint32_t n3 = 4u * (uint32_t)p->nx * p->ny * p->nz;
  int grid = (int)((n3 + 255) / 256);
  if (grid > 152 * 32) grid = 152 * 32;
  fixed_to_float_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(n3, pdrag_fix, pdrag);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

}  // extern "C"
