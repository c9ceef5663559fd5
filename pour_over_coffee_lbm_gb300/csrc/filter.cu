// filter.cu -- filter-paper dynamics (FilterPaperSystem, src/physics/filter_paper.py:616-750):
// particles meeting the paper bounce and accumulate on it, and the accumulation raises the
// band's flow resistance (the blockage field the step kernel reads).  The reference's
// ti.random() roughness kicks come from a counter-based hash here, so runs repeat exactly.
#include "common.cuh"

namespace pog {

// lowbias32 integer hash (C. Wellons, "Prospecting for Hash Functions", 2018).
__host__ __device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
// uniform in [0, 1) with 24 random bits
__host__ __device__ __forceinline__ float hash_uniform(uint32_t seed, uint32_t step, uint32_t id, uint32_t lane) {
  const uint32_t h = lowbias32(seed ^ lowbias32(step ^ lowbias32(id * 2u + lane)));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

__global__ void filter_particles_kernel(uint32_t nx, uint32_t ny, uint32_t nz, const uint32_t* __restrict__ flags,
                                        const float* __restrict__ pos, float* __restrict__ vel,
                                        const int32_t* __restrict__ active, int np, float* __restrict__ accum,
                                        uint32_t seed, uint32_t step) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= np || !active[q]) return;
  const float x = pos[q], y = pos[np + q], z = pos[2 * np + q];
  // int() truncation of the reference; only cells inside the grid
  if (!(x >= 0.0f && y >= 0.0f && z >= 0.0f)) return;
  const uint32_t i = (uint32_t)x, j = (uint32_t)y, k = (uint32_t)z;
  if (i >= nx || j >= ny || k >= nz) return;
  for (int o = -2; o <= 2; ++o) {
    const int kk = (int)k + o;
    if (kk < 0 || kk >= (int)nz) continue;
    const uint32_t c = ((uint32_t)kk * ny + j) * nx + i;
    if (!(flags[c] & POG_CELL_POROUS)) continue;
    const float vz = vel[2 * np + q];
    if (vz < 0.0f) {
      vel[2 * np + q] = -vz * 0.3f;  // restitution 0.3 (:676)
      vel[q] = vel[q] + (hash_uniform(seed, step, (uint32_t)q, 0u) - 0.5f) * 0.01f;
      vel[np + q] = vel[np + q] + (hash_uniform(seed, step, (uint32_t)q, 1u) - 0.5f) * 0.01f;
      atomicAdd(accum + c, 0.01f);
    }
    break;
  }
}

__global__ void filter_update_kernel(uint32_t n, const uint32_t* __restrict__ flags, float* __restrict__ accum,
                                     float* __restrict__ blockage) {
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    if (!(flags[c] & POG_CELL_POROUS)) continue;
    const float a = accum[c];
    const float nb = 0.9f * (1.0f - expf(-0.1f * a));
    blockage[c] = 0.95f * blockage[c] + 0.05f * nb;
    accum[c] = a * 0.999f;
  }
}

}  // namespace pog

using namespace pog;

extern "C" {

int pog_filter_particles(const pog_params* p, const uint32_t* flags, const float* pos, float* vel,
                         const int32_t* active, int np, float* accum, uint32_t seed, long long step, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (np < 0) return set_error(POG_E_ARG, "np=%d", np);
  if (np == 0) return POG_OK;
  if (!flags || !pos || !vel || !active || !accum) return set_error(POG_E_ARG, "NULL pointer");
  filter_particles_kernel<<<(np + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      (uint32_t)p->nx, (uint32_t)p->ny, (uint32_t)p->nz, flags, pos, vel, active, np, accum, seed, (uint32_t)step);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_filter_update(const pog_params* p, const uint32_t* flags, float* accum, float* blockage, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!flags || !accum || !blockage) return set_error(POG_E_ARG, "NULL pointer");
  const uint32_t n = (uint32_t)p->nx * p->ny * p->nz;
  long long want = ((long long)n + 255) / 256;
  filter_update_kernel<<<(int)(want < 152 * 16 ? want : 152 * 16), 256, 0, (cudaStream_t)stream>>>(n, flags, accum,
                                                                                                  blockage);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

}  // extern "C"
