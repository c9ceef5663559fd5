// geometry.cu -- V60 cell flags (replaces FilterPaperSystem._setup_v60_geometry and
// _setup_filter_zones, src/physics/filter_paper.py:206-364, and the LES-mask copy :199-204).
//
// Integer output computed in FP64; this translation unit is compiled with -fmad=false and
// tan() is evaluated on the host, so every cell decision is bit-identical with the CPU
// restatement.  Two passes: the solid mask, then inlet/outlet/porous/near-solid bits that
// need the neighbours' solidity.
#include <math.h>

#include "common.cuh"

namespace pog {

struct GeoParams {
  int nx, ny, nz;
  double cx, cy, tanth, apex, wall, hole, rin, band;
};

__device__ inline double radius_at(const GeoParams& g, int i, int j) {
  double dx = (double)i - g.cx, dy = (double)j - g.cy;
  return sqrt(dx * dx + dy * dy);
}

__global__ void solid_kernel(GeoParams g, uint32_t* flags) {
  long long n = (long long)g.nx * g.ny * g.nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    int i = (int)(c % g.nx);
    int j = (int)((c / g.nx) % g.ny);
    int k = (int)(c / ((long long)g.nx * g.ny));
    double r = radius_at(g, i, j);
    double z = (double)k;
    bool s = (i == 0 || j == 0 || k == 0 || i == g.nx - 1 || j == g.ny - 1 || k == g.nz - 1);
    double rc = (z - g.apex) * g.tanth;
    if (z < g.apex) {
      s = s || (r > g.hole);
    } else if (r > rc && r <= rc + g.wall && r > g.hole) {
      s = true;
    }
    flags[c] = s ? POG_CELL_SOLID : 0;
  }
}

__global__ void fluid_bits_kernel(GeoParams g, uint32_t* flags) {
  long long n = (long long)g.nx * g.ny * g.nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    if (flags[c] & POG_CELL_SOLID) continue;
    int i = (int)(c % g.nx);
    int j = (int)((c / g.nx) % g.ny);
    int k = (int)(c / ((long long)g.nx * g.ny));
    double r = radius_at(g, i, j);
    double z = (double)k;
    double rc = (z - g.apex) * g.tanth;
    uint32_t fl = 0;
    if (k == g.nz - 2 && r <= g.rin) fl |= POG_CELL_INLET;
    if (k == 1 && r <= g.hole) fl |= POG_CELL_OUTLET;
    if (!(fl & (POG_CELL_INLET | POG_CELL_OUTLET)) && g.band > 0 && z >= g.apex &&
        r > rc - g.band && r <= rc + g.wall)
      fl |= POG_CELL_POROUS;
    // Fluid cells are never on the outer shell, so every neighbour is in the grid.
    uint32_t links = 0;
#pragma unroll
    for (int q = 1; q < 19; ++q) {
      long long nb = c + cx(q) + (long long)cy(q) * g.nx + (long long)cz(q) * g.nx * g.ny;
      if (flags[nb] & POG_CELL_SOLID) links |= 1u << (POG_LINK_SHIFT + q);
    }
    if (links) fl |= POG_CELL_NEAR_SOLID | links;
    flags[c] = fl;
  }
}

}  // namespace pog

using namespace pog;

extern "C" int pog_build_flags(const pog_params* p, uint32_t* flags, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!flags) return set_error(POG_E_ARG, "flags is NULL");
  GeoParams g;
  g.nx = p->nx;
  g.ny = p->ny;
  g.nz = p->nz;
  g.cx = p->center_x < 0 ? 0.5 * p->nx : (double)p->center_x;
  g.cy = p->center_y < 0 ? 0.5 * p->ny : (double)p->center_y;
  g.tanth = tan((double)p->cone_half_angle_deg * M_PI / 180.0);  // host libm, as the oracle
  g.apex = p->cone_apex_z;
  g.wall = p->cone_wall;
  g.hole = p->hole_radius;
  g.rin = p->inlet_radius;
  g.band = p->band_thickness;
  cudaStream_t s = (cudaStream_t)stream;
  long long n = (long long)p->nx * p->ny * p->nz;
  int block = 256;
  long long want = (n + block - 1) / block;
  int grid = (int)(want < 65535 * 16 ? want : 65535 * 16);
  solid_kernel<<<grid, block, 0, s>>>(g, flags);
  POG_TRY_CUDA(cudaGetLastError());
  // fluid_bits reads only the solid bit of neighbours and writes only non-solid cells, so the
  // in-place second pass is race-free.
  fluid_bits_kernel<<<grid, block, 0, s>>>(g, flags);
  POG_TRY_CUDA(cudaGetLastError());
  count_launch(2);
  return POG_OK;
}
