// multiphase.cu -- the Cahn-Hilliard phase field of MultiphaseFlow3D (src/core/multiphase_3d.py)
// and the pour stream's phase change (PrecisePouringSystem.apply_gradual_phase_change,
// src/physics/precise_pouring.py:166-193).
//
// phi in [-1, 1] (-1 air, +1 water) lives in two [NZ][NY][NX] float buffers used in turn.  The
// stencil passes touch interior cells only (1 <= i < NX-1, ...), as the reference's ndrange
// loops do; the outer shell of the normal field stays zero.  Everything is float32 and compiled
// without contraction, so the CPU restatement reproduces it bit for bit.
#include "common.cuh"

namespace pog {

struct PhaseGrid {
  uint32_t nx, ny, nz, plane, n;
};

static PhaseGrid phase_grid(const pog_params* p) {
  PhaseGrid g;
  g.nx = (uint32_t)p->nx;
  g.ny = (uint32_t)p->ny;
  g.nz = (uint32_t)p->nz;
  g.plane = g.nx * g.ny;
  g.n = g.plane * g.nz;
  return g;
}

// One thread per cell on a (x, y, z) grid of PHASE_BX x PHASE_BY blocks, one plane per grid z:
// the cell indices come without divisions and a warp covers 32 consecutive x.
constexpr int PHASE_BX = 64, PHASE_BY = 4;

struct PhaseCell {
  uint32_t i, j, k, c;
  bool valid, interior;
};

__device__ __forceinline__ PhaseCell phase_cell(const PhaseGrid& g) {
  PhaseCell p;
  p.i = blockIdx.x * PHASE_BX + threadIdx.x;
  p.j = blockIdx.y * PHASE_BY + threadIdx.y;
  p.k = blockIdx.z;
  p.valid = p.i < g.nx && p.j < g.ny;
  p.c = (p.k * g.ny + p.j) * g.nx + p.i;
  p.interior = p.valid && p.i >= 1 && p.i + 1 < g.nx && p.j >= 1 && p.j + 1 < g.ny && p.k >= 1 && p.k + 1 < g.nz;
  return p;
}

// 6-neighbour sum minus 6 x centre, in the reference's order (x+, x-, y+, y-, z+, z-)
__device__ __forceinline__ float lap7(const float* __restrict__ a, const PhaseGrid& g, uint32_t c) {
  return a[c + 1] + a[c - 1] + a[c + g.nx] + a[c - g.nx] + a[c + g.plane] + a[c - g.plane] - 6.0f * a[c];
}

// compute_chemical_potential (:80-109): mu = phi^3 - phi - kappa lap(phi)
__global__ void phase_mu_kernel(PhaseGrid g, const float* __restrict__ phi, float kappa, float* __restrict__ mu) {
  const PhaseCell pc_ = phase_cell(g);
  if (!pc_.interior) return;
  const uint32_t c = pc_.c;
  const float p = phi[c];
  const float lap = lap7(phi, g, c);
  mu[c] = (p * p * p - p) + (-kappa * lap);
}

// compute_gradients (:111-132): grad phi by central differences, unit normal where |grad| > 1e-10
__global__ void phase_normals_kernel(PhaseGrid g, const float* __restrict__ phi, float* __restrict__ normal,
                                     float* __restrict__ gmag) {
  const PhaseCell pc_ = phase_cell(g);
  if (!pc_.interior) return;
  const uint32_t c = pc_.c;
  const float gx = (phi[c + 1] - phi[c - 1]) * 0.5f;
  const float gy = (phi[c + g.nx] - phi[c - g.nx]) * 0.5f;
  const float gz = (phi[c + g.plane] - phi[c - g.plane]) * 0.5f;
  const float m = sqrtf(gx * gx + gy * gy + gz * gz);
  float nx = 0.0f, ny = 0.0f, nz = 0.0f;
  if (m > 1e-10f) {
    nx = gx / m;
    ny = gy / m;
    nz = gz / m;
  }
  normal[c] = nx;
  normal[g.n + c] = ny;
  normal[2 * g.n + c] = nz;
  gmag[c] = m;
}

// compute_curvature (:134-149), compute_surface_tension_force (:313-331) and
// apply_surface_tension (:354-363): kappa = div n, F = sigma kappa |grad phi| n where |phi| < 0.9,
// body_force += F / rho on non-solid cells with rho > 1e-10.  The normal is nonzero exactly
// where |grad phi| > 1e-10, so that test stands for the reference's |n| > 1e-10.  Cells where F
// is zero (the bulk of either phase) read |grad phi| only and leave the body force alone (the
// reference adds 0 / rho there).
__global__ void phase_tension_kernel(PhaseGrid g, const uint32_t* __restrict__ flags, const float* __restrict__ phi,
                                     const float* __restrict__ normal, const float* __restrict__ gmag,
                                     const float* __restrict__ rho, float sigma, float* __restrict__ body_force,
                                     float* __restrict__ curvature, float* __restrict__ sforce) {
  const PhaseCell pc_ = phase_cell(g);
  if (!pc_.interior) return;
  const uint32_t c = pc_.c;
  const float m = gmag[c];
  float kap = 0.0f, fx = 0.0f, fy = 0.0f, fz = 0.0f;
  bool on = false;
  if (m > 1e-10f) {
    on = fabsf(phi[c]) < 0.9f;
    if (on || curvature) {
      const float* nx = normal;
      const float* ny = normal + g.n;
      const float* nz = normal + 2 * g.n;
      kap = (nx[c + 1] - nx[c - 1]) * 0.5f + (ny[c + g.nx] - ny[c - g.nx]) * 0.5f +
            (nz[c + g.plane] - nz[c - g.plane]) * 0.5f;
    }
    if (on) {
      const float fm = sigma * kap * m;
      fx = fm * normal[c];
      fy = fm * normal[g.n + c];
      fz = fm * normal[2 * g.n + c];
    }
  }
  if (curvature) curvature[c] = kap;
  if (sforce) {
    sforce[c] = fx;
    sforce[g.n + c] = fy;
    sforce[2 * g.n + c] = fz;
  }
  if (on && body_force && !(flags[c] & POG_CELL_SOLID)) {
    const float r = rho[c];
    if (r > 1e-10f) {
      body_force[c] += fx / r;
      body_force[g.n + c] += fy / r;
      body_force[2 * g.n + c] += fz / r;
    }
  }
}

// update_phase_field_cahn_hilliard (:151-197) + apply_phase_separation (:334-352) +
// update_density_from_phase (:365-381) in one pass.  Interior cells: first-order upwind
// advection by the fluid velocity (zero in solid cells), M lap(mu) (mu NULL = 0), clamp, then
// the phase-separation relaxation where |phi| < 0.99.  Other cells carry phi over.  rho and the
// phase indicator (phi + 1)/2 follow from the clamped new phi, for every cell.
__global__ void phase_update_kernel(PhaseGrid g, const uint32_t* __restrict__ flags, const float* __restrict__ phi,
                                    float* __restrict__ phi_new, const float* __restrict__ u,
                                    const float* __restrict__ mu, float mobility, float dt, float rho_air,
                                    float drho, float* __restrict__ rho_out, float* __restrict__ phase_out) {
  const PhaseCell pc_ = phase_cell(g);
  if (!pc_.valid) return;
  const uint32_t c = pc_.c;
  const float p = phi[c];
  float pn = p;
  if (pc_.interior) {
    float ux = 0.0f, uy = 0.0f, uz = 0.0f;
    if (!(flags[c] & POG_CELL_SOLID)) {
      ux = u[c];
      uy = u[g.n + c];
      uz = u[2 * g.n + c];
    }
    const float dx = ux > 0.0f ? p - phi[c - 1] : phi[c + 1] - p;
    const float dy = uy > 0.0f ? p - phi[c - g.nx] : phi[c + g.nx] - p;
    const float dz = uz > 0.0f ? p - phi[c - g.plane] : phi[c + g.plane] - p;
    const float conv = -(ux * dx + uy * dy + uz * dz);
    float diff = 0.0f;
    if (mu) diff = mobility * lap7(mu, g, c);
    pn = p + dt * (conv + diff);
    pn = fmaxf(-1.0f, fminf(1.0f, pn));
    if (fabsf(p) < 0.99f) {
      const float lap = lap7(phi, g, c);
      const float chem = p * (p * p - 1.0f) - 0.01f * lap;
      pn = pn + -0.001f * chem * dt;
    }
  }
  phi_new[c] = pn;
  if (rho_out) {
    const float pc = fmaxf(-1.0f, fminf(1.0f, pn));
    rho_out[c] = rho_air + drho * (pc + 1.0f) / 2.0f;
    phase_out[c] = (pc + 1.0f) / 2.0f;
  }
}

// update_density_from_phase (:365-381) alone
__global__ void phase_properties_kernel(PhaseGrid g, const float* __restrict__ phi, float rho_air, float drho,
                                        float* __restrict__ rho_out, float* __restrict__ phase_out) {
  const PhaseCell pc_ = phase_cell(g);
  if (!pc_.valid) return;
  const uint32_t c = pc_.c;
  const float pc = fmaxf(-1.0f, fminf(1.0f, phi[c]));
  rho_out[c] = rho_air + drho * (pc + 1.0f) / 2.0f;
  phase_out[c] = (pc + 1.0f) / 2.0f;
}

// apply_gradual_phase_change (precise_pouring.py:166-193): non-solid cells of the stream move
// toward water, d phi = clamp((1 - phi) / 0.05, +-2) * I * dt * flow, I the stream intensity
// of pour_accel.  Only the stream's planes are visited.
__global__ void pour_phase_kernel(PhaseGrid g, const float* __restrict__ b, const uint32_t* __restrict__ flags,
                                  float* __restrict__ phi, float dt) {
  if (b[POG_POUR_ACTIVE] == 0.0f) return;
  const float ztop = b[POG_POUR_ZTOP];
  const float klo = ceilf(ztop - b[POG_POUR_HEIGHT]), khi = floorf(ztop);
  if (!(khi >= 0.0f) || klo > (float)(g.nz - 1) || khi < klo) return;
  const uint32_t c0 = (uint32_t)fmaxf(klo, 0.0f) * g.plane;
  const uint32_t c1 = ((uint32_t)fminf(khi, (float)(g.nz - 1)) + 1u) * g.plane;
  const float R = b[POG_POUR_RADIUS], px = b[POG_POUR_X], py = b[POG_POUR_Y], flow = b[POG_POUR_FLOW];
  for (uint32_t c = c0 + blockIdx.x * blockDim.x + threadIdx.x; c < c1; c += gridDim.x * blockDim.x) {
    if (flags[c] & POG_CELL_SOLID) continue;
    const uint32_t k = c / g.plane, rem = c - k * g.plane, j = rem / g.nx, i = rem - j * g.nx;
    const float dx = (float)i - px, dy = (float)j - py;
    const float d = sqrtf(dx * dx + dy * dy);
    if (!(d <= R)) continue;
    const float dr = d / R;
    const float I = expf(-0.5f * dr * dr) * expf(-(ztop - (float)k) / 2.0f);
    if (!(I > 0.0f)) continue;
    const float cur = phi[c];
    float rate = (1.0f - cur) / 0.05f;
    rate = fmaxf(-2.0f, fminf(2.0f, rate));
    const float nw = cur + rate * I * dt * flow;
    phi[c] = fmaxf(-1.0f, fminf(1.0f, nw));
  }
}

static int phase_blocks(uint32_t n) {
  const long long want = ((long long)n + 255) / 256;
  return (int)(want < 152 * 16 ? want : 152 * 16);
}
static dim3 phase_grid3(const PhaseGrid& g) {
  return dim3((g.nx + PHASE_BX - 1) / PHASE_BX, (g.ny + PHASE_BY - 1) / PHASE_BY, g.nz);
}
static const dim3 kPhaseBlock(PHASE_BX, PHASE_BY, 1);

}  // namespace pog

using namespace pog;

extern "C" {

int pog_phase_chemical_potential(const pog_params* p, const float* phi, float kappa, float* mu, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!phi || !mu) return set_error(POG_E_ARG, "NULL pointer");
  const PhaseGrid g = phase_grid(p);
  phase_mu_kernel<<<phase_grid3(g), kPhaseBlock, 0, (cudaStream_t)stream>>>(g, phi, kappa, mu);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_phase_normals(const pog_params* p, const float* phi, float* normal, float* gmag, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!phi || !normal || !gmag) return set_error(POG_E_ARG, "NULL pointer");
  const PhaseGrid g = phase_grid(p);
  phase_normals_kernel<<<phase_grid3(g), kPhaseBlock, 0, (cudaStream_t)stream>>>(g, phi, normal, gmag);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_phase_surface_tension(const pog_params* p, const uint32_t* flags, const float* phi, const float* normal,
                              const float* gmag, const float* rho, float sigma, float* body_force,
                              float* curvature, float* surface_force, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!flags || !phi || !normal || !gmag) return set_error(POG_E_ARG, "NULL pointer");
  if (body_force && !rho) return set_error(POG_E_ARG, "body_force needs rho");
  const PhaseGrid g = phase_grid(p);
  phase_tension_kernel<<<phase_grid3(g), kPhaseBlock, 0, (cudaStream_t)stream>>>(g, flags, phi, normal, gmag, rho, sigma,
                                                                            body_force, curvature, surface_force);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_phase_update(const pog_params* p, const uint32_t* flags, const float* phi, float* phi_new, const float* u,
                     const float* mu, float mobility, float dt, float rho_air, float rho_water, float* rho,
                     float* phase, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!flags || !phi || !phi_new || !u) return set_error(POG_E_ARG, "NULL pointer");
  if (phi == phi_new) return set_error(POG_E_ARG, "phi and phi_new must differ");
  if (!rho != !phase) return set_error(POG_E_ARG, "rho and phase go together");
  const PhaseGrid g = phase_grid(p);
  phase_update_kernel<<<phase_grid3(g), kPhaseBlock, 0, (cudaStream_t)stream>>>(
      g, flags, phi, phi_new, u, mu, mobility, dt, rho_air, (float)((double)rho_water - (double)rho_air), rho, phase);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_phase_properties(const pog_params* p, const float* phi, float rho_air, float rho_water, float* rho,
                         float* phase, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!phi || !rho || !phase) return set_error(POG_E_ARG, "NULL pointer");
  const PhaseGrid g = phase_grid(p);
  phase_properties_kernel<<<phase_grid3(g), kPhaseBlock, 0, (cudaStream_t)stream>>>(
      g, phi, rho_air, (float)((double)rho_water - (double)rho_air), rho, phase);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_pour_phase(const pog_params* p, const uint32_t* flags, float* phi, float dt, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!p->pour_control) return set_error(POG_E_ARG, "pour_control is NULL");
  if (!flags || !phi) return set_error(POG_E_ARG, "NULL pointer");
  const PhaseGrid g = phase_grid(p);
  pour_phase_kernel<<<phase_blocks(g.plane * 8u), 256, 0, (cudaStream_t)stream>>>(g, p->pour_control, flags, phi,
                                                                                  dt);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

}  // extern "C"
