// drive.cu -- pressure-gradient drive (PressureGradientDrive, src/physics/pressure_gradient_drive.py):
// the force drive adds F = -c_s^2 grad(rho) / rho, capped at |F| <= max_force, to the explicit
// force field the step reads (compute_pressure_gradient :124-177 + the accumulation :188-193 /
// :274-279), and the density drive relaxes rho toward a per-plane target (apply_density_drive
// :95-122).  Both are plain stencil passes over [NZ][NY][NX] fields, HBM-bound.
#include "common.cuh"

namespace pog {

__global__ void pressure_force_kernel(uint32_t nx, uint32_t ny, uint32_t nz, const uint32_t* __restrict__ flags,
                                      const float* __restrict__ rho, float* __restrict__ force, float scale,
                                      float max_force) {
  const uint32_t n = nx * ny * nz;
  const uint32_t plane = nx * ny;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    if (flags[c] & POG_CELL_SOLID) continue;
    const uint32_t i = c % nx, j = (c / nx) % ny, k = c / plane;
    const float r = rho[c];
    // central differences inside, one-sided on the domain faces (:137-160)
    float gx, gy, gz;
    if (i > 0 && i < nx - 1) gx = (rho[c + 1] - rho[c - 1]) * 0.5f;
    else if (i == 0) gx = rho[c + 1] - r;
    else gx = r - rho[c - 1];
    if (j > 0 && j < ny - 1) gy = (rho[c + nx] - rho[c - nx]) * 0.5f;
    else if (j == 0) gy = rho[c + nx] - r;
    else gy = r - rho[c - nx];
    if (k > 0 && k < nz - 1) gz = (rho[c + plane] - rho[c - plane]) * 0.5f;
    else if (k == 0) gz = rho[c + plane] - r;
    else gz = r - rho[c - plane];
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    if (r > 1e-12f) {
      const float cs2 = 1.0f / 3.0f;
      fx = -(gx * cs2) / r;
      fy = -(gy * cs2) / r;
      fz = -(gz * cs2) / r;
      const float m = sqrtf(fx * fx + fy * fy + fz * fz);
      if (m > max_force) {
        const float s = max_force / m;
        fx *= s;
        fy *= s;
        fz *= s;
      }
    }
    force[c] += scale * fx;
    force[n + c] += scale * fy;
    force[2 * n + c] += scale * fz;
  }
}

__global__ void density_drive_kernel(uint32_t nx, uint32_t ny, uint32_t nz, const uint32_t* __restrict__ flags,
                                     float* __restrict__ rho, const float* __restrict__ target, float rate,
                                     float max_adjust, float lo, float hi) {
  const uint32_t n = nx * ny * nz;
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    if (flags[c] & POG_CELL_SOLID) continue;
    const float r = rho[c];
    float a = (target[c / (nx * ny)] - r) * rate;
    if (fabsf(a) > max_adjust) a = a > 0.0f ? max_adjust : -max_adjust;
    rho[c] = fmaxf(lo, fminf(hi, r + a));
  }
}

static int grid_for(uint32_t n) {
  const long long want = ((long long)n + 255) / 256;
  return (int)(want < 152 * 16 ? want : 152 * 16);
}

}  // namespace pog

using namespace pog;

extern "C" {

int pog_pressure_force(const pog_params* p, const uint32_t* flags, const float* rho, float* force, float scale,
                       float max_force, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!flags || !rho || !force) return set_error(POG_E_ARG, "NULL pointer");
  if (!(max_force >= 0.0f)) return set_error(POG_E_ARG, "max_force must be >= 0");
  const uint32_t n = (uint32_t)p->nx * p->ny * p->nz;
  pressure_force_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((uint32_t)p->nx, (uint32_t)p->ny,
                                                                       (uint32_t)p->nz, flags, rho, force, scale,
                                                                       max_force);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

int pog_density_drive(const pog_params* p, const uint32_t* flags, float* rho, const float* target, float rate,
                      float max_adjust, float rho_min, float rho_max, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!flags || !rho || !target) return set_error(POG_E_ARG, "NULL pointer");
  if (!(max_adjust >= 0.0f) || !(rho_min <= rho_max)) return set_error(POG_E_ARG, "bad drive limits");
  const uint32_t n = (uint32_t)p->nx * p->ny * p->nz;
  density_drive_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((uint32_t)p->nx, (uint32_t)p->ny,
                                                                      (uint32_t)p->nz, flags, rho, target, rate,
                                                                      max_adjust, rho_min, rho_max);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

}  // extern "C"
