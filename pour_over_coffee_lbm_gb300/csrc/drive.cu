// drive.cu -- pressure-gradient drive (PressureGradientDrive, src/physics/pressure_gradient_drive.py):
// the force drive adds F = -c_s^2 grad(rho) / rho, capped at |F| <= max_force, to the explicit
// force field the step reads (compute_pressure_gradient :124-177 + the accumulation :188-193 /
// :274-279), and the density drive relaxes rho toward a per-plane target (apply_density_drive
// :95-122).  Both are plain stencil passes over [NZ][NY][NX] fields, HBM-bound.
#include "common.cuh"

namespace pog {

constexpr int DRIVE_BX = 64, DRIVE_BY = 4;

__global__ void pressure_force_kernel(uint32_t nx, uint32_t ny, uint32_t nz, const uint32_t* __restrict__ flags,
                                      const float* __restrict__ rho, float* __restrict__ force, float scale,
                                      float max_force) {
  const uint32_t n = nx * ny * nz;
  const uint32_t plane = nx * ny;
  // one thread per cell, one plane per grid z: the indices come without divisions
  const uint32_t i = blockIdx.x * DRIVE_BX + threadIdx.x, j = blockIdx.y * DRIVE_BY + threadIdx.y, k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const uint32_t c = (k * ny + j) * nx + i;
  if (flags[c] & POG_CELL_SOLID) return;
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

__global__ void density_drive_kernel(uint32_t nx, uint32_t ny, uint32_t nz, const uint32_t* __restrict__ flags,
                                     float* __restrict__ rho, const float* __restrict__ target, float rate,
                                     float max_adjust, float lo, float hi) {
  const uint32_t i = blockIdx.x * DRIVE_BX + threadIdx.x, j = blockIdx.y * DRIVE_BY + threadIdx.y, k = blockIdx.z;
  if (i >= nx || j >= ny) return;
  const uint32_t c = (k * ny + j) * nx + i;
  if (flags[c] & POG_CELL_SOLID) return;
  const float r = rho[c];
  float a = (target[k] - r) * rate;
  if (fabsf(a) > max_adjust) a = a > 0.0f ? max_adjust : -max_adjust;
  rho[c] = fmaxf(lo, fminf(hi, r + a));
}

static dim3 grid_for(const pog_params* p) {
  return dim3((p->nx + DRIVE_BX - 1) / DRIVE_BX, (p->ny + DRIVE_BY - 1) / DRIVE_BY, p->nz);
}
static const dim3 kDriveBlock(DRIVE_BX, DRIVE_BY, 1);

}  // namespace pog

using namespace pog;

extern "C" {

int pog_pressure_force(const pog_params* p, const uint32_t* flags, const float* rho, float* force, float scale,
                       float max_force, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!flags || !rho || !force) return set_error(POG_E_ARG, "NULL pointer");
  if (!(max_force >= 0.0f)) return set_error(POG_E_ARG, "max_force must be >= 0");
  pressure_force_kernel<<<grid_for(p), kDriveBlock, 0, (cudaStream_t)stream>>>((uint32_t)p->nx, (uint32_t)p->ny,
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
  density_drive_kernel<<<grid_for(p), kDriveBlock, 0, (cudaStream_t)stream>>>((uint32_t)p->nx, (uint32_t)p->ny,
                                                                      (uint32_t)p->nz, flags, rho, target, rate,
                                                                      max_adjust, rho_min, rho_max);
  count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}

}  // extern "C"
