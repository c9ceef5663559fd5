// api.cu -- library-level entry points: version, errors, parameter checks, launch counting.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>

#include "common.cuh"

namespace pog {

static thread_local char g_err[512] = "";
static thread_local long long g_launches = 0;

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  return set_error(POG_E_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

void count_launch(int n) { g_launches += n; }

int persistent_blocks(const void* kernel, int block, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess)
    return 0;
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

KParams make_kparams(const pog_params* p) {
  KParams k;
  k.nx = (uint32_t)p->nx;
  k.ny = (uint32_t)p->ny;
  k.nz = (uint32_t)p->nz;
  k.nxny = k.nx * k.ny;
  k.n = k.nxny * k.nz;
  k.guard_lo = k.nxny + k.nx + 1;
  k.guard_hi = k.n - 1 - k.guard_lo;
  for (int q = 0; q < 19; ++q)
    k.off[q] = cx(q) + cy(q) * (int32_t)k.nx + cz(q) * (int32_t)k.nxny;
  for (int q = 0; q < 19; ++q) {
    k.pl[q] = (uint32_t)q * k.n;
    k.rd[q] = (uint32_t)opp(q) * k.n - (uint32_t)k.off[q];
    k.wr[q] = (uint32_t)q * k.n + (uint32_t)k.off[q];
  }
  k.les_mode = p->les_mode;
  k.drag_mode = p->drag_mode;
  k.forcing_mode = p->forcing_mode;
  k.clamp_tau = p->clamp_tau;
  k.storage = p->storage;
  k.tau = p->tau;
  k.rho0 = p->rho0;
  k.gx = p->gx;
  k.gy = p->gy;
  k.gz = p->gz;
  k.cs2 = p->cs_smag * p->cs_smag;
  k.strain_floor = p->les_strain_floor;
  k.nu_max = p->les_nu_max;
  k.tau_min = p->tau_min;
  k.tau_max = p->tau_max;
  k.nu0 = (p->tau - 0.5f) / 3.0f;
  k.K0 = p->permeability;
  k.CF0 = p->forchheimer;
  k.eps0 = p->porosity;
  float e0 = p->porosity;
  k.g0 = e0 * e0 * e0 / ((1.0f - e0) * (1.0f - e0));
  k.drag_cap = p->drag_cap;
  k.u_inlet = p->u_inlet;
  k.inlet_R = p->inlet_radius;
  k.cxf = (float)(p->center_x < 0 ? 0.5 * p->nx : (double)p->center_x);
  k.cyf = (float)(p->center_y < 0 ? 0.5 * p->ny : (double)p->center_y);
  k.rho_out = p->rho_outlet;
  for (int i = 0; i < POG_INLET_NCOEF; ++i) k.coef[i] = p->inlet_coef[i];
  k.inlet_ctl = p->inlet_control;
  k.pour = p->pour_control;
  k.blockage = p->filter_blockage;
  k.phase = p->phase;
  k.tau_air = p->tau_air;
  k.dmask = p->deposit_mask;
  k.dref = (__half*)p->density_ref;
  return k;
}

}  // namespace pog

using namespace pog;

extern "C" {

int pog_version(void) { return POG_VERSION; }

const char* pog_last_error(void) { return g_err; }

int pog_zero(void* p, size_t bytes, void* stream) {
  if (!p && bytes) return set_error(POG_E_ARG, "NULL pointer");
  if (bytes) POG_TRY_CUDA(cudaMemsetAsync(p, 0, bytes, (cudaStream_t)stream));
  return POG_OK;
}

long long pog_launch_count(int reset) {
  long long v = g_launches;
  if (reset) g_launches = 0;
  return v;
}

int pog_validate_params(const pog_params* p) {
  if (!p) return set_error(POG_E_ARG, "params is NULL");
  if (p->nx < 4 || p->ny < 4 || p->nz < 4)
    return set_error(POG_E_ARG, "grid %dx%dx%d: every extent must be >= 4", p->nx, p->ny, p->nz);
  double n = (double)p->nx * p->ny * p->nz;
  // 32-bit element indexing of the 19 distribution planes.
  if (n * 19.0 >= 4294967296.0)
    return set_error(POG_E_RANGE, "grid of %.0f cells exceeds the 19*ncell < 2^32 limit", n);
  if (p->storage < POG_STORE_F32 || p->storage > POG_STORE_F64)
    return set_error(POG_E_ARG, "storage %d unknown", p->storage);
  if (p->les_mode < POG_LES_OFF || p->les_mode > POG_LES_LOCAL)
    return set_error(POG_E_ARG, "les_mode %d unknown", p->les_mode);
  if (p->drag_mode < 0 || p->drag_mode > 1) return set_error(POG_E_ARG, "drag_mode %d unknown", p->drag_mode);
  if (p->forcing_mode < 0 || p->forcing_mode > 1)
    return set_error(POG_E_ARG, "forcing_mode %d unknown", p->forcing_mode);
  if (!(p->tau > 0.5f)) return set_error(POG_E_ARG, "tau=%g must be > 0.5", (double)p->tau);
  if (p->phase && !(p->tau_air > 0.5f))
    return set_error(POG_E_ARG, "tau_air=%g must be > 0.5 with a phase field", (double)p->tau_air);
  if (!(p->rho0 > 0.0f)) return set_error(POG_E_ARG, "rho0 must be > 0");
  if (p->band_thickness > 0) {
    if (!(p->porosity > 0.0f && p->porosity < 1.0f))
      return set_error(POG_E_ARG, "porosity=%g must be in (0,1)", (double)p->porosity);
    if (!(p->permeability > 0.0f)) return set_error(POG_E_ARG, "permeability must be > 0");
    if (!(p->forchheimer >= 0.0f)) return set_error(POG_E_ARG, "forchheimer must be >= 0");
  }
  if (!(p->cone_half_angle_deg > 0.0f && p->cone_half_angle_deg < 89.0f))
    return set_error(POG_E_ARG, "cone half angle must be in (0, 89) degrees");
  if (p->wall_cells && p->n_wall_cells < 0)
    return set_error(POG_E_ARG, "n_wall_cells=%d must be >= 0", p->n_wall_cells);
  if (p->step_kernel != POG_STEP_AUTO && p->step_kernel != POG_STEP_CELLS)
    return set_error(POG_E_ARG, "step_kernel=%d unknown", p->step_kernel);
  if (p->density_ref && p->storage != POG_STORE_F16S)
    return set_error(POG_E_ARG, "density_ref needs FP16S storage (storage=%d)", p->storage);
  if (p->clamp_tau && !(p->tau_min > 0.5f && p->tau_max >= p->tau_min))
    return set_error(POG_E_ARG, "tau clamp [%g,%g] invalid", (double)p->tau_min, (double)p->tau_max);
  return POG_OK;
}

}  // extern "C"
