// pour.cu -- the pour nozzle's motion (PrecisePouringSystem._get_current_pour_position and the
// pour_time update of apply_pouring_force, src/physics/precise_pouring.py:81-98,142-146), kept on
// the device so a replayed CUDA graph moves the nozzle step by step.  The force it exerts is
// applied inside the step kernel (collide.cuh pour_accel) and the particle kernel (pour_impact).
#include "common.cuh"

namespace pog {

__global__ void pour_advance_kernel(float* __restrict__ b, float nx, float ny) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || b[POG_POUR_ACTIVE] == 0.0f) return;
  const float time = b[POG_POUR_TIME] + b[POG_POUR_DT];
  b[POG_POUR_TIME] = time;
  float x = b[POG_POUR_CX], y = b[POG_POUR_CY];
  if (b[POG_POUR_PATTERN] == 1.0f) {
    const float t = time * b[POG_POUR_SPIRAL_SPEED];
    const float r = b[POG_POUR_SPIRAL_R] * (1.0f + 0.1f * t);
    const float d = b[POG_POUR_DIAMETER];
    x = fmaxf(d, fminf(nx - d, x + r * cosf(t)));
    y = fmaxf(d, fminf(ny - d, y + r * sinf(t)));
  }
  b[POG_POUR_X] = x;
  b[POG_POUR_Y] = y;
}

}  // namespace pog

extern "C" int pog_pour_advance(const pog_params* p, void* stream) {
  int rc = pog_validate_params(p);
  if (rc) return rc;
  if (!p->pour_control) return pog::set_error(POG_E_ARG, "pour_control is NULL");
  pog::pour_advance_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(const_cast<float*>(p->pour_control),
                                                                 (float)p->nx, (float)p->ny);
  pog::count_launch();
  POG_TRY_CUDA(cudaGetLastError());
  return POG_OK;
}
