// particles_noalloc.cu -- particle binning and cell sort without caller-provided scratch.
//
// pog_particles_bin needs a few megabytes of device scratch for its radix sort, which the caller
// allocates.  Some callers cannot: a host application that hands this library a fixed device
// memory budget and forbids any further device allocation once it is running (its own memory
// manager owns the GPU), or a loop that must never block on, or fail in, an allocator.  For them,
// pog_particles_bin_noalloc runs the same binning and sort with its scratch in a device array
// that is part of this library's image.  CUDA loads a library's device code lazily, per device:
// the 20 MiB array is reserved on a GPU by the first call on that GPU (which also resolves its
// address) and stays reserved there until the process exits.  A caller with a fixed memory budget
// therefore makes one call with np = 0 on each device at set-up time -- before its budget is fixed
// and before any stream capture -- and then never allocates again.
//
// The address is resolved once per device ordinal and cached.  The current device must be the
// device of `stream`, and the cache does not survive cudaDeviceReset (the device's code and its
// array are reloaded at a new address): do not use this entry point across a reset.
//
// Limit: POG_NOALLOC_MAX_PARTICLES particles (the array is sized for exactly that many).
// The array is shared by every call on a device and keeps the previous call's contents; the
// sort writes every histogram entry, prefix sum and key/value slot before it reads it, so no
// part of it needs clearing between calls.  Calls whose work overlaps on the GPU (different
// streams, or different host threads on one stream without ordering) race on the array and
// must be serialised by the caller.
#include <mutex>

#include "common.cuh"

namespace pog {

// Radix-sort scratch for POG_NOALLOC_MAX_PARTICLES particles: 4 key/value ping-pong arrays of
// 4 MiB, a 2 MiB digit histogram and the scan's chunk sums (see pog_particles_bin).
constexpr size_t NOALLOC_SCRATCH_BYTES = 20u * 1024u * 1024u;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device ordinal, resolved once per device.
constexpr int NOALLOC_MAX_DEVICES = 64;
static void* g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mutex;

static int noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return check_cuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return set_error(POG_E_RANGE, "device ordinal %d beyond %d", dev, NOALLOC_MAX_DEVICES);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    // Host code may not use g_noalloc_scratch's name as a device address: resolve it with the
    // device current (it is: cudaGetDevice above returned it).
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return check_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return POG_OK;
}

}  // namespace pog

using namespace pog;

extern "C" int pog_particles_bin_noalloc(const pog_params* p, const float* pos, const int32_t* active,
                                         int np, int32_t* keys, int32_t* perm, void* stream) {
  if (np < 0) return set_error(POG_E_ARG, "np=%d < 0", np);
  if (np > POG_NOALLOC_MAX_PARTICLES)
    return set_error(POG_E_RANGE,
                     "pog_particles_bin_noalloc handles at most %d particles (got %d); use "
                     "pog_particles_bin with caller scratch for more",
                     POG_NOALLOC_MAX_PARTICLES, np);
  const size_t need = pog_particles_bin_scratch_bytes(np);
  if (need > NOALLOC_SCRATCH_BYTES)
    return set_error(POG_E_RANGE, "sort scratch %zu bytes exceeds the static %zu", need,
                     NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  return pog_particles_bin(p, pos, active, np, keys, perm, perm ? scratch : nullptr, stream);
}
