// gal_integrate_noalloc: orbit integration for callers that cannot allocate
// device memory.
//
// gal_integrate takes its scratch (the work-queue counter and, for the two-pass
// schedule, one resume record per orbit) from a caller-provided workspace. Some
// callers cannot provide one: host plug-ins that are handed only their input
// and output buffers (an XLA custom call registered without a scratch
// allocator, for instance), services that forbid device allocation after
// start-up, and hosts with a fixed device-memory budget. For them this entry
// point takes the scratch from a fixed array that lives in the library's own
// device memory (allocated by the CUDA runtime when the library's module loads,
// and held by every GPU that loads the library until the process exits), and
// then runs the same integration path as gal_integrate.
//
// The array's device address is looked up once per device and cached. A
// cudaDeviceReset unloads the module, so the cached address is then stale; the
// header tells callers not to use this entry point on a device after a reset.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/galax_gb300.h"
#include "handle.h"

namespace gal {

// The scratch array. In host code this symbol is only a handle: its device
// address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GAL_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
static void* g_noalloc_ptr[kMaxDevices] = {};
static std::mutex g_noalloc_mutex;

// Device address of the scratch array on the current device (set-up on first use).
static gal_status noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(GAL_ERR_UNSUPPORTED, "device index beyond 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch array)");
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return GAL_OK;
}

}  // namespace gal

using namespace gal;

extern "C" {

gal_status gal_integrate_noalloc(const gal_potential* pot, const gal_solver_config* cfg, const double* y0,
                                 const double* t0, const double* t1, const int64_t* save_offsets,
                                 const double* save_ts, int64_t n_saves, double* out, int32_t* status,
                                 int64_t* steps, const int32_t* order, int64_t n, gal_stream_t stream) {
  if (!cfg) return fail(GAL_ERR_INVALID_ARGUMENT, "config is NULL");
  if (n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "n < 0");
  size_t need = 0;
  gal_status st = gal_integrate_workspace_size(cfg, n, &need);
  if (st != GAL_OK) return st;
  if (need > (size_t)GAL_NOALLOC_SCRATCH_BYTES)
    return fail(GAL_ERR_TOO_LARGE,
                "gal_integrate_noalloc: this call needs " + std::to_string(need) +
                    " bytes of scratch but the built-in array holds " +
                    std::to_string((size_t)GAL_NOALLOC_SCRATCH_BYTES) +
                    " (the two-pass schedule takes 136 bytes per orbit); use schedule = 0, fewer orbits per call, "
                    "or gal_integrate with a workspace");
  void* scratch = nullptr;
  st = noalloc_scratch(&scratch);
  if (st != GAL_OK) return st;
  return gal_integrate(pot, cfg, y0, t0, t1, save_offsets, save_ts, n_saves, out, status, steps, order, n, scratch,
                       (size_t)GAL_NOALLOC_SCRATCH_BYTES, stream);
}

}  // extern "C"
