// C ABI of the galax_gb300 library (declared in include/galax_gb300.h):
// potential handles, batched potential / gradient / Hessian evaluation, the
// orbit-integration entry point and small utilities.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/galax_gb300.h"
#include "handle.h"
#include "launch.h"

namespace gal {

thread_local std::string g_last_error;
// SMs given to four-warp teams for the longest orbits (gal_set_team); atomic
// because calls on other threads may read it while it is set
static std::atomic<int> g_team_blocks{32};
// Fraction of every span the first pass of the two-pass schedule covers
// (gal_set_split_fraction), in millionths
static std::atomic<int> g_split_ppm{100000};

// One library-owned stream per device for the team kernel, created on first use.
static cudaError_t team_stream(cudaStream_t* out) {
  static std::mutex mu;
  static cudaStream_t streams[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!streams[dev]) {
    e = cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
  }
  *out = streams[dev];
  return cudaSuccess;
}

// The fork/join event pair that orders the team stream after, and the caller's
// stream before, one team launch. Created once per thread and device and then
// reused: an event is re-recorded by every call, and cudaStreamWaitEvent takes
// the record current at the time of the wait, so a pair must not be shared
// between threads that launch concurrently.
struct TeamEvents {
  cudaEvent_t ev[64][2] = {};
  ~TeamEvents() {
    for (auto& p : ev)
      for (cudaEvent_t e : p)
        if (e) cudaEventDestroy(e);
  }
};

static cudaError_t team_events(cudaEvent_t* fork, cudaEvent_t* join) {
  thread_local TeamEvents cache;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  for (int k = 0; k < 2; ++k) {
    if (!cache.ev[dev][k]) {
      e = cudaEventCreateWithFlags(&cache.ev[dev][k], cudaEventDisableTiming);
      if (e != cudaSuccess) {
        cache.ev[dev][k] = nullptr;
        return e;
      }
    }
  }
  *fork = cache.ev[dev][0];
  *join = cache.ev[dev][1];
  return cudaSuccess;
}

// Launch shape per [method == 8][adaptive], set by gal_set_launch. Dopri5 fits
// 3 blocks of 128 per SM without spills (variant 0); Dopri8 needs the uncapped
// variant 2 to avoid spilling. Adaptive batches default to one warp per SM
// sub-partition (128 threads, one block per SM): their longest orbits then run
// at their own latency instead of sharing an FP64 pipe. Read and written under
// g_shape_mu so that a shape is never seen half-set.
static LaunchShape g_shape[2][2] = {{{0, 0, 0, 0}, {128, 1, 2, 0}}, {{0, 0, 2, 0}, {128, 1, 2, 0}}};
static std::mutex g_shape_mu;

// Component tables: 0 = choose one thread or one warp per orbit automatically,
// 1 / 32 = always that (gal_set_table_lanes).
static std::atomic<int> g_table_lanes{0};

static LaunchShape launch_shape(int method, int adaptive) {
  std::lock_guard<std::mutex> lock(g_shape_mu);
  LaunchShape s = g_shape[method == 8][adaptive ? 1 : 0];
  s.table_lanes = g_table_lanes.load(std::memory_order_relaxed);
  return s;
}

gal_status fail(gal_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

gal_status cuda_fail(cudaError_t e, const char* where) {
  return fail(GAL_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// SM count of the current device, looked up once per device (so that launches
// made while a stream is being captured query nothing)
int device_sm_count() {
  static std::atomic<int> cache[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  int sms = cache[dev].load(std::memory_order_relaxed);
  if (sms <= 0) {
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    cache[dev].store(sms, std::memory_order_relaxed);
  }
  return sms;
}

static DevComp fold(const gal_component& c, double G) {
  return fold_comp(c.kind, c.m, c.l1, c.l2, c.origin[0], c.origin[1], c.origin[2], G);
}

static bool milky_way_shape(const gal_component* c, int n) {
  if (n != 4) return false;
  const int32_t want[4] = {MIYAMOTO_NAGAI, NFW, HERNQUIST, HERNQUIST};
  for (int i = 0; i < 4; ++i) {
    if (c[i].kind != want[i]) return false;
    if (c[i].origin[0] != 0.0 || c[i].origin[1] != 0.0 || c[i].origin[2] != 0.0) return false;
  }
  return true;
}

static MWParams mw_params(const gal_component* c, double G) {
  MWParams p{};
  p.Gm_d = G * c[0].m;
  p.a_d = c[0].l1;
  p.b2_d = c[0].l2 * c[0].l2;
  p.Gm_h = G * c[1].m;
  p.rs_h = c[1].l1;
  p.irs_h = 1.0 / c[1].l1;
  p.Gm_b = G * c[2].m;
  p.rs_b = c[2].l1;
  p.Gm_n = G * c[3].m;
  p.rs_n = c[3].l1;
  return p;
}

static gal_status validate_components(const gal_component* comps, int32_t n) {
  if (!comps || n < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "need at least one component");
  if (n > GAL_MAX_COMPONENTS) return fail(GAL_ERR_TOO_LARGE, "too many components (max GAL_MAX_COMPONENTS)");
  for (int i = 0; i < n; ++i) {
    const gal_component& c = comps[i];
    if (c.kind < GAL_KEPLER || c.kind > GAL_POWERLAW_CUTOFF)
      return fail(GAL_ERR_UNSUPPORTED, "unsupported component kind");
    if (c.flags != 0) return fail(GAL_ERR_INVALID_ARGUMENT, "component flags must be 0");
    const double v[6] = {c.m, c.l1, c.l2, c.origin[0], c.origin[1], c.origin[2]};
    for (double x : v)
      if (!std::isfinite(x)) return fail(GAL_ERR_INVALID_ARGUMENT, "non-finite component parameter");
    if ((c.kind == GAL_HERNQUIST || c.kind == GAL_NFW) && !(c.l1 > 0.0))
      return fail(GAL_ERR_INVALID_ARGUMENT, "r_s must be > 0");
    // a < 0 occurs in the three-disk (MN3) fits; a > -b keeps sqrt(z^2 + b^2) + a > 0
    if (c.kind == GAL_MIYAMOTO_NAGAI && !(c.l2 > 0.0 && c.l1 > -c.l2))
      return fail(GAL_ERR_INVALID_ARGUMENT, "Miyamoto-Nagai needs b > 0 and a > -b");
    if (c.kind == GAL_PLUMMER && c.l1 < 0.0) return fail(GAL_ERR_INVALID_ARGUMENT, "Plummer r_s must be >= 0");
    if ((c.kind == GAL_ISOCHRONE || c.kind == GAL_LOGARITHMIC) && !(c.l1 > 0.0))
      return fail(GAL_ERR_INVALID_ARGUMENT, "isochrone b / logarithmic r_s must be > 0");
    if (c.kind == GAL_POWERLAW_CUTOFF && (!(c.l1 > 0.0) || !(c.l2 >= 0.0 && c.l2 < 2.0)))
      return fail(GAL_ERR_INVALID_ARGUMENT, "power law with cutoff needs r_c > 0 and 0 <= alpha < 2");
  }
  return GAL_OK;
}

// ----------------------------------------------------------------- eval kernels
template <class Pot>
__global__ void k_eval_gradient(Pot pot, const double* __restrict__ x, int64_t n, double* __restrict__ out,
                                double sign) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double gx, gy, gz;
    pot.grad(x[i], x[n + i], x[2 * n + i], gx, gy, gz);
    out[i] = sign * gx;
    out[n + i] = sign * gy;
    out[2 * n + i] = sign * gz;
  }
}

__global__ void k_eval_gradient_table(const DevComp* comps, const DevLinear* lin, double t, int ncomp,
                                      const double* __restrict__ x, int64_t n, double* __restrict__ out,
                                      double sign) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevComp* s = reinterpret_cast<DevComp*>(smem_raw);
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) s[i] = lin ? comp_at_time(comps[i], lin[i], t) : comps[i];
  __syncthreads();
  const TablePot pot{s, ncomp};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double gx, gy, gz;
    pot.grad(x[i], x[n + i], x[2 * n + i], gx, gy, gz);
    out[i] = sign * gx;
    out[n + i] = sign * gy;
    out[2 * n + i] = sign * gz;
  }
}

// Components staged into shared memory, refolded at time t when time-dependent.
__device__ __forceinline__ void stage_at_time(const DevComp* comps, const DevLinear* lin, int ncomp, double t,
                                              DevComp* s) {
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) s[i] = lin ? comp_at_time(comps[i], lin[i], t) : comps[i];
}

__global__ void k_eval_phi(const DevComp* comps, const DevLinear* lin, double t, int ncomp,
                           const double* __restrict__ x, int64_t n, double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevComp* s = reinterpret_cast<DevComp*>(smem_raw);
  stage_at_time(comps, lin, ncomp, t, s);
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double phi = 0.0;
    for (int c = 0; c < ncomp; ++c) phi += comp_phi(s[c], x[i], x[n + i], x[2 * n + i]);
    out[i] = phi;
  }
}

__global__ void k_eval_hessian(const DevComp* comps, const DevLinear* lin, double t, int ncomp,
                               const double* __restrict__ x, int64_t n, double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevComp* s = reinterpret_cast<DevComp*>(smem_raw);
  stage_at_time(comps, lin, ncomp, t, s);
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < ncomp; ++c) comp_hessian(s[c], x[i], x[n + i], x[2 * n + i], H);
#pragma unroll
    for (int k = 0; k < 9; ++k) out[k * n + i] = H[k];
  }
}

__global__ void k_fp64_probe(int64_t iters, double seed, double* sink) {
  double a0 = seed + threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
  const double m = 0.999999999, c = 1e-9;
  for (int64_t i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) sink[threadIdx.x] = s;  // keep the chain alive
}

gal_status validate_cfg(const gal_solver_config* c) {
  if (!c) return fail(GAL_ERR_INVALID_ARGUMENT, "config is NULL");
  if (c->method != 5 && c->method != 8) return fail(GAL_ERR_UNSUPPORTED, "method must be 5 (Dopri5) or 8 (Dopri8)");
  if (c->schedule != 0 && c->schedule != 1) return fail(GAL_ERR_INVALID_ARGUMENT, "schedule must be 0 or 1");
  if (c->max_steps < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "max_steps must be >= 1");
  if (!c->adaptive && !(c->dt0 > 0.0)) return fail(GAL_ERR_INVALID_ARGUMENT, "constant step needs dt0 > 0");
  if (c->adaptive) {
    if (!(c->rtol >= 0.0) || !(c->atol >= 0.0) || (c->rtol == 0.0 && c->atol == 0.0))
      return fail(GAL_ERR_INVALID_ARGUMENT, "rtol/atol must be >= 0 and not both 0");
    if (!(c->safety > 0.0) || !(c->factormin > 0.0) || !(c->factormax >= 1.0))
      return fail(GAL_ERR_INVALID_ARGUMENT, "bad safety/factormin/factormax");
  }
  return GAL_OK;
}

// ---- two-phase schedule: order parked orbits by estimated remaining work
constexpr int kBuckets = 64;

__global__ void k_sched_keys(const OrbitResume* __restrict__ r, int64_t n, unsigned* __restrict__ hist,
                             int* __restrict__ bucket) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (r[i].paused) {
      const double p = r[i].progress;
      const double key = (double)r[i].nsteps * (1.0 - p) / fmax(p, 1e-12);
      int b = (int)(2.0f * log2f(1.0f + (float)key));  // half-octave buckets
      b = b < 0 ? 0 : (b >= kBuckets ? kBuckets - 1 : b);
      bucket[i] = b;
      atomicAdd(&hist[b], 1u);
    } else {
      bucket[i] = -1;
    }
  }
}

__global__ void k_sched_scan(const unsigned* __restrict__ hist, unsigned* __restrict__ cursor,
                             unsigned long long* __restrict__ qlen) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    unsigned acc = 0;
    for (int b = kBuckets - 1; b >= 0; --b) {  // most remaining work first
      cursor[b] = acc;
      acc += hist[b];
    }
    *qlen = acc;
  }
}

__global__ void k_sched_scatter(const int* __restrict__ bucket, int64_t n, unsigned* __restrict__ cursor,
                                int32_t* __restrict__ order) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int b = bucket[i];
    if (b >= 0) order[atomicAdd(&cursor[b], 1u)] = (int32_t)i;
  }
}

struct SchedLayout {
  size_t header, resume, bucket, order, total;
};

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

static SchedLayout sched_layout(int64_t n) {
  SchedLayout L{};
  L.header = 0;  // [0] queue counter, [8] queue length, [16] hist[64], [272] cursor[64]
  L.resume = 1024;
  L.bucket = L.resume + align256(sizeof(OrbitResume) * (size_t)n);
  L.order = L.bucket + align256(sizeof(int) * (size_t)n);
  L.total = L.order + align256(sizeof(int32_t) * (size_t)n);
  return L;
}

static void grid_for(int64_t n, int block, unsigned* grid) {
  int64_t g = (n + block - 1) / block;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  *grid = (unsigned)g;
}

}  // namespace gal

using namespace gal;


extern "C" {

int32_t gal_abi_version(void) { return 1; }

const char* gal_last_error(void) { return g_last_error.c_str(); }

const char* gal_status_string(int32_t st) {
  switch (st) {
    case GAL_OK: return "ok";
    case GAL_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GAL_ERR_UNSUPPORTED: return "unsupported";
    case GAL_ERR_CUDA: return "CUDA error";
    case GAL_ERR_WORKSPACE: return "workspace too small";
    case GAL_ERR_TOO_LARGE: return "size beyond the supported maximum";
    case GAL_ERR_HOST_ALLOC: return "host allocation failed";
    default: return "unknown status";
  }
}

gal_status gal_potential_create(const gal_component* comps, int32_t n, double G, gal_potential** out) {
  return no_throw([&]() -> gal_status {
    if (!out) return fail(GAL_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    gal_status st = validate_components(comps, n);
    if (st != GAL_OK) return st;
    if (!(G > 0.0) || !std::isfinite(G)) return fail(GAL_ERR_INVALID_ARGUMENT, "G must be finite and > 0");
    std::unique_ptr<gal_potential> holder(new gal_potential());
    gal_potential* p = holder.get();
    p->comps.assign(comps, comps + n);
    p->G = G;
    p->n = n;
    p->is_mw = milky_way_shape(comps, n);
    p->mw = p->is_mw ? mw_params(comps, G) : MWParams{};
    std::vector<DevComp> h(n);
    for (int i = 0; i < n; ++i) h[i] = fold(comps[i], G);
    cudaError_t e = cudaMalloc(&p->d_comps, sizeof(DevComp) * n);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(component table)");
    e = cudaMemcpy(p->d_comps, h.data(), sizeof(DevComp) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(p->d_comps);
      return cuda_fail(e, "cudaMemcpy(component table)");
    }
    *out = holder.release();
    return GAL_OK;
  });
}

gal_status gal_potential_destroy(gal_potential* p) {
  if (!p) return GAL_OK;
  cudaError_t e = cudaFree(p->d_comps);
  if (p->d_lin) {
    const cudaError_t e2 = cudaFree(p->d_lin);
    if (e == cudaSuccess) e = e2;
  }
  delete p;
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "cudaFree(component table)");
}

gal_status gal_potential_set_linear(gal_potential* p, const double* slopes) {
  return no_throw([&]() -> gal_status {
    if (!p) return fail(GAL_ERR_INVALID_ARGUMENT, "potential is NULL");
    if (slopes) {
      for (int i = 0; i < 3 * p->n; ++i)
        if (!std::isfinite(slopes[i])) return fail(GAL_ERR_INVALID_ARGUMENT, "non-finite slope");
    }
    bool any = false;
    std::vector<DevLinear> h(p->n);
    for (int i = 0; i < p->n; ++i) {
      const gal_component& c = p->comps[i];
      DevLinear& L = h[i];
      L.kind = c.kind;
      L.m0 = c.m;
      L.l10 = c.l1;
      L.l20 = c.l2;
      L.G = p->G;
      L.dm = slopes ? slopes[3 * i] : 0.0;
      L.dl1 = slopes ? slopes[3 * i + 1] : 0.0;
      L.dl2 = slopes ? slopes[3 * i + 2] : 0.0;
      L.active = (L.dm != 0.0 || L.dl1 != 0.0 || L.dl2 != 0.0) ? 1 : 0;
      any = any || L.active;
    }
    if (p->d_lin) {
      cudaError_t e = cudaFree(p->d_lin);
      p->d_lin = nullptr;
      if (e != cudaSuccess) return cuda_fail(e, "cudaFree(linear table)");
    }
    (void)any;
    if (slopes) {  // time-dependent even when every slope is zero: the adjoint then gives d/d(slope)
      cudaError_t e = cudaMalloc(&p->d_lin, sizeof(DevLinear) * p->n);
      if (e != cudaSuccess) {
        p->d_lin = nullptr;
        return cuda_fail(e, "cudaMalloc(linear table)");
      }
      e = cudaMemcpy(p->d_lin, h.data(), sizeof(DevLinear) * p->n, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(linear table)");
    }
    // the specialised Milky Way model has constant parameters
    p->is_mw = !p->d_lin && milky_way_shape(p->comps.data(), p->n);
    return GAL_OK;
  });
}

gal_status gal_potential_update(gal_potential* p, const gal_component* comps, int32_t n, gal_stream_t stream) {
  return no_throw([&]() -> gal_status {
    if (!p) return fail(GAL_ERR_INVALID_ARGUMENT, "potential is NULL");
    if (n != p->n) return fail(GAL_ERR_INVALID_ARGUMENT, "component count differs from the handle's");
    gal_status st = validate_components(comps, n);
    if (st != GAL_OK) return st;
    for (int i = 0; i < n; ++i)
      if (comps[i].kind != p->comps[i].kind) return fail(GAL_ERR_INVALID_ARGUMENT, "component kinds differ");
    std::vector<DevComp> h(n);
    for (int i = 0; i < n; ++i) h[i] = fold(comps[i], p->G);
    // pageable source: the call returns once the bytes are staged, so h may go out of scope
    cudaError_t e = cudaMemcpyAsync(p->d_comps, h.data(), sizeof(DevComp) * n, cudaMemcpyHostToDevice,
                                    (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(component table)");
    e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    p->comps.assign(comps, comps + n);
    p->is_mw = !p->d_lin && milky_way_shape(comps, n);
    p->mw = milky_way_shape(comps, n) ? mw_params(comps, p->G) : MWParams{};
    if (p->d_lin) {  // new values at t = 0, same slopes
      std::vector<DevLinear> L(n);
      e = cudaMemcpy(L.data(), p->d_lin, sizeof(DevLinear) * n, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(linear table)");
      for (int i = 0; i < n; ++i) {
        L[i].m0 = comps[i].m;
        L[i].l10 = comps[i].l1;
        L[i].l20 = comps[i].l2;
      }
      e = cudaMemcpy(p->d_lin, L.data(), sizeof(DevLinear) * n, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(linear table)");
    }
    return GAL_OK;
  });
}

int32_t gal_potential_num_components(const gal_potential* p) { return p ? p->n : 0; }
int32_t gal_potential_is_milky_way(const gal_potential* p) { return p && p->is_mw ? 1 : 0; }

int32_t gal_potential_is_time_dependent(const gal_potential* p) { return time_dependent(p) ? 1 : 0; }

static gal_status eval_grad_common(const gal_potential* p, const double* x, double t, int64_t n, double* out,
                                   double sign, gal_stream_t stream) {
  if (!p || (!x && n) || (!out && n) || n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "bad pointer or size");
  if (n == 0) return GAL_OK;
  const int block = 256;
  unsigned grid;
  grid_for(n, block, &grid);
  if (p->is_mw) {
    k_eval_gradient<MWPot><<<grid, block, 0, (cudaStream_t)stream>>>(MWPot{p->mw}, x, n, out, sign);
  } else {
    const size_t smem = sizeof(DevComp) * p->n;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_eval_gradient_table, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_eval_gradient_table<<<grid, block, smem, (cudaStream_t)stream>>>(p->d_comps, p->d_lin, t, p->n, x, n, out,
                                                                       sign);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "gradient kernel launch");
}

gal_status gal_eval_gradient(const gal_potential* p, const double* x, double t, int64_t n, double* out,
                             gal_stream_t stream) {
  return eval_grad_common(p, x, t, n, out, 1.0, stream);
}

gal_status gal_eval_acceleration(const gal_potential* p, const double* x, double t, int64_t n, double* out,
                                 gal_stream_t stream) {
  return eval_grad_common(p, x, t, n, out, -1.0, stream);
}

gal_status gal_eval_potential(const gal_potential* p, const double* x, double t, int64_t n, double* phi,
                              gal_stream_t stream) {
  if (!p || (!x && n) || (!phi && n) || n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "bad pointer or size");
  if (n == 0) return GAL_OK;
  const int block = 256;
  unsigned grid;
  grid_for(n, block, &grid);
  const size_t smem = sizeof(DevComp) * p->n;
  if (smem > 48 * 1024) cudaFuncSetAttribute(k_eval_phi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_eval_phi<<<grid, block, smem, (cudaStream_t)stream>>>(p->d_comps, p->d_lin, t, p->n, x, n, phi);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "potential kernel launch");
}

gal_status gal_eval_hessian(const gal_potential* p, const double* x, double t, int64_t n, double* out,
                            gal_stream_t stream) {
  if (!p || (!x && n) || (!out && n) || n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "bad pointer or size");
  if (n == 0) return GAL_OK;
  const int block = 128;
  unsigned grid;
  grid_for(n, block, &grid);
  const size_t smem = sizeof(DevComp) * p->n;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_eval_hessian, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_eval_hessian<<<grid, block, smem, (cudaStream_t)stream>>>(p->d_comps, p->d_lin, t, p->n, x, n, out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "hessian kernel launch");
}

gal_status gal_integrate_workspace_size(const gal_solver_config* cfg, int64_t n, size_t* bytes) {
  if (!bytes || !cfg || n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "bad workspace query");
  *bytes = cfg->schedule ? sched_layout(n).total : 256;  // one 8-byte work-queue counter, padded
  return GAL_OK;
}

gal_status gal_set_team(int32_t blocks) {
  if (blocks < 0 || blocks > 1024) return fail(GAL_ERR_INVALID_ARGUMENT, "team blocks must be in [0, 1024]");
  g_team_blocks.store(blocks, std::memory_order_relaxed);
  return GAL_OK;
}

gal_status gal_set_split_fraction(double fraction) {
  if (!(fraction >= 1e-3 && fraction <= 0.9)) return fail(GAL_ERR_INVALID_ARGUMENT, "fraction must be in [0.001, 0.9]");
  g_split_ppm.store((int)(fraction * 1e6 + 0.5), std::memory_order_relaxed);
  return GAL_OK;
}

gal_status gal_set_table_lanes(int32_t lanes) {
  if (lanes != 0 && lanes != 1 && lanes != 32) return fail(GAL_ERR_INVALID_ARGUMENT, "lanes must be 0, 1 or 32");
  g_table_lanes.store(lanes, std::memory_order_relaxed);
  return GAL_OK;
}

gal_status gal_set_launch(int32_t method, int32_t adaptive, int32_t block_threads, int32_t blocks_per_sm,
                          int32_t variant) {
  if ((method != 5 && method != 8) || block_threads < 0 || block_threads > 256 || (block_threads % 32) ||
      blocks_per_sm < 0 || variant < 0 || variant > 2 || (variant != 2 && block_threads > 128))
    return fail(GAL_ERR_INVALID_ARGUMENT, "bad launch shape");
  std::lock_guard<std::mutex> lock(g_shape_mu);
  g_shape[method == 8][adaptive ? 1 : 0] = LaunchShape{block_threads, blocks_per_sm, variant, 0};
  return GAL_OK;
}

gal_status gal_integrate(const gal_potential* p, const gal_solver_config* cfg, const double* y0, const double* t0,
                         const double* t1, const int64_t* save_offsets, const double* save_ts, int64_t n_saves,
                         double* out, int32_t* status, int64_t* steps, const int32_t* order, int64_t n,
                         void* workspace, size_t workspace_bytes, gal_stream_t stream) {
  if (!p) return fail(GAL_ERR_INVALID_ARGUMENT, "potential is NULL");
  gal_status st = validate_cfg(cfg);
  if (st != GAL_OK) return st;
  if (n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "n < 0");
  if (n == 0) return GAL_OK;
  if (n > (int64_t)2147483647) return fail(GAL_ERR_TOO_LARGE, "at most 2^31-1 orbits per call");
  if (!y0 || !t0 || !t1) return fail(GAL_ERR_INVALID_ARGUMENT, "y0/t0/t1 NULL");
  if (n_saves < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "n_saves < 0");
  if ((save_offsets || n_saves > 0) && (!save_ts || !out)) return fail(GAL_ERR_INVALID_ARGUMENT, "saves need save_ts and out");
  size_t need = 0;
  gal_integrate_workspace_size(cfg, n, &need);
  if (!workspace || workspace_bytes < need) return fail(GAL_ERR_WORKSPACE, "workspace too small");
  // CSR saves: n_saves is the total count (save_offsets[n]); shared grid: saves per orbit
  const int64_t total = save_offsets ? n_saves : n_saves * n;
  IntegrateArgs a{};
  a.adaptive = cfg->adaptive;
  a.force_dtmin = cfg->force_dtmin;
  a.max_steps = cfg->max_steps;
  a.dt0 = cfg->dt0;
  a.rtol = cfg->rtol;
  a.atol = cfg->atol;
  a.dtmin = cfg->dtmin;
  a.dtmax = cfg->dtmax;
  const double morder = cfg->method == 8 ? 8.0 : 5.0;
  a.c1 = (cfg->icoeff + cfg->pcoeff + cfg->dcoeff) / morder;
  a.c2 = -(cfg->pcoeff + 2.0 * cfg->dcoeff) / morder;
  a.c3 = cfg->dcoeff / morder;
  a.i_controller = (cfg->pcoeff == 0.0 && cfg->dcoeff == 0.0 && cfg->icoeff == 1.0) ? 1 : 0;
  a.safety = cfg->safety;
  a.factormin = cfg->factormin;
  a.factormax = cfg->factormax;
  a.y0 = y0;
  a.t0 = t0;
  a.t1 = t1;
  a.save_offsets = save_offsets;
  a.save_ts = save_ts;
  a.n_saves = n_saves;
  a.out = out;
  a.out_stride = total;
  a.status = status;
  a.steps = steps;
  a.order = order;
  a.n = n;
  a.lin = p->d_lin;
  cudaStream_t s = (cudaStream_t)stream;
  char* ws = static_cast<char*>(workspace);
  a.queue = reinterpret_cast<unsigned long long*>(ws);
  a.phase = 0;
  a.split_frac = 0.0;
  a.resume = nullptr;
  a.queue_len = nullptr;
  const LaunchShape shape = launch_shape(cfg->method, cfg->adaptive);
  auto launch = [&]() {
    return cfg->method == 8 ? launch_integrate_dopri8(a, p->is_mw, p->mw, p->d_comps, p->n, shape, s)
                            : launch_integrate_dopri5(a, p->is_mw, p->mw, p->d_comps, p->n, shape, s);
  };
  if (!cfg->schedule) {
    cudaError_t e = cudaMemsetAsync(ws, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_fail(e, "clearing the work queue");
    e = launch();
    return e == cudaSuccess ? GAL_OK : cuda_fail(e, "integrate kernel launch");
  }
  // two phases: a fraction of every span (a tenth by default), then longest remaining work first
  const SchedLayout L = sched_layout(n);
  auto* qlen = reinterpret_cast<unsigned long long*>(ws + 8);
  auto* hist = reinterpret_cast<unsigned*>(ws + 16);
  auto* cursor = reinterpret_cast<unsigned*>(ws + 16 + 4 * kBuckets);
  auto* resume = reinterpret_cast<OrbitResume*>(ws + L.resume);
  auto* bucket = reinterpret_cast<int*>(ws + L.bucket);
  auto* order2 = reinterpret_cast<int32_t*>(ws + L.order);
  cudaError_t e = cudaMemsetAsync(ws, 0, L.resume + sizeof(OrbitResume) * (size_t)n, s);
  if (e != cudaSuccess) return cuda_fail(e, "clearing the schedule scratch");
  a.split_frac = 1e-6 * g_split_ppm.load(std::memory_order_relaxed);
  a.resume = resume;
  e = launch();
  if (e != cudaSuccess) return cuda_fail(e, "integrate kernel launch (first pass)");
  unsigned grid;
  grid_for(n, 256, &grid);
  k_sched_keys<<<grid, 256, 0, s>>>(resume, n, hist, bucket);
  k_sched_scan<<<1, 32, 0, s>>>(hist, cursor, qlen);
  k_sched_scatter<<<grid, 256, 0, s>>>(bucket, n, cursor, order2);
  e = cudaMemsetAsync(ws, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "ordering the parked orbits");
  a.phase = 1;
  a.order = order2;
  a.queue_len = qlen;
  const int sms = device_sm_count();
  const int team_blocks = g_team_blocks.load(std::memory_order_relaxed);
  const int blocks = team_blocks < sms - 1 ? team_blocks : sms - 1;
  if (blocks > 0 && p->is_mw) {
    // The longest orbits go to four-warp teams on `blocks` SMs of their own
    // (second stream), the rest to the one-thread kernel on the other SMs, one
    // block per SM; results are the same either way.
    const long long tcap = (long long)kTeamLanes * blocks;
    cudaStream_t ts = nullptr;
    e = team_stream(&ts);
    cudaEvent_t fork = nullptr, join = nullptr;
    if (e == cudaSuccess) e = team_events(&fork, &join);
    if (e == cudaSuccess) e = cudaEventRecord(fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ts, fork, 0);
    bool team_launched = false, joinable = false;
    if (e == cudaSuccess) {
      unsigned long long* tq = reinterpret_cast<unsigned long long*>(ws + 528);
      e = cfg->method == 8 ? launch_integrate_team8(a, p->mw, tq, tcap, blocks, kExclusiveSmem, ts)
                           : launch_integrate_team(a, p->mw, tq, tcap, blocks, kExclusiveSmem, ts);
      team_launched = e == cudaSuccess;
    }
    if (e == cudaSuccess) {
      e = cudaEventRecord(join, ts);
      joinable = e == cudaSuccess;
    }
    if (e == cudaSuccess) {
      a.queue_base = tcap;
      // one warp per sub-partition: two (256 threads) made the step 1.4x longer
      e = cfg->method == 8
              ? launch_integrate_dopri8_exclusive(a, p->mw, shape.variant, 128, sms - blocks, kExclusiveSmem, s)
              : launch_integrate_dopri5_exclusive(a, p->mw, shape.variant, 128, sms - blocks, kExclusiveSmem, s);
    }
    // Whatever failed after the team kernel was queued, the caller's stream
    // still waits for it, so the caller never frees buffers it is using.
    if (joinable) {
      const cudaError_t ej = cudaStreamWaitEvent(s, join, 0);
      if (e == cudaSuccess) e = ej;
    } else if (team_launched) {
      // Under stream capture nothing has run yet and a synchronize would
      // invalidate the caller's capture; the caller discards it on this error.
      cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap == cudaStreamCaptureStatusNone)
        cudaStreamSynchronize(ts);
    }
    return e == cudaSuccess ? GAL_OK : cuda_fail(e, "integrate kernel launch (second pass, teams)");
  }
  e = launch();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "integrate kernel launch (second pass)");
}

int32_t gal_tableau(int32_t method, double* c, double* a, double* b, double* e) {
  if (method != 5 && method != 8) return 0;
  for (int i = 0; i < 13; ++i) {
    c[i] = b[i] = e[i] = 0.0;
    for (int j = 0; j < 13; ++j) a[13 * i + j] = 0.0;
  }
  auto copy = [&](auto tb) {
    using TB = decltype(tb);
    for (int i = 0; i < TB::S; ++i) {
      c[i] = TB::C[i];
      b[i] = TB::B[i];
      e[i] = TB::E[i];
      for (int j = 0; j < TB::S; ++j) a[13 * i + j] = TB::A[i][j];
    }
    return TB::S;
  };
  return method == 5 ? copy(Dopri5{}) : copy(Dopri8{});
}

gal_status gal_fp64_peak_probe(int64_t iters, double* ms, double* flops, gal_stream_t stream) {
  if (iters < 1 || !ms || !flops) return fail(GAL_ERR_INVALID_ARGUMENT, "bad probe arguments");
  const int block = 256;
  const unsigned grid = (unsigned)device_sm_count() * 8;
  double* sink = nullptr;
  cudaError_t e = cudaMalloc(&sink, block * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(probe)");
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fp64_probe<<<grid, block, 0, (cudaStream_t)stream>>>(iters / 8 + 1, 1.0, sink);  // warm-up
  cudaEventRecord(a, (cudaStream_t)stream);
  k_fp64_probe<<<grid, block, 0, (cudaStream_t)stream>>>(iters, 1.0, sink);
  cudaEventRecord(b, (cudaStream_t)stream);
  e = cudaEventSynchronize(b);
  float t = 0.f;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  if (e != cudaSuccess) return cuda_fail(e, "probe");
  *ms = t;
  *flops = 2.0 * 8.0 * (double)iters * (double)grid * (double)block;
  return GAL_OK;
}

// The adjoint entry points live in adjoint.cu.

}  // extern "C"
