// Orbit integration with the learned surrogate: analytic FP64 part + MLP part.
//
// Dopri5 with a constant step over a batch of orbits, stepped at batch level:
// per stage one FP64 kernel forms the stage state Y = y + h sum_l a_il F_l,
// writes F_i = (Y_v, -grad Phi_analytic(Y_q)) and the stage positions, then the
// tensor-core MLP kernel adds -grad Phi_MLP(Y_q) into F_i. The seventh stage is
// evaluated at y_{n+1} (FSAL), so it becomes the next step's first slope in
// place. One step (12 kernels) is captured once as a CUDA graph and replayed.
// The analytic part is any gal_potential (the Milky Way model runs its
// specialised gradient).
#include <cuda_runtime.h>

#include <cmath>

#include "handle.h"
#include "integrate.cuh"
#include "split.cuh"

struct gal_mlp;
extern "C" gal_status gal_mlp_eval(const gal_mlp* mlp, const double* x, int64_t n, double* grad, int32_t accumulate,
                                   double grad_sign, double* phi, gal_stream_t stream);

namespace gal {

// Stage I of a constant step of signed length hs. F is [7][6][n] (slot 0 holds the
// step's first slope, slot I receives this stage; the FSAL stage I = 6 writes
// slot 0 and the state). Yq receives the stage positions [3][n].
template <int I, class Pot>
__global__ void __launch_bounds__(256) k_stage(Pot pot, double* __restrict__ y, double* __restrict__ F,
                                               double* __restrict__ Yq, double hs, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double Y[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      double acc = 0.0;
      bool first = true;
      static_for<0, I>([&](auto l) {
        constexpr int L = decltype(l)::value;
        constexpr double c = Dopri5::A[I][L];
        if constexpr (c != 0.0) {
          const double f = F[((int64_t)L * 6 + j) * n + i];
          acc = first ? c * f : fma(c, f, acc);
          first = false;
        }
      });
      Y[j] = fma(hs, acc, y[(int64_t)j * n + i]);
    }
    double gx, gy, gz;
    pot.grad(Y[0], Y[1], Y[2], gx, gy, gz);
    constexpr int slot = (I == Dopri5::S - 1) ? 0 : I;
    double* Fo = F + (int64_t)slot * 6 * n;
    Fo[0 * n + i] = Y[3];
    Fo[1 * n + i] = Y[4];
    Fo[2 * n + i] = Y[5];
    Fo[3 * n + i] = -gx;
    Fo[4 * n + i] = -gy;
    Fo[5 * n + i] = -gz;
    Yq[0 * n + i] = Y[0];
    Yq[1 * n + i] = Y[1];
    Yq[2 * n + i] = Y[2];
    if constexpr (I == Dopri5::S - 1) {
#pragma unroll
      for (int j = 0; j < 6; ++j) y[(int64_t)j * n + i] = Y[j];  // y_{n+1} = Y_7 (a_7 = b)
    }
  }
}

// slope at the current state (stage 0 of the first step)
template <class Pot>
__global__ void __launch_bounds__(256) k_slope0(Pot pot, const double* __restrict__ y, double* __restrict__ F,
                                                double* __restrict__ Yq, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double gx, gy, gz;
    pot.grad(y[i], y[n + i], y[2 * n + i], gx, gy, gz);
    F[0 * n + i] = y[3 * n + i];
    F[1 * n + i] = y[4 * n + i];
    F[2 * n + i] = y[5 * n + i];
    F[3 * n + i] = -gx;
    F[4 * n + i] = -gy;
    F[5 * n + i] = -gz;
    Yq[0 * n + i] = y[i];
    Yq[1 * n + i] = y[n + i];
    Yq[2 * n + i] = y[2 * n + i];
  }
}

template <class Pot>
static cudaError_t launch_step(const Pot& pot, double* y, double* F, double* Yq, double hs, int64_t n,
                               const gal_mlp* mlp, cudaStream_t s, unsigned grid) {
  auto mlp_add = [&](double* Fslot) -> cudaError_t {
    if (!mlp) return cudaSuccess;
    return gal_mlp_eval(mlp, Yq, n, Fslot + 3 * n, 1, -1.0, nullptr, s) == GAL_OK ? cudaSuccess
                                                                                    : cudaErrorLaunchFailure;
  };
  cudaError_t e;
  k_stage<1><<<grid, 256, 0, s>>>(pot, y, F, Yq, hs, n);
  if ((e = mlp_add(F + 1 * 6 * n)) != cudaSuccess) return e;
  k_stage<2><<<grid, 256, 0, s>>>(pot, y, F, Yq, hs, n);
  if ((e = mlp_add(F + 2 * 6 * n)) != cudaSuccess) return e;
  k_stage<3><<<grid, 256, 0, s>>>(pot, y, F, Yq, hs, n);
  if ((e = mlp_add(F + 3 * 6 * n)) != cudaSuccess) return e;
  k_stage<4><<<grid, 256, 0, s>>>(pot, y, F, Yq, hs, n);
  if ((e = mlp_add(F + 4 * 6 * n)) != cudaSuccess) return e;
  k_stage<5><<<grid, 256, 0, s>>>(pot, y, F, Yq, hs, n);
  if ((e = mlp_add(F + 5 * 6 * n)) != cudaSuccess) return e;
  k_stage<6><<<grid, 256, 0, s>>>(pot, y, F, Yq, hs, n);  // FSAL: slot 0 and y_{n+1}
  if ((e = mlp_add(F)) != cudaSuccess) return e;
  return cudaGetLastError();
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace gal

using namespace gal;

extern "C" {

gal_status gal_surrogate_workspace_size(int64_t n, size_t* bytes) {
  if (!bytes || n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "bad workspace query");
  *bytes = align256(sizeof(double) * 7 * 6 * (size_t)n) + align256(sizeof(double) * 3 * (size_t)n);
  return GAL_OK;
}

gal_status gal_integrate_surrogate(const gal_potential* pot, const gal_mlp* mlp, const gal_split* near, double dt,
                                   double t0, double t1, double* y, int64_t n, int32_t use_graph, void* workspace,
                                   size_t workspace_bytes, gal_stream_t stream) {
  if (!pot || !y || n < 0 || !(dt > 0.0)) return fail(GAL_ERR_INVALID_ARGUMENT, "bad surrogate arguments");
  if (time_dependent(pot)) return fail(GAL_ERR_UNSUPPORTED, "time-dependent parameters: evaluation, integration and the orbit adjoint only");
  if (!std::isfinite(t0) || !std::isfinite(t1)) return fail(GAL_ERR_INVALID_ARGUMENT, "t0 and t1 must be finite");
  if (n == 0 || t0 == t1) return GAL_OK;
  size_t need = 0;
  gal_surrogate_workspace_size(n, &need);
  if (!workspace || workspace_bytes < need) return fail(GAL_ERR_WORKSPACE, "workspace too small");
  double* F = static_cast<double*>(workspace);
  double* Yq = reinterpret_cast<double*>(static_cast<char*>(workspace) + align256(sizeof(double) * 7 * 6 * (size_t)n));
  cudaStream_t caller = (cudaStream_t)stream;
  // graphs are captured on a private non-blocking stream (the legacy default
  // stream cannot be captured), ordered after and before the caller's stream
  cudaStream_t s = caller;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  if (use_graph) {
    s = nullptr;
    cudaError_t e0 = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e0 == cudaSuccess) e0 = cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming);
    if (e0 == cudaSuccess) e0 = cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming);
    if (e0 == cudaSuccess) e0 = cudaEventRecord(ev_in, caller);
    if (e0 == cudaSuccess) e0 = cudaStreamWaitEvent(s, ev_in, 0);
    if (e0 != cudaSuccess) {  // nothing was queued on s: release what was created
      if (ev_in) cudaEventDestroy(ev_in);
      if (ev_out) cudaEventDestroy(ev_out);
      if (s) cudaStreamDestroy(s);
      return cuda_fail(e0, "setting up the capture stream");
    }
  }
  auto finish = [&](gal_status st) -> gal_status {
    if (use_graph) {
      cudaEventRecord(ev_out, s);
      cudaStreamWaitEvent(caller, ev_out, 0);
      cudaEventDestroy(ev_in);
      cudaEventDestroy(ev_out);
      cudaStreamDestroy(s);  // returns at once; queued work still completes
    }
    return st;
  };
  const double dir = (t0 < t1) ? 1.0 : -1.0;
  // constant-step time grid as for gal_integrate: the step that would pass t1 - 1e-10 ends on t1
  const double tau1 = dir * t1;
  double tprev = dir * t0, tnext = fmin(tprev + dt, tau1);
  int64_t grid64 = (n + 255) / 256;
  const int64_t cap = (int64_t)device_sm_count() * 8;
  const unsigned grid = (unsigned)(grid64 > cap ? cap : grid64);
  cudaError_t e;
  // the analytic part, with the exact short-range Plummer sum when a split is given
  const SplitDev* spd = gal_split_device(near);
  auto with_pot = [&](auto&& fn) -> cudaError_t {
    if (pot->is_mw) {
      const MWPot base{pot->mw};
      return spd ? fn(WithShort<MWPot>{base, *spd}) : fn(base);
    }
    const TablePot base{pot->d_comps, pot->n};
    return spd ? fn(WithShort<TablePot>{base, *spd}) : fn(base);
  };
  auto run_slope0 = [&]() -> cudaError_t {
    cudaError_t e0 = with_pot([&](auto P) -> cudaError_t {
      k_slope0<<<grid, 256, 0, s>>>(P, y, F, Yq, n);
      return cudaSuccess;
    });
    if (e0 != cudaSuccess) return e0;
    if (mlp && gal_mlp_eval(mlp, Yq, n, F + 3 * n, 1, -1.0, nullptr, s) != GAL_OK) return cudaErrorLaunchFailure;
    return cudaGetLastError();
  };
  auto run_step = [&](double hs) -> cudaError_t {
    return with_pot([&](auto P) -> cudaError_t { return launch_step(P, y, F, Yq, hs, n, mlp, s, grid); });
  };
  if ((e = run_slope0()) != cudaSuccess) return finish(cuda_fail(e, "surrogate first slope"));
  cudaGraphExec_t exec = nullptr;
  double graph_hs = 0.0;
  while (tprev < tau1) {
    if (!(tnext > tprev)) {  // dt below the spacing of the times: the grid would never reach t1
      if (exec) cudaGraphExecDestroy(exec);
      return finish(fail(GAL_ERR_INVALID_ARGUMENT, "dt does not advance the time"));
    }
    const double hs = dir * (tnext - tprev);
    if (use_graph && hs == dir * dt) {
      if (!exec || graph_hs != hs) {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        cudaGraph_t g;
        e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
          cudaError_t e2 = run_step(hs);
          e = cudaStreamEndCapture(s, &g);
          if (e2 != cudaSuccess) e = e2;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
        if (e == cudaSuccess) cudaGraphDestroy(g);
        if (e != cudaSuccess) return finish(cuda_fail(e, "capturing the surrogate step"));
        graph_hs = hs;
      }
      e = cudaGraphLaunch(exec, s);
    } else {
      e = run_step(hs);
    }
    if (e != cudaSuccess) {
      if (exec) cudaGraphExecDestroy(exec);
      return finish(cuda_fail(e, "surrogate step"));
    }
    double nt1 = tnext + dt;
    tprev = fmin(tnext, tau1);
    if (nt1 > tau1 - 1e-10) nt1 = tau1;
    tnext = nt1;
  }
  if (exec) cudaGraphExecDestroy(exec);
  return finish(GAL_OK);
}

}  // extern "C"
