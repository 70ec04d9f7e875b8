// Discrete adjoint of the constant-step Runge-Kutta orbit map, with
// checkpointing: gradients of a terminal loss with respect to the initial
// phase-space point of every orbit and to every component parameter.
//
// galax differentiates through diffrax (ForwardMode by default,
// src/galax/dynamics/_src/orbit/solver.py:133; RecursiveCheckpointAdjoint as
// in orbit/solver.py:99-108). Here the reverse pass is written out by hand: for
// y1 = y0 + h sum_i b_i F_i with F_i = f(Y_i) and Y_i = y0 + h sum_l a_il F_l,
// given lambda = dL/dy1,
//     Fbar_i = h b_i lambda + h sum_{j>i} a_ji Ybar_j,   Ybar_i = J(Y_i)^T Fbar_i,
//     dL/dy0 = lambda + sum_i Ybar_i,   dL/dtheta += sum_i (df/dtheta)(Y_i)^T Fbar_i,
// with f = (p, -grad Phi(q)), so J^T (u, v) = (-H(q) v, u) and
// (df/dtheta)^T (u, v) = -d(grad Phi . v)/dtheta.
//
// One thread owns one orbit: it integrates forward storing the state every
// k_ckpt steps, then walks the segments backwards, recomputing each segment's
// states from its checkpoint into scratch and sweeping the stages in reverse.
// Per-orbit parameter gradients go to scratch and are summed over orbits by a
// fixed-order reduction, so results are bitwise reproducible.
//
// Time-dependent potentials (galax's LinearParameter,
// src/galax/potential/_src/params/core.py:25-110): every stage runs at its own
// time t_i, with each component's (m, l1, l2) = values at t = 0 + slopes t_i.
// Their parameter cotangent at t_i, dL/dp(t_i), adds to dL/dp(0) and, times
// t_i, to dL/d(slope).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "handle.h"
#include "integrate.cuh"
#include "vjp.cuh"

namespace gal {

struct AdjointArgs {
  const double* y0;      // [6][n]
  const double* lambda;  // [6][n] or NULL
  const double* target;  // [6][n] when lambda is NULL
  double* yT;            // [6][n]
  double* grad_y0;       // [6][n]
  const double* ts;      // [N+1] time grid (same for every orbit); ts[k+1] - ts[k] is the signed step
  double* ckpt;          // [nseg][6][n]
  double* seg;           // [K][6][n]
  double* gp_orbit;      // [ncomp*NP][n]: NP = 3 (m, l1, l2), or 6 with the slopes
  const DevLinear* lin;  // time-dependent parameters, or NULL
  int64_t nsteps;
  int32_t k_ckpt;
  int64_t n;
};

template <class TB, class Pot, bool TIMED = false>
__global__ void __launch_bounds__(128) k_adjoint(AdjointArgs a, Pot pot, const DevComp* comps, int ncomp) {
  constexpr int NP = TIMED ? 6 : 3;
  __shared__ DevComp s_comps[kAdjMaxComps];
  __shared__ DevLinear s_lin[TIMED ? kAdjMaxComps : 1];
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) {
    s_comps[i] = comps[i];
    if constexpr (TIMED) s_lin[i] = a.lin[i];
  }
  __syncthreads();
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= a.n) return;
  const int64_t n = a.n;
  const int K = a.k_ckpt;
  double y[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) y[j] = a.y0[j * n + o];
  // forward sweep with checkpoints
  for (int64_t k = 0; k < a.nsteps; ++k) {
    if (k % K == 0) {
      const int64_t c = k / K;
#pragma unroll
      for (int j = 0; j < 6; ++j) a.ckpt[(c * 6 + j) * n + o] = y[j];
    }
    rk_step_plain<TB>(pot, y, a.ts[k + 1] - a.ts[k], a.ts[k]);
  }
  double lam[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    a.yT[j * n + o] = y[j];
    lam[j] = a.lambda ? a.lambda[j * n + o] : 2.0 * (y[j] - a.target[j * n + o]);
  }
  double gp[kAdjMaxComps * NP];
#pragma unroll
  for (int i = 0; i < kAdjMaxComps * NP; ++i) gp[i] = 0.0;
  const int64_t nseg = (a.nsteps + K - 1) / K;
  for (int64_t sgi = nseg - 1; sgi >= 0; --sgi) {
    const int64_t k0 = sgi * K;
    const int64_t k1 = (k0 + K < a.nsteps) ? k0 + K : a.nsteps;
#pragma unroll
    for (int j = 0; j < 6; ++j) y[j] = a.ckpt[(sgi * 6 + j) * n + o];
    for (int64_t k = k0; k < k1; ++k) {
#pragma unroll
      for (int j = 0; j < 6; ++j) a.seg[((k - k0) * 6 + j) * n + o] = y[j];
      if (k + 1 < k1) rk_step_plain<TB>(pot, y, a.ts[k + 1] - a.ts[k], a.ts[k]);
    }
    for (int64_t k = k1 - 1; k >= k0; --k) {
      const double hs = a.ts[k + 1] - a.ts[k];  // signed step (the grid carries the direction)
      const double tk = a.ts[k];
      double yk[6];
#pragma unroll
      for (int j = 0; j < 6; ++j) yk[j] = a.seg[((k - k0) * 6 + j) * n + o];
      // recompute the stages, keeping each stage position
      double F[TB::S][6], Yq[TB::S][3];
      field(pot, yk, F[0], tk);
      Yq[0][0] = yk[0];
      Yq[0][1] = yk[1];
      Yq[0][2] = yk[2];
      static_for<1, TB::S>([&](auto i) {
        constexpr int I = decltype(i)::value;
        double Y[6];
        stage_state<TB, I>(yk, hs, F, Y);
        Yq[I][0] = Y[0];
        Yq[I][1] = Y[1];
        Yq[I][2] = Y[2];
        constexpr double ci = TB::C[I];
        field(pot, Y, F[I], fma(ci, hs, tk));
      });
      // reverse sweep (F is reused as Fbar)
      static_for<0, TB::S>([&](auto i) {
        constexpr int I = decltype(i)::value;
        constexpr double bi = TB::B[I];
#pragma unroll
        for (int j = 0; j < 6; ++j) F[I][j] = hs * bi * lam[j];
      });
      static_for<0, TB::S>([&](auto r) {
        constexpr int I = TB::S - 1 - decltype(r)::value;
        double Hv[3] = {0.0, 0.0, 0.0};
        const double v[3] = {F[I][3], F[I][4], F[I][5]};
        constexpr double ci = TB::C[I];
        const double ti = fma(ci, hs, tk);  // the stage's time, as in the forward pass
        for (int c = 0; c < ncomp; ++c) {
          double dp[3] = {0.0, 0.0, 0.0};
          if constexpr (TIMED)
            comp_vjp(comp_at_time(s_comps[c], s_lin[c], ti), Yq[I], v, Hv, dp);
          else
            comp_vjp(s_comps[c], Yq[I], v, Hv, dp);
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            gp[NP * c + j] -= dp[j];
            if constexpr (TIMED) gp[NP * c + 3 + j] -= dp[j] * ti;
          }
        }
        const double Yb[6] = {-Hv[0], -Hv[1], -Hv[2], F[I][0], F[I][1], F[I][2]};
#pragma unroll
        for (int j = 0; j < 6; ++j) lam[j] += Yb[j];
        static_for<0, I>([&](auto l) {
          constexpr int L = decltype(l)::value;
          constexpr double c = TB::A[I][L];
          if constexpr (c != 0.0) {
#pragma unroll
            for (int j = 0; j < 6; ++j) F[L][j] = fma(hs * c, Yb[j], F[L][j]);
          }
        });
      });
    }
  }
#pragma unroll
  for (int j = 0; j < 6; ++j) a.grad_y0[j * n + o] = lam[j];
  for (int i = 0; i < ncomp * NP; ++i) a.gp_orbit[(int64_t)i * n + o] = gp[i];
}

// grad_params[p] = sum over orbits of gp_orbit[p][:], in a fixed order.
__global__ void k_reduce_rows(const double* __restrict__ in, int64_t n, double* __restrict__ out) {
  __shared__ double red[256];
  const double* row = in + (int64_t)blockIdx.x * n;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += row[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// Constant-step time grid exactly as the forward kernels build it
// (ts[k+1] - ts[k] == dir * h_k exactly: negation is exact). False when t0 or
// t1 is not finite, when the grid would need more than max_steps steps, or
// when a step of dt no longer moves the time (dt below its spacing); the
// host grid holds at most 2^28 steps whatever max_steps says.
constexpr int64_t kMaxGridSteps = int64_t(1) << 28;  // 2 GiB of step times on the host

static bool time_grid(double t0, double t1, double dt, int64_t max_steps, std::vector<double>& ts) {
  ts.clear();
  if (max_steps > kMaxGridSteps) max_steps = kMaxGridSteps;
  if (!std::isfinite(t0) || !std::isfinite(t1) || !(dt > 0.0)) return false;
  if (std::fabs(t1 - t0) / dt > (double)max_steps + 1.0) return false;
  const double dir = (t0 < t1) ? 1.0 : -1.0;
  const double tau1 = dir * t1;
  double tprev = dir * t0, tnext = tprev + dt;
  if (tnext > tau1) tnext = tau1;
  ts.push_back(dir * tprev);
  while (tprev < tau1) {
    if (!(tnext > tprev) || (int64_t)ts.size() > max_steps) return false;
    ts.push_back(dir * tnext);
    double nt1 = tnext + dt;
    tprev = tnext < tau1 ? tnext : tau1;
    if (nt1 > tau1 - 1e-10) nt1 = tau1;
    tnext = nt1;
  }
  return true;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct AdjLayout {
  size_t ts, ckpt, seg, gp, total;
  int64_t nsteps, nseg;
};

static AdjLayout adj_layout(int ncomp, int np, const std::vector<double>& ts, int k, int64_t n) {
  AdjLayout L{};
  L.nsteps = (int64_t)ts.size() - 1;
  L.nseg = (L.nsteps + k - 1) / k;
  size_t off = 0;
  L.ts = off;
  off += align256(sizeof(double) * ts.size());
  L.ckpt = off;
  off += align256(sizeof(double) * 6 * (size_t)L.nseg * n);
  L.seg = off;
  off += align256(sizeof(double) * 6 * (size_t)k * n);
  L.gp = off;
  off += align256(sizeof(double) * np * (size_t)ncomp * n);
  L.total = off;
  return L;
}

}  // namespace gal

using namespace gal;

extern "C" {

gal_status gal_adjoint_workspace_size(const gal_potential* pot, const gal_solver_config* cfg, double t0, double t1,
                                      int32_t k_ckpt, int64_t n, size_t* bytes) {
  return no_throw([&]() -> gal_status {
    if (!pot || !cfg || !bytes || k_ckpt < 1 || n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "bad adjoint arguments");
    if (cfg->adaptive || !(cfg->dt0 > 0.0)) return fail(GAL_ERR_UNSUPPORTED, "the adjoint needs a constant step");
    std::vector<double> ts;
    if (!time_grid(t0, t1, cfg->dt0, cfg->max_steps, ts))
      return fail(GAL_ERR_INVALID_ARGUMENT, "t0 and t1 must be finite and at most max_steps steps of dt0 apart");
    *bytes = adj_layout(pot->n, time_dependent(pot) ? 6 : 3, ts, k_ckpt, n).total;
    return GAL_OK;
  });
}

gal_status gal_adjoint(const gal_potential* pot, const gal_solver_config* cfg, const double* y0, double t0,
                       double t1, const double* lambda, const double* target, double* yT, double* grad_y0,
                       double* grad_params, int32_t k_ckpt, int64_t n, void* workspace, size_t workspace_bytes,
                       gal_stream_t stream) {
  return no_throw([&]() -> gal_status {
    if (!pot) return fail(GAL_ERR_INVALID_ARGUMENT, "potential is NULL");
    const bool timed = time_dependent(pot);
    gal_status st = validate_cfg(cfg);
    if (st != GAL_OK) return st;
    if (cfg->adaptive) return fail(GAL_ERR_UNSUPPORTED, "the adjoint needs a constant step (adaptive = 0)");
    if (pot->n > kAdjMaxComps) return fail(GAL_ERR_UNSUPPORTED, "the adjoint supports at most 8 components");
    if (k_ckpt < 1 || n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "k_ckpt >= 1 and n >= 0 required");
    if (n == 0) return GAL_OK;
    if (!y0 || !yT || !grad_y0 || !grad_params || (!lambda && !target))
      return fail(GAL_ERR_INVALID_ARGUMENT, "NULL array");
    if (!(t0 != t1)) return fail(GAL_ERR_INVALID_ARGUMENT, "t0 == t1");
    std::vector<double> ts;
    if (!time_grid(t0, t1, cfg->dt0, cfg->max_steps, ts))
      return fail(GAL_ERR_INVALID_ARGUMENT, "t0 and t1 must be finite and at most max_steps steps of dt0 apart");
    const int np = timed ? 6 : 3;
    const AdjLayout L = adj_layout(pot->n, np, ts, k_ckpt, n);
    if (!workspace || workspace_bytes < L.total) return fail(GAL_ERR_WORKSPACE, "workspace too small");
    char* ws = static_cast<char*>(workspace);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(ws + L.ts, ts.data(), sizeof(double) * ts.size(), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "copying the time grid");
    AdjointArgs a{};
    a.y0 = y0;
    a.lambda = lambda;
    a.target = target;
    a.yT = yT;
    a.grad_y0 = grad_y0;
    a.ts = reinterpret_cast<const double*>(ws + L.ts);
    a.ckpt = reinterpret_cast<double*>(ws + L.ckpt);
    a.seg = reinterpret_cast<double*>(ws + L.seg);
    a.gp_orbit = reinterpret_cast<double*>(ws + L.gp);
    a.nsteps = L.nsteps;
    a.k_ckpt = k_ckpt;
    a.n = n;
    a.lin = pot->d_lin;
    const int block = 64;
    const unsigned grid = (unsigned)((n + block - 1) / block);
    if (timed) {
      const TimedTablePot tp{pot->d_comps, pot->n, pot->d_lin};
      if (cfg->method == 8)
        k_adjoint<Dopri8, TimedTablePot, true><<<grid, block, 0, s>>>(a, tp, pot->d_comps, pot->n);
      else
        k_adjoint<Dopri5, TimedTablePot, true><<<grid, block, 0, s>>>(a, tp, pot->d_comps, pot->n);
    } else if (cfg->method == 8) {
      if (pot->is_mw)
        k_adjoint<Dopri8, MWPot><<<grid, block, 0, s>>>(a, MWPot{pot->mw}, pot->d_comps, pot->n);
      else
        k_adjoint<Dopri8, TablePot><<<grid, block, 0, s>>>(a, TablePot{pot->d_comps, pot->n}, pot->d_comps, pot->n);
    } else {
      if (pot->is_mw)
        k_adjoint<Dopri5, MWPot><<<grid, block, 0, s>>>(a, MWPot{pot->mw}, pot->d_comps, pot->n);
      else
        k_adjoint<Dopri5, TablePot><<<grid, block, 0, s>>>(a, TablePot{pot->d_comps, pot->n}, pot->d_comps, pot->n);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "adjoint kernel launch");
    k_reduce_rows<<<(unsigned)(pot->n * np), 256, 0, s>>>(a.gp_orbit, n, grad_params);
    e = cudaGetLastError();
    return e == cudaSuccess ? GAL_OK : cuda_fail(e, "adjoint reduction launch");
  });
}

}  // extern "C"
