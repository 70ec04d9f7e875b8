// Mock stream with a moving progenitor: the forward simulation and the
// discrete adjoint of the whole pipeline (progenitor orbit -> release
// conditions -> particle orbits -> loss).
//
// Reference pipeline: src/galax/dynamics/_src/experimental/stream.py:121-230
// (StreamSimulator.init: integrate the progenitor back to the first release
// time, then forwards through the release times), stream.py:380-446 (run: every
// particle from its release time to the present), with the progenitor's own
// potential moved along its orbit as legacy/mockstream/_moving.py:20-42 does
// (TimeDependentSpatialTranslationOperator), and the release model built on the
// King (1962) tidal radius (dynamics/_src/cluster/radius.py:198-214,
// r_t = cbrt(G M / (Omega^2 - d2Phi/dr2)); Omega = |x x v| / r^2,
// dynamics/_src/register_api.py:82-88; d2Phi/dr2 = rhat . H . rhat,
// potential/_src/register_funcs.py:444-457). galax differentiates all of it
// with jax (diffrax ForwardMode); here the reverse pass is written out.
//
// Grid. Constant steps dt. The progenitor starts at w_now (time t_now), is
// integrated n_rel steps backwards, then n_rel steps forwards; the forward pass
// records its state P[k] at every grid point and its position Q[k][i] at every
// Runge-Kutta stage i of every step k. Release r (r = 0..n_rel-1) happens at
// grid point r and sends two particles, p = 2r (leading) and 2r + 1 (trailing):
//     x_p = x_r + s r_t rhat + 0.1 r_t xi_p,   v_p = v_r + 0.1 Omega r_t eta_p,
// s = -1 / +1, xi and eta caller-given standard-normal draws. Each particle is
// integrated from grid point r to n_rel in the host potential plus a Plummer
// sphere centred on Q[k][i] at stage i of step k: since the progenitor does not
// feel the particles, this is exactly the particle half of the coupled
// (particle, progenitor) system, with no interpolation of the progenitor track.
//
// Kernels. The progenitor runs on one block whose four warps split each stage
// (it is one serial orbit; see k_stream_progenitor_team); the
// release map on one thread per release; the particles 32 to a block of four
// warps that split each stage the same way (k_stream_particles_team). The
// particle adjoint walks the global step grid backwards in
// lockstep across the warp (a lane joins once the walk reaches its release
// step), so that at every step and stage the warp can sum its lanes'
// cotangents on the progenitor's stage position (mu) with shuffles and write
// one partial per warp; a fixed-order reduction over warps follows, then the
// release-map adjoint (forward-mode dual numbers for d(d2Phi/dr2)) and the
// progenitor adjoint: Hessians at all its stage points in parallel, the serial
// reverse recurrence on one warp (a lane per state component, no potential
// evaluations), and the parameter terms of all stage points in parallel.
// Parameter gradients are written per column and summed in a fixed order, so
// results are bitwise reproducible.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <vector>

#include "handle.h"
#include "integrate.cuh"
#include "vjp.cuh"

namespace gal {

struct StreamDev {
  int64_t n_rel, np, nwarps, ncol;
  double dt, GMp, b2;
  double w_now[6];
  int32_t k_ckpt, ncomp;
  int32_t df;            // release model (GAL_STREAM_DF_*)
  double dfp[8];         // its parameters
  double* B;             // [n_rel + 1][6] backwards progenitor track, B[0] = w_now
  double* P;             // [n_rel + 1][6] forwards progenitor track
  double* Q;             // [n_rel][S][3] progenitor stage positions (forwards track)
  double* Qb;            // [n_rel][S][3] stage positions of the backwards track (gradient only)
  double* Hst;           // [2][n_rel][S][6] host Hessians at both tracks' stage points (xx xy xz yy yz zz)
  double* vst;           // [2][n_rel][S][3] velocity cotangents at those stage points
  double* rt_om;         // [2][n_rel] tidal radius, angular frequency
  const double* noise;   // [12][n_rel] or [4][n_rel] normal draws of the release model
  double* ics;           // [6][np]
  double* fin;           // [6][np]
  double* ckpt;          // [nseg][6][np] (gradient with k_ckpt >= 1)
  double* Ys;            // particle stage positions, Hessians and velocity cotangents at every
  double* Hs;            // stage point (gradient with k_ckpt = 0); step k holds the 2(k+1) released
  double* vs;            // particles: [S][E][2(k+1)] after k(k+1) S E earlier entries (E = 3, 12, 3)
  int64_t pg_col0;       // first gp_all column of the stored-stage parameter partials
  double* seg;           // [K][6][np]
  const double* target;  // [6][np]
  double* lam_rel;       // [6][np] dL/dy_p at the release step
  double* mu_warp;       // [nwarps][n_rel][S * 3]
  double* mu;            // [n_rel][S * 3]
  double* nu;            // [n_rel][6] dL/dP[r] through the release map
  double* gp_all;        // [ncomp * 3 + 1][ncol]: parameter partials per column, last row the loss
                         // (columns: particles, releases, progenitor stage points)
  double* grad_w_now;    // [6] or NULL
};


__device__ __forceinline__ void stage_comps(const DevComp* comps, int ncomp, DevComp* s_comps) {
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) s_comps[i] = comps[i];
  __syncthreads();
}

// Particle field: host potential plus the progenitor's Plummer sphere at q,
// summed in the order of the four-warp particle kernel: partial sum w
// (w = 0..3) holds components w, w + 4, ... and partial 3 also the Plummer
// sphere; the partials are added in order w = 0..3. Recomputed particle steps
// therefore reproduce the forward pass bitwise.
__device__ __forceinline__ void pfield(const DevComp* comps, int ncomp, double GMp, double b2, const double* q,
                                       const double* Y, double* F) {
  double g[4][3];
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    g[w][0] = g[w][1] = g[w][2] = 0.0;
    for (int c = w; c < ncomp; c += 4) comp_grad(comps[c], Y[0], Y[1], Y[2], g[w][0], g[w][1], g[w][2]);
  }
  const double d0 = Y[0] - q[0], d1 = Y[1] - q[1], d2 = Y[2] - q[2];
  const double r2 = fma(d0, d0, fma(d1, d1, fma(d2, d2, TINY)));
  const double is = rsqrt(r2 + b2);
  const double f = GMp * (is * is) * is;
  g[3][0] = fma(f, d0, g[3][0]);
  g[3][1] = fma(f, d1, g[3][1]);
  g[3][2] = fma(f, d2, g[3][2]);
  F[0] = Y[3];
  F[1] = Y[4];
  F[2] = Y[5];
#pragma unroll
  for (int j = 0; j < 3; ++j) F[3 + j] = -(((g[0][j] + g[1][j]) + g[2][j]) + g[3][j]);
}

template <class TB>
__device__ __forceinline__ void particle_step(const DevComp* comps, int ncomp, double GMp, double b2,
                                              const double* Qk, double* y, double hs) {
  double F[TB::S][6];
  pfield(comps, ncomp, GMp, b2, Qk, y, F[0]);
  static_for<1, TB::S>([&](auto i) {
    constexpr int I = decltype(i)::value;
    double Y[6];
    stage_state<TB, I>(y, hs, F, Y);
    pfield(comps, ncomp, GMp, b2, Qk + 3 * I, Y, F[I]);
  });
  double y1[6];
  rk_combine<TB>(y, hs, F, y1, nullptr);
#pragma unroll
  for (int j = 0; j < 6; ++j) y[j] = y1[j];
}

// H v of the Plummer sphere GMp / sqrt(|d|^2 + b^2) at offset d.
__device__ __forceinline__ void plummer_hv(double GMp, double b2, const double* d, const double* v, double* Hv) {
  const double r2 = fma(d[0], d[0], fma(d[1], d[1], fma(d[2], d[2], TINY)));
  const double is = rsqrt(r2 + b2), is2 = is * is;
  const double g = GMp * is2 * is;
  const double gpr = -3.0 * g * is2;
  const double dv = fma(d[0], v[0], fma(d[1], v[1], d[2] * v[2]));
#pragma unroll
  for (int j = 0; j < 3; ++j) Hv[j] = fma(g, v[j], gpr * dv * d[j]);
}

// Stored-stage layout: entry e of stage i of particle p at step k.
__host__ __device__ __forceinline__ int64_t stage_idx(int64_t k, int i, int e, int64_t p, int S, int E) {
  return k * (k + 1) * S * E + ((int64_t)i * E + e) * (2 * (k + 1)) + p;
}

// ------------------------------------------------------------------ forward
// The progenitor on one block of four warps, one per SM sub-partition: a GB300
// FP64 instruction holds its sub-partition's pipe for ~64 cycles however few
// lanes are active, so a single orbit advances faster when the independent
// parts of each stage run on different sub-partitions. Per stage: lanes 0-5 of
// warp 0 form the stage state (one state component each), then the host
// components' gradients run in parallel (component c on lane 0 of warp c % 4),
// then warp 0 sums them in component order into the stage slope. Records the
// same tracks and stage positions as the single-thread kernel.
template <class TB>
__device__ __forceinline__ void team_step(const DevComp* comps, int ncomp, double hs, double* Qk, double* sy,
                                          double (*sF)[6], double* sY, double (*sg)[3], int warp, int lane) {
  constexpr int S = TB::S;
  const bool comb = warp == 0 && lane < 6;
  auto slope = [&](int I) {
    __syncthreads();  // sY complete
    if (lane == 0)
      for (int c = warp; c < ncomp; c += 4) {
        double gx = 0.0, gy = 0.0, gz = 0.0;
        comp_grad(comps[c], sY[0], sY[1], sY[2], gx, gy, gz);
        sg[c][0] = gx;
        sg[c][1] = gy;
        sg[c][2] = gz;
      }
    __syncthreads();  // sg complete
    if (comb) {
      double f;
      if (lane < 3) {
        f = sY[lane + 3];
      } else {
        double g = 0.0;
        for (int c = 0; c < ncomp; ++c) g += sg[c][lane - 3];
        f = -g;
      }
      sF[I][lane] = f;
      if (Qk && lane < 3) Qk[3 * I + lane] = sY[lane];
    }
  };
  if (comb) sY[lane] = sy[lane];
  slope(0);
  static_for<1, S>([&](auto i) {
    constexpr int I = decltype(i)::value;
    __syncthreads();  // sF[I-1] written, sY free for reuse
    if (comb) {
      double acc = 0.0;
      bool first = true;
      static_for<0, I>([&](auto l) {
        constexpr int L = decltype(l)::value;
        constexpr double c = TB::A[I][L];
        if constexpr (c != 0.0) {
          acc = first ? c * sF[L][lane] : fma(c, sF[L][lane], acc);
          first = false;
        }
      });
      sY[lane] = fma(hs, acc, sy[lane]);
    }
    slope(I);
  });
  __syncthreads();
  if (comb) {
    double acc = 0.0;
    bool first = true;
    static_for<0, S>([&](auto l) {
      constexpr int L = decltype(l)::value;
      constexpr double c = TB::B[L];
      if constexpr (c != 0.0) {
        acc = first ? c * sF[L][lane] : fma(c, sF[L][lane], acc);
        first = false;
      }
    });
    sy[lane] = fma(hs, acc, sy[lane]);
  }
  __syncthreads();
}

// team_step for a Milky Way host: the gradient split as in the integrators'
// four-warp teams (warp 0: radius and shared reciprocal, warp 1: NFW log,
// warp 3: disk; mw_* pieces), combined on lanes 0-2 of warp 0. The NFW log,
// the longest chain, no longer shares a warp with the rest of its component.
template <class TB>
__device__ __forceinline__ void team_step_mw(const MWParams& p, double hs, double* Qk, double* sy,
                                             double (*sF)[6], double* sY, double* sw, int warp, int lane) {
  constexpr int S = TB::S;
  const bool comb = warp == 0 && lane < 6;
  // sw: [0] ir, [1] inv_dh, [2] inv_db2, [3] inv_dn2, [4] L, [5] u, [6] us, [7] izb
  auto slope = [&](int I) {
    __syncthreads();  // sY complete
    if (lane == 0) {
      const double x = sY[0], y = sY[1], z = sY[2];
      if (warp == 0) {
        double r;
        const double ir = mw_ir(x, y, z, r);
        const MWRecip c = mw_recip(p, r);
        sw[0] = ir;
        sw[1] = c.inv_dh;
        sw[2] = c.inv_db2;
        sw[3] = c.inv_dn2;
      } else if (warp == 1) {
        double r;
        mw_ir(x, y, z, r);
        sw[4] = mw_halo_log(p, r);
      } else if (warp == 3) {
        const MWDisk d = mw_disk(p, x, y, z);
        sw[5] = d.u;
        sw[6] = d.us;
        sw[7] = d.izb;
      }
    }
    __syncthreads();  // pieces complete
    if (comb) {
      double f;
      if (lane < 3) {
        f = sY[lane + 3];
      } else {
        const MWRecip c{sw[1], sw[2], sw[3]};
        const double fr = mw_f(p, sw[0], sw[4], c);
        const int j = lane - 3;
        const double g = (j == 2) ? fma(sw[6], sw[7], fr) * sY[2] : (sw[5] + fr) * sY[j];
        f = -g;
      }
      sF[I][lane] = f;
      if (Qk && lane < 3) Qk[3 * I + lane] = sY[lane];
    }
  };
  if (comb) sY[lane] = sy[lane];
  slope(0);
  static_for<1, S>([&](auto i) {
    constexpr int I = decltype(i)::value;
    __syncthreads();  // sF[I-1] written, sY free for reuse
    if (comb) {
      double acc = 0.0;
      bool first = true;
      static_for<0, I>([&](auto l) {
        constexpr int L = decltype(l)::value;
        constexpr double c = TB::A[I][L];
        if constexpr (c != 0.0) {
          acc = first ? c * sF[L][lane] : fma(c, sF[L][lane], acc);
          first = false;
        }
      });
      sY[lane] = fma(hs, acc, sy[lane]);
    }
    slope(I);
  });
  __syncthreads();
  if (comb) {
    double acc = 0.0;
    bool first = true;
    static_for<0, S>([&](auto l) {
      constexpr int L = decltype(l)::value;
      constexpr double c = TB::B[L];
      if constexpr (c != 0.0) {
        acc = first ? c * sF[L][lane] : fma(c, sF[L][lane], acc);
        first = false;
      }
    });
    sy[lane] = fma(hs, acc, sy[lane]);
  }
  __syncthreads();
}

template <class TB>
__global__ void __launch_bounds__(128) k_stream_progenitor_mw(StreamDev a, MWParams p) {
  __shared__ double sy[6], sY[6], sF[TB::S][6], sw[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < 6) {
    sy[threadIdx.x] = a.w_now[threadIdx.x];
    a.B[threadIdx.x] = sy[threadIdx.x];
  }
  __syncthreads();
  for (int64_t k = 0; k < a.n_rel; ++k) {
    team_step_mw<TB>(p, -a.dt, a.Qb ? a.Qb + k * TB::S * 3 : nullptr, sy, sF, sY, sw, warp, lane);
    if (threadIdx.x < 6) a.B[(k + 1) * 6 + threadIdx.x] = sy[threadIdx.x];
  }
  if (threadIdx.x < 6) a.P[threadIdx.x] = sy[threadIdx.x];
  for (int64_t k = 0; k < a.n_rel; ++k) {
    team_step_mw<TB>(p, a.dt, a.Q + k * TB::S * 3, sy, sF, sY, sw, warp, lane);
    if (threadIdx.x < 6) a.P[(k + 1) * 6 + threadIdx.x] = sy[threadIdx.x];
  }
}

template <class TB>
__global__ void __launch_bounds__(128) k_stream_progenitor_team(StreamDev a, const DevComp* comps) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  __shared__ double sy[6], sY[6], sF[TB::S][6], sg[kAdjMaxComps][3];
  stage_comps(comps, a.ncomp, s_comps);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < 6) {
    sy[threadIdx.x] = a.w_now[threadIdx.x];
    a.B[threadIdx.x] = sy[threadIdx.x];
  }
  __syncthreads();
  for (int64_t k = 0; k < a.n_rel; ++k) {
    team_step<TB>(s_comps, a.ncomp, -a.dt, a.Qb ? a.Qb + k * TB::S * 3 : nullptr, sy, sF, sY, sg, warp, lane);
    if (threadIdx.x < 6) a.B[(k + 1) * 6 + threadIdx.x] = sy[threadIdx.x];
  }
  if (threadIdx.x < 6) a.P[threadIdx.x] = sy[threadIdx.x];
  for (int64_t k = 0; k < a.n_rel; ++k) {
    team_step<TB>(s_comps, a.ncomp, a.dt, a.Q + k * TB::S * 3, sy, sF, sY, sg, warp, lane);
    if (threadIdx.x < 6) a.P[(k + 1) * 6 + threadIdx.x] = sy[threadIdx.x];
  }
}


// Particles on teams of four warps: block b integrates particles 32b .. 32b+31
// (one per lane). Warps 0-2 own state components (w, w+3) of their lane's
// particle and form the stage states; every warp evaluates its share of the
// host components (component c on warp c % 4) and warp 3 also the progenitor's
// Plummer sphere; warps 0-2 then sum the four partial gradients in warp order.
// A lane joins when the global step reaches its release step. Writes the final
// states and either the checkpoints or the stored stage positions.
template <class TB>
__global__ void __launch_bounds__(128) k_stream_particles_team(StreamDev a, const DevComp* comps) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  __shared__ double sY[3][32], sg[4][3][32];
  stage_comps(comps, a.ncomp, s_comps);
  constexpr int S = TB::S;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t p = (int64_t)blockIdx.x * 32 + lane;
  const int64_t n = a.np;
  const bool valid = p < n;
  const int64_t rp = valid ? (p >> 1) : LLONG_MAX;
  const int64_t rmin = ((int64_t)blockIdx.x * 32) >> 1;
  const bool own = warp < 3;
  const int j0 = warp, j1 = warp + 3;  // state components owned by warps 0-2
  const int K = a.k_ckpt;
  double y0 = 0.0, y1 = 0.0;  // this warp's two components of the lane's particle
  if (own) {  // lanes past the last particle follow a circular-ish orbit at 8 kpc
    y0 = valid ? a.ics[j0 * n + p] : (j0 == 0 ? 8.0 : 0.0);
    y1 = valid ? a.ics[j1 * n + p] : (j1 == 4 ? 0.2 : 0.0);
  }
  for (int64_t k = rmin; k < a.n_rel; ++k) {
    const bool act = valid && k >= rp;
    if (own && act && a.ckpt && (k == rp || k % K == 0)) {
      const int64_t g = k / K;
      a.ckpt[(g * 6 + j0) * n + p] = y0;
      a.ckpt[(g * 6 + j1) * n + p] = y1;
    }
    const double* Qk = a.Q + k * S * 3;
    double F0[S] = {}, F1[S] = {};  // this warp's components of the stage slopes
    static_for<0, S>([&](auto i) {
      constexpr int I = decltype(i)::value;
      double Y0 = y0, Y1 = y1;
      if (own && I > 0) {
        double c0 = 0.0, c1 = 0.0;
        bool first = true;
        static_for<0, I>([&](auto l) {
          constexpr int L = decltype(l)::value;
          constexpr double c = TB::A[I][L];
          if constexpr (c != 0.0) {
            c0 = first ? c * F0[L] : fma(c, F0[L], c0);
            c1 = first ? c * F1[L] : fma(c, F1[L], c1);
            first = false;
          }
        });
        Y0 = fma(a.dt, c0, y0);
        Y1 = fma(a.dt, c1, y1);
      }
      if (own) {
        sY[j0][lane] = Y0;
        if (a.Ys && act) a.Ys[stage_idx(k, I, j0, p, S, 3)] = Y0;
      }
      __syncthreads();
      const double x0 = sY[0][lane], x1 = sY[1][lane], x2 = sY[2][lane];
      double gx = 0.0, gy = 0.0, gz = 0.0;
      for (int c = warp; c < a.ncomp; c += 4) comp_grad(s_comps[c], x0, x1, x2, gx, gy, gz);
      if (warp == 3) {  // the progenitor's Plummer sphere at its stage position
        const double d0 = x0 - Qk[3 * I], d1 = x1 - Qk[3 * I + 1], d2 = x2 - Qk[3 * I + 2];
        const double r2 = fma(d0, d0, fma(d1, d1, fma(d2, d2, TINY)));
        const double is = rsqrt(r2 + a.b2);
        const double f = a.GMp * (is * is) * is;
        gx = fma(f, d0, gx);
        gy = fma(f, d1, gy);
        gz = fma(f, d2, gz);
      }
      sg[warp][0][lane] = gx;
      sg[warp][1][lane] = gy;
      sg[warp][2][lane] = gz;
      __syncthreads();
      if (own) {
        F0[I] = Y1;  // dq/dt = p
        F1[I] = -(((sg[0][j0][lane] + sg[1][j0][lane]) + sg[2][j0][lane]) + sg[3][j0][lane]);
      }
    });
    if (own && act) {
      double c0 = 0.0, c1 = 0.0;
      bool first = true;
      static_for<0, S>([&](auto l) {
        constexpr int L = decltype(l)::value;
        constexpr double c = TB::B[L];
        if constexpr (c != 0.0) {
          c0 = first ? c * F0[L] : fma(c, F0[L], c0);
          c1 = first ? c * F1[L] : fma(c, F1[L], c1);
          first = false;
        }
      });
      y0 = fma(a.dt, c0, y0);
      y1 = fma(a.dt, c1, y1);
    }
  }
  if (own && valid) {
    a.fin[j0 * n + p] = y0;
    a.fin[j1 * n + p] = y1;
  }
}

// ------------------------------------------------------------------ adjoint
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

template <class TB>
__global__ void __launch_bounds__(32) k_stream_particles_adj(StreamDev a, const DevComp* comps) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  stage_comps(comps, a.ncomp, s_comps);
  constexpr int S = TB::S;
  const int lane = threadIdx.x;
  const int64_t w = blockIdx.x;
  const int64_t p = w * 32 + lane;
  const int64_t n = a.np;
  const bool valid = p < n;
  const int64_t rp = valid ? (p >> 1) : LLONG_MAX;
  const int64_t rmin = (w * 32) >> 1;
  const int K = a.k_ckpt;
  const int ncomp = a.ncomp;
  const double dt = a.dt;
  double lam[6], loss = 0.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double d = valid ? a.fin[j * n + p] - a.target[j * n + p] : 0.0;
    lam[j] = 2.0 * d;
    loss = fma(d, d, loss);
  }
  double gp[kAdjMaxComps * 3];
#pragma unroll
  for (int i = 0; i < kAdjMaxComps * 3; ++i) gp[i] = 0.0;
  const int64_t nseg = (a.n_rel + K - 1) / K;
  for (int64_t g = nseg - 1; g >= rmin / K; --g) {
    const int64_t k0 = g * K;
    const int64_t k1 = (k0 + K < a.n_rel) ? k0 + K : a.n_rel;
    if (valid && rp < k1) {
      const int64_t ks = rp > k0 ? rp : k0;
      double y[6];
#pragma unroll
      for (int j = 0; j < 6; ++j) y[j] = a.ckpt[(g * 6 + j) * n + p];
      for (int64_t k = ks; k < k1; ++k) {
#pragma unroll
        for (int j = 0; j < 6; ++j) a.seg[((k - k0) * 6 + j) * n + p] = y[j];
        if (k + 1 < k1) particle_step<TB>(s_comps, ncomp, a.GMp, a.b2, a.Q + k * S * 3, y, dt);
      }
    }
    const int64_t kstop = k0 > rmin ? k0 : rmin;
    for (int64_t k = k1 - 1; k >= kstop; --k) {
      const bool act = valid && k >= rp;
      const double* Qk = a.Q + k * S * 3;
      double yk[6] = {8.0, 0.0, 0.0, 0.0, 0.2, 0.0};  // finite stand-in for lanes not yet released
      if (act) {
#pragma unroll
        for (int j = 0; j < 6; ++j) yk[j] = a.seg[((k - k0) * 6 + j) * n + p];
      }
      double F[S][6], Yq[S][3];
      pfield(s_comps, ncomp, a.GMp, a.b2, Qk, yk, F[0]);
      Yq[0][0] = yk[0];
      Yq[0][1] = yk[1];
      Yq[0][2] = yk[2];
      static_for<1, S>([&](auto i) {
        constexpr int I = decltype(i)::value;
        double Y[6];
        stage_state<TB, I>(yk, dt, F, Y);
        Yq[I][0] = Y[0];
        Yq[I][1] = Y[1];
        Yq[I][2] = Y[2];
        pfield(s_comps, ncomp, a.GMp, a.b2, Qk + 3 * I, Y, F[I]);
      });
      static_for<0, S>([&](auto i) {
        constexpr int I = decltype(i)::value;
        constexpr double bi = TB::B[I];
#pragma unroll
        for (int j = 0; j < 6; ++j) F[I][j] = dt * bi * lam[j];
      });
      double* mw_out = a.mu_warp + (w * a.n_rel + k) * (S * 3);
      static_for<0, S>([&](auto rr) {
        constexpr int I = S - 1 - decltype(rr)::value;
        const double v[3] = {F[I][3], F[I][4], F[I][5]};
        double Hv[3] = {0.0, 0.0, 0.0};
        for (int c = 0; c < ncomp; ++c) {
          double dp[3] = {0.0, 0.0, 0.0};
          comp_vjp(s_comps[c], Yq[I], v, Hv, dp);
          if (act) {
            gp[3 * c + 0] -= dp[0];
            gp[3 * c + 1] -= dp[1];
            gp[3 * c + 2] -= dp[2];
          }
        }
        const double d[3] = {Yq[I][0] - Qk[3 * I], Yq[I][1] - Qk[3 * I + 1], Yq[I][2] - Qk[3 * I + 2]};
        double Hp[3];
        plummer_hv(a.GMp, a.b2, d, v, Hp);
        // cotangent on the progenitor's stage position: +H_prog v, summed over the warp
        const double m0 = warp_sum(act ? Hp[0] : 0.0);
        const double m1 = warp_sum(act ? Hp[1] : 0.0);
        const double m2 = warp_sum(act ? Hp[2] : 0.0);
        if (lane == 0) {
          mw_out[3 * I + 0] = m0;
          mw_out[3 * I + 1] = m1;
          mw_out[3 * I + 2] = m2;
        }
        const double Yb[6] = {-(Hv[0] + Hp[0]), -(Hv[1] + Hp[1]), -(Hv[2] + Hp[2]), F[I][0], F[I][1], F[I][2]};
        if (act) {
#pragma unroll
          for (int j = 0; j < 6; ++j) lam[j] += Yb[j];
        }
        static_for<0, I>([&](auto l) {
          constexpr int L = decltype(l)::value;
          constexpr double c = TB::A[I][L];
          if constexpr (c != 0.0) {
#pragma unroll
            for (int j = 0; j < 6; ++j) F[L][j] = fma(dt * c, Yb[j], F[L][j]);
          }
        });
      });
      if (valid && k == rp) {
#pragma unroll
        for (int j = 0; j < 6; ++j) a.lam_rel[j * n + p] = lam[j];
      }
    }
  }
  if (valid) {
    for (int c = 0; c < 3 * ncomp; ++c) a.gp_all[(int64_t)c * a.ncol + p] = gp[c];
    a.gp_all[(int64_t)(3 * ncomp) * a.ncol + p] = loss;
  }
}

// ---- stored-stage particle adjoint (k_ckpt = 0)
// (k, p) of particle-step q in the stored layout: step k holds particles 0 .. 2k+1
__device__ __forceinline__ void particle_step_of(int64_t q, int64_t& k, int64_t& p) {
  int64_t kk = (int64_t)((sqrt(4.0 * (double)q + 1.0) - 1.0) * 0.5);
  while ((kk + 1) * (kk + 2) <= q) ++kk;
  while (kk * (kk + 1) > q) --kk;
  k = kk;
  p = q - kk * (kk + 1);
}

// Hessians at every particle stage point: host + progenitor (0..5) and progenitor alone (6..11).
template <class TB>
__global__ void __launch_bounds__(128) k_stream_particle_hess(StreamDev a, const DevComp* comps) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  stage_comps(comps, a.ncomp, s_comps);
  constexpr int S = TB::S;
  const int64_t nq = a.n_rel * (a.n_rel + 1);
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nq) return;
  int64_t k, p;
  particle_step_of(q, k, p);
  for (int i = 0; i < S; ++i) {
    const double Y[3] = {a.Ys[stage_idx(k, i, 0, p, S, 3)], a.Ys[stage_idx(k, i, 1, p, S, 3)],
                         a.Ys[stage_idx(k, i, 2, p, S, 3)]};
    double H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < a.ncomp; ++c) comp_hessian(s_comps[c], Y[0], Y[1], Y[2], H);
    const double* Qi = a.Q + (k * S + i) * 3;
    const double d[3] = {Y[0] - Qi[0], Y[1] - Qi[1], Y[2] - Qi[2]};
    const double r2 = fma(d[0], d[0], fma(d[1], d[1], fma(d[2], d[2], TINY)));
    const double is = rsqrt(r2 + a.b2), is2 = is * is;
    const double g = a.GMp * is2 * is, gpr = -3.0 * g * is2;
    const double Hp[6] = {fma(gpr * d[0], d[0], g), gpr * d[0] * d[1], gpr * d[0] * d[2],
                          fma(gpr * d[1], d[1], g), gpr * d[1] * d[2], fma(gpr * d[2], d[2], g)};
    const double Ht[6] = {H[0] + Hp[0], H[1] + Hp[1], H[2] + Hp[2], H[4] + Hp[3], H[5] + Hp[4], H[8] + Hp[5]};
#pragma unroll
    for (int e = 0; e < 6; ++e) {
      a.Hs[stage_idx(k, i, e, p, S, 12)] = Ht[e];
      a.Hs[stage_idx(k, i, 6 + e, p, S, 12)] = Hp[e];
    }
  }
}

__device__ __forceinline__ void sym_mv(const double* H, const double* v, double* o) {
  o[0] = fma(H[0], v[0], fma(H[1], v[1], H[2] * v[2]));
  o[1] = fma(H[1], v[0], fma(H[3], v[1], H[4] * v[2]));
  o[2] = fma(H[2], v[0], fma(H[4], v[1], H[5] * v[2]));
}

// Reverse sweep with the stored Hessians: no potential evaluations on the serial chain.
template <class TB>
__global__ void __launch_bounds__(32) k_stream_particles_sweep(StreamDev a) {
  constexpr int S = TB::S;
  const int lane = threadIdx.x;
  const int64_t w = blockIdx.x;
  const int64_t p = w * 32 + lane;
  const int64_t n = a.np;
  const bool valid = p < n;
  const int64_t rp = valid ? (p >> 1) : LLONG_MAX;
  const int64_t rmin = (w * 32) >> 1;
  const double dt = a.dt;
  double lam[6], loss = 0.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double d = valid ? a.fin[j * n + p] - a.target[j * n + p] : 0.0;
    lam[j] = 2.0 * d;
    loss = fma(d, d, loss);
  }
  for (int64_t k = a.n_rel - 1; k >= rmin; --k) {
    const bool act = valid && k >= rp;
    double F[S][6];
    static_for<0, S>([&](auto i) {
      constexpr int I = decltype(i)::value;
      constexpr double bi = TB::B[I];
#pragma unroll
      for (int j = 0; j < 6; ++j) F[I][j] = dt * bi * lam[j];
    });
    double* mw_out = a.mu_warp + (w * a.n_rel + k) * (S * 3);
    static_for<0, S>([&](auto rr) {
      constexpr int I = S - 1 - decltype(rr)::value;
      const double v[3] = {F[I][3], F[I][4], F[I][5]};
      double Ht[6] = {0, 0, 0, 0, 0, 0}, Hp[6] = {0, 0, 0, 0, 0, 0};
      if (act) {
#pragma unroll
        for (int e = 0; e < 6; ++e) {
          Ht[e] = a.Hs[stage_idx(k, I, e, p, S, 12)];
          Hp[e] = a.Hs[stage_idx(k, I, 6 + e, p, S, 12)];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) a.vs[stage_idx(k, I, c, p, S, 3)] = v[c];
      }
      double Hv[3], Hpv[3];
      sym_mv(Ht, v, Hv);
      sym_mv(Hp, v, Hpv);
      const double m0 = warp_sum(act ? Hpv[0] : 0.0);
      const double m1 = warp_sum(act ? Hpv[1] : 0.0);
      const double m2 = warp_sum(act ? Hpv[2] : 0.0);
      if (lane == 0) {
        mw_out[3 * I + 0] = m0;
        mw_out[3 * I + 1] = m1;
        mw_out[3 * I + 2] = m2;
      }
      const double Yb[6] = {-Hv[0], -Hv[1], -Hv[2], F[I][0], F[I][1], F[I][2]};
      if (act) {
#pragma unroll
        for (int j = 0; j < 6; ++j) lam[j] += Yb[j];
      }
      static_for<0, I>([&](auto l) {
        constexpr int L = decltype(l)::value;
        constexpr double c = TB::A[I][L];
        if constexpr (c != 0.0) {
#pragma unroll
          for (int j = 0; j < 6; ++j) F[L][j] = fma(dt * c, Yb[j], F[L][j]);
        }
      });
    });
    if (valid && k == rp) {
#pragma unroll
      for (int j = 0; j < 6; ++j) a.lam_rel[j * n + p] = lam[j];
    }
  }
  if (valid) {
    for (int c = 0; c < 3 * a.ncomp; ++c) a.gp_all[(int64_t)c * a.ncol + p] = 0.0;
    a.gp_all[(int64_t)(3 * a.ncomp) * a.ncol + p] = loss;
  }
}

// Parameter terms -sum d(grad Phi_host . v)/dtheta over all particle stage points,
// one column of partial sums per block.
template <class TB>
__global__ void __launch_bounds__(256) k_stream_particles_pgrad(StreamDev a, const DevComp* comps) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  __shared__ double red[kAdjMaxComps * 3][8];
  stage_comps(comps, a.ncomp, s_comps);
  constexpr int S = TB::S;
  const int64_t nq = a.n_rel * (a.n_rel + 1);
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int nc3 = 3 * a.ncomp;
  double acc[kAdjMaxComps * 3];
#pragma unroll
  for (int i = 0; i < kAdjMaxComps * 3; ++i) acc[i] = 0.0;
  if (q < nq) {
    int64_t k, p;
    particle_step_of(q, k, p);
    for (int i = 0; i < S; ++i) {
      const double Y[3] = {a.Ys[stage_idx(k, i, 0, p, S, 3)], a.Ys[stage_idx(k, i, 1, p, S, 3)],
                           a.Ys[stage_idx(k, i, 2, p, S, 3)]};
      const double v[3] = {a.vs[stage_idx(k, i, 0, p, S, 3)], a.vs[stage_idx(k, i, 1, p, S, 3)],
                           a.vs[stage_idx(k, i, 2, p, S, 3)]};
      for (int c = 0; c < a.ncomp; ++c) {
        double Hv[3] = {0, 0, 0}, dp[3] = {0, 0, 0};
        comp_vjp(s_comps[c], Y, v, Hv, dp);
        acc[3 * c + 0] -= dp[0];
        acc[3 * c + 1] -= dp[1];
        acc[3 * c + 2] -= dp[2];
      }
    }
  }
  // warp sums, then the block's eight warps in order
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = 0; c < nc3; ++c) {
    const double v = warp_sum(acc[c]);
    if (lane == 0) red[c][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < nc3) {
    double t = 0.0;
    for (int j = 0; j < (int)(blockDim.x >> 5); ++j) t += red[threadIdx.x][j];
    a.gp_all[(int64_t)threadIdx.x * a.ncol + a.pg_col0 + blockIdx.x] = t;
  }
  if (threadIdx.x == 0) a.gp_all[(int64_t)nc3 * a.ncol + a.pg_col0 + blockIdx.x] = 0.0;
}

// mu[k][:] = sum over the warps that had released particles by step k, in warp order.
__global__ void k_stream_mu_reduce(StreamDev a, int S3) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= a.n_rel * S3) return;
  const int64_t k = idx / S3;
  int64_t wmax = k / 16;
  if (wmax > a.nwarps - 1) wmax = a.nwarps - 1;
  double s = 0.0;
  for (int64_t w = 0; w <= wmax; ++w) s += a.mu_warp[w * a.n_rel * S3 + idx];
  a.mu[idx] = s;
}

// Forward-mode dual numbers (value + N tangents) for the release-map adjoint.
template <int N>
struct Dual {
  double v, d[N];
  __device__ Dual() : v(0.0) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  __device__ Dual(double x) : v(x) {  // NOLINT: implicit promotion of constants
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
};
template <int N>
__device__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v + b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__device__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v - b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__device__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r(-a.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
__device__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v * b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = fma(a.d[i], b.v, a.v * b.d[i]);
  return r;
}
template <int N>
__device__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  const double ib = 1.0 / b.v;
  Dual<N> r(a.v * ib);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N>
__device__ Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N>
__device__ Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N>
__device__ Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N>
__device__ Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N>
__device__ Dual<N> operator*(const Dual<N>& a, double b) { return a * Dual<N>(b); }
template <int N>
__device__ Dual<N> operator*(double a, const Dual<N>& b) { return Dual<N>(a) * b; }
template <int N>
__device__ Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N>
__device__ Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N>
__device__ Dual<N> sqrt(const Dual<N>& a) {
  const double s = ::sqrt(a.v);
  Dual<N> r(s);
  const double f = 0.5 / s;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = f * a.d[i];
  return r;
}
template <int N>
__device__ Dual<N> log1p(const Dual<N>& a) {
  Dual<N> r(::log1p(a.v));
  const double f = 1.0 / (1.0 + a.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = f * a.d[i];
  return r;
}

// The power law with cutoff's radial factors g (grad Phi = g x) and g'(r)/r,
// and their partial derivatives in r^2, G m, r_c and alpha, at the
// component's parameters (cc's folded constants: 1 / r_c^2, 1 / Gamma(a1),
// psi(a1)). With x = r^2 / r_c^2, a1 = 3/2 - alpha/2, P = gamma(a1, x) /
// Gamma(a1) and eN = x^a1 e^-x / Gamma(a1):
//   g = G m P r^-3,  g'/r = 2 G m eN r^-5 - 3 g r^-2,
//   dP/dx = eN / x,  deN/dx = eN (a1 / x - 1),  deN/da1 = eN (log x - psi(a1)),
//   dP/da1 from the series or continued fraction's a-derivative (as in plc_g).
struct PlcHess {
  double g, gpr;
  double g_r2, g_gm, g_rc, g_al;      // dg / d(r^2, G m, r_c, alpha)
  double p_r2, p_gm, p_rc, p_al;      // d(g'/r) / d(...)
};

__device__ __noinline__ PlcHess plc_hess(const DevComp& c, double Gm, double rc, double r2) {
  const double a1 = fma(-0.5, c.l2, 1.5);
  const double irc2 = c.inv_l1;
  const double x = r2 * irc2;
  const IncGamma ig = inc_gamma(a1, x, true);
  const double eN = ig.e * c.l2sq;
  const double P = ig.series ? eN * ig.sum : 1.0 - eN * ig.sum;
  const double dPda = ig.series ? fma(eN, fma(ig.lx, ig.sum, ig.dsum), -P * c.aux0)
                                : -fma(eN, fma(ig.lx, ig.sum, ig.dsum), -(1.0 - P) * c.aux0);
  const double ir = 1.0 / ::sqrt(r2), ir2 = ir * ir, ir3 = ir2 * ir, ir5 = ir3 * ir2, ir7 = ir5 * ir2;
  const double dPdx = eN / x, deNdx = eN * (a1 / x - 1.0), deNda = eN * (ig.lx - c.aux0);
  PlcHess o;
  o.g = Gm * P * ir3;
  o.gpr = 2.0 * Gm * eN * ir5 - 3.0 * o.g * ir2;
  o.g_r2 = Gm * (dPdx * irc2 * ir3 - 1.5 * P * ir5);
  o.g_gm = P * ir3;
  o.g_rc = Gm * eN * (-2.0 / rc) * ir3;          // dx/dr_c = -2 x / r_c
  o.g_al = Gm * dPda * (-0.5) * ir3;              // da1/dalpha = -1/2
  o.p_r2 = 2.0 * Gm * (deNdx * irc2 * ir5 - 2.5 * eN * ir7) - 3.0 * (o.g_r2 * ir2 - o.g * ir2 * ir2);
  o.p_gm = 2.0 * eN * ir5 - 3.0 * o.g_gm * ir2;
  o.p_rc = 2.0 * Gm * deNdx * (-2.0 * x / rc) * ir5 - 3.0 * o.g_rc * ir2;
  o.p_al = 2.0 * Gm * deNda * (-0.5) * ir5 - 3.0 * o.g_al * ir2;
  return o;
}

__device__ __forceinline__ void plc_radial(const DevComp& c, double Gm, double rc, double al, double r2, double& g,
                                           double& gpr) {
  const PlcHess h = plc_hess(c, Gm, rc, r2);
  g = h.g;
  gpr = h.gpr;
}
template <int N>
__device__ void plc_radial(const DevComp& c, const Dual<N>& Gm, const Dual<N>& rc, const Dual<N>& al,
                           const Dual<N>& r2, Dual<N>& g, Dual<N>& gpr) {
  const PlcHess h = plc_hess(c, Gm.v, rc.v, r2.v);
  g = Dual<N>(h.g);
  gpr = Dual<N>(h.gpr);
#pragma unroll
  for (int i = 0; i < N; ++i) {
    g.d[i] = h.g_r2 * r2.d[i] + h.g_gm * Gm.d[i] + h.g_rc * rc.d[i] + h.g_al * al.d[i];
    gpr.d[i] = h.p_r2 * r2.d[i] + h.p_gm * Gm.d[i] + h.p_rc * rc.d[i] + h.p_al * al.d[i];
  }
}

// Hessian of one component at offset d from its centre (same closed forms as
// comp_hessian), generic in the number type so parameters and positions can
// carry tangents. cc: the component (the power law with cutoff reads its
// folded constants; its parameters' tangents come from Gm, l1, l2).
template <class T>
__device__ void comp_hessian_t(const DevComp& cc, int kind, const T& Gm, const T& l1, const T& l2, const T* d,
                               T* H) {
  if (kind == MIYAMOTO_NAGAI) {
    const T zb = sqrt(d[2] * d[2] + l2 * l2);
    const T s = zb + l1;
    const T D2 = d[0] * d[0] + d[1] * d[1] + s * s;
    const T D = sqrt(D2);
    const T u = Gm / (D2 * D);
    const T w = 3.0 * Gm / (D2 * D2 * D);
    const T v[3] = {d[0], d[1], d[2] * s / zb};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) H[3 * i + j] = H[3 * i + j] - w * v[i] * v[j];
    H[0] = H[0] + u;
    H[4] = H[4] + u;
    H[8] = H[8] + u * (1.0 + l1 * l2 * l2 / (zb * zb * zb));
    return;
  }
  const T r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + TINY;
  const T r = sqrt(r2);
  T g, gpr;
  if (kind == KEPLER) {
    g = Gm / (r2 * r);
    gpr = -3.0 * Gm / (r2 * r2 * r);
  } else if (kind == HERNQUIST) {
    const T dd = r + l1;
    g = Gm / (r * dd * dd);
    gpr = -Gm * (3.0 * r + l1) / (r2 * r * dd * dd * dd);
  } else if (kind == NFW) {
    const T Lg = log1p(r / l1), q = l1 + r;
    g = Gm * (Lg / (r2 * r) - 1.0 / (r2 * q));
    gpr = Gm * (3.0 / (r2 * r2 * q) - 3.0 * Lg / (r2 * r2 * r) + 1.0 / (r2 * r * q * q));
  } else if (kind == ISOCHRONE) {
    const T s2 = r2 + l1 * l1, s = sqrt(s2), d = l1 + s;
    g = Gm / (d * d * s);
    gpr = -g * (2.0 / (d * s) + 1.0 / s2);
  } else if (kind == LOGARITHMIC) {
    const T q = r2 + l1 * l1;
    g = Gm / q;
    gpr = -2.0 * g / q;
  } else if (kind == POWERLAW_CUTOFF) {
    plc_radial(cc, Gm, l1, l2, r2, g, gpr);
  } else {  // PLUMMER
    const T s2 = r2 + l1 * l1, s = sqrt(s2);
    g = Gm / (s2 * s);
    gpr = -3.0 * Gm / (s2 * s2 * s);
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) H[3 * i + j] = H[3 * i + j] + gpr * d[i] * d[j];
  H[0] = H[0] + g;
  H[4] = H[4] + g;
  H[8] = H[8] + g;
}

template <class T>
__device__ T contract_rhat(const T* H, const T* rh) {
  T s(0.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) s = s + rh[i] * H[3 * i + j] * rh[j];
  return s;
}

__device__ __forceinline__ double vsqrt(double x) { return ::sqrt(x); }
constexpr double kChenRho = 0.71414284285428499980;  // sqrt(1 - 0.7^2)
template <int N>
__device__ __forceinline__ Dual<N> vsqrt(const Dual<N>& x) {
  return sqrt(x);
}

// Release conditions of release r's two particles (out[0] leading, s = -1;
// out[1] trailing, s = +1) from the progenitor point (x, v), its tidal radius
// rt and angular frequency om; T = double, or dual numbers for the adjoint.
// noise[q * stride + r] is draw q of release r.
//   DF_OFFSETS:    x + s rt rhat + 0.1 rt xi,  v + 0.1 om rt eta (12 draws)
//   DF_FARDAL2015: kr = kr_bar + s_kr n0, kvphi = kr (kvphi_bar + s_kvphi n1),
//                  kz = kz_bar + s_kz n2, kvz = kvz_bar + s_kvz n3;
//                  x + rt (s kr rhat + kz zhat),  v + om rt (s kvphi phihat + kvz zhat)
//                  with zhat along x cross v and phihat along v - (v.rhat) rhat
//                  (legacy/mockstream/df/fardal15.py:62-94, experimental/df.py:148-177;
//                  both particles share the four draws).
//   DF_CHEN2024:   posvel = mean + A z from six standard-normal draws z, A the
//                  lower-triangular factor of galax's covariance (only posvel_0
//                  and posvel_4 are correlated, coefficient -0.7; posvel_3 has
//                  no spread), then Dr = posvel_0 rt, Dv = posvel_3
//                  sqrt(2 GM / Dr), angles phi, theta, alpha, beta = posvel_1,2,4,5
//                  in degrees; x +/- Dr (ct cp xhat + ct sp yhat) + Dr st zhat,
//                  v +/- Dv (cb ca xhat + cb sa yhat) + Dv sb zhat (+ trailing,
//                  - leading; legacy/mockstream/df/chen24.py:21-137).
template <class T>
__device__ void release_pair(int df, const double* dfp, const double* noise, int64_t stride, int64_t r, const T* x,
                             const T* v, const T& rt, const T& om, double GM, T (*out)[6]) {
  const T rr = vsqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  const T rh[3] = {x[0] / rr, x[1] / rr, x[2] / rr};
  if (df == GAL_STREAM_DF_CHEN2024) {
    double z[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) z[q] = noise[q * stride + r];
    const double pv0 = 1.6 + 0.35 * z[0];
    const double pv1 = -30.0 + 23.0 * z[1];
    const double pv2 = 12.0 * z[2];
    const double pv3 = 1.0;
    const double pv4 = 20.0 + 20.0 * fma(-0.7, z[0], kChenRho * z[4]);
    const double pv5 = 22.0 * z[5];
    constexpr double DEG = 0.017453292519943295;
    double sp, cp, st, ct, sa, ca, sb, cb;
    sincos(pv1 * DEG, &sp, &cp);
    sincos(pv2 * DEG, &st, &ct);
    sincos(pv4 * DEG, &sa, &ca);
    sincos(pv5 * DEG, &sb, &cb);
    const T L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
    const T Lm = vsqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
    const T vr = v[0] * rh[0] + v[1] * rh[1] + v[2] * rh[2];
    const T ph[3] = {v[0] - vr * rh[0], v[1] - vr * rh[1], v[2] - vr * rh[2]};
    const T pm = vsqrt(ph[0] * ph[0] + ph[1] * ph[1] + ph[2] * ph[2]);
    const T Dr = pv0 * rt;
    const T Dv = pv3 * vsqrt((2.0 * GM) / Dr);
    for (int side = 0; side < 2; ++side) {
      const double s = side ? 1.0 : -1.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T zh = L[j] / Lm, yh = ph[j] / pm;
        out[side][j] = x[j] + s * (Dr * (ct * cp) * rh[j] + Dr * (ct * sp) * yh) + Dr * st * zh;
        out[side][3 + j] = v[j] + s * (Dv * (cb * ca) * rh[j] + Dv * (cb * sa) * yh) + Dv * sb * zh;
      }
    }
    return;
  }
  if (df == GAL_STREAM_DF_FARDAL2015) {
    const double kr = dfp[0] + dfp[4] * noise[r];
    const double kvphi = kr * (dfp[1] + dfp[5] * noise[stride + r]);
    const double kz = dfp[2] + dfp[6] * noise[2 * stride + r];
    const double kvz = dfp[3] + dfp[7] * noise[3 * stride + r];
    const T L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
    const T Lm = vsqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
    const T vr = v[0] * rh[0] + v[1] * rh[1] + v[2] * rh[2];
    const T ph[3] = {v[0] - vr * rh[0], v[1] - vr * rh[1], v[2] - vr * rh[2]};
    const T pm = vsqrt(ph[0] * ph[0] + ph[1] * ph[1] + ph[2] * ph[2]);
    const T vc = om * rt;
    for (int side = 0; side < 2; ++side) {
      const double s = side ? 1.0 : -1.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const T zh = L[j] / Lm;
        out[side][j] = x[j] + rt * (s * kr * rh[j] + kz * zh);
        out[side][3 + j] = v[j] + vc * (s * kvphi * (ph[j] / pm) + kvz * zh);
      }
    }
  } else {
    for (int side = 0; side < 2; ++side) {
      const double s = side ? 1.0 : -1.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double xi = noise[(6 * side + j) * stride + r];
        const double eta = noise[(6 * side + 3 + j) * stride + r];
        out[side][j] = x[j] + s * rt * rh[j] + 0.1 * rt * xi;
        out[side][3 + j] = v[j] + 0.1 * om * rt * eta;
      }
    }
  }
}

// King (1962) tidal radius r_t = cbrt(GM / (Omega^2 - d2Phi/dr2)) and Omega =
// |x cross v| / |x|^2 at (x, v) (cluster/radius.py:198-214, register_api.py:82-88).
__device__ __forceinline__ void king_rt_om(const DevComp* comps, int ncomp, double GM, const double* x,
                                           const double* v, double& rt, double& om) {
  const double rr = ::sqrt(fma(x[0], x[0], fma(x[1], x[1], x[2] * x[2])));
  const double rh[3] = {x[0] / rr, x[1] / rr, x[2] / rr};
  const double L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
  om = ::sqrt(fma(L[0], L[0], fma(L[1], L[1], L[2] * L[2]))) / (rr * rr);
  double H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int c = 0; c < ncomp; ++c) comp_hessian(comps[c], x[0], x[1], x[2], H);
  double prr = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) prr = fma(rh[i] * H[3 * i + j], rh[j], prr);
  rt = cbrt(GM / (om * om - prr));
}

// Release map, one thread per release: tidal radius, angular frequency and
// the two particles' release conditions.
__global__ void __launch_bounds__(128) k_stream_release(StreamDev a, const DevComp* comps) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  stage_comps(comps, a.ncomp, s_comps);
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= a.n_rel) return;
  const double* w = a.P + 6 * r;
  double rt, om, out[2][6];
  king_rt_om(s_comps, a.ncomp, a.GMp, w, w + 3, rt, om);
  a.rt_om[r] = rt;
  a.rt_om[a.n_rel + r] = om;
  release_pair<double>(a.df, a.dfp, a.noise, a.n_rel, r, w, w + 3, rt, om, a.GMp, out);
  for (int side = 0; side < 2; ++side)
#pragma unroll
    for (int e = 0; e < 6; ++e) a.ics[e * a.np + 2 * r + side] = out[side][e];
}

// Release conditions at n independent progenitor points (SoA [6][n] in and
// out), one thread per point.
struct DfSampleArgs {
  const double* w;
  const double* mass;
  const double* noise;
  double* lead;
  double* trail;
  double* rt;
  int64_t n;
  double G;
  int df, ncomp;
  double dfp[8];
};

__global__ void __launch_bounds__(128) k_stream_df_sample(DfSampleArgs a, const DevComp* comps) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  stage_comps(comps, a.ncomp, s_comps);
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= a.n) return;
  double x[3], v[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    x[j] = a.w[j * a.n + r];
    v[j] = a.w[(3 + j) * a.n + r];
  }
  double rt, om, out[2][6];
  const double GM = a.G * a.mass[r];
  king_rt_om(s_comps, a.ncomp, GM, x, v, rt, om);
  if (a.rt) a.rt[r] = rt;
  release_pair<double>(a.df, a.dfp, a.noise, a.n, r, x, v, rt, om, GM, out);
#pragma unroll
  for (int e = 0; e < 6; ++e) {
    a.lead[e * a.n + r] = out[0][e];
    a.trail[e * a.n + r] = out[1][e];
  }
}

// The release map's transpose: (dL/dx_p, dL/dv_p) of both particles ->
// dL/dP[r] (nu) and dL/d(component parameters) through d2Phi/dr2.
__global__ void __launch_bounds__(128) k_stream_release_adj(StreamDev a, const DevComp* comps) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  stage_comps(comps, a.ncomp, s_comps);
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= a.n_rel) return;
  const double* w = a.P + 6 * r;
  const double x[3] = {w[0], w[1], w[2]}, v[3] = {w[3], w[4], w[5]};
  const double rt = a.rt_om[r], om = a.rt_om[a.n_rel + r];
  const double rr = ::sqrt(fma(x[0], x[0], fma(x[1], x[1], x[2] * x[2])));
  const double rh[3] = {x[0] / rr, x[1] / rr, x[2] / rr};
  // release map by forward mode: tangents x (0-2), v (3-5), r_t (6), Omega (7)
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  {
    Dual<8> X8[3], V8[3], RT(rt), OM(om), out[2][6];
    for (int j = 0; j < 3; ++j) {
      X8[j] = Dual<8>(x[j]);
      X8[j].d[j] = 1.0;
      V8[j] = Dual<8>(v[j]);
      V8[j].d[3 + j] = 1.0;
    }
    RT.d[6] = 1.0;
    OM.d[7] = 1.0;
    release_pair<Dual<8>>(a.df, a.dfp, a.noise, a.n_rel, r, X8, V8, RT, OM, a.GMp, out);
    for (int side = 0; side < 2; ++side)
      for (int e = 0; e < 6; ++e) {
        const double lam = a.lam_rel[e * a.np + 2 * r + side];
#pragma unroll
        for (int t = 0; t < 8; ++t) acc[t] = fma(lam, out[side][e].d[t], acc[t]);
      }
  }
  double xb[3] = {acc[0], acc[1], acc[2]}, vb[3] = {acc[3], acc[4], acc[5]};
  const double g_rt = acc[6];
  double g_om = acc[7];
  // d2Phi/dr2 and its gradient in x (three tangents)
  Dual<3> X[3], RH[3], Hd[9];
  for (int j = 0; j < 3; ++j) {
    X[j] = Dual<3>(x[j]);
    X[j].d[j] = 1.0;
  }
  const Dual<3> R = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
  for (int j = 0; j < 3; ++j) RH[j] = X[j] / R;
  for (int c = 0; c < a.ncomp; ++c) {
    const DevComp& cc = s_comps[c];
    const Dual<3> dd[3] = {X[0] - cc.ox, X[1] - cc.oy, X[2] - cc.oz};
    comp_hessian_t<Dual<3>>(cc, cc.kind, Dual<3>(cc.Gm), Dual<3>(cc.l1), Dual<3>(cc.l2), dd, Hd);
  }
  const Dual<3> prr = contract_rhat(Hd, RH);
  const double D = om * om - prr.v;
  const double Db = g_rt * (-rt / (3.0 * D));
  g_om += 2.0 * om * Db;
  const double prr_b = -Db;
#pragma unroll
  for (int j = 0; j < 3; ++j) xb[j] += prr_b * prr.d[j];
  // parameters: d2Phi/dr2 is linear in each mass; (l1, l2) by two tangents
  for (int c = 0; c < a.ncomp; ++c) {
    const DevComp& cc = s_comps[c];
    Dual<2> l1(cc.l1), l2(cc.l2), Hc[9], dd[3], rhd[3];
    l1.d[0] = 1.0;
    l2.d[1] = 1.0;
    dd[0] = Dual<2>(x[0] - cc.ox);
    dd[1] = Dual<2>(x[1] - cc.oy);
    dd[2] = Dual<2>(x[2] - cc.oz);
    for (int j = 0; j < 3; ++j) rhd[j] = Dual<2>(rh[j]);
    comp_hessian_t<Dual<2>>(cc, cc.kind, Dual<2>(cc.Gm), l1, l2, dd, Hc);
    const Dual<2> pc = contract_rhat(Hc, rhd);
    a.gp_all[(int64_t)(3 * c + 0) * a.ncol + a.np + r] = prr_b * pc.v * cc.inv_m;
    a.gp_all[(int64_t)(3 * c + 1) * a.ncol + a.np + r] = prr_b * pc.d[0];
    a.gp_all[(int64_t)(3 * c + 2) * a.ncol + a.np + r] = prr_b * pc.d[1];
  }
  a.gp_all[(int64_t)(3 * a.ncomp) * a.ncol + a.np + r] = 0.0;
  // Omega = |x x v| / |x|^2
  const double L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
  const double Lm = ::sqrt(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
  const double Lh[3] = {L[0] / Lm, L[1] / Lm, L[2] / Lm};
  const double ir2 = 1.0 / (rr * rr);
  const double vxL[3] = {v[1] * Lh[2] - v[2] * Lh[1], v[2] * Lh[0] - v[0] * Lh[2], v[0] * Lh[1] - v[1] * Lh[0]};
  const double Lxx[3] = {Lh[1] * x[2] - Lh[2] * x[1], Lh[2] * x[0] - Lh[0] * x[2], Lh[0] * x[1] - Lh[1] * x[0]};
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    xb[j] += g_om * (vxL[j] * ir2 - 2.0 * om * x[j] * ir2);
    vb[j] += g_om * Lxx[j] * ir2;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    a.nu[6 * r + j] = xb[j];
    a.nu[6 * r + 3 + j] = vb[j];
  }
}

// Progenitor adjoint, in three kernels. Its stage positions are known from the
// forward pass, so the Hessians there are computed for all stage points at
// once (k_stream_prog_hess); the serial reverse recurrence then needs no
// potential evaluations, only H v and the Runge-Kutta combinations, and runs on
// one warp with a lane per state component (k_stream_prog_sweep), recording the
// velocity cotangent v of every stage; the parameter gradient
// -sum d(grad Phi . v)/dtheta over all stage points is again parallel
// (k_stream_prog_pgrad).
__global__ void __launch_bounds__(128) k_stream_prog_hess(StreamDev a, const DevComp* comps, int S) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  stage_comps(comps, a.ncomp, s_comps);
  const int64_t npts = 2 * a.n_rel * S;
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int64_t per = a.n_rel * S;
  const double* Y = (p < per ? a.Q + 3 * p : a.Qb + 3 * (p - per));
  double H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int c = 0; c < a.ncomp; ++c) comp_hessian(s_comps[c], Y[0], Y[1], Y[2], H);
  double* o = a.Hst + 6 * p;
  o[0] = H[0];
  o[1] = H[1];
  o[2] = H[2];
  o[3] = H[4];
  o[4] = H[5];
  o[5] = H[8];
}

// One track of the reverse recurrence (track 0: forwards, hs = +dt, with the
// particles' cotangents mu on the stage positions and the release-map
// cotangents nu on the grid states; track 1: backwards, hs = -dt). Lane j < 6
// owns component j of lambda and of every stage cotangent Fbar_i.
template <class TB>
__device__ __forceinline__ void prog_sweep_track(const StreamDev& a, int track, double hs, double& lam, int lane) {
  constexpr int S = TB::S;
  const bool mine = lane < 6;
  const int hrow = lane < 3 ? lane : 0;
  const int h0 = hrow == 0 ? 0 : (hrow == 1 ? 1 : 2);
  const int h1 = hrow == 0 ? 1 : (hrow == 1 ? 3 : 4);
  const int h2 = hrow == 0 ? 2 : (hrow == 1 ? 4 : 5);
  const int src = (lane >= 3 && lane < 6) ? lane - 3 : lane;
  for (int64_t k = a.n_rel - 1; k >= 0; --k) {
    const int64_t base = (int64_t)track * a.n_rel * S + k * S;  // stage-point index of (k, 0)
    double Hr[S][3], Mu[S];
    // all of this step's inputs in flight together
    static_for<0, S>([&](auto i) {
      constexpr int I = decltype(i)::value;
      const double* Hp = a.Hst + 6 * (base + I);
      Hr[I][0] = lane < 3 ? Hp[h0] : 0.0;
      Hr[I][1] = lane < 3 ? Hp[h1] : 0.0;
      Hr[I][2] = lane < 3 ? Hp[h2] : 0.0;
      Mu[I] = (track == 0 && lane < 3) ? a.mu[(k * S + I) * 3 + lane] : 0.0;
    });
    const double nu = (track == 0 && mine) ? a.nu[6 * k + lane] : 0.0;
    double Fb[S];
    static_for<0, S>([&](auto i) {
      constexpr int I = decltype(i)::value;
      constexpr double bi = TB::B[I];
      Fb[I] = hs * bi * lam;
    });
    static_for<0, S>([&](auto rr) {
      constexpr int I = S - 1 - decltype(rr)::value;
      const double f = Fb[I];
      const double v0 = __shfl_sync(0xffffffffu, f, 3);
      const double v1 = __shfl_sync(0xffffffffu, f, 4);
      const double v2 = __shfl_sync(0xffffffffu, f, 5);
      const double pos = __shfl_sync(0xffffffffu, f, src);
      if (lane >= 3 && mine) a.vst[3 * (base + I) + (lane - 3)] = f;
      double Yb;
      if (lane < 3)
        Yb = Mu[I] - fma(Hr[I][0], v0, fma(Hr[I][1], v1, Hr[I][2] * v2));
      else
        Yb = mine ? pos : 0.0;
      lam += Yb;
      static_for<0, I>([&](auto l) {
        constexpr int L = decltype(l)::value;
        constexpr double c = TB::A[I][L];
        if constexpr (c != 0.0) Fb[L] = fma(hs * c, Yb, Fb[L]);
      });
    });
    lam += nu;
  }
}

template <class TB>
__global__ void __launch_bounds__(32) k_stream_prog_sweep(StreamDev a) {
  const int lane = threadIdx.x;
  double lam = 0.0;
  prog_sweep_track<TB>(a, 0, a.dt, lam, lane);
  prog_sweep_track<TB>(a, 1, -a.dt, lam, lane);
  if (a.grad_w_now && lane < 6) a.grad_w_now[lane] = lam;
}

__global__ void __launch_bounds__(128) k_stream_prog_pgrad(StreamDev a, const DevComp* comps, int S) {
  __shared__ DevComp s_comps[kAdjMaxComps];
  stage_comps(comps, a.ncomp, s_comps);
  const int64_t npts = 2 * a.n_rel * S;
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= npts) return;
  const int64_t per = a.n_rel * S;
  const double* Y = (p < per ? a.Q + 3 * p : a.Qb + 3 * (p - per));
  const double* v = a.vst + 3 * p;
  const int64_t col = a.np + a.n_rel + p;
  for (int c = 0; c < a.ncomp; ++c) {
    double Hv[3] = {0.0, 0.0, 0.0}, dp[3] = {0.0, 0.0, 0.0};
    comp_vjp(s_comps[c], Y, v, Hv, dp);
    a.gp_all[(int64_t)(3 * c + 0) * a.ncol + col] = -dp[0];
    a.gp_all[(int64_t)(3 * c + 1) * a.ncol + col] = -dp[1];
    a.gp_all[(int64_t)(3 * c + 2) * a.ncol + col] = -dp[2];
  }
  a.gp_all[(int64_t)(3 * a.ncomp) * a.ncol + col] = 0.0;
}

__global__ void k_stream_reduce_rows(const double* __restrict__ in, int64_t n, double* __restrict__ out) {
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

// ------------------------------------------------------------------ host side
static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

struct StreamLayout {
  size_t B, P, Q, Qb, Hst, vst, rt_om, ics, fin, ckpt, seg, Ys, Hs, vs, lam_rel, mu_warp, mu, nu, gp_all, red, total;
  int64_t np, nwarps, nseg, ncol, pg_col0, pg_blocks;
  int S;
};

static StreamLayout stream_layout(int ncomp, const gal_stream_config& c, bool grad) {
  StreamLayout L{};
  L.S = c.method == 5 ? Dopri5::S : Dopri8::S;
  L.np = 2 * c.n_release;
  L.nwarps = (L.np + 31) / 32;
  const bool stored = c.k_ckpt == 0;
  const int K = c.k_ckpt > 0 ? c.k_ckpt : 1;
  L.nseg = (c.n_release + K - 1) / K;
  const int64_t nq = c.n_release * (c.n_release + 1);  // particle-steps
  L.pg_col0 = L.np + c.n_release + 2 * c.n_release * L.S;
  L.pg_blocks = stored ? (nq + 255) / 256 : 0;
  L.ncol = L.pg_col0 + L.pg_blocks;
  const size_t d = sizeof(double);
  const size_t nr = (size_t)c.n_release;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += al256(bytes);
    return o;
  };
  L.B = take(d * 6 * (nr + 1));
  L.P = take(d * 6 * (nr + 1));
  L.Q = take(d * 3 * L.S * nr);
  L.rt_om = take(d * 2 * nr);
  L.ics = take(d * 6 * L.np);
  L.fin = take(d * 6 * L.np);
  if (grad) {
    L.Qb = take(d * 3 * L.S * nr);
    L.Hst = take(d * 6 * 2 * L.S * nr);
    L.vst = take(d * 3 * 2 * L.S * nr);
    if (stored) {
      L.Ys = take(d * 3 * L.S * (size_t)nq);
      L.Hs = take(d * 12 * L.S * (size_t)nq);
      L.vs = take(d * 3 * L.S * (size_t)nq);
    } else {
      L.ckpt = take(d * 6 * L.nseg * L.np);
      L.seg = take(d * 6 * (size_t)K * L.np);
    }
    L.lam_rel = take(d * 6 * L.np);
    L.mu_warp = take(d * 3 * L.S * nr * L.nwarps);
    L.mu = take(d * 3 * L.S * nr);
    L.nu = take(d * 6 * nr);
    L.gp_all = take(d * (3 * (size_t)ncomp + 1) * L.ncol);
    L.red = take(d * (3 * (size_t)ncomp + 1));
  }
  L.total = off;
  return L;
}

static gal_status df_validate(int32_t df, const double* p) {
  if (df != GAL_STREAM_DF_OFFSETS && df != GAL_STREAM_DF_FARDAL2015 && df != GAL_STREAM_DF_CHEN2024)
    return fail(GAL_ERR_INVALID_ARGUMENT, "df must be GAL_STREAM_DF_OFFSETS, _FARDAL2015 or _CHEN2024");
  if (df == GAL_STREAM_DF_FARDAL2015) {
    if (!p) return fail(GAL_ERR_INVALID_ARGUMENT, "NULL df_params");
    for (int j = 0; j < 8; ++j)
      if (!std::isfinite(p[j])) return fail(GAL_ERR_INVALID_ARGUMENT, "df_params must be finite");
  }
  return GAL_OK;
}

static gal_status stream_validate(const gal_potential* pot, const gal_stream_config* c) {
  if (!pot || !c) return fail(GAL_ERR_INVALID_ARGUMENT, "NULL potential or stream configuration");
  if (c->method != 5 && c->method != 8) return fail(GAL_ERR_INVALID_ARGUMENT, "method must be 5 or 8");
  if (!(c->dt > 0.0)) return fail(GAL_ERR_INVALID_ARGUMENT, "dt must be > 0");
  if (c->n_release < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "n_release must be >= 1");
  // the particle-step grids (n_release (n_release + 1) entries) must fit one launch
  if (c->n_release > (int64_t(1) << 18)) return fail(GAL_ERR_TOO_LARGE, "n_release must be <= 2^18");
  if (c->k_ckpt < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "k_ckpt must be >= 0");
  if (!(c->prog_m > 0.0) || !(c->prog_b > 0.0)) return fail(GAL_ERR_INVALID_ARGUMENT, "progenitor m, b must be > 0");
  if (pot->n > kAdjMaxComps) return fail(GAL_ERR_UNSUPPORTED, "stream host potentials have at most 8 components");
  if (time_dependent(pot)) return fail(GAL_ERR_UNSUPPORTED, "time-dependent parameters: evaluation, integration and the orbit adjoint only");
  return df_validate(c->df, c->df_params);
}

static StreamDev stream_args(const gal_potential* pot, const gal_stream_config* c, const StreamLayout& L, char* ws,
                             const double* noise, bool grad) {
  StreamDev a{};
  a.n_rel = c->n_release;
  a.np = L.np;
  a.nwarps = L.nwarps;
  a.ncol = L.ncol;
  a.pg_col0 = L.pg_col0;
  a.dt = c->dt;
  a.GMp = pot->G * c->prog_m;
  a.b2 = c->prog_b * c->prog_b;
  for (int j = 0; j < 6; ++j) a.w_now[j] = c->w_now[j];
  a.k_ckpt = c->k_ckpt;
  a.ncomp = pot->n;
  a.df = c->df;
  for (int j = 0; j < 8; ++j) a.dfp[j] = c->df_params[j];
  auto at = [&](size_t o) { return reinterpret_cast<double*>(ws + o); };
  a.B = at(L.B);
  a.P = at(L.P);
  a.Q = at(L.Q);
  a.rt_om = at(L.rt_om);
  a.noise = noise;
  a.ics = at(L.ics);
  a.fin = at(L.fin);
  if (grad) {
    a.Qb = at(L.Qb);
    a.Hst = at(L.Hst);
    a.vst = at(L.vst);
    if (c->k_ckpt == 0) {
      a.Ys = at(L.Ys);
      a.Hs = at(L.Hs);
      a.vs = at(L.vs);
    } else {
      a.ckpt = at(L.ckpt);
      a.seg = at(L.seg);
    }
    a.lam_rel = at(L.lam_rel);
    a.mu_warp = at(L.mu_warp);
    a.mu = at(L.mu);
    a.nu = at(L.nu);
    a.gp_all = at(L.gp_all);
  }
  return a;
}

template <class TB>
static cudaError_t stream_forward(const StreamDev& a, const gal_potential* pot, cudaStream_t s) {
  const DevComp* comps = pot->d_comps;
  if (pot->is_mw)
    k_stream_progenitor_mw<TB><<<1, 128, 0, s>>>(a, pot->mw);
  else
    k_stream_progenitor_team<TB><<<1, 128, 0, s>>>(a, comps);
  k_stream_release<<<(unsigned)((a.n_rel + 127) / 128), 128, 0, s>>>(a, comps);
  k_stream_particles_team<TB><<<(unsigned)((a.np + 31) / 32), 128, 0, s>>>(a, comps);
  return cudaGetLastError();
}

template <class TB>
static cudaError_t stream_backward(const StreamDev& a, const DevComp* comps, cudaStream_t s) {
  if (a.Ys) {
    const int64_t nq = a.n_rel * (a.n_rel + 1);
    k_stream_particle_hess<TB><<<(unsigned)((nq + 127) / 128), 128, 0, s>>>(a, comps);
    k_stream_particles_sweep<TB><<<(unsigned)a.nwarps, 32, 0, s>>>(a);
    k_stream_particles_pgrad<TB><<<(unsigned)((nq + 255) / 256), 256, 0, s>>>(a, comps);
  } else {
    k_stream_particles_adj<TB><<<(unsigned)a.nwarps, 32, 0, s>>>(a, comps);
  }
  const int S3 = 3 * TB::S;
  k_stream_mu_reduce<<<(unsigned)((a.n_rel * S3 + 255) / 256), 256, 0, s>>>(a, S3);
  k_stream_release_adj<<<(unsigned)((a.n_rel + 127) / 128), 128, 0, s>>>(a, comps);
  const int64_t npts = 2 * a.n_rel * TB::S;
  k_stream_prog_hess<<<(unsigned)((npts + 127) / 128), 128, 0, s>>>(a, comps, TB::S);
  k_stream_prog_sweep<TB><<<1, 32, 0, s>>>(a);
  k_stream_prog_pgrad<<<(unsigned)((npts + 127) / 128), 128, 0, s>>>(a, comps, TB::S);
  return cudaGetLastError();
}

template <class Fn>
static cudaError_t dispatch(int method, Fn&& fn) {
  if (method == 8) return fn(Dopri8{});
  return fn(Dopri5{});
}

}  // namespace gal

using namespace gal;

extern "C" {

gal_status gal_stream_df_sample(const gal_potential* pot, int32_t df, const double* df_params, const double* prog_w,
                                const double* prog_mass, const double* noise, int64_t n, double* lead, double* trail,
                                double* r_tidal, gal_stream_t stream) {
  if (!pot) return fail(GAL_ERR_INVALID_ARGUMENT, "NULL potential");
  if (time_dependent(pot)) return fail(GAL_ERR_UNSUPPORTED, "time-dependent parameters: evaluation, integration and the orbit adjoint only");
  gal_status st = df_validate(df, df_params);
  if (st != GAL_OK) return st;
  if (n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "n must be >= 0");
  if (pot->n > kAdjMaxComps) return fail(GAL_ERR_UNSUPPORTED, "stream host potentials have at most 8 components");
  if (n == 0) return GAL_OK;
  if (!prog_w || !prog_mass || !noise || !lead || !trail)
    return fail(GAL_ERR_INVALID_ARGUMENT, "NULL progenitor points, masses, noise or output");
  DfSampleArgs a{prog_w, prog_mass, noise, lead, trail, r_tidal, n, pot->G, df, pot->n, {}};
  if (df == GAL_STREAM_DF_FARDAL2015)
    for (int j = 0; j < 8; ++j) a.dfp[j] = df_params[j];
  k_stream_df_sample<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(a, pot->d_comps);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "k_stream_df_sample");
}

gal_status gal_stream_workspace_size(const gal_potential* pot, const gal_stream_config* cfg, int32_t with_grad,
                                     size_t* bytes) {
  gal_status st = stream_validate(pot, cfg);
  if (st != GAL_OK) return st;
  if (!bytes) return fail(GAL_ERR_INVALID_ARGUMENT, "bytes is NULL");
  *bytes = stream_layout(pot->n, *cfg, with_grad != 0).total;
  return GAL_OK;
}

gal_status gal_stream_run(const gal_potential* pot, const gal_stream_config* cfg, const double* noise,
                          double* final_states, double* ics, double* prog_track, void* workspace,
                          size_t workspace_bytes, gal_stream_t stream) {
  gal_status st = stream_validate(pot, cfg);
  if (st != GAL_OK) return st;
  if (!noise || !final_states) return fail(GAL_ERR_INVALID_ARGUMENT, "NULL noise or output");
  const StreamLayout L = stream_layout(pot->n, *cfg, false);
  if (!workspace || workspace_bytes < L.total) return fail(GAL_ERR_WORKSPACE, "workspace too small");
  char* ws = static_cast<char*>(workspace);
  StreamDev a = stream_args(pot, cfg, L, ws, noise, false);
  a.fin = final_states;
  if (ics) a.ics = ics;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = dispatch(cfg->method, [&](auto tb) { return stream_forward<decltype(tb)>(a, pot, s); });
  if (e != cudaSuccess) return cuda_fail(e, "stream kernels");
  if (prog_track) {
    e = cudaMemcpyAsync(prog_track, a.P, sizeof(double) * 6 * (size_t)(cfg->n_release + 1), cudaMemcpyDeviceToDevice,
                        s);
    if (e != cudaSuccess) return cuda_fail(e, "copying the progenitor track");
  }
  return GAL_OK;
}

gal_status gal_stream_grad(const gal_potential* pot, const gal_stream_config* cfg, const double* noise,
                           const double* target, double* final_states, double* grad_params, double* grad_w_now,
                           double* loss, void* workspace, size_t workspace_bytes, gal_stream_t stream) {
  gal_status st = stream_validate(pot, cfg);
  if (st != GAL_OK) return st;
  if (!noise || !target || !grad_params) return fail(GAL_ERR_INVALID_ARGUMENT, "NULL noise, target or gradient");
  const StreamLayout L = stream_layout(pot->n, *cfg, true);
  if (!workspace || workspace_bytes < L.total) return fail(GAL_ERR_WORKSPACE, "workspace too small");
  char* ws = static_cast<char*>(workspace);
  StreamDev a = stream_args(pot, cfg, L, ws, noise, true);
  if (final_states) a.fin = final_states;
  a.target = target;
  a.grad_w_now = grad_w_now;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = dispatch(cfg->method, [&](auto tb) {
    cudaError_t e1 = stream_forward<decltype(tb)>(a, pot, s);
    if (e1 != cudaSuccess) return e1;
    return stream_backward<decltype(tb)>(a, pot->d_comps, s);
  });
  if (e != cudaSuccess) return cuda_fail(e, "stream gradient kernels");
  double* red = reinterpret_cast<double*>(ws + L.red);
  k_stream_reduce_rows<<<(unsigned)(3 * pot->n + 1), 256, 0, s>>>(a.gp_all, L.ncol, red);
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(grad_params, red, sizeof(double) * 3 * pot->n, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, red + 3 * pot->n, sizeof(double), cudaMemcpyDeviceToDevice, s);
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "stream gradient reduction");
}

}  // extern "C"
