// Orbit integration kernels: explicit embedded Runge-Kutta (Dopri5 / Dopri8),
// constant step or diffrax's PID controller, saves at per-orbit times.
//
// One thread owns one orbit at a time and keeps the state and every stage slope
// in registers. The launch is persistent: each lane takes its next orbit from a
// device work queue (an atomic counter in caller-provided scratch) as soon as
// its current orbit ends, so orbits of very different lengths keep every lane
// busy and the expensive stage code runs converged across the warp.
//
// Semantics follow what galax asks of diffrax
// (src/galax/dynamics/_src/legacy/integrator.py:179-245,
//  src/galax/dynamics/_src/orbit/solver.py:774-803):
//  * time runs in tau = d t with d = sign(t1 - t0) (reversed integration);
//  * ConstantStepSize: t_{k+1} = t_k + dt0, the step that would pass t1 - 1e-10
//    ends on t1;
//  * PIDController: error = h sum_i e_i F_i, RMS of err / (atol + rtol max(|y0|,|y1|)),
//    accept when < 1 (or when the previous step sat at dtmin),
//    factor = clip(safety inv^(i+p+d)/order prev^-(p+2d)/order prevprev^d/order,
//    accepted ? 1 : factormin, factormax), dt = (t1 - t0) factor, clamps to
//    [dtmin, dtmax], next step clipped onto t1 (half the remainder after a
//    rejection); initial step by the Hairer-Norsett-Wanner rule with exponent
//    1/(order + 1);
//  * saves in (t_k, t_{k+1}] of an accepted step: Dopri5 uses the quartic through
//    y0, y1, y(t_k + h/2) (Shampine's weights), f0, f1; Dopri8 takes one Dopri8
//    step of the partial length from (t_k, y_k).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "potentials.cuh"
#include "tableaux.cuh"

namespace gal {

enum { ORBIT_OK = 0, ORBIT_MAX_STEPS = 1, ORBIT_DT_MIN = 2, ORBIT_NONFINITE = 3 };

constexpr int kTeamLanes = 32;  // orbits per four-warp team block (integrate_team.cuh)

// Everything needed to continue an orbit exactly where a first pass parked it
// (state, step times, controller memory, counters, save cursor). 128 bytes.
struct OrbitResume {
  double y[6];
  double tau, tnext, prev_inv, prev_prev_inv, progress;
  int64_t nsteps, naccepted, save_i;
  int32_t at_dtmin, status, paused, pad;
};
static_assert(sizeof(OrbitResume) == 128, "OrbitResume layout");

struct IntegrateArgs {
  // solver
  int32_t adaptive;
  int32_t force_dtmin;
  int64_t max_steps;
  double dt0, rtol, atol, dtmin, dtmax;
  double c1, c2, c3;  // PID exponents (i+p+d)/order, -(p+2d)/order, d/order
  int32_t i_controller;  // 1 when pcoeff = dcoeff = 0 and icoeff = 1 (diffrax's default)
  double safety, factormin, factormax;
  // data
  const double* y0;  // [6][n]
  const double* t0;
  const double* t1;
  const int64_t* save_offsets;  // NULL -> shared grid
  const double* save_ts;
  int64_t n_saves;  // shared grid size
  double* out;
  int64_t out_stride;  // elements between components of out
  int32_t* status;
  int64_t* steps;
  const int32_t* order;
  int64_t n;
  unsigned long long* queue;  // work-queue counter (scratch)
  const DevLinear* lin;       // time-dependent component parameters (table kernel), or NULL
  long long queue_base;       // first queue position of this launch (earlier ones belong to a team kernel)
  // two-phase schedule: phase 0 parks every orbit once it has covered split_frac
  // of its span; phase 1 resumes the parked orbits from `resume` in `order`
  int32_t phase;
  double split_frac;                     // <= 0: single pass
  OrbitResume* resume;                   // [n]
  const unsigned long long* queue_len;   // phase 1: number of entries in order (device)
};

// Hamiltonian field without the time-direction sign: F = (p, -grad Phi(q, t)).
// Static potential models ignore t, so its arithmetic vanishes from their code.
template <class Pot>
__device__ __forceinline__ void field(const Pot& pot, const double* Y, double* F, double t = 0.0) {
  double gx, gy, gz;
  pot_grad_t(pot, t, Y[0], Y[1], Y[2], gx, gy, gz);
  F[0] = Y[3];
  F[1] = Y[4];
  F[2] = Y[5];
  F[3] = -gx;
  F[4] = -gy;
  F[5] = -gz;
}

// Y = y + hs * sum_{l<I} A[I][l] F[l] (row I of the tableau).
template <class TB, int I>
__device__ __forceinline__ void stage_state(const double* y, double hs, const double (&F)[TB::S][6], double* Y) {
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double acc = 0.0;
    bool first = true;
    static_for<0, I>([&](auto l) {
      constexpr int L = decltype(l)::value;
      constexpr double c = TB::A[I][L];
      if constexpr (c != 0.0) {
        acc = first ? c * F[L][j] : fma(c, F[L][j], acc);
        first = false;
      }
    });
    Y[j] = fma(hs, acc, y[j]);
  }
}

// Stages 1..S-1 of one RK step of signed length hs from (t, y) (F[0] preset).
template <class TB, class Pot>
__device__ __forceinline__ void rk_stages(const Pot& pot, const double* y, double hs, double (&F)[TB::S][6],
                                          double t = 0.0) {
  static_for<1, TB::S>([&](auto i) {
    constexpr int I = decltype(i)::value;
    double Y[6];
    stage_state<TB, I>(y, hs, F, Y);
    constexpr double ci = TB::C[I];
    field(pot, Y, F[I], fma(ci, hs, t));
  });
}

enum Weights { W_SOLUTION = 0, W_ERROR = 1, W_MIDPOINT = 2 };

template <class TB, int WHICH, int L>
__host__ __device__ constexpr double weight() {
  if constexpr (WHICH == W_SOLUTION) return TB::B[L];
  else if constexpr (WHICH == W_ERROR) return TB::E[L];
  else return TB::CMID[L];  // Dopri5 dense output only
}

// out = y + hs * sum_l w_l F[l] for a compile-time weight vector (y may be NULL).
template <class TB, int WHICH>
__device__ __forceinline__ void weighted(const double* y, double hs, const double (&F)[TB::S][6], double* out) {
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double acc = 0.0;
    bool first = true;
    static_for<0, TB::S>([&](auto l) {
      constexpr int L = decltype(l)::value;
      constexpr double c = weight<TB, WHICH, L>();
      if constexpr (c != 0.0) {
        acc = first ? c * F[L][j] : fma(c, F[L][j], acc);
        first = false;
      }
    });
    out[j] = y ? fma(hs, acc, y[j]) : hs * acc;
  }
}

template <class TB>
__device__ __forceinline__ void rk_combine(const double* y, double hs, const double (&F)[TB::S][6], double* y1,
                                           double* err) {
  weighted<TB, W_SOLUTION>(y, hs, F, y1);
  if (err != nullptr) weighted<TB, W_ERROR>(nullptr, hs, F, err);
}

// Dopri5 dense output at theta in [0, 1] of a step of signed length hs: the
// quartic p with p(0) = y0, p(1) = y1, p(1/2) = y_mid (Shampine's weights),
// p'(0) = hs F0, p'(1) = hs F6 (diffrax's FourthOrderPolynomialInterpolation),
// written in its basis form
//   p = y0 + H1 (y1 - y0) + Hm (y_mid - y0) + Hf0 hs F0 + Hf1 hs F6,
//   H1 = th^2 (-8 th^2 + 14 th - 5), Hm = 16 th^2 (1 - th)^2,
//   Hf0 = th (1 - th)^2 (1 - 2 th), Hf1 = th^2 (th - 1) (2 th - 1),
// so that p = y0 + hs sum_i W_i F_i with W_i = H1 b_i + Hm cmid_i (+ Hf0, Hf1).
// One weight vector per save time; no per-step set-up.
__device__ __forceinline__ void dopri5_dense(const double* y0, double hs, const double (&F)[Dopri5::S][6],
                                             double th, double* out) {
  const double t2 = th * th;
  const double u = 1.0 - th;
  const double H1 = t2 * fma(th, fma(-8.0, th, 14.0), -5.0);
  const double Hm = 16.0 * t2 * (u * u);
  const double Hf0 = th * (u * u) * fma(-2.0, th, 1.0);
  const double Hf1 = t2 * (-u) * fma(2.0, th, -1.0);
  double W[Dopri5::S];
  static_for<0, Dopri5::S>([&](auto i) {
    constexpr int I = decltype(i)::value;
    constexpr double b = Dopri5::B[I], c = Dopri5::CMID[I];
    double w = (b != 0.0) ? H1 * b : 0.0;
    if constexpr (c != 0.0) w = fma(Hm, c, w);
    if constexpr (I == 0) w += Hf0;
    if constexpr (I == Dopri5::S - 1) w += Hf1;
    W[I] = w;
  });
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double acc = W[0] * F[0][j];
    static_for<1, Dopri5::S>([&](auto i) {
      constexpr int I = decltype(i)::value;
      if constexpr (I != 1) acc = fma(W[I], F[I][j], acc);  // b_1 = cmid_1 = 0
    });
    out[j] = fma(hs, acc, y0[j]);
  }
}

__device__ __forceinline__ double rms6(const double* q) {
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) s = fma(q[j], q[j], s);
  return sqrt(s / 6.0);
}

struct OrbitState {
  int64_t orbit;       // < 0: no orbit
  int64_t save_base;   // index of this orbit's first save (CSR) or orbit (shared grid)
  int64_t save_i, save_end;
  int64_t nsteps, naccepted;
  double y[6], F0[6];
  double tau, tnext, tau0, tau1, dir;
  double prev_inv, prev_prev_inv;
  int32_t at_dtmin;
  int32_t status;      // sticky: set when the controller reports dt < dtmin
  int32_t pending;     // Dopri8: saves of the accepted step still to write
  double ynew[6];      // Dopri8: accepted end state while its saves are written
  double tau_new;      // end time of that accepted step
  double tnext_new;
};

__device__ __forceinline__ int64_t save_index(const IntegrateArgs& a, const OrbitState& s, int64_t k) {
  return a.save_offsets ? (s.save_base + k) : (k * a.n + s.save_base);
}

__device__ __forceinline__ void write_save(const IntegrateArgs& a, const OrbitState& s, int64_t k, const double* v) {
  const int64_t idx = save_index(a, s, k);
#pragma unroll
  for (int j = 0; j < 6; ++j) a.out[j * a.out_stride + idx] = v[j];
}

__device__ __forceinline__ double save_tau(const IntegrateArgs& a, const OrbitState& s, int64_t k) {
  const double ts = a.save_offsets ? a.save_ts[s.save_base + k] : a.save_ts[k];
  return s.dir * ts;
}

__device__ __forceinline__ void finish_orbit(const IntegrateArgs& a, OrbitState& s, int32_t st) {
  const double nanv[6] = {__longlong_as_double(0x7ff8000000000000LL), __longlong_as_double(0x7ff8000000000000LL),
                          __longlong_as_double(0x7ff8000000000000LL), __longlong_as_double(0x7ff8000000000000LL),
                          __longlong_as_double(0x7ff8000000000000LL), __longlong_as_double(0x7ff8000000000000LL)};
  for (int64_t k = s.save_i; k < s.save_end; ++k) write_save(a, s, k, nanv);
  if (a.status) a.status[s.orbit] = st;
  if (a.steps) a.steps[s.orbit] = s.naccepted;
  s.orbit = -1;
}

template <class TB, class Pot>
__device__ __forceinline__ double initial_step(const IntegrateArgs& a, const Pot& pot, const double* y,
                                               const double* F0, double dir, double t) {
  // Hairer, Norsett & Wanner (1993) II.4, as used by diffrax when dt0 is None.
  double sc[6], q[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) sc[j] = fma(fabs(y[j]), a.rtol, a.atol);
#pragma unroll
  for (int j = 0; j < 6; ++j) q[j] = y[j] / sc[j];
  const double d0 = rms6(q);
#pragma unroll
  for (int j = 0; j < 6; ++j) q[j] = F0[j] / sc[j];
  const double d1 = rms6(q);
  const bool cond = (d0 < 1e-5) || (d1 < 1e-5);
  const double h0 = cond ? 1e-6 : 0.01 * (d0 / d1);
  double Y[6], F1[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) Y[j] = fma(h0 * dir, F0[j], y[j]);
  field(pot, Y, F1, fma(h0, dir, t));
#pragma unroll
  for (int j = 0; j < 6; ++j) q[j] = (F1[j] - F0[j]) / sc[j];
  const double d2 = rms6(q) / h0;
  const double maxd = fmax(d1, d2);
  const double h1 = (maxd <= 1e-15) ? fmax(1e-6, h0 * 1e-3) : pow(0.01 / maxd, 1.0 / (TB::ORDER + 1.0));
  return fmin(100.0 * h0, h1);
}

// Queue position of a thread's first orbit. The queue is ordered longest work
// first; handing the first positions out in stripes (lane 0 of warp 0 of every
// block, then lane 0 of warp 1, ..., then lane 1) puts the longest orbits on
// different SMs and sub-partitions, so the tail they form at the end of a batch
// does not queue up on a few FP64 pipes. Later positions are dequeued
// atomically after the gridDim.x * blockDim.x striped ones.
//
// With LANES = 32 a whole warp owns one orbit (warp-per-orbit mode, for
// composites with many components): the positions are handed out per warp,
// and lane 0 takes the next one from the queue for the warp.
template <int LANES>
__device__ __forceinline__ unsigned long long first_position() {
  const unsigned long long W = blockDim.x >> 5, w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if constexpr (LANES == 32) return w * gridDim.x + blockIdx.x;
  return (l * W + w) * gridDim.x + blockIdx.x;
}

template <int LANES>
__device__ __forceinline__ unsigned long long next_position(unsigned long long* queue) {
  if constexpr (LANES == 32) {
    unsigned long long k = 0;
    if ((threadIdx.x & 31) == 0) k = atomicAdd(queue, 1ULL);
    return __shfl_sync(0xffffffffu, k, 0);
  }
  return atomicAdd(queue, 1ULL);
}

// Returns false when the queue is empty.
template <class TB, class Pot, int LANES = 1>
__device__ __forceinline__ bool start_orbit(const IntegrateArgs& a, const Pot& pot, OrbitState& s,
                                            bool& first) {
  const unsigned long long qlen = a.queue_len ? *a.queue_len : (unsigned long long)a.n;
  const unsigned long long striped = (unsigned long long)gridDim.x * (blockDim.x / LANES);
  const unsigned long long base = (unsigned long long)a.queue_base;
  while (true) {
    unsigned long long k;
    if (first) {
      first = false;
      k = base + first_position<LANES>();
    } else {
      k = base + striped + next_position<LANES>(a.queue);
    }
    if (k >= qlen) return false;
    const int64_t o = a.order ? (int64_t)a.order[k] : (int64_t)k;
    s.orbit = o;
    const double t0 = a.t0[o], t1 = a.t1[o];
    if (a.save_offsets) {
      s.save_base = a.save_offsets[o];
      s.save_end = a.save_offsets[o + 1] - s.save_base;
    } else {
      s.save_base = o;
      s.save_end = a.n_saves;
    }
    s.pending = 0;
    s.dir = (t0 < t1) ? 1.0 : -1.0;
    s.tau0 = s.dir * t0;
    s.tau1 = s.dir * t1;
    if (a.phase == 1) {  // continue a parked orbit exactly
      const OrbitResume& r = a.resume[o];
#pragma unroll
      for (int j = 0; j < 6; ++j) s.y[j] = r.y[j];
      s.tau = r.tau;
      s.tnext = r.tnext;
      s.prev_inv = r.prev_inv;
      s.prev_prev_inv = r.prev_prev_inv;
      s.nsteps = r.nsteps;
      s.naccepted = r.naccepted;
      s.save_i = r.save_i;
      s.at_dtmin = r.at_dtmin;
      s.status = r.status;
      field(pot, s.y, s.F0, s.dir * s.tau);
      return true;
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) s.y[j] = a.y0[j * a.n + o];
    s.save_i = 0;
    s.nsteps = 0;
    s.naccepted = 0;
    s.tau = s.tau0;
    s.prev_inv = 1.0;
    s.prev_prev_inv = 1.0;
    s.at_dtmin = 0;
    s.status = ORBIT_OK;
    if (t0 == t1) {  // nothing to integrate: every save is the initial state
      for (; s.save_i < s.save_end; ++s.save_i) write_save(a, s, s.save_i, s.y);
      finish_orbit(a, s, ORBIT_OK);
      continue;
    }
    if (!isfinite(t0) || !isfinite(t1)) {  // an infinite span never ends: report it at once
      finish_orbit(a, s, ORBIT_NONFINITE);
      continue;
    }
    field(pot, s.y, s.F0, t0);
    double dt;
    if (a.adaptive) {
      dt = a.dt0 > 0.0 ? a.dt0 : initial_step<TB>(a, pot, s.y, s.F0, s.dir, t0);
      if (a.dtmax > 0.0) dt = fmin(dt, a.dtmax);
      if (a.dtmin > 0.0) {
        s.at_dtmin = dt <= a.dtmin;
        dt = fmax(dt, a.dtmin);
      }
    } else {
      dt = a.dt0;
    }
    s.tnext = fmin(s.tau + dt, s.tau1);
    return true;
  }
}

// Phase 0 of the two-phase schedule: park the orbit once it has covered
// split_frac of its span (only between steps, never with saves pending).
__device__ __forceinline__ bool maybe_park(const IntegrateArgs& a, OrbitState& s) {
  if (a.phase != 0 || a.split_frac <= 0.0) return false;
  const double span = s.tau1 - s.tau0;
  const double done = s.tau - s.tau0;
  if (done < a.split_frac * span) return false;
  OrbitResume& r = a.resume[s.orbit];
#pragma unroll
  for (int j = 0; j < 6; ++j) r.y[j] = s.y[j];
  r.tau = s.tau;
  r.tnext = s.tnext;
  r.prev_inv = s.prev_inv;
  r.prev_prev_inv = s.prev_prev_inv;
  r.progress = done / span;
  r.nsteps = s.nsteps;
  r.naccepted = s.naccepted;
  r.save_i = s.save_i;
  r.at_dtmin = s.at_dtmin;
  r.status = s.status;
  r.paused = 1;
  if (a.steps) a.steps[s.orbit] = s.naccepted;
  s.orbit = -1;
  return true;
}

// y = ms^(-1/(2*ORDER)) to FP64 accuracy: an FP32 seed and two FP64 Newton
// steps on ms * y^(2*ORDER) = 1 (y <- y (1 + e / (2*ORDER)), e = 1 - ms y^(2*ORDER);
// the error squares each step). Valid for ms in [1e-30, 1e30].
template <int ORDER>
__device__ __forceinline__ double inv_root(double ms) {
  constexpr int P = 2 * ORDER;
  double y = (double)powf((float)ms, -1.0f / P);
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    double p = y;  // y^P by repeated multiplication (P = 10 or 16)
    if constexpr (P == 16) {
      p = p * p; p = p * p; p = p * p; p = p * p;
    } else {
      const double y2 = y * y, y4 = y2 * y2, y8 = y4 * y4;
      p = y8 * y2;
    }
    const double e = fma(-ms, p, 1.0);
    y = fma(y * (1.0 / P), e, y);
  }
  return y;
}

// Controller after a step of length h = tnext - tau with error estimate err.
// Sets keep, the next (t0, t1) and the controller state.
template <int ORDER>
__device__ __forceinline__ bool pid_adapt(const IntegrateArgs& a, OrbitState& s, const double* y1,
                                          const double* err, double h, double& next_t0, double& next_t1) {
  // RMS of err_j / d_j with d_j = atol + rtol max(|y0_j|, |y1_j|); the six
  // reciprocals come from one division (prefix/suffix products).
  double d[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double y1c = isnan(y1[j]) ? s.y[j] : y1[j];
    d[j] = fma(fmax(fabs(s.y[j]), fabs(y1c)), a.rtol, a.atol);
  }
  const double p01 = d[0] * d[1], p23 = d[2] * d[3], p45 = d[4] * d[5];
  const double p0123 = p01 * p23;
  const double P = p0123 * p45;
  double ms = 0.0;
  if (P > 1e-280 && P < 1e280) {
    const double iP = 1.0 / P;
    const double i01 = iP * p23 * p45, i23 = iP * p01 * p45, i45 = iP * p0123;
    const double r[6] = {i01 * d[1], i01 * d[0], i23 * d[3], i23 * d[2], i45 * d[5], i45 * d[4]};
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const double q = err[j] * r[j];
      ms = fma(q, q, ms);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const double q = err[j] / d[j];
      ms = fma(q, q, ms);
    }
  }
  ms = ms / 6.0;
  bool keep = ms < 1.0;  // scaled error = sqrt(ms) < 1
  if (a.dtmin > 0.0) keep = keep || s.at_dtmin;
  const double fmin_ = keep ? 1.0 : a.factormin;
  double factor;
  if (a.i_controller && ms >= 1e-30 && ms <= 1e30) {
    // integral controller: factor = safety * (1/scaled)^(1/order) = safety * ms^(-1/(2 order))
    factor = fmin(fmax(a.safety * inv_root<ORDER>(ms), fmin_), a.factormax);
  } else {
    double inv = 1.0 / sqrt(ms);
    const double f1 = (a.c1 == 0.0) ? 1.0 : pow(inv, a.c1);
    const double f2 = (a.c2 == 0.0) ? 1.0 : pow(s.prev_inv, a.c2);
    const double f3 = (a.c3 == 0.0) ? 1.0 : pow(s.prev_prev_inv, a.c3);
    factor = fmin(fmax(a.safety * f1 * f2 * f3, fmin_), a.factormax);
    if (inv == 0.0 || isinf(inv)) inv = 1.0;
    if (keep) {
      s.prev_prev_inv = s.prev_inv;
      s.prev_inv = inv;
    }
  }
  double dt = h * factor;
  if (a.dtmax > 0.0) dt = fmin(dt, a.dtmax);
  if (a.dtmin > 0.0) {
    if (!a.force_dtmin && dt < a.dtmin) s.status = ORBIT_DT_MIN;
    s.at_dtmin = dt <= a.dtmin;
    dt = fmax(dt, a.dtmin);
  }
  next_t0 = keep ? s.tnext : s.tau;
  next_t1 = next_t0 + dt;
  return keep;
}

__device__ __forceinline__ double clip_to_end(double tprev, double tnext, double tau1, bool keep) {
  // diffrax _clip_to_end: float64 tolerance 1e-10
  if (tnext > tau1 - 1e-10) return keep ? tau1 : tprev + 0.5 * (tau1 - tprev);
  return tnext;
}

// LANES = 1: one thread per orbit. LANES = 32: one warp per orbit; Pot must
// then give every lane of the warp the bitwise-same gradient (WarpTablePot), so
// the 32 lanes run the orbit's steps in lockstep on identical values and their
// identical stores of saves, status and steps coincide.
template <class TB, class Pot, int LANES = 1>
__device__ void integrate_loop(const IntegrateArgs& a, const Pot& pot) {
  OrbitState s;
  s.orbit = -1;
  bool first = true;
  if (!start_orbit<TB, Pot, LANES>(a, pot, s, first)) return;
  double F[TB::S][6];
  while (true) {
    // One RK evaluation per iteration: either the main step from (tau, y) or,
    // for Dopri8, the sub-step from (tau, y) to a save time of the step just accepted.
    double hs;
    if (TB::FSAL || !s.pending) {
      hs = s.dir * (s.tnext - s.tau);
    } else {
      hs = s.dir * (save_tau(a, s, s.save_i) - s.tau);
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) F[0][j] = s.F0[j];
    rk_stages<TB>(pot, s.y, hs, F, s.dir * s.tau);
    double y1[6], err[6];
    int32_t st = ORBIT_OK;
    bool done = false;
    if (!TB::FSAL && s.pending) {
      rk_combine<TB>(s.y, hs, F, y1, nullptr);
      write_save(a, s, s.save_i, y1);
      ++s.save_i;
      if (s.save_i < s.save_end && save_tau(a, s, s.save_i) <= s.tau_new) continue;
      // all saves of the accepted step written: commit it
      s.pending = 0;
#pragma unroll
      for (int j = 0; j < 6; ++j) s.y[j] = s.ynew[j];
      s.tau = fmin(s.tau_new, s.tau1);
      field(pot, s.y, s.F0, s.dir * s.tau);
      s.tnext = s.tnext_new;
      if (s.status != ORBIT_OK) { done = true; st = s.status; }
      else if (s.tau >= s.tau1) done = true;
      else if (s.nsteps >= a.max_steps) { done = true; st = ORBIT_MAX_STEPS; }
      else if (maybe_park(a, s)) {
        if (!start_orbit<TB, Pot, LANES>(a, pot, s, first)) return;
        continue;
      }
    } else {
      rk_combine<TB>(s.y, hs, F, y1, a.adaptive ? err : nullptr);
      ++s.nsteps;
      const double h = s.tnext - s.tau;
      double next_t0, next_t1;
      bool keep;
      if (a.adaptive) {
        keep = pid_adapt<TB::ORDER>(a, s, y1, err, h, next_t0, next_t1);
      } else {
        keep = true;
        next_t0 = s.tnext;
        next_t1 = s.tnext + a.dt0;
      }
      bool finite = true;
#pragma unroll
      for (int j = 0; j < 6; ++j) finite = finite && isfinite(y1[j]);
      if (!finite) {
        done = true;
        st = ORBIT_NONFINITE;
      } else {
        const double tprev_new = fmin(next_t0, s.tau1);
        const double tnext_new = clip_to_end(tprev_new, next_t1, s.tau1, keep);
        if (keep) {
          ++s.naccepted;
          if constexpr (TB::FSAL) {
            // Dopri5: saves in (tau, tnext] from the quartic dense output
            if (s.save_i < s.save_end && save_tau(a, s, s.save_i) <= next_t0) {
              const double ih = 1.0 / h;
              do {
                const double th = (save_tau(a, s, s.save_i) - s.tau) * ih;
                double v[6];
                dopri5_dense(s.y, hs, F, th, v);
                write_save(a, s, s.save_i, v);
                ++s.save_i;
              } while (s.save_i < s.save_end && save_tau(a, s, s.save_i) <= next_t0);
            }
#pragma unroll
            for (int j = 0; j < 6; ++j) {
              s.y[j] = y1[j];
              s.F0[j] = F[TB::S - 1][j];
            }
            s.tau = tprev_new;
            s.tnext = tnext_new;
          } else {
            if (s.save_i < s.save_end && save_tau(a, s, s.save_i) <= next_t0) {
              // Dopri8 with saves inside this step: keep (tau, y) for the sub-steps
              s.pending = 1;
#pragma unroll
              for (int j = 0; j < 6; ++j) s.ynew[j] = y1[j];
              s.tau_new = next_t0;
              s.tnext_new = tnext_new;
              continue;
            }
#pragma unroll
            for (int j = 0; j < 6; ++j) s.y[j] = y1[j];
            s.tau = tprev_new;
            s.tnext = tnext_new;
            field(pot, s.y, s.F0, s.dir * s.tau);
          }
        } else {
          s.tau = tprev_new;
          s.tnext = tnext_new;
        }
        if (s.status != ORBIT_OK) { done = true; st = s.status; }
        else if (s.tau >= s.tau1) done = true;
        else if (s.nsteps >= a.max_steps) { done = true; st = ORBIT_MAX_STEPS; }
        else if (maybe_park(a, s)) {
          if (!start_orbit<TB, Pot, LANES>(a, pot, s, first)) return;
          continue;
        }
      }
    }
    if (done) {
      finish_orbit(a, s, st);
      if (!start_orbit<TB, Pot, LANES>(a, pot, s, first)) return;
    }
  }
}

}  // namespace gal
