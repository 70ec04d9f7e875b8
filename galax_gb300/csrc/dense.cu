// Dense output: the integrator records, for every accepted step, what is needed
// to evaluate the orbit anywhere inside that step afterwards. Replaces
// diffrax's DenseInterpolation as galax wraps it in PhaseSpaceInterpolation
// (src/galax/dynamics/_src/orbit/interp.py:42-145) for evaluate_orbit(...,
// dense=True) (dynamics/_src/legacy/funcs.py:42-51).
//
// Per orbit: the step boundaries ts[0..nsteps] (original time) and per step
//   Dopri5: the quartic p(theta) = a0 + a1 theta + ... + a4 theta^4 (5 x 6
//           doubles), the same polynomial the save path evaluates (through y0,
//           y1, the Shampine midpoint, f0 and f1; diffrax's
//           FourthOrderPolynomialInterpolation), in monomial form;
//   Dopri8: the step's start state (6 doubles); evaluation takes one Dopri8
//           step of the partial length from it, exactly as the save path.
// One thread per orbit, own controller, no work queue; evaluation is one
// thread per query (binary search for the step, then Horner or the sub-step).
#include <cuda_runtime.h>

#include "handle.h"
#include "integrate.cuh"

namespace gal {

__device__ __forceinline__ MWPot bind_table(const MWPot& p, const DevComp*) { return p; }
__device__ __forceinline__ TablePot bind_table(const TablePot& p, const DevComp* s) { return TablePot{s, p.n}; }
__device__ __forceinline__ TimedTablePot bind_table(const TimedTablePot& p, const DevComp* s) {
  return TimedTablePot{s, p.n, p.lin};
}

// Solver fields of gal_integrate's argument block (the same mapping as gal_integrate).
static IntegrateArgs make_integrate_args(const gal_solver_config* cfg) {
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
  return a;
}

template <class TB>
struct DenseCoef;
template <>
struct DenseCoef<Dopri5> {
  static constexpr int NC = 5;
};
template <>
struct DenseCoef<Dopri8> {
  static constexpr int NC = 1;
};

// Monomial coefficients (powers 1..4) of the four basis polynomials of the
// Dopri5 quartic (integrate.cuh::dopri5_dense):
//   H1 = -5 th^2 + 14 th^3 - 8 th^4, Hm = 16 th^2 - 32 th^3 + 16 th^4,
//   Hf0 = th - 4 th^2 + 5 th^3 - 2 th^4, Hf1 = th^2 - 3 th^3 + 2 th^4.
template <int K, int I>
__host__ __device__ constexpr double quartic_weight() {
  constexpr double h1[5] = {0, 0, -5, 14, -8};
  constexpr double hm[5] = {0, 0, 16, -32, 16};
  constexpr double hf0[5] = {0, 1, -4, 5, -2};
  constexpr double hf1[5] = {0, 0, 1, -3, 2};
  double w = h1[K] * Dopri5::B[I] + hm[K] * Dopri5::CMID[I];
  if (I == 0) w += hf0[K];
  if (I == Dopri5::S - 1) w += hf1[K];
  return w;
}

template <class TB>
__device__ __forceinline__ void record_step(double* c, const double* y, double hs, const double (&F)[TB::S][6]) {
  if constexpr (DenseCoef<TB>::NC == 1) {
#pragma unroll
    for (int j = 0; j < 6; ++j) c[j] = y[j];
  } else {
#pragma unroll
    for (int j = 0; j < 6; ++j) c[j] = y[j];
    static_for<1, 5>([&](auto kk) {
      constexpr int K = decltype(kk)::value;
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        double acc = 0.0;
        static_for<0, TB::S>([&](auto i) {
          constexpr int I = decltype(i)::value;
          constexpr double w = quartic_weight<K, I>();
          if constexpr (w != 0.0) acc = fma(w, F[I][j], acc);
        });
        c[6 * K + j] = hs * acc;
      }
    });
  }
}

template <class TB, class Pot>
__global__ void __launch_bounds__(128) k_integrate_dense(IntegrateArgs a, Pot pot, const DevComp* comps, int ncomp,
                                                         int64_t cap, double* __restrict__ ts,
                                                         double* __restrict__ coef, int64_t* __restrict__ nsteps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevComp* s_comps = reinterpret_cast<DevComp*>(smem_raw);
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) s_comps[i] = comps[i];
  __syncthreads();
  const Pot P = bind_table(pot, s_comps);
  const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= a.n) return;
  constexpr int NC = DenseCoef<TB>::NC;
  double* tso = ts + o * (cap + 1);
  double* co = coef + o * cap * NC * 6;
  OrbitState s;
  s.orbit = o;
  const double t0 = a.t0[o], t1 = a.t1[o];
  s.dir = (t0 < t1) ? 1.0 : -1.0;
  s.tau0 = s.dir * t0;
  s.tau1 = s.dir * t1;
  s.tau = s.tau0;
#pragma unroll
  for (int j = 0; j < 6; ++j) s.y[j] = a.y0[j * a.n + o];
  s.nsteps = 0;
  s.naccepted = 0;
  s.prev_inv = 1.0;
  s.prev_prev_inv = 1.0;
  s.at_dtmin = 0;
  s.status = ORBIT_OK;
  tso[0] = t0;
  int64_t m = 0;
  int32_t st = ORBIT_OK;
  if (t0 == t1) {  // nothing to integrate: the interpolant is the initial state
#pragma unroll
    for (int j = 0; j < 6; ++j) co[j] = s.y[j];
  } else if (!isfinite(t0) || !isfinite(t1)) {  // an infinite span never ends: report it at once
#pragma unroll
    for (int j = 0; j < 6; ++j) co[j] = __longlong_as_double(0x7ff8000000000000LL);
    st = ORBIT_NONFINITE;
  } else {
    field(P, s.y, s.F0, t0);
    double dt;
    if (a.adaptive) {
      dt = a.dt0 > 0.0 ? a.dt0 : initial_step<TB>(a, P, s.y, s.F0, s.dir, t0);
      if (a.dtmax > 0.0) dt = fmin(dt, a.dtmax);
      if (a.dtmin > 0.0) {
        s.at_dtmin = dt <= a.dtmin;
        dt = fmax(dt, a.dtmin);
      }
    } else {
      dt = a.dt0;
    }
    s.tnext = fmin(s.tau + dt, s.tau1);
    double F[TB::S][6];
    while (true) {
      const double hs = s.dir * (s.tnext - s.tau);
#pragma unroll
      for (int j = 0; j < 6; ++j) F[0][j] = s.F0[j];
      rk_stages<TB>(P, s.y, hs, F, s.dir * s.tau);
      double y1[6], err[6];
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
        st = ORBIT_NONFINITE;
        break;
      }
      const double tprev_new = fmin(next_t0, s.tau1);
      const double tnext_new = clip_to_end(tprev_new, next_t1, s.tau1, keep);
      if (keep) {
        if (m >= cap) {
          st = ORBIT_MAX_STEPS;
          break;
        }
        record_step<TB>(co + m * NC * 6, s.y, hs, F);
        tso[m + 1] = s.dir * tprev_new;
        ++m;
#pragma unroll
        for (int j = 0; j < 6; ++j) s.y[j] = y1[j];
        if constexpr (TB::FSAL) {
#pragma unroll
          for (int j = 0; j < 6; ++j) s.F0[j] = F[TB::S - 1][j];
        } else {
          field(P, s.y, s.F0, s.dir * tprev_new);
        }
      }
      s.tau = tprev_new;
      s.tnext = tnext_new;
      if (s.status != ORBIT_OK) {
        st = s.status;
        break;
      }
      if (s.tau >= s.tau1) break;
      if (s.nsteps >= a.max_steps) {
        st = ORBIT_MAX_STEPS;
        break;
      }
    }
  }
  nsteps[o] = m;
  if (a.status) a.status[o] = st;
}

template <class TB, class Pot>
__global__ void __launch_bounds__(128) k_dense_eval(Pot pot, const DevComp* comps, int ncomp, const double* ts,
                                                    const double* coef, const int64_t* nsteps, int64_t cap,
                                                    int64_t n, const int64_t* orbit, const double* tq, int64_t m,
                                                    double* out, unsigned long long* oob) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevComp* s_comps = reinterpret_cast<DevComp*>(smem_raw);
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) s_comps[i] = comps[i];
  __syncthreads();
  const Pot P = bind_table(pot, s_comps);
  constexpr int NC = DenseCoef<TB>::NC;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = orbit[q];
    const double t = tq[q];
    double v[6];
    const double nanv = __longlong_as_double(0x7ff8000000000000LL);
    bool ok = o >= 0 && o < n;
    int64_t ns = ok ? nsteps[o] : 0;
    const double* tso = ok ? ts + o * (cap + 1) : ts;
    const double dir = (ok && ns > 0 && tso[ns] < tso[0]) ? -1.0 : 1.0;
    const double tau = dir * t;
    if (ok) ok = ns > 0 ? (tau >= dir * tso[0] && tau <= dir * tso[ns]) : (t == tso[0]);
    if (!ok) {
#pragma unroll
      for (int j = 0; j < 6; ++j) v[j] = nanv;
      atomicAdd(oob, 1ULL);
    } else if (ns == 0) {  // t0 == t1: the orbit is its initial state
      const double* c = coef + o * cap * NC * 6;
#pragma unroll
      for (int j = 0; j < 6; ++j) v[j] = cap > 0 ? c[j] : nanv;
    } else {
      // last step k with dir * ts[k] <= tau (the final time belongs to the last step)
      int64_t lo = 0, hi = ns - 1;
      while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (dir * tso[mid] <= tau) lo = mid;
        else hi = mid - 1;
      }
      const double* c = coef + (o * cap + lo) * NC * 6;
      const double ta = dir * tso[lo], tb = dir * tso[lo + 1];
      if constexpr (NC == 5) {
        const double th = (tau - ta) / (tb - ta);
#pragma unroll
        for (int j = 0; j < 6; ++j)
          v[j] = fma(th, fma(th, fma(th, fma(th, c[24 + j], c[18 + j]), c[12 + j]), c[6 + j]), c[j]);
      } else {
        double y[6], F[TB::S][6];
#pragma unroll
        for (int j = 0; j < 6; ++j) y[j] = c[j];
        const double hs = dir * (tau - ta);
        field(P, y, F[0], tso[lo]);  // tso[lo]: the step's start time
        rk_stages<TB>(P, y, hs, F, tso[lo]);
        rk_combine<TB>(y, hs, F, v, nullptr);
      }
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) out[j * m + q] = v[j];
  }
}

}  // namespace gal

using namespace gal;

extern "C" {

int32_t gal_dense_coef_per_step(int32_t method) { return method == 5 ? 30 : (method == 8 ? 6 : 0); }

gal_status gal_integrate_dense(const gal_potential* pot, const gal_solver_config* cfg, const double* y0,
                               const double* t0, const double* t1, int64_t n, int64_t cap, double* ts, double* coef,
                               int64_t* nsteps, int32_t* status, gal_stream_t stream) {
  if (!pot) return fail(GAL_ERR_INVALID_ARGUMENT, "potential is NULL");
  gal_status st = validate_cfg(cfg);
  if (st != GAL_OK) return st;
  if (n < 0 || cap < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "n >= 0 and cap >= 1 required");
  if (n == 0) return GAL_OK;
  if (!y0 || !t0 || !t1 || !ts || !coef || !nsteps) return fail(GAL_ERR_INVALID_ARGUMENT, "NULL array");
  IntegrateArgs a = make_integrate_args(cfg);
  a.y0 = y0;
  a.t0 = t0;
  a.t1 = t1;
  a.status = status;
  a.n = n;
  const unsigned grid = (unsigned)((n + 127) / 128);
  const size_t smem = pot->is_mw ? 0 : sizeof(DevComp) * (size_t)pot->n;
  cudaStream_t s = (cudaStream_t)stream;
  if (smem > 48 * 1024) return fail(GAL_ERR_UNSUPPORTED, "dense output supports tables up to 48 KB");
  auto run = [&](auto tb) {
    using TB = decltype(tb);
    if (pot->is_mw)
      k_integrate_dense<TB, MWPot><<<grid, 128, 0, s>>>(a, MWPot{pot->mw}, pot->d_comps, 0, cap, ts, coef, nsteps);
    else if (pot->d_lin)  // LinearParameter components, refolded at every stage time
      k_integrate_dense<TB, TimedTablePot><<<grid, 128, smem, s>>>(
          a, TimedTablePot{pot->d_comps, pot->n, pot->d_lin}, pot->d_comps, pot->n, cap, ts, coef, nsteps);
    else
      k_integrate_dense<TB, TablePot><<<grid, 128, smem, s>>>(a, TablePot{pot->d_comps, pot->n}, pot->d_comps,
                                                              pot->n, cap, ts, coef, nsteps);
  };
  if (cfg->method == 8)
    run(Dopri8{});
  else
    run(Dopri5{});
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "dense integration launch");
}

gal_status gal_dense_evaluate(const gal_potential* pot, int32_t method, const double* ts, const double* coef,
                              const int64_t* nsteps, int64_t cap, int64_t n, const int64_t* orbit, const double* t,
                              int64_t m, double* out, unsigned long long* out_of_bounds, gal_stream_t stream) {
  if (!pot || (method != 5 && method != 8)) return fail(GAL_ERR_INVALID_ARGUMENT, "bad potential or method");
  if (m < 0 || n < 0 || cap < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "bad sizes");
  if (m == 0) return GAL_OK;
  if (!ts || !coef || !nsteps || !orbit || !t || !out || !out_of_bounds)
    return fail(GAL_ERR_INVALID_ARGUMENT, "NULL array");
  int64_t grid = (m + 127) / 128;
  const int64_t capg = (int64_t)device_sm_count() * 16;
  if (grid > capg) grid = capg;
  const size_t smem = pot->is_mw ? 0 : sizeof(DevComp) * (size_t)pot->n;
  if (smem > 48 * 1024) return fail(GAL_ERR_UNSUPPORTED, "dense output supports tables up to 48 KB");
  cudaStream_t s = (cudaStream_t)stream;
  auto run = [&](auto tb) {
    using TB = decltype(tb);
    const unsigned g = (unsigned)grid;
    if (pot->is_mw)
      k_dense_eval<TB, MWPot><<<g, 128, 0, s>>>(MWPot{pot->mw}, pot->d_comps, 0, ts, coef, nsteps, cap, n, orbit, t,
                                                m, out, out_of_bounds);
    else if (pot->d_lin && TB::S == Dopri8::S)  // Dopri8 re-evaluates the field: at the step's own times
      k_dense_eval<TB, TimedTablePot><<<g, 128, smem, s>>>(TimedTablePot{pot->d_comps, pot->n, pot->d_lin},
                                                           pot->d_comps, pot->n, ts, coef, nsteps, cap, n, orbit, t,
                                                           m, out, out_of_bounds);
    else
      k_dense_eval<TB, TablePot><<<g, 128, smem, s>>>(TablePot{pot->d_comps, pot->n}, pot->d_comps, pot->n, ts,
                                                      coef, nsteps, cap, n, orbit, t, m, out, out_of_bounds);
  };
  if (method == 8)
    run(Dopri8{});
  else
    run(Dopri5{});
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "dense evaluation launch");
}

}  // extern "C"
