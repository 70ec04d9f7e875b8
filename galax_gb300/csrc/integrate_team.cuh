// Four-warp teams for the longest orbits of an adaptive Dopri5 or Dopri8
// batch in the Milky Way model.
//
// The orbits that run longest set the duration of an uneven batch, and a lone
// orbit is latency-bound: a GB300 FP64 warp instruction holds its
// sub-partition's FP64 pipe for ~64 cycles however few lanes are active. A
// team block (4 warps, one per sub-partition) integrates 32 orbits, one per
// lane, and splits every field evaluation over the four warps:
//   warp 0: the spheres' radius and the shared reciprocal (mw_ir, mw_recip);
//   warp 1: the radius and the NFW halo's log(1 + r / r_s) (mw_halo_log);
//   warp 3: the Miyamoto-Nagai disk (mw_disk);
// and warps 0-2 own state components (w, w + 3), form the stage states and
// combine the pieces (mw_f) into their gradient component. Step control is
// computed redundantly by all four warps from the same shared-memory values.
// Every operation matches the one-thread-per-orbit kernel (k_integrate_mw with
// MWPot::grad, integrate_loop), so results are bitwise identical.
//
// Dopri5 is FSAL: a step's last stage is the next step's first slope. Dopri8
// is not, and follows integrate_loop's non-FSAL branch: after an accepted step
// the slope at the new state is one more team round, and saves inside an
// accepted step are written by sub-steps of the partial length from the
// step's start (the orbit stays "pending" until its last save of the step),
// each one RK evaluation of its own.
//
// Used for the second pass of the two-pass schedule only: every orbit resumes
// from its parked state.
#pragma once

#include "integrate.cuh"

namespace gal {

struct TeamShared {
  // field-evaluation exchange, double-buffered by round parity
  double pos[2][3][kTeamLanes];
  double u[2][kTeamLanes], us[2][kTeamLanes], izb[2][kTeamLanes];
  double ir[2][kTeamLanes], L[2][kTeamLanes];
  double inv_dh[2][kTeamLanes], inv_db2[2][kTeamLanes], inv_dn2[2][kTeamLanes];
  // controller exchange
  double y1[6][kTeamLanes], err[6][kTeamLanes];
  long long slot[kTeamLanes];
};

// Y_j = y_j + hs sum_{l<I} A[I][l] F_l,j for one component (stage_state's arithmetic).
template <class TB, int I>
__device__ __forceinline__ double stage_comp(double yj, double hs, const double (&Fj)[TB::S]) {
  double acc = 0.0;
  bool first = true;
  static_for<0, I>([&](auto l) {
    constexpr int L = decltype(l)::value;
    constexpr double c = TB::A[I][L];
    if constexpr (c != 0.0) {
      acc = first ? c * Fj[L] : fma(c, Fj[L], acc);
      first = false;
    }
  });
  return fma(hs, acc, yj);
}

// weighted<TB, WHICH> for one component: y_j + hs sum_l w_l F_l,j, or
// hs sum_l w_l F_l,j without y.
template <class TB, int WHICH, bool WITH_Y>
__device__ __forceinline__ double weighted_comp(double yj, double hs, const double (&Fj)[TB::S]) {
  double acc = 0.0;
  bool first = true;
  static_for<0, TB::S>([&](auto l) {
    constexpr int L = decltype(l)::value;
    constexpr double c = weight<TB, WHICH, L>();
    if constexpr (c != 0.0) {
      acc = first ? c * Fj[L] : fma(c, Fj[L], acc);
      first = false;
    }
  });
  if constexpr (WITH_Y) return fma(hs, acc, yj);
  return hs * acc;
}

// dopri5_dense for one component.
__device__ __forceinline__ double dense_comp(double y0j, double hs, const double (&Fj)[Dopri5::S], double th) {
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
  double acc = W[0] * Fj[0];
  static_for<1, Dopri5::S>([&](auto i) {
    constexpr int I = decltype(i)::value;
    if constexpr (I != 1) acc = fma(W[I], Fj[I], acc);
  });
  return fma(hs, acc, y0j);
}

// One team field evaluation: the owners (warps 0-2) have put the position
// components in pos[b][w]; returns warp w's gradient component (w < 3).
__device__ __forceinline__ double team_grad(TeamShared& sh, int b, int warp, int lane, const MWParams& p) {
  __syncthreads();  // positions written
  const double x = sh.pos[b][0][lane], y = sh.pos[b][1][lane], z = sh.pos[b][2][lane];
  if (warp == 0) {
    double r;
    const double ir = mw_ir(x, y, z, r);
    const MWRecip c = mw_recip(p, r);
    sh.ir[b][lane] = ir;
    sh.inv_dh[b][lane] = c.inv_dh;
    sh.inv_db2[b][lane] = c.inv_db2;
    sh.inv_dn2[b][lane] = c.inv_dn2;
  } else if (warp == 1) {
    double r;
    mw_ir(x, y, z, r);
    sh.L[b][lane] = mw_halo_log(p, r);
  } else if (warp == 3) {
    const MWDisk d = mw_disk(p, x, y, z);
    sh.u[b][lane] = d.u;
    sh.us[b][lane] = d.us;
    sh.izb[b][lane] = d.izb;
  }
  __syncthreads();  // pieces written
  if (warp > 2) return 0.0;
  const MWRecip c{sh.inv_dh[b][lane], sh.inv_db2[b][lane], sh.inv_dn2[b][lane]};
  const double f = mw_f(p, sh.ir[b][lane], sh.L[b][lane], c);
  const double u = sh.u[b][lane];
  if (warp == 0) return (u + f) * x;
  if (warp == 1) return (u + f) * y;
  return fma(sh.us[b][lane], sh.izb[b][lane], f) * z;
}

__device__ __forceinline__ void team_write_save(const IntegrateArgs& a, const OrbitState& s, int64_t k, int j,
                                                double v) {
  a.out[j * a.out_stride + save_index(a, s, k)] = v;
}

// tqueue: the team's position counter; positions [0, min(tcap, *a.queue_len))
// of a.order are the team's.
template <class TB>
__global__ void __launch_bounds__(128, 1) k_integrate_mw_team(IntegrateArgs a, MWParams p,
                                                              unsigned long long* tqueue, long long tcap) {
  constexpr int S = TB::S;
  __shared__ TeamShared sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool owner = warp < 3;
  const int j0 = warp, j1 = warp + 3;  // owned components (warps 0-2)
  const long long qlen = (long long)*a.queue_len;
  const long long tlen = qlen < tcap ? qlen : tcap;
  OrbitState s{};
  s.orbit = -1;
  bool need_orbit = true, queue_open = true;
  double yo0 = 0.0, yo1 = 0.0;  // owned state components j0, j1 (s.y holds all six for the controller)
  double yn0 = 0.0, yn1 = 0.0;  // Dopri8: owned components of the accepted end state while saves are pending
  double F0[2] = {0.0, 0.0};    // owned components of the slope at (tau, y)
  bool need_f0 = false;         // Dopri8: the slope at a newly committed state is still to be evaluated
  int round = 0;
  while (true) {
    // ---- lanes without an orbit take the next queue position (warp 0 dequeues)
    if (warp == 0 && need_orbit && queue_open) {
      const unsigned long long k = atomicAdd(tqueue, 1ULL);
      sh.slot[lane] = ((long long)k < tlen) ? (long long)a.order[k] : -1;
    }
    __syncthreads();
    bool fresh = false;
    if (need_orbit && queue_open) {
      const long long o = sh.slot[lane];
      if (o < 0) {
        queue_open = false;
      } else {  // resume a parked orbit (start_orbit, phase 1)
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
        const OrbitResume& r = a.resume[o];
#pragma unroll
        for (int j = 0; j < 6; ++j) s.y[j] = r.y[j];
        yo0 = r.y[j0 < 6 ? j0 : 0];
        yo1 = r.y[j1 < 6 ? j1 : 0];
        s.tau = r.tau;
        s.tnext = r.tnext;
        s.prev_inv = r.prev_inv;
        s.prev_prev_inv = r.prev_prev_inv;
        s.nsteps = r.nsteps;
        s.naccepted = r.naccepted;
        s.save_i = r.save_i;
        s.at_dtmin = r.at_dtmin;
        s.status = r.status;
        fresh = true;
        need_orbit = false;
      }
    }
    const bool active = s.orbit >= 0;
    if (!__syncthreads_or(active)) break;
    // ---- slope at resumed (and, for Dopri8, newly committed) states: one team
    // round, only when a lane needs it
    const bool want_f0 = fresh || (need_f0 && active);
    if (__syncthreads_or(want_f0)) {
      const int b = round++ & 1;
      if (owner) sh.pos[b][warp][lane] = want_f0 ? yo0 : 8.0;
      const double g = team_grad(sh, b, warp, lane, p);
      if (owner && want_f0) {
        F0[0] = yo1;
        F0[1] = -g;
      }
    }
    need_f0 = false;
    // ---- one RK evaluation (integrate_loop): a step from (tau, y), or for
    // Dopri8 with saves pending the sub-step from (tau, y) to the next save
    const bool sub = !TB::FSAL && s.pending && active;
    const double hs = sub ? s.dir * (save_tau(a, s, s.save_i) - s.tau) : s.dir * (s.tnext - s.tau);
    double Fp[S], Fv[S];  // owned components of the stage slopes: position j0, velocity j1
    Fp[0] = F0[0];
    Fv[0] = F0[1];
    static_for<1, S>([&](auto i) {
      constexpr int I = decltype(i)::value;
      const int b = round++ & 1;
      double Yv = 0.0;
      if (owner) {
        const double Yp = stage_comp<TB, I>(yo0, hs, Fp);
        Yv = stage_comp<TB, I>(yo1, hs, Fv);
        sh.pos[b][warp][lane] = active ? Yp : 8.0;
      }
      const double g = team_grad(sh, b, warp, lane, p);
      Fp[I] = Yv;
      Fv[I] = -g;
    });
    // solution and error for the owned components, then the shared controller
    double y1o0 = 0.0, y1o1 = 0.0;
    if (owner) {
      y1o0 = weighted_comp<TB, W_SOLUTION, true>(yo0, hs, Fp);
      y1o1 = weighted_comp<TB, W_SOLUTION, true>(yo1, hs, Fv);
      sh.y1[j0][lane] = y1o0;
      sh.y1[j1][lane] = y1o1;
      if (a.adaptive && !sub) {
        sh.err[j0][lane] = weighted_comp<TB, W_ERROR, false>(0.0, hs, Fp);
        sh.err[j1][lane] = weighted_comp<TB, W_ERROR, false>(0.0, hs, Fv);
      }
    }
    __syncthreads();
    double y1[6], err[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      y1[j] = sh.y1[j][lane];
      err[j] = a.adaptive ? sh.err[j][lane] : 0.0;
    }
    __syncthreads();  // the exchange arrays are reused next step
    if (!active) continue;
    if constexpr (!TB::FSAL) {
      if (sub) {  // the partial step's end is a save of the accepted step
        if (owner) {
          team_write_save(a, s, s.save_i, j0, y1o0);
          team_write_save(a, s, s.save_i, j1, y1o1);
        }
        ++s.save_i;
        if (s.save_i < s.save_end && save_tau(a, s, s.save_i) <= s.tau_new) continue;
        // all saves of the accepted step written: commit it
        s.pending = 0;
#pragma unroll
        for (int j = 0; j < 6; ++j) s.y[j] = s.ynew[j];
        yo0 = yn0;
        yo1 = yn1;
        s.tau = fmin(s.tau_new, s.tau1);
        need_f0 = true;
        s.tnext = s.tnext_new;
        bool done = false;
        int32_t st = ORBIT_OK;
        if (s.status != ORBIT_OK) {
          done = true;
          st = s.status;
        } else if (s.tau >= s.tau1) {
          done = true;
        } else if (s.nsteps >= a.max_steps) {
          done = true;
          st = ORBIT_MAX_STEPS;
        }
        if (done) {
          if (warp == 0) {
            finish_orbit(a, s, st);
          } else {
            s.orbit = -1;
          }
          need_orbit = true;
          need_f0 = false;
        }
        continue;
      }
    }
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
    bool done = false;
    int32_t st = ORBIT_OK;
    if (!finite) {
      done = true;
      st = ORBIT_NONFINITE;
    } else {
      const double tprev_new = fmin(next_t0, s.tau1);
      const double tnext_new = clip_to_end(tprev_new, next_t1, s.tau1, keep);
      if (keep) {
        ++s.naccepted;
        if constexpr (TB::FSAL) {
          if (s.save_i < s.save_end && save_tau(a, s, s.save_i) <= next_t0) {
            const double ih = 1.0 / h;
            do {
              const double th = (save_tau(a, s, s.save_i) - s.tau) * ih;
              if (owner) {
                team_write_save(a, s, s.save_i, j0, dense_comp(yo0, hs, Fp, th));
                team_write_save(a, s, s.save_i, j1, dense_comp(yo1, hs, Fv, th));
              }
              ++s.save_i;
            } while (s.save_i < s.save_end && save_tau(a, s, s.save_i) <= next_t0);
          }
#pragma unroll
          for (int j = 0; j < 6; ++j) s.y[j] = y1[j];
          yo0 = y1o0;
          yo1 = y1o1;
          F0[0] = Fp[S - 1];
          F0[1] = Fv[S - 1];
          s.tau = tprev_new;
          s.tnext = tnext_new;
        } else {
          if (s.save_i < s.save_end && save_tau(a, s, s.save_i) <= next_t0) {
            // saves inside this step: keep (tau, y) for the sub-steps
            s.pending = 1;
#pragma unroll
            for (int j = 0; j < 6; ++j) s.ynew[j] = y1[j];
            yn0 = y1o0;
            yn1 = y1o1;
            s.tau_new = next_t0;
            s.tnext_new = tnext_new;
            continue;
          }
#pragma unroll
          for (int j = 0; j < 6; ++j) s.y[j] = y1[j];
          yo0 = y1o0;
          yo1 = y1o1;
          s.tau = tprev_new;
          s.tnext = tnext_new;
          need_f0 = true;
        }
      } else {
        s.tau = tprev_new;
        s.tnext = tnext_new;
      }
      if (s.status != ORBIT_OK) {
        done = true;
        st = s.status;
      } else if (s.tau >= s.tau1) {
        done = true;
      } else if (s.nsteps >= a.max_steps) {
        done = true;
        st = ORBIT_MAX_STEPS;
      }
    }
    if (done) {
      if (warp == 0) {
        finish_orbit(a, s, st);
      } else {
        s.orbit = -1;
      }
      need_orbit = true;
      need_f0 = false;
    }
  }
}

}  // namespace gal
