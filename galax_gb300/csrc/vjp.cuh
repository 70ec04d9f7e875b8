// Reverse-mode pieces shared by the adjoint kernels: the Hessian-vector
// product and parameter derivatives of one component (the transposed Jacobian
// of the Hamiltonian field, f = (p, -grad Phi(q)) so J^T (u, v) = (-H(q) v, u)),
// and a plain constant-step Runge-Kutta step.
#pragma once

#include "integrate.cuh"

namespace gal {

constexpr int kAdjMaxComps = 8;

// H(x) v and d(grad Phi(x) . v)/d(m, l1, l2) of one component, accumulated.
__device__ __forceinline__ void comp_vjp(const DevComp& c, const double* x, const double* v, double* Hv,
                                         double* dp) {
  const double d0 = x[0] - c.ox, d1 = x[1] - c.oy, d2 = x[2] - c.oz;
  if (c.kind == MIYAMOTO_NAGAI) {
    const double zb2 = fma(d2, d2, c.l2sq);
    const double izb = rsqrt(zb2);
    const double zb = zb2 * izb;
    const double s = zb + c.l1;
    const double iD = rsqrt(fma(d0, d0, fma(d1, d1, s * s)));
    const double iD2 = iD * iD;
    const double u = c.Gm * iD2 * iD;
    const double w = 3.0 * u * iD2;
    const double vz = d2 * s * izb;
    const double vv = fma(d0, v[0], fma(d1, v[1], vz * v[2]));
    const double izb3 = izb * izb * izb;
    Hv[0] += fma(u, v[0], -w * vv * d0);
    Hv[1] += fma(u, v[1], -w * vv * d1);
    Hv[2] += fma(u * fma(c.l1 * c.l2sq, izb3, 1.0), v[2], -w * vv * vz);
    dp[0] += u * vv * c.inv_m;
    dp[1] += fma(-w * s, vv, u * d2 * izb * v[2]);
    dp[2] += fma(-w * s * c.l2 * izb, vv, -u * c.l1 * c.l2 * d2 * izb3 * v[2]);
    return;
  }
  const double r2 = fma(d0, d0, fma(d1, d1, fma(d2, d2, TINY)));
  const double ir = rsqrt(r2);
  const double ir2 = ir * ir;
  const double r = r2 * ir;
  const double xv = fma(d0, v[0], fma(d1, v[1], d2 * v[2]));
  double g, gpr, dl1 = 0.0, dl2 = 0.0;
  switch (c.kind) {
    case KEPLER:
      g = c.Gm * ir2 * ir;
      gpr = -3.0 * g * ir2;
      break;
    case HERNQUIST: {
      const double dd = r + c.l1, idd = 1.0 / dd;
      g = c.Gm * ir * idd * idd;
      gpr = -c.Gm * (3.0 * r + c.l1) * ir2 * ir * idd * idd * idd;
      dl1 = -2.0 * g * idd * xv;
      break;
    }
    case NFW: {
      const double L = log1p_pos(r * c.inv_l1), q = c.l1 + r, iq = 1.0 / q;
      g = c.Gm * ir2 * fma(L, ir, -iq);
      gpr = c.Gm * ir2 * ir * (3.0 * ir * iq - 3.0 * L * ir2 + iq * iq);
      dl1 = -c.Gm * ir * c.inv_l1 * iq * iq * xv;
      break;
    }
    case ISOCHRONE: {  // g = G m / ((b + s)^2 s); dg/db = -g (2 (1 + b/s) / (b + s) + b / s^2)
      const double s2 = r2 + c.l2sq, is = rsqrt(s2), s = s2 * is, d = c.l1 + s, id = 1.0 / d;
      g = c.Gm * is * id * id;
      gpr = -g * (2.0 * id * is + is * is);
      dl1 = -g * fma(2.0 * id, fma(c.l1, is, 1.0), c.l1 * is * is) * xv;
      break;
    }
    case LOGARITHMIC: {  // g = v^2 / (r_s^2 + r^2); dg/dr_s = -2 r_s g / q
      const double iq = 1.0 / (r2 + c.l2sq);
      g = c.Gm * iq;
      gpr = -2.0 * g * iq;
      dl1 = -2.0 * c.l1 * g * iq * xv;
      break;
    }
    case POWERLAW_CUTOFF: {
      const PlcG t = plc_g(c, r2, ir, true, true);
      g = t.g;
      gpr = t.gpr;
      dl1 = t.dg_drc * xv;
      dl2 = t.dg_dalpha * xv;
      break;
    }
    default: {  // PLUMMER
      const double is = rsqrt(r2 + c.l2sq), is2 = is * is;
      g = c.Gm * is2 * is;
      gpr = -3.0 * g * is2;
      dl1 = -3.0 * g * is2 * c.l1 * xv;
      break;
    }
  }
  Hv[0] += fma(g, v[0], gpr * xv * d0);
  Hv[1] += fma(g, v[1], gpr * xv * d1);
  Hv[2] += fma(g, v[2], gpr * xv * d2);
  dp[0] += g * xv * c.inv_m;
  dp[1] += dl1;
  dp[2] += dl2;
}

// One constant step of signed length hs from time t (static models ignore t).
template <class TB, class Pot>
__device__ __forceinline__ void rk_step_plain(const Pot& pot, double* y, double hs, double t = 0.0) {
  double F[TB::S][6], y1[6];
  field(pot, y, F[0], t);
  rk_stages<TB>(pot, y, hs, F, t);
  rk_combine<TB>(y, hs, F, y1, nullptr);
#pragma unroll
  for (int j = 0; j < 6; ++j) y[j] = y1[j];
}

}  // namespace gal
