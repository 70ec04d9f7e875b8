// Device-side potentials: value, gradient and Hessian of the closed-form
// components galax's orbit path uses, and of their sums.
//
// Formulas (r = sqrt(x^2 + y^2 + z^2 + DBL_MIN) as galax's r_spherical /
// safe_sqrt, src/galax/potential/_src/utils.py:45-125):
//   Kepler          Phi = -G m / r                       builtin/kepler.py
//   Hernquist       Phi = -G m / (r + r_s)               builtin/hernquist.py:80-82
//   Miyamoto-Nagai  Phi = -G m / sqrt(R^2 + (sqrt(z^2 + b^2) + a)^2)   builtin/miyamotonagai.py:73-78
//   NFW             Phi = -G m log1p(r / r_s) / r        builtin/nfw/base.py:326-338
//   Plummer         Phi = -G m / sqrt(r^2 + b^2)         builtin/plummer.py:122-133
//   Isochrone       Phi = -G m / (b + sqrt(r^2 + b^2))    builtin/isochrone.py:61-110
//   Logarithmic     Phi = v_c^2 / 2 log(r_s^2 + r^2)      builtin/logarithmic.py:45-53
//   Power law with cutoff  Phi = -G m P(a1, s^2) / r - G m Gamma(a2, s^2) / (r_c Gamma(a1)),
//                   s = r / r_c, a1 = (3 - alpha) / 2, a2 = 1 - alpha / 2
//                   builtin/powerlawcutoff.py:21-120 (galax: jax gammainc * gamma)
// galax differentiates these with jax.grad (src/galax/potential/_src/base.py:170-179);
// here the derivatives are written out analytically and arranged for the FP64
// pipe: reciprocal square roots instead of sqrt + divide, one shared radius for
// all centred spherical components, and one reciprocal for the three
// (r + r_s) factors of the Milky Way model.
#pragma once

#include <cstdint>

#include "log_table.h"

namespace gal {

enum Kind : int32_t { KEPLER = 0, HERNQUIST = 1, MIYAMOTO_NAGAI = 2, NFW = 3, PLUMMER = 4, ISOCHRONE = 5,
                      LOGARITHMIC = 6, POWERLAW_CUTOFF = 7 };

constexpr double TINY = 2.2250738585072014e-308;  // DBL_MIN, galax's safe_sqrt offset

// log(1 + u) for u >= 0 (the NFW halo's log(1 + r / r_s)) by Tang's
// table-driven method (P. T. P. Tang, "Table-driven implementation of the
// logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990):
// 1 + u = 2^k F_j (1 + r) with F_j = 1 + j/128 the nearest table point, so
// |r| <= 1/256; log(F_j) is tabulated as hi + lo and log(1 + r) is its Taylor
// polynomial to r^7 (truncation below 2e-18 relative). The rounding error of
// 1 + u is folded into r. About 20 FP64 operations, where a lone FP64 chain
// pays ~64 cycles for each; within ~1 unit in the last place.
__device__ __forceinline__ double log1p_pos(double u) {
  const double x = 1.0 + u;
  const double c = (u <= 1.0) ? u - (x - 1.0) : 1.0 - (x - u);  // x + c = 1 + u exactly
  const long long bits = __double_as_longlong(x);
  const int k = (int)(bits >> 52) - 1023;
  const long long mant = bits & 0x000FFFFFFFFFFFFFLL;
  const double m = __longlong_as_double(mant | 0x3FF0000000000000LL);  // x = 2^k m, 1 <= m < 2
  const int j = (int)((mant + (1LL << 44)) >> 45);                      // nearest j / 128, 0..128
  const double F = 1.0 + (double)j * 0.0078125;                         // exact
  const double scale = __longlong_as_double((long long)(1023 - k) << 52);  // 2^-k
  const double r = fma(c, scale, m - F) * __ldg(&kLogTable[j][0]);       // m - F is exact
  double q = fma(0.14285714285714285, r, -0.16666666666666666);
  q = fma(q, r, 0.2);
  q = fma(q, r, -0.25);
  q = fma(q, r, 0.3333333333333333);
  q = fma(q, r, -0.5);
  const double p = fma(r * r, q, r);
  const double dk = (double)k;
  const double hi = fma(dk, 0.6931471805599453, __ldg(&kLogTable[j][1]));   // ln 2 = hi + lo
  const double lo = fma(dk, 2.3190468138462996e-17, __ldg(&kLogTable[j][2]));
  return hi + (lo + p);
}

// Component with parameters folded for evaluation (96 bytes).
struct DevComp {
  int32_t kind;
  int32_t centered;  // 1 when origin == 0
  double Gm;         // G * m (v_c^2 for the logarithmic potential)
  double l1;         // a (MN) or r_s / b / r_c
  double l2;         // b (MN) or alpha (power law with cutoff)
  double l2sq;       // b^2 (MN), l1^2 (Plummer, isochrone, logarithmic) or 1 / Gamma(a1) (cutoff)
  double inv_l1;     // 1 / r_s (NFW) or 1 / r_c^2 (cutoff)
  double ox, oy, oz;
  double inv_m;      // d(log Gm)/dm: 1 / m, or 2 / v_c for the logarithmic potential
  double aux0;       // digamma(a1) (cutoff)
  double aux1;       // Gamma(a2) (cutoff)
};
static_assert(sizeof(DevComp) == 96, "DevComp layout");

// ----------------------------------------------------------- incomplete gamma
// gamma(a, x) for the power law with cutoff, 0 < a <= 3/2, x > 0: with
// e = x^a exp(-x), the lower function is e S (power series S = sum_n x^n /
// (a (a+1) ... (a+n)), Abramowitz & Stegun 6.5.29) for x < a + 1, and the upper
// one is e h (continued fraction h, A&S 6.5.31, modified Lentz evaluation)
// otherwise. With want_da the a-derivatives S' and h' are carried along the
// same recurrences. Both loops stop once the terms (and their derivatives)
// no longer change the sums, and after 400 terms at most.
struct IncGamma {
  bool series;  // true: lower = e sum; false: upper = e sum
  double lx;    // log x
  double e;     // x^a exp(-x)
  double sum, dsum;
};

__device__ __forceinline__ IncGamma inc_gamma(double a, double x, bool want_da) {
  IncGamma o;
  o.lx = log(x);
  o.e = exp(fma(a, o.lx, -x));
  o.dsum = 0.0;
  if (x < a + 1.0) {
    o.series = true;
    double t = 1.0 / a, h = -t, S = t, dS = t * h;
    for (int n = 1; n < 400; ++n) {
      const double ian = 1.0 / (a + n);
      t *= x * ian;
      S += t;
      if (want_da) {
        h -= ian;
        dS = fma(t, h, dS);
      }
      if (fabs(t) < 1e-17 * fabs(S) && (!want_da || fabs(t * h) < 1e-17 * fabs(dS))) break;
    }
    o.sum = S;
    o.dsum = dS;
    return o;
  }
  o.series = false;
  const double FP = 1e-300;
  double b = x + 1.0 - a, c = 1.0 / FP, d = 1.0 / b, hh = d;
  double dc = 0.0, dd = d * d, dh = dd;  // d/da: db/da = -1
  for (int i = 1; i < 400; ++i) {
    const double an = -i * (i - a);
    b += 2.0;
    double dp = fma(an, d, b);
    if (fabs(dp) < FP) dp = FP;
    const double cn = b + an / c;
    double ddel = 0.0;
    const double dnew = 1.0 / dp;
    if (want_da) {
      const double ddp = fma((double)i, d, fma(an, dd, -1.0));
      const double dcn = -1.0 + (i * c - an * dc) / (c * c);
      dc = dcn;
      dd = -ddp * dnew * dnew;
    }
    c = fabs(cn) < FP ? FP : cn;
    d = dnew;
    const double del = d * c;
    if (want_da) {
      ddel = fma(dd, c, d * dc);
      dh = fma(dh, del, hh * ddel);
    }
    hh *= del;
    if (fabs(del - 1.0) < 1e-17 && (!want_da || fabs(ddel) < 1e-17 * (1.0 + fabs(dh / hh)))) break;
  }
  o.sum = hh;
  o.dsum = dh;
  return o;
}

// Power law with cutoff: g(r) with grad Phi = g(r) x, and optionally g'(r)/r and
// the partials of g with respect to r_c and alpha.
struct PlcG {
  double g, gpr, dg_drc, dg_dalpha;
};

// Not inlined: the series / fraction loops would otherwise add to the register
// budget of every kernel that evaluates component tables.
static __device__ __noinline__ PlcG plc_g(const DevComp& c, double r2, double ir, bool want_hess, bool want_params) {
  const double a1 = fma(-0.5, c.l2, 1.5);
  const double x = r2 * c.inv_l1;  // (r / r_c)^2
  const IncGamma ig = inc_gamma(a1, x, want_params);
  const double eN = ig.e * c.l2sq;  // x^a1 e^-x / Gamma(a1)
  const double P = ig.series ? eN * ig.sum : 1.0 - eN * ig.sum;
  const double ir3 = ir * ir * ir;
  PlcG o;
  o.g = c.Gm * P * ir3;
  o.gpr = 0.0;
  o.dg_drc = 0.0;
  o.dg_dalpha = 0.0;
  if (want_hess) o.gpr = fma(2.0 * c.Gm * eN, ir3 * ir * ir, -3.0 * o.g * ir * ir);
  if (want_params) {
    // dP/da = e (log x S + S') / Gamma(a) - P psi(a) (lower), or -(e (log x h + h') / Gamma(a) - Q psi(a))
    const double dPda = ig.series ? fma(eN, fma(ig.lx, ig.sum, ig.dsum), -P * c.aux0)
                                  : -fma(eN, fma(ig.lx, ig.sum, ig.dsum), -(1.0 - P) * c.aux0);
    o.dg_drc = -2.0 * c.Gm * eN * ir3 * sqrt(c.inv_l1);
    o.dg_dalpha = -0.5 * c.Gm * dPda * ir3;
  }
  return o;
}

static __device__ __noinline__ double plc_phi(const DevComp& c, double dx, double dy, double dz) {
  const double r = sqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, TINY))));
  const double x = (r * r) * c.inv_l1;
  const double a1 = fma(-0.5, c.l2, 1.5), a2 = fma(-0.5, c.l2, 1.0);
  const IncGamma g1 = inc_gamma(a1, x, false), g2 = inc_gamma(a2, x, false);
  const double P1 = g1.series ? g1.e * g1.sum * c.l2sq : 1.0 - g1.e * g1.sum * c.l2sq;
  const double up2 = g2.series ? c.aux1 - g2.e * g2.sum : g2.e * g2.sum;  // Gamma(a2, x)
  return -c.Gm * (P1 / r + up2 * c.l2sq * sqrt(c.inv_l1));
}

// ----------------------------------------------------------- single components
__device__ __forceinline__ void comp_grad(const DevComp& c, double x, double y, double z, double& gx, double& gy,
                                          double& gz) {
  const double dx = x - c.ox, dy = y - c.oy, dz = z - c.oz;
  if (c.kind == MIYAMOTO_NAGAI) {
    const double zb2 = fma(dz, dz, c.l2sq);
    const double izb = rsqrt(zb2);
    const double zb = zb2 * izb;
    const double s = zb + c.l1;
    const double D2 = fma(dx, dx, fma(dy, dy, s * s));
    const double iD = rsqrt(D2);
    const double u = c.Gm * (iD * iD) * iD;
    gx = fma(u, dx, gx);
    gy = fma(u, dy, gy);
    gz = fma(u * s * izb, dz, gz);
    return;
  }
  const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, TINY)));
  const double ir = rsqrt(r2);
  double f;
  switch (c.kind) {
    case KEPLER:
      f = c.Gm * (ir * ir) * ir;
      break;
    case HERNQUIST: {
      const double d = fma(r2, ir, c.l1);
      f = c.Gm * ir / (d * d);
      break;
    }
    case NFW: {
      const double r = r2 * ir;
      const double L = log1p_pos(r * c.inv_l1);
      f = c.Gm * (ir * ir) * fma(L, ir, -1.0 / (c.l1 + r));
      break;
    }
    case ISOCHRONE: {
      const double s2 = r2 + c.l2sq;
      const double is = rsqrt(s2);
      const double d = fma(s2, is, c.l1);
      f = c.Gm * is / (d * d);
      break;
    }
    case LOGARITHMIC:
      f = c.Gm / (r2 + c.l2sq);
      break;
    case POWERLAW_CUTOFF:
      f = plc_g(c, r2, ir, false, false).g;
      break;
    default: {  // PLUMMER
      const double s2 = r2 + c.l2sq;
      const double is = rsqrt(s2);
      f = c.Gm * (is * is) * is;
      break;
    }
  }
  gx = fma(f, dx, gx);
  gy = fma(f, dy, gy);
  gz = fma(f, dz, gz);
}

__device__ __forceinline__ double comp_phi(const DevComp& c, double x, double y, double z) {
  const double dx = x - c.ox, dy = y - c.oy, dz = z - c.oz;
  switch (c.kind) {
    case MIYAMOTO_NAGAI: {
      const double zp = sqrt(fma(dz, dz, c.l2sq)) + c.l1;
      return -c.Gm / sqrt(fma(dx, dx, fma(dy, dy, zp * zp)));
    }
    case KEPLER:
      return -c.Gm / sqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, TINY))));
    case HERNQUIST:
      return -c.Gm / (sqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, TINY)))) + c.l1);
    case NFW: {
      const double r = sqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, TINY))));
      const double s = r * c.inv_l1;
      return -c.Gm * c.inv_l1 * log1p_pos(s) / s;
    }
    case ISOCHRONE: {
      const double r = sqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, TINY))));
      return -c.Gm / (c.l1 + sqrt(fma(r, r, c.l2sq)));
    }
    case LOGARITHMIC: {
      const double r = sqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, TINY))));
      return 0.5 * c.Gm * log(fma(r, r, c.l2sq));
    }
    case POWERLAW_CUTOFF: {
      return plc_phi(c, dx, dy, dz);
    }
    default: {
      const double r = sqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, TINY))));
      return -c.Gm / sqrt(fma(r, r, c.l2sq));
    }
  }
}

// Hessian accumulated into H[9] (row-major, symmetric).
__device__ __forceinline__ void comp_hessian(const DevComp& c, double x, double y, double z, double* H) {
  const double d[3] = {x - c.ox, y - c.oy, z - c.oz};
  if (c.kind == MIYAMOTO_NAGAI) {
    const double zb = sqrt(fma(d[2], d[2], c.l2sq));
    const double s = zb + c.l1;
    const double D2 = fma(d[0], d[0], fma(d[1], d[1], s * s));
    const double D = sqrt(D2);
    const double u = c.Gm / (D2 * D);
    const double w = 3.0 * c.Gm / (D2 * D2 * D);
    const double v[3] = {d[0], d[1], d[2] * s / zb};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) H[3 * i + j] -= w * v[i] * v[j];
    H[0] += u;
    H[4] += u;
    H[8] += u * (1.0 + c.l1 * c.l2sq / (zb * zb * zb));
    return;
  }
  const double r2 = fma(d[0], d[0], fma(d[1], d[1], fma(d[2], d[2], TINY)));
  const double r = sqrt(r2);
  double g, gpr;  // g(r) with grad = g x, and g'(r)/r
  switch (c.kind) {
    case KEPLER:
      g = c.Gm / (r2 * r);
      gpr = -3.0 * c.Gm / (r2 * r2 * r);
      break;
    case HERNQUIST: {
      const double dd = r + c.l1;
      g = c.Gm / (r * dd * dd);
      gpr = -c.Gm * (3.0 * r + c.l1) / (r2 * r * dd * dd * dd);
      break;
    }
    case NFW: {
      const double L = log1p_pos(r * c.inv_l1), q = c.l1 + r;
      g = c.Gm * (L / (r2 * r) - 1.0 / (r2 * q));
      gpr = c.Gm * (3.0 / (r2 * r2 * q) - 3.0 * L / (r2 * r2 * r) + 1.0 / (r2 * r * q * q));
      break;
    }
    case ISOCHRONE: {  // g = G m / ((b + s)^2 s), s = sqrt(r^2 + b^2)
      const double s2 = r2 + c.l2sq, s = sqrt(s2), d = c.l1 + s;
      g = c.Gm / (d * d * s);
      gpr = -g * (2.0 / (d * s) + 1.0 / s2);
      break;
    }
    case LOGARITHMIC: {  // g = v^2 / (r_s^2 + r^2)
      const double q = r2 + c.l2sq;
      g = c.Gm / q;
      gpr = -2.0 * g / q;
      break;
    }
    case POWERLAW_CUTOFF: {
      const PlcG t = plc_g(c, r2, 1.0 / r, true, false);
      g = t.g;
      gpr = t.gpr;
      break;
    }
    default: {
      const double s2 = r2 + c.l2sq, s = sqrt(s2);
      g = c.Gm / (s2 * s);
      gpr = -3.0 * c.Gm / (s2 * s2 * s);
      break;
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) H[3 * i + j] += gpr * d[i] * d[j];
  H[0] += g;
  H[4] += g;
  H[8] += g;
}

// ----------------------------------------------------------- folding
// digamma by upward recurrence to x >= 8 and the asymptotic series
// (Abramowitz & Stegun 6.3.18).
__host__ __device__ inline double digamma_fn(double x) {
  double acc = 0.0;
  // at most 8 shifts: the power law with cutoff needs x = (3 - alpha)/2 in
  // (0.5, 1.5]; outside that the result is not used, and the bound keeps a
  // huge negative x (x + 1 == x) from looping
  for (int i = 0; i < 8 && x < 8.0; ++i) {
    acc -= 1.0 / x;
    x += 1.0;
  }
  const double i2 = 1.0 / (x * x);
  return acc + log(x) - 0.5 / x -
         i2 * (1.0 / 12 - i2 * (1.0 / 120 - i2 * (1.0 / 252 - i2 * (1.0 / 240 - i2 * (1.0 / 132)))));
}

// Component parameters folded for evaluation (shared by the host, which folds
// static tables once, and by kernels that refold time-dependent components).
__host__ __device__ inline DevComp fold_comp(int32_t kind, double m, double l1, double l2, double ox, double oy,
                                             double oz, double G) {
  DevComp d{};
  d.kind = kind;
  d.centered = (ox == 0.0 && oy == 0.0 && oz == 0.0) ? 1 : 0;
  const bool log_kind = kind == LOGARITHMIC;  // m holds v_c: Phi scales with v_c^2, not G m
  d.Gm = log_kind ? m * m : G * m;
  d.l1 = l1;
  d.l2 = l2;
  d.l2sq = (kind == PLUMMER || kind == ISOCHRONE || log_kind) ? l1 * l1 : l2 * l2;
  d.inv_l1 = (kind == NFW) ? 1.0 / l1 : 0.0;
  d.inv_m = (m != 0.0) ? (log_kind ? 2.0 / m : 1.0 / m) : 0.0;
  d.ox = ox;
  d.oy = oy;
  d.oz = oz;
  if (kind == POWERLAW_CUTOFF) {
    const double a1 = 1.5 - 0.5 * l2, a2 = 1.0 - 0.5 * l2;
    d.l2sq = 1.0 / tgamma(a1);
    d.inv_l1 = 1.0 / (l1 * l1);
    d.aux0 = digamma_fn(a1);
    d.aux1 = tgamma(a2);
  }
  return d;
}

// Linear time dependence of one component (galax's LinearParameter,
// src/galax/potential/_src/params/core.py:25-110): p(t) = p0 + slope t for
// p in (m, l1, l2), with p0 the value at t = 0.
struct DevLinear {
  int32_t kind, active;
  double m0, l10, l20, dm, dl1, dl2, G;
};

__device__ __forceinline__ DevComp comp_at_time(const DevComp& c, const DevLinear& L, double t) {
  if (!L.active) return c;
  return fold_comp(L.kind, fma(L.dm, t, L.m0), fma(L.dl1, t, L.l10), fma(L.dl2, t, L.l20), c.ox, c.oy, c.oz, L.G);
}

// ----------------------------------------------------------- potential models
// General composite: a table of components (in shared memory inside kernels).
struct TablePot {
  const DevComp* c;
  int n;
  __device__ __forceinline__ void grad(double x, double y, double z, double& gx, double& gy, double& gz) const {
    gx = gy = gz = 0.0;
    for (int i = 0; i < n; ++i) comp_grad(c[i], x, y, z, gx, gy, gz);
  }
};

// A table whose components have linear time dependence: refolded at every
// evaluation time.
struct TimedTablePot {
  const DevComp* c;
  int n;
  const DevLinear* lin;
  __device__ __forceinline__ void grad_t(double t, double x, double y, double z, double& gx, double& gy,
                                         double& gz) const {
    gx = gy = gz = 0.0;
    for (int i = 0; i < n; ++i) comp_grad(comp_at_time(c[i], lin[i], t), x, y, z, gx, gy, gz);
  }
};

// A table evaluated by a whole warp for one orbit (integrate_loop with
// LANES = 32, for composites with many components): lane l sums components
// l, l + 32, ..., then a butterfly of xor-shuffles gives every lane the total.
// At each level a lane adds its partner's partial sum to its own while the
// partner adds the same two numbers in the other order; IEEE addition is
// commutative, so both get the same bits, and after five levels all 32 lanes
// hold bitwise-identical sums. Every lane of the warp must call it.
template <bool TIMED>
struct WarpTablePot {
  const DevComp* c;
  int n;
  const DevLinear* lin;  // TIMED: time-dependent parameters
  __device__ __forceinline__ void grad_t(double t, double x, double y, double z, double& gx, double& gy,
                                         double& gz) const {
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int i = threadIdx.x & 31; i < n; i += 32) {
      if constexpr (TIMED)
        comp_grad(comp_at_time(c[i], lin[i], t), x, y, z, ax, ay, az);
      else
        comp_grad(c[i], x, y, z, ax, ay, az);
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      ax += __shfl_xor_sync(0xffffffffu, ax, m);
      ay += __shfl_xor_sync(0xffffffffu, ay, m);
      az += __shfl_xor_sync(0xffffffffu, az, m);
    }
    gx = ax;
    gy = ay;
    gz = az;
  }
};

// Gradient of any potential model at time t: static models ignore t.
template <class Pot>
__device__ __forceinline__ void pot_grad_t(const Pot& p, double, double x, double y, double z, double& gx,
                                           double& gy, double& gz) {
  p.grad(x, y, z, gx, gy, gz);
}
__device__ __forceinline__ void pot_grad_t(const TimedTablePot& p, double t, double x, double y, double z,
                                           double& gx, double& gy, double& gz) {
  p.grad_t(t, x, y, z, gx, gy, gz);
}
template <bool TIMED>
__device__ __forceinline__ void pot_grad_t(const WarpTablePot<TIMED>& p, double t, double x, double y, double z,
                                           double& gx, double& gy, double& gz) {
  p.grad_t(t, x, y, z, gx, gy, gz);
}

// galax's MilkyWayPotential structure: Miyamoto-Nagai disk, NFW halo and two
// Hernquist spheres (bulge, nucleus), all centred on the origin
// (src/galax/potential/_src/builtin/milkyway.py:203-229).
struct MWParams {
  double Gm_d, a_d, b2_d;   // disk
  double Gm_h, rs_h, irs_h; // halo
  double Gm_b, rs_b;        // bulge
  double Gm_n, rs_n;        // nucleus
};

// The Milky Way gradient in four pieces, shared by MWPot::grad and the
// four-warp team kernel (which evaluates the pieces on different warps), so
// that both produce bitwise-identical results.
struct MWDisk {
  double u, us, izb;  // Gm_d / D^3, u s, 1 / sqrt(z^2 + b^2)
};
__device__ __forceinline__ MWDisk mw_disk(const MWParams& p, double x, double y, double z) {
  const double zb2 = fma(z, z, p.b2_d);
  const double izb = rsqrt(zb2);
  const double s = fma(zb2, izb, p.a_d);
  const double R2 = fma(x, x, y * y);
  const double iD = rsqrt(fma(s, s, R2));
  const double u = p.Gm_d * (iD * iD) * iD;
  return MWDisk{u, u * s, izb};
}
// centred spheres: 1/r and r
__device__ __forceinline__ double mw_ir(double x, double y, double z, double& r) {
  const double R2 = fma(x, x, y * y);
  const double r2 = fma(z, z, R2 + TINY);
  const double ir = rsqrt(r2);
  r = r2 * ir;
  return ir;
}
struct MWRecip {
  double inv_dh, inv_db2, inv_dn2;
};
// one reciprocal for 1/(r + rs_h), 1/(r + rs_b)^2, 1/(r + rs_n)^2
__device__ __forceinline__ MWRecip mw_recip(const MWParams& p, double r) {
  const double dh = p.rs_h + r, db = r + p.rs_b, dn = r + p.rs_n;
  const double db2 = db * db, dn2 = dn * dn;
  const double q = db2 * dn2;
  const double iP = 1.0 / (dh * q);
  return MWRecip{iP * q, iP * dh * dn2, iP * dh * db2};
}
__device__ __forceinline__ double mw_halo_log(const MWParams& p, double r) { return log1p_pos(r * p.irs_h); }
// radial factor of the three spheres
__device__ __forceinline__ double mw_f(const MWParams& p, double ir, double L, const MWRecip& c) {
  return p.Gm_h * (ir * ir) * fma(L, ir, -c.inv_dh) + ir * fma(p.Gm_b, c.inv_db2, p.Gm_n * c.inv_dn2);
}

struct MWPot {
  MWParams p;
  __device__ __forceinline__ void grad(double x, double y, double z, double& gx, double& gy, double& gz) const {
    const MWDisk d = mw_disk(p, x, y, z);
    double r;
    const double ir = mw_ir(x, y, z, r);
    const MWRecip c = mw_recip(p, r);
    const double L = mw_halo_log(p, r);
    const double f = mw_f(p, ir, L, c);
    gx = (d.u + f) * x;
    gy = (d.u + f) * y;
    gz = fma(d.us, d.izb, f) * z;
  }
};

}  // namespace gal
