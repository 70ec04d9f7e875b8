// CPU FP64 oracle for the galax orbit-integration hot path.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain C++17, the arithmetic
// that GalacticDynamics/galax (and its pinned ODE engine diffrax 0.7.0)
// performs on the `evaluate_orbit` / `AbstractPotential.gradient` path. The
// tests compare the CUDA library against it and the benchmark times it as the
// CPU baseline; nothing in the shipped package links or calls it.
//
// What is restated, and from where:
//   * closed-form potentials
//       Kepler     Phi = -G m / r                 src/galax/potential/_src/builtin/kepler.py
//       Hernquist  Phi = -G m / (r + r_s)         src/galax/potential/_src/builtin/hernquist.py:80-82
//       Miyamoto-Nagai                            src/galax/potential/_src/builtin/miyamotonagai.py:73-78
//       NFW        Phi = -G m log1p(r/r_s) / r    src/galax/potential/_src/builtin/nfw/base.py:326-338
//       Plummer    Phi = -G m / sqrt(r^2 + b^2)   src/galax/potential/_src/builtin/plummer.py:122-133
//       Isochrone  Phi = -G m / (b + sqrt(r^2 + b^2))  src/galax/potential/_src/builtin/isochrone.py:61-110
//       Logarithmic Phi = v_c^2 / 2 log(r_s^2 + r^2)  src/galax/potential/_src/builtin/logarithmic.py:45-53
//                  (the component's m field holds v_c)
//     with r = sqrt(x^2+y^2+z^2 + DBL_MIN)        src/galax/potential/_src/utils.py:45-77
//     composite = sum over components             src/galax/potential/_src/base_multi.py:39-55
//   * gradient = analytic derivative of Phi (the reference uses jax.grad of the
//     same closed form, src/galax/potential/_src/base.py:170-179); Hessians the
//     same (base.py:230-239).
//   * Hamilton's equations dq/dt = p, dp/dt = -grad Phi
//                                              src/galax/dynamics/_src/orbit/field_hamiltonian.py:240-249
//   * explicit Runge-Kutta steps with the published Dormand-Prince 5(4)
//     (Dormand & Prince 1980) and Prince-Dormand 8(7) 13-stage "RK8(7)13M"
//     (Prince & Dormand 1981) pairs, the Dopri5 midpoint dense output of
//     Shampine (1986), and diffrax's documented step-size logic: PID controller
//     (rtol/atol RMS error norm, safety 0.9, factor clip [0.2, 10], factor >= 1
//     after an accepted step), Hairer-Norsett-Wanner initial-step selection
//     (h1 = (0.01 / max(d1, d2))^(1/(p+1))),
//     clipping of the last step onto t1 with a 1e-10 tolerance, and reversed
//     time for t1 < t0. Callers in the reference:
//       src/galax/dynamics/_src/legacy/integrator.py:161-168, 228-230
//       src/galax/dynamics/_src/orbit/solver.py:121-141
//       src/galax/dynamics/_src/fields.py:168-188
//   * saves at requested times. Dopri5 uses the quartic through y0, y1, y_mid,
//     f0, f1 as diffrax does. For Dopri8 the value at a save time inside a step
//     is one Dopri8 step of size (t_save - t_n) from the step's start point:
//     the same order as the integrator itself (diffrax's own 7th-order Dopri8
//     interpolant is not a published formula that can be restated).
//   * a discrete adjoint of the fixed-step RK map (gradients of a terminal loss
//     with respect to the initial conditions and every component parameter).
//
// Build: g++ -O2 -fopenmp -shared -fPIC (see oracle/build_oracle.py).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---------------------------------------------------------------------------
// Operation counter (used to fix the algorithmic flop count of one step).
// ---------------------------------------------------------------------------
struct OpCount {
  long long add = 0, mul = 0, div = 0, sqrt = 0, log1p = 0, cmp = 0;
};
static OpCount g_ops;

struct CD {  // counted double
  double v;
  CD() : v(0) {}
  CD(double x) : v(x) {}
};
inline CD operator+(CD a, CD b) { g_ops.add++; return CD(a.v + b.v); }
inline CD operator-(CD a, CD b) { g_ops.add++; return CD(a.v - b.v); }
inline CD operator-(CD a) { return CD(-a.v); }
inline CD operator*(CD a, CD b) { g_ops.mul++; return CD(a.v * b.v); }
inline CD operator/(CD a, CD b) { g_ops.div++; return CD(a.v / b.v); }
inline CD& operator+=(CD& a, CD b) { a = a + b; return a; }
inline CD& operator-=(CD& a, CD b) { a = a - b; return a; }
inline CD& operator*=(CD& a, CD b) { a = a * b; return a; }
inline CD sqrt(CD a) { g_ops.sqrt++; return CD(std::sqrt(a.v)); }
inline CD log1p(CD a) { g_ops.log1p++; return CD(std::log1p(a.v)); }
inline double val(CD a) { return a.v; }
inline double val(double a) { return a; }
using std::sqrt;
using std::log1p;

// ---------------------------------------------------------------------------
// Potential components. Same memory layout as the product's gal_component.
// ---------------------------------------------------------------------------
enum Kind : int32_t { KEPLER = 0, HERNQUIST = 1, MIYAMOTO_NAGAI = 2, NFW = 3, PLUMMER = 4, ISOCHRONE = 5, LOGARITHMIC = 6,
                      POWERLAW_CUTOFF = 7 };

struct Comp {
  int32_t kind;
  int32_t flags;
  double m;       // mass: m_tot (Kepler, Hernquist, MN, Plummer) or m (NFW)
  double l1;      // r_s (Hernquist, NFW, Plummer) or a (MN)
  double l2;      // b (MN)
  double origin[3];
};
static_assert(sizeof(Comp) == 56, "component layout");

static const double TINY = std::numeric_limits<double>::min();  // 2.2250738585072014e-308

// ---------------------------------------------------------------------------
// Incomplete gamma function for the power-law-with-cutoff sphere (galax
// builtin/powerlawcutoff.py:21-23, jax.scipy gammainc * gamma). Regularised
// P(a, x) = gamma(a, x) / Gamma(a) by the power series (Abramowitz & Stegun
// 6.5.29) for x < a + 1 and by the continued fraction of Q = 1 - P (A&S 6.5.31,
// modified Lentz evaluation) otherwise; dP/da by differentiating the same
// series / fraction term by term. psi = digamma by recurrence to x >= 8 and
// the asymptotic series (A&S 6.3.18).
// ---------------------------------------------------------------------------
static double digamma(double x) {
  double acc = 0.0;
  for (int i = 0; i < 8 && x < 8.0; ++i) {  // x in (0.5, 1.5] here; bounded for any input
    acc -= 1.0 / x;
    x += 1.0;
  }
  const double i2 = 1.0 / (x * x);
  return acc + std::log(x) - 0.5 / x -
         i2 * (1.0 / 12 - i2 * (1.0 / 120 - i2 * (1.0 / 252 - i2 * (1.0 / 240 - i2 * (1.0 / 132)))));
}

struct GammaP {
  double P, dPda;  // regularised lower incomplete gamma and its a-derivative
  double upper;    // unregularised upper incomplete gamma Gamma(a, x)
};

static GammaP gamma_p(double a, double x) {
  GammaP o{0.0, 0.0, std::tgamma(a)};
  if (!(x > 0.0)) return o;
  const double lga = std::lgamma(a), psi = digamma(a);
  const double lx = std::log(x);
  const double pre = std::exp(a * lx - x - lga);  // x^a e^-x / Gamma(a)
  if (x < a + 1.0) {
    double t = 1.0 / a, h = -1.0 / a, S = t, dS = t * h;
    for (int n = 1; n < 1000; ++n) {
      t *= x / (a + n);
      h -= 1.0 / (a + n);
      S += t;
      dS += t * h;
      if (std::fabs(t) < std::fabs(S) * 1e-17 && std::fabs(t * h) < std::fabs(dS) * 1e-17) break;
    }
    o.P = pre * S;
    o.dPda = o.P * (lx - psi) + pre * dS;
    o.upper = std::tgamma(a) * (1.0 - o.P);
    return o;
  }
  // Lentz on (value, d/da) pairs
  const double FP = 1e-300;
  double b = x + 1.0 - a, db = -1.0;
  double c = 1.0 / FP, dc = 0.0;
  double d = 1.0 / b, dd = -db / (b * b);
  double hh = d, dh = dd;
  for (int i = 1; i < 1000; ++i) {
    const double an = -i * (i - a), dan = i;
    b += 2.0;
    double dpre = an * d + b, ddpre = dan * d + an * dd + db;
    if (std::fabs(dpre) < FP) dpre = FP;
    const double cn = b + an / c, dcn = db + (dan * c - an * dc) / (c * c);
    c = std::fabs(cn) < FP ? FP : cn;
    dc = dcn;
    d = 1.0 / dpre;
    dd = -ddpre / (dpre * dpre);
    const double del = d * c, ddel = dd * c + d * dc;
    dh = dh * del + hh * ddel;
    hh *= del;
    // the value can converge before its a-derivative (a fraction that ends,
    // an = 0, at integer a): both must have settled
    if (std::fabs(del - 1.0) < 1e-17 && std::fabs(ddel) < 1e-17 * (1.0 + std::fabs(dh / hh))) break;
  }
  const double Q = pre * hh;
  o.P = 1.0 - Q;
  o.dPda = -(Q * (lx - psi) + pre * dh);
  o.upper = std::exp(a * lx - x) * hh;
  return o;
}

// g(r) of grad Phi = g(r) x for the power law with cutoff: g = G M P(a1, s^2) / r^3,
// a1 = 3/2 - alpha/2, s = r / r_c, and its partials.
struct PlcTerms {
  double g, gpr, dg_drc, dg_dalpha;
};
static PlcTerms plc_terms(double Gm, double rc, double alpha, double r2) {
  const double a1 = 1.5 - 0.5 * alpha, x = r2 / (rc * rc), r = std::sqrt(r2);
  const GammaP gp = gamma_p(a1, x);
  const double dens = std::exp(a1 * std::log(x) - x - std::lgamma(a1));  // x^a1 e^-x / Gamma(a1)
  PlcTerms t;
  t.g = Gm * gp.P / (r2 * r);
  t.gpr = 2.0 * Gm * dens / (r2 * r2 * r) - 3.0 * t.g / r2;
  t.dg_drc = -2.0 * Gm * dens / (r2 * r * rc);
  t.dg_dalpha = -0.5 * Gm * gp.dPda / (r2 * r);
  return t;
}

template <class T>
inline T rsph2(const T* x) { return x[0] * x[0] + x[1] * x[1] + x[2] * x[2]; }

template <class T>
T comp_potential(const Comp& c, double G, const T* xin) {
  T x[3] = {xin[0] - T(c.origin[0]), xin[1] - T(c.origin[1]), xin[2] - T(c.origin[2])};
  const T Gm = T(G) * T(c.m);
  switch (c.kind) {
    case KEPLER: {
      T r = sqrt(rsph2(x) + T(TINY));
      return -Gm / r;
    }
    case HERNQUIST: {
      T r = sqrt(rsph2(x) + T(TINY));
      return -Gm / (r + T(c.l1));
    }
    case MIYAMOTO_NAGAI: {
      T R2 = x[0] * x[0] + x[1] * x[1];
      T zp = sqrt(x[2] * x[2] + T(c.l2) * T(c.l2)) + T(c.l1);
      return -Gm / sqrt(R2 + zp * zp);
    }
    case NFW: {
      T r = sqrt(rsph2(x) + T(TINY));
      T s = r / T(c.l1);
      return -Gm / T(c.l1) * log1p(s) / s;
    }
    case PLUMMER: {
      T r = sqrt(rsph2(x) + T(TINY));
      return -Gm / sqrt(r * r + T(c.l1) * T(c.l1));
    }
    case ISOCHRONE: {
      T r = sqrt(rsph2(x) + T(TINY));
      return -Gm / (T(c.l1) + sqrt(r * r + T(c.l1) * T(c.l1)));
    }
    case LOGARITHMIC: {
      T r = sqrt(rsph2(x) + T(TINY));
      return T(0.5) * T(c.m) * T(c.m) * log(T(c.l1) * T(c.l1) + r * r);
    }
    case POWERLAW_CUTOFF: {  // -G M P(a1, s^2) / r - G M Gamma(a2, s^2) / (r_c Gamma(a1)), a2 = 1 - alpha/2
      const double rv = std::sqrt(val(rsph2(x)) + TINY), rc = c.l1, a1 = 1.5 - 0.5 * c.l2;
      const double s2 = (rv / rc) * (rv / rc);
      const GammaP p1 = gamma_p(a1, s2), p2 = gamma_p(1.0 - 0.5 * c.l2, s2);
      return T(-val(Gm) * p1.P / rv - val(Gm) * p2.upper / (rc * std::tgamma(a1)));
    }
  }
  return T(0);
}

// g(r) such that grad Phi = g(r) * x for spherical components.
template <class T>
void comp_gradient(const Comp& c, double G, const T* xin, T* g) {
  T x[3] = {xin[0] - T(c.origin[0]), xin[1] - T(c.origin[1]), xin[2] - T(c.origin[2])};
  const T Gm = T(G) * T(c.m);
  if (c.kind == MIYAMOTO_NAGAI) {
    T a = T(c.l1), b = T(c.l2);
    T zb = sqrt(x[2] * x[2] + b * b);
    T s = zb + a;
    T D2 = x[0] * x[0] + x[1] * x[1] + s * s;
    T D = sqrt(D2);
    T u = Gm / (D2 * D);
    g[0] += u * x[0];
    g[1] += u * x[1];
    g[2] += u * x[2] * s / zb;
    return;
  }
  T r2 = rsph2(x) + T(TINY);
  T r = sqrt(r2);
  T f;
  switch (c.kind) {
    case KEPLER: f = Gm / (r2 * r); break;
    case HERNQUIST: { T d = r + T(c.l1); f = Gm / (r * d * d); break; }
    case NFW: {
      T rs = T(c.l1);
      f = Gm * (log1p(r / rs) / r - T(1) / (rs + r)) / r2;
      break;
    }
    case PLUMMER: { T s2 = r2 + T(c.l1) * T(c.l1); f = Gm / (s2 * sqrt(s2)); break; }
    case ISOCHRONE: {
      T b = T(c.l1), s = sqrt(r2 + b * b), d = b + s;
      f = Gm / (d * d * s);
      break;
    }
    case LOGARITHMIC: { f = T(c.m) * T(c.m) / (r2 + T(c.l1) * T(c.l1)); break; }
    case POWERLAW_CUTOFF: { f = T(plc_terms(val(Gm), c.l1, c.l2, val(r2)).g); break; }
    default: f = T(0);
  }
  g[0] += f * x[0];
  g[1] += f * x[1];
  g[2] += f * x[2];
}

// Hessian (row-major 3x3) accumulated into H.
void comp_hessian(const Comp& c, double G, const double* xin, double* H) {
  double x[3] = {xin[0] - c.origin[0], xin[1] - c.origin[1], xin[2] - c.origin[2]};
  const double Gm = G * c.m;
  if (c.kind == MIYAMOTO_NAGAI) {
    double a = c.l1, b = c.l2;
    double zb = std::sqrt(x[2] * x[2] + b * b);
    double s = zb + a;
    double D2 = x[0] * x[0] + x[1] * x[1] + s * s;
    double D = std::sqrt(D2);
    double u = Gm / (D2 * D);
    double w = 3.0 * Gm / (D2 * D2 * D);
    double vz = x[2] * s / zb;  // d(D^2/2)/dz
    double v[3] = {x[0], x[1], vz};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) H[3 * i + j] -= w * v[i] * v[j];
    H[0] += u;
    H[4] += u;
    H[8] += u * (1.0 + a * b * b / (zb * zb * zb));
    return;
  }
  double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + TINY;
  double r = std::sqrt(r2);
  double g = 0, gpr = 0;  // g(r), g'(r)/r
  switch (c.kind) {
    case KEPLER: g = Gm / (r2 * r); gpr = -3.0 * Gm / (r2 * r2 * r); break;
    case HERNQUIST: {
      double d = r + c.l1;
      g = Gm / (r * d * d);
      gpr = -Gm * (3.0 * r + c.l1) / (r2 * r * d * d * d);
      break;
    }
    case NFW: {
      double rs = c.l1, L = std::log1p(r / rs), q = rs + r;
      g = Gm * (L / (r2 * r) - 1.0 / (r2 * q));
      gpr = Gm * (3.0 / (r2 * r2 * q) - 3.0 * L / (r2 * r2 * r) + 1.0 / (r2 * r * q * q));
      break;
    }
    case PLUMMER: {
      double s2 = r2 + c.l1 * c.l1, s = std::sqrt(s2);
      g = Gm / (s2 * s);
      gpr = -3.0 * Gm / (s2 * s2 * s);
      break;
    }
    case ISOCHRONE: {  // g = G m / ((b + s)^2 s), g'/r = -g (2 / ((b + s) s) + 1 / s^2)
      double b = c.l1, s2 = r2 + b * b, s = std::sqrt(s2), d = b + s;
      g = Gm / (d * d * s);
      gpr = -g * (2.0 / (d * s) + 1.0 / s2);
      break;
    }
    case LOGARITHMIC: {  // g = v^2 / (r_s^2 + r^2), g'/r = -2 g / (r_s^2 + r^2)
      double q = r2 + c.l1 * c.l1;
      g = c.m * c.m / q;
      gpr = -2.0 * g / q;
      break;
    }
    case POWERLAW_CUTOFF: {
      const PlcTerms t = plc_terms(Gm, c.l1, c.l2, r2);
      g = t.g;
      gpr = t.gpr;
      break;
    }
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) H[3 * i + j] += gpr * x[i] * x[j];
  H[0] += g;
  H[4] += g;
  H[8] += g;
}

// d(grad Phi)/d(param) dotted with v, accumulated into out[3] = (d/dm, d/dl1, d/dl2).
void comp_dgrad_dparams_dot(const Comp& c, double G, const double* xin, const double* v, double* out) {
  double x[3] = {xin[0] - c.origin[0], xin[1] - c.origin[1], xin[2] - c.origin[2]};
  const double Gm = G * c.m;
  double gr[3] = {0, 0, 0};
  comp_gradient<double>(c, G, xin, gr);
  double gv = gr[0] * v[0] + gr[1] * v[1] + gr[2] * v[2];
  out[0] += c.kind == LOGARITHMIC ? 2.0 * gv / c.m : gv / c.m;  // grad Phi ~ v_c^2 for the logarithmic
  if (c.kind == MIYAMOTO_NAGAI) {
    double a = c.l1, b = c.l2;
    double zb = std::sqrt(x[2] * x[2] + b * b);
    double s = zb + a;
    double D2 = x[0] * x[0] + x[1] * x[1] + s * s;
    double D = std::sqrt(D2);
    double u = Gm / (D2 * D);
    double w = 3.0 * Gm / (D2 * D2 * D);
    double vz = x[2] * s / zb;
    double xv = x[0] * v[0] + x[1] * v[1] + vz * v[2];  // (x, y, z s/zb) . v
    // d/da: du/da = -w s ; d(z s/zb)/da = z/zb
    out[1] += -w * s * xv + u * (x[2] / zb) * v[2];
    // d/db: du/db = -w s b/zb ; d(z s/zb)/db = -a b z / zb^3
    out[2] += -w * s * b / zb * xv + u * (-a * b * x[2] / (zb * zb * zb)) * v[2];
    return;
  }
  double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + TINY;
  double r = std::sqrt(r2);
  double xv = x[0] * v[0] + x[1] * v[1] + x[2] * v[2];
  switch (c.kind) {
    case HERNQUIST: { double d = r + c.l1; out[1] += -2.0 * Gm / (r * d * d * d) * xv; break; }
    case NFW: { double rs = c.l1, q = rs + r; out[1] += -Gm / (r * rs * q * q) * xv; break; }
    case PLUMMER: { double s2 = r2 + c.l1 * c.l1; out[1] += -3.0 * Gm * c.l1 / (s2 * s2 * std::sqrt(s2)) * xv; break; }
    case ISOCHRONE: {  // d/db [G m / ((b + s)^2 s)] = -g (b / s^2 + 2 (1 + b / s) / (b + s))
      double b = c.l1, s2 = r2 + b * b, s = std::sqrt(s2), d = b + s, g = Gm / (d * d * s);
      out[1] += -g * (b / s2 + 2.0 * (1.0 + b / s) / d) * xv;
      break;
    }
    case LOGARITHMIC: {  // d/dr_s [v^2 / (r_s^2 + r^2)] = -2 r_s v^2 / (r_s^2 + r^2)^2
      double q = r2 + c.l1 * c.l1;
      out[1] += -2.0 * c.l1 * c.m * c.m / (q * q) * xv;
      break;
    }
    case POWERLAW_CUTOFF: {
      const PlcTerms t = plc_terms(Gm, c.l1, c.l2, r2);
      out[1] += t.dg_drc * xv;
      out[2] += t.dg_dalpha * xv;
      break;
    }
    default: break;
  }
}

// Components; slopes (n x 3, or NULL) make (m, l1, l2) linear in time,
// p(t) = p + slope t, with the table holding the values at t = 0 (galax's
// LinearParameter, src/galax/potential/_src/params/core.py:25-110, in
// point-slope form p(t) = slope (t - t_i) + p(t_i)).
struct Pot {
  const Comp* comps;
  int n;
  double G;
  const double* slopes = nullptr;
};

inline Comp comp_at(const Pot& P, int i, double t) {
  Comp c = P.comps[i];
  if (P.slopes) {
    c.m += P.slopes[3 * i] * t;
    c.l1 += P.slopes[3 * i + 1] * t;
    c.l2 += P.slopes[3 * i + 2] * t;
  }
  return c;
}

template <class T>
inline void gradient(const Pot& P, const T* x, T* g, double t = 0.0) {
  g[0] = g[1] = g[2] = T(0);
  for (int i = 0; i < P.n; ++i) comp_gradient<T>(comp_at(P, i, t), P.G, x, g);
}

// Hamiltonian field with optional time reversal (sign = -1).
template <class T>
inline void field(const Pot& P, double sign, const T* y, T* dy, double t = 0.0) {
  T g[3];
  gradient<T>(P, y, g, t);
  dy[0] = T(sign) * y[3];
  dy[1] = T(sign) * y[4];
  dy[2] = T(sign) * y[5];
  dy[3] = T(-sign) * g[0];
  dy[4] = T(-sign) * g[1];
  dy[5] = T(-sign) * g[2];
}

// ---------------------------------------------------------------------------
// Butcher tableaux.
// ---------------------------------------------------------------------------
struct Tableau {
  int s;                 // stages
  int order;             // error order used by the controller
  bool fsal;
  double c[13];
  double a[13][13];
  double b[13];
  double e[13];          // b - bhat
};

static Tableau make_dopri5() {
  Tableau T{};
  T.s = 7; T.order = 5; T.fsal = true;
  double c[7] = {0, 1.0 / 5, 3.0 / 10, 4.0 / 5, 8.0 / 9, 1, 1};
  for (int i = 0; i < 7; ++i) T.c[i] = c[i];
  T.a[1][0] = 1.0 / 5;
  T.a[2][0] = 3.0 / 40; T.a[2][1] = 9.0 / 40;
  T.a[3][0] = 44.0 / 45; T.a[3][1] = -56.0 / 15; T.a[3][2] = 32.0 / 9;
  T.a[4][0] = 19372.0 / 6561; T.a[4][1] = -25360.0 / 2187; T.a[4][2] = 64448.0 / 6561; T.a[4][3] = -212.0 / 729;
  T.a[5][0] = 9017.0 / 3168; T.a[5][1] = -355.0 / 33; T.a[5][2] = 46732.0 / 5247; T.a[5][3] = 49.0 / 176;
  T.a[5][4] = -5103.0 / 18656;
  T.a[6][0] = 35.0 / 384; T.a[6][2] = 500.0 / 1113; T.a[6][3] = 125.0 / 192; T.a[6][4] = -2187.0 / 6784;
  T.a[6][5] = 11.0 / 84;
  double b[7] = {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84, 0};
  double bh[7] = {5179.0 / 57600, 0, 7571.0 / 16695, 393.0 / 640, -92097.0 / 339200, 187.0 / 2100, 1.0 / 40};
  for (int i = 0; i < 7; ++i) { T.b[i] = b[i]; T.e[i] = b[i] - bh[i]; }
  return T;
}

static Tableau make_dopri8() {
  Tableau T{};
  T.s = 13; T.order = 8; T.fsal = false;
  double c[13] = {0, 1.0 / 18, 1.0 / 12, 1.0 / 8, 5.0 / 16, 3.0 / 8, 59.0 / 400, 93.0 / 200,
                  5490023248.0 / 9719169821.0, 13.0 / 20, 1201146811.0 / 1299019798.0, 1, 1};
  for (int i = 0; i < 13; ++i) T.c[i] = c[i];
  T.a[1][0] = 1.0 / 18;
  T.a[2][0] = 1.0 / 48; T.a[2][1] = 1.0 / 16;
  T.a[3][0] = 1.0 / 32; T.a[3][2] = 3.0 / 32;
  T.a[4][0] = 5.0 / 16; T.a[4][2] = -75.0 / 64; T.a[4][3] = 75.0 / 64;
  T.a[5][0] = 3.0 / 80; T.a[5][3] = 3.0 / 16; T.a[5][4] = 3.0 / 20;
  T.a[6][0] = 29443841.0 / 614563906.0; T.a[6][3] = 77736538.0 / 692538347.0;
  T.a[6][4] = -28693883.0 / 1125000000.0; T.a[6][5] = 23124283.0 / 1800000000.0;
  T.a[7][0] = 16016141.0 / 946692911.0; T.a[7][3] = 61564180.0 / 158732637.0;
  T.a[7][4] = 22789713.0 / 633445777.0; T.a[7][5] = 545815736.0 / 2771057229.0;
  T.a[7][6] = -180193667.0 / 1043307555.0;
  T.a[8][0] = 39632708.0 / 573591083.0; T.a[8][3] = -433636366.0 / 683701615.0;
  T.a[8][4] = -421739975.0 / 2616292301.0; T.a[8][5] = 100302831.0 / 723423059.0;
  T.a[8][6] = 790204164.0 / 839813087.0; T.a[8][7] = 800635310.0 / 3783071287.0;
  T.a[9][0] = 246121993.0 / 1340847787.0; T.a[9][3] = -37695042795.0 / 15268766246.0;
  T.a[9][4] = -309121744.0 / 1061227803.0; T.a[9][5] = -12992083.0 / 490766935.0;
  T.a[9][6] = 6005943493.0 / 2108947869.0; T.a[9][7] = 393006217.0 / 1396673457.0;
  T.a[9][8] = 123872331.0 / 1001029789.0;
  T.a[10][0] = -1028468189.0 / 846180014.0; T.a[10][3] = 8478235783.0 / 508512852.0;
  T.a[10][4] = 1311729495.0 / 1432422823.0; T.a[10][5] = -10304129995.0 / 1701304382.0;
  T.a[10][6] = -48777925059.0 / 3047939560.0; T.a[10][7] = 15336726248.0 / 1032824649.0;
  T.a[10][8] = -45442868181.0 / 3398467696.0; T.a[10][9] = 3065993473.0 / 597172653.0;
  T.a[11][0] = 185892177.0 / 718116043.0; T.a[11][3] = -3185094517.0 / 667107341.0;
  T.a[11][4] = -477755414.0 / 1098053517.0; T.a[11][5] = -703635378.0 / 230739211.0;
  T.a[11][6] = 5731566787.0 / 1027545527.0; T.a[11][7] = 5232866602.0 / 850066563.0;
  T.a[11][8] = -4093664535.0 / 808688257.0; T.a[11][9] = 3962137247.0 / 1805957418.0;
  T.a[11][10] = 65686358.0 / 487910083.0;
  T.a[12][0] = 403863854.0 / 491063109.0; T.a[12][3] = -5068492393.0 / 434740067.0;
  T.a[12][4] = -411421997.0 / 543043805.0; T.a[12][5] = 652783627.0 / 914296604.0;
  T.a[12][6] = 11173962825.0 / 925320556.0; T.a[12][7] = -13158990841.0 / 6184727034.0;
  T.a[12][8] = 3936647629.0 / 1978049680.0; T.a[12][9] = -160528059.0 / 685178525.0;
  T.a[12][10] = 248638103.0 / 1413531060.0;
  double b[13] = {14005451.0 / 335480064.0, 0, 0, 0, 0, -59238493.0 / 1068277825.0,
                  181606767.0 / 758867731.0, 561292985.0 / 797845732.0, -1041891430.0 / 1371343529.0,
                  760417239.0 / 1151165299.0, 118820643.0 / 751138087.0, -528747749.0 / 2220607170.0, 1.0 / 4};
  double bh[13] = {13451932.0 / 455176623.0, 0, 0, 0, 0, -808719846.0 / 976000145.0,
                   1757004468.0 / 5645159321.0, 656045339.0 / 265891186.0, -3867574721.0 / 1518517206.0,
                   465885868.0 / 322736535.0, 53011238.0 / 667516719.0, 2.0 / 45, 0};
  for (int i = 0; i < 13; ++i) { T.b[i] = b[i]; T.e[i] = b[i] - bh[i]; }
  return T;
}

static const Tableau DOPRI5 = make_dopri5();
static const Tableau DOPRI8 = make_dopri8();

// Shampine (1986) midpoint weights for the Dopri5 dense output (already halved,
// i.e. y(t0 + h/2) ~= y0 + sum_i cmid_i k_i with k_i = h f_i).
static const double DOPRI5_CMID[7] = {
    6025192743.0 / 30085553152.0 / 2, 0, 51252292925.0 / 65400821598.0 / 2,
    -2691868925.0 / 45128329728.0 / 2, 187940372067.0 / 1594534317056.0 / 2,
    -1776094331.0 / 19743644256.0 / 2, 11237099.0 / 235043384.0 / 2};

// ---------------------------------------------------------------------------
// One RK step for an m-orbit lockstep system (6m doubles).
// Stage values are kept as slopes F_i = f(Y_i); increments are h * F_i.
// ---------------------------------------------------------------------------
template <class T>
struct System {
  const Pot* P;
  int m;            // orbits in lockstep
  double sign;      // +1 forward, -1 reversed time
  // tau: the integration variable sign * t
  void f(double tau, const T* y, T* dy) const {
    for (int o = 0; o < m; ++o) field<T>(*P, sign, y + 6 * o, dy + 6 * o, sign * tau);
  }
};

// F holds the stage slopes f(Y_i) (s x n); Y is an n-scratch. The step is
// y1 = y0 + h sum_i b_i F_i and err = h sum_i e_i F_i (diffrax's ODE form).
template <class T>
void rk_step(const System<T>& S, const Tableau& TB, double tau, const T* y0, const T* f0, double h,
             T* F, T* Y, T* y1, T* err) {
  const int n = 6 * S.m;
  for (int j = 0; j < n; ++j) F[j] = f0[j];
  for (int i = 1; i < TB.s; ++i) {
    for (int j = 0; j < n; ++j) {
      T acc = T(0);
      bool first = true;
      for (int l = 0; l < i; ++l)
        if (TB.a[i][l] != 0.0) {
          T t = T(TB.a[i][l]) * F[(size_t)l * n + j];
          acc = first ? t : acc + t;
          first = false;
        }
      Y[j] = y0[j] + T(h) * acc;
    }
    S.f(tau + TB.c[i] * h, Y, F + (size_t)i * n);
  }
  for (int j = 0; j < n; ++j) {
    T acc = T(0), e = T(0);
    bool fb = true, fe = true;
    for (int l = 0; l < TB.s; ++l) {
      if (TB.b[l] != 0.0) { T t = T(TB.b[l]) * F[(size_t)l * n + j]; acc = fb ? t : acc + t; fb = false; }
      if (err && TB.e[l] != 0.0) { T t = T(TB.e[l]) * F[(size_t)l * n + j]; e = fe ? t : e + t; fe = false; }
    }
    y1[j] = y0[j] + T(h) * acc;
    if (err) err[j] = T(h) * e;
  }
}

static double rms(const std::vector<double>& v) {
  double s = 0;
  for (double x : v) s += x * x;
  return v.empty() ? 0.0 : std::sqrt(s / (double)v.size());
}

}  // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------
// Solver configuration (same layout as the product's gal_solver_config).
// ---------------------------------------------------------------------------
extern "C" {

struct OrcSolverCfg {
  int32_t method;        // 5 = Dopri5, 8 = Dopri8
  int32_t adaptive;      // 0 = constant step dt0, 1 = PID controller
  int64_t max_steps;     // bound on step attempts (accepted + rejected)
  double dt0;            // constant step, or initial step for PID (<= 0: select)
  double rtol, atol;
  double dtmin, dtmax;   // <= 0 : none
  double pcoeff, icoeff, dcoeff;
  double safety, factormin, factormax;
  int32_t force_dtmin;
  int32_t lockstep;      // oracle only: 1 = all orbits share one controller
};

enum { ORC_OK = 0, ORC_MAX_STEPS = 1, ORC_DT_MIN = 2, ORC_NONFINITE = 3 };

}  // extern "C"

namespace orc {

struct SolveOut {
  int status = ORC_OK;
  long long accepted = 0, rejected = 0;
};

// Integrate an m-orbit lockstep group. y0: 6m, saves: ns times, out: ns x 6m.
static SolveOut solve_group(const Pot& P, const OrcSolverCfg& cfg, const double* y0, double t0, double t1,
                            const double* ts, int64_t ns, double* out, int m) {
  SolveOut R;
  const Tableau& TB = (cfg.method == 5) ? DOPRI5 : DOPRI8;
  const int n = 6 * m;
  const double dir = (t0 < t1) ? 1.0 : -1.0;  // diffrax: direction = where(t0 < t1, 1, -1)
  const double tau0 = dir * t0, tau1 = dir * t1;
  System<double> S{&P, m, dir};
  std::vector<double> y(y0, y0 + n), f0(n), y1(n), err(n), F((size_t)TB.s * n), Fs((size_t)TB.s * n), Y(n),
      ysave(n), q(n);
  int64_t si = 0;
  auto tau_s = [&](int64_t i) { return dir * ts[i]; };
  if (t0 == t1) {
    for (; si < ns; ++si) std::memcpy(out + si * n, y.data(), sizeof(double) * n);
    return R;
  }
  if (!std::isfinite(t0) || !std::isfinite(t1)) {  // an infinite span never ends: report it at once
    for (; si < ns; ++si)
      for (int j = 0; j < n; ++j) out[si * n + j] = std::numeric_limits<double>::quiet_NaN();
    R.status = ORC_NONFINITE;
    return R;
  }
  S.f(tau0, y.data(), f0.data());
  double tprev = tau0, tnext;
  // controller state
  bool at_dtmin = false;
  double prev_inv = 1.0, prev_prev_inv = 1.0;
  const double order = (double)TB.order;
  if (cfg.adaptive) {
    double dt0 = cfg.dt0;
    if (!(dt0 > 0)) {
      // Hairer-Norsett-Wanner II.4 initial step, as diffrax's _select_initial_step.
      std::vector<double> sc(n);
      for (int j = 0; j < n; ++j) sc[j] = cfg.atol + std::fabs(y[j]) * cfg.rtol;
      for (int j = 0; j < n; ++j) q[j] = y[j] / sc[j];
      double d0 = rms(q);
      for (int j = 0; j < n; ++j) q[j] = f0[j] / sc[j];
      double d1 = rms(q);
      bool cond = (d0 < 1e-5) || (d1 < 1e-5);
      double d1_ = cond ? 1.0 : d1;
      double h0 = cond ? 1e-6 : 0.01 * (d0 / d1_);
      std::vector<double> yy(n), f1(n);
      for (int j = 0; j < n; ++j) yy[j] = y[j] + h0 * f0[j];
      S.f(tau0 + h0, yy.data(), f1.data());
      for (int j = 0; j < n; ++j) q[j] = (f1[j] - f0[j]) / sc[j];
      double d2 = rms(q) / h0;
      double maxd = std::max(d1, d2);
      // exponent 1/(p+1) with p the method order (Hairer-Norsett-Wanner II.4 eq. 4.14)
      double h1 = (maxd <= 1e-15) ? std::max(1e-6, h0 * 1e-3) : std::pow(0.01 / maxd, 1.0 / (order + 1.0));
      dt0 = std::min(100 * h0, h1);
    }
    if (cfg.dtmax > 0) dt0 = std::min(dt0, cfg.dtmax);
    if (cfg.dtmin > 0) { at_dtmin = dt0 <= cfg.dtmin; dt0 = std::max(dt0, cfg.dtmin); }
    tnext = tau0 + dt0;
  } else {
    tnext = tau0 + cfg.dt0;
  }
  tnext = std::min(tnext, tau1);

  const double tol = 1e-10;
  long long nsteps = 0;
  while (tprev < tau1 && nsteps < cfg.max_steps) {
    const double h = tnext - tprev;
    rk_step<double>(S, TB, tprev, y.data(), f0.data(), h, F.data(), Y.data(), y1.data(),
                    cfg.adaptive ? err.data() : nullptr);
    ++nsteps;
    bool finite = true;
    for (int j = 0; j < n; ++j) finite = finite && std::isfinite(y1[j]);
    bool keep;
    double next_t0, next_t1;
    if (cfg.adaptive) {
      for (int j = 0; j < n; ++j) {
        double y1c = std::isnan(y1[j]) ? y[j] : y1[j];
        double yy = std::max(std::fabs(y[j]), std::fabs(y1c));
        q[j] = err[j] / (cfg.atol + yy * cfg.rtol);
      }
      double scaled = rms(q);
      keep = scaled < 1.0;
      if (cfg.dtmin > 0) keep = keep || at_dtmin;
      double inv = 1.0 / scaled;
      double c1 = (cfg.icoeff + cfg.pcoeff + cfg.dcoeff) / order;
      double c2 = -(cfg.pcoeff + 2 * cfg.dcoeff) / order;
      double c3 = cfg.dcoeff / order;
      double f1 = (c1 == 0) ? 1.0 : std::pow(inv, c1);
      double f2 = (c2 == 0) ? 1.0 : std::pow(prev_inv, c2);
      double f3 = (c3 == 0) ? 1.0 : std::pow(prev_prev_inv, c3);
      double fmin = keep ? 1.0 : cfg.factormin;
      double factor = std::min(std::max(cfg.safety * f1 * f2 * f3, fmin), cfg.factormax);
      double dt = h * factor;  // prev_dt = t1 - t0 (no jumps)
      if (inv == 0.0 || std::isinf(inv)) inv = 1.0;
      if (cfg.dtmax > 0) dt = std::min(dt, cfg.dtmax);
      if (cfg.dtmin > 0) {
        if (!cfg.force_dtmin && dt < cfg.dtmin) { R.status = ORC_DT_MIN; }
        at_dtmin = dt <= cfg.dtmin;
        dt = std::max(dt, cfg.dtmin);
      }
      next_t0 = keep ? tnext : tprev;
      next_t1 = next_t0 + dt;
      if (keep) { prev_prev_inv = prev_inv; prev_inv = inv; }
    } else {
      keep = true;
      next_t0 = tnext;
      next_t1 = tnext + cfg.dt0;
    }
    if (!finite) { R.status = ORC_NONFINITE; break; }
    if (keep) {
      ++R.accepted;
      // saves inside (tprev, tnext]
      while (si < ns && tau_s(si) <= next_t0) {
        double ts_ = tau_s(si);
        if (cfg.method == 5) {
          double th = (ts_ - tprev) / h;
          for (int j = 0; j < n; ++j) {
            double ymid = y[j];
            for (int l = 0; l < 7; ++l) ymid += DOPRI5_CMID[l] * (h * F[(size_t)l * n + j]);
            double F0 = h * F[j], F1 = h * F[(size_t)6 * n + j], Y0 = y[j], Y1 = y1[j];
            double A = 2 * (F1 - F0) - 8 * (Y1 + Y0) + 16 * ymid;
            double B = 5 * F0 - 3 * F1 + 18 * Y0 + 14 * Y1 - 32 * ymid;
            double C = F1 - 4 * F0 - 11 * Y0 - 5 * Y1 + 16 * ymid;
            ysave[j] = (((A * th + B) * th + C) * th + F0) * th + Y0;
          }
        } else {
          rk_step<double>(S, TB, tprev, y.data(), f0.data(), ts_ - tprev, Fs.data(), Y.data(), ysave.data(),
                          nullptr);
        }
        std::memcpy(out + si * n, ysave.data(), sizeof(double) * n);
        ++si;
      }
      y = y1;
      if (TB.fsal) {
        for (int j = 0; j < n; ++j) f0[j] = F[(size_t)(TB.s - 1) * n + j];
      } else {
        S.f(tnext, y.data(), f0.data());
      }
    } else {
      ++R.rejected;
    }
    tprev = std::min(next_t0, tau1);
    // diffrax _clip_to_end
    if (next_t1 > tau1 - tol) next_t1 = keep ? tau1 : tprev + 0.5 * (tau1 - tprev);
    tnext = next_t1;
    if (R.status == ORC_DT_MIN) break;  // an unsuccessful result ends diffrax's loop after this step
  }
  if (R.status == ORC_OK && tprev < tau1) R.status = ORC_MAX_STEPS;
  // Unreached saves stay NaN.
  for (; si < ns; ++si)
    for (int j = 0; j < n; ++j) out[si * n + j] = std::numeric_limits<double>::quiet_NaN();
  return R;
}

}  // namespace orc

extern "C" {

int orc_abi_version() { return 1; }

// P(a, x), dP/da and Gamma(a, x) (see gamma_p), for tests.
void orc_gamma_p(double a, double x, double* out) {
  const GammaP g = gamma_p(a, x);
  out[0] = g.P;
  out[1] = g.dPda;
  out[2] = g.upper;
}

// Phi, grad Phi, Hessian at n points (x: n x 3 row-major).
// slopes: n_comp x 3 or NULL (static); t: evaluation time.
void orc_potential(const Comp* comps, int ncomp, double G, const double* x, int64_t n, double* out,
                   const double* slopes, double t) {
  Pot P{comps, ncomp, G, slopes};
  for (int64_t i = 0; i < n; ++i) {
    double s = 0;
    for (int c = 0; c < ncomp; ++c) s += comp_potential<double>(comp_at(P, c, t), G, x + 3 * i);
    out[i] = s;
  }
}

void orc_gradient(const Comp* comps, int ncomp, double G, const double* x, int64_t n, double* out,
                  const double* slopes, double t) {
  Pot P{comps, ncomp, G, slopes};
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) gradient<double>(P, x + 3 * i, out + 3 * i, t);
}

void orc_hessian(const Comp* comps, int ncomp, double G, const double* x, int64_t n, double* out,
                 const double* slopes, double t) {
  Pot P{comps, ncomp, G, slopes};
  for (int64_t i = 0; i < n; ++i) {
    double* H = out + 9 * i;
    for (int j = 0; j < 9; ++j) H[j] = 0;
    for (int c = 0; c < ncomp; ++c) comp_hessian(comp_at(P, c, t), G, x + 3 * i, H);
  }
}

// d(grad Phi . v)/d(params): out is n x ncomp x 3.
void orc_dgrad_dparams(const Comp* comps, int ncomp, double G, const double* x, const double* v, int64_t n,
                       double* out) {
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < ncomp; ++c) {
      double* o = out + (i * ncomp + c) * 3;
      o[0] = o[1] = o[2] = 0;
      comp_dgrad_dparams_dot(comps[c], G, x + 3 * i, v + 3 * i, o);
    }
}

// Copy out a tableau (c[13], a[13*13], b[13], e[13]); returns number of stages.
int orc_tableau(int method, double* c, double* a, double* b, double* e) {
  const Tableau& T = (method == 5) ? DOPRI5 : DOPRI8;
  for (int i = 0; i < 13; ++i) {
    c[i] = T.c[i];
    b[i] = T.b[i];
    e[i] = T.e[i];
    for (int j = 0; j < 13; ++j) a[13 * i + j] = T.a[i][j];
  }
  return T.s;
}

void orc_dopri5_cmid(double* out) {
  for (int i = 0; i < 7; ++i) out[i] = DOPRI5_CMID[i];
}

// Integrate n orbits. y0: n x 6; t0,t1: n; save_offsets: n+1 (CSR into save_ts);
// out: total_saves x 6 (row-major, orbit-major order). status/accepted/rejected: n.
// lockstep=1: all n orbits form one system with a shared step (requires equal
// t0, t1 and save grids: orbit 0's are used); out then holds ns x n x 6.
int orc_integrate(const Comp* comps, int ncomp, double G, const OrcSolverCfg* cfg, const double* y0,
                  const double* t0, const double* t1, const int64_t* save_offsets, const double* save_ts,
                  double* out, int32_t* status, int64_t* accepted, int64_t* rejected, int64_t n, int nthreads,
                  const double* slopes) {
  Pot P{comps, ncomp, G, slopes};
  if (cfg->lockstep) {
    int64_t ns = save_offsets[1] - save_offsets[0];
    SolveOut R = solve_group(P, *cfg, y0, t0[0], t1[0], save_ts + save_offsets[0], ns, out, (int)n);
    for (int64_t i = 0; i < n; ++i) {
      status[i] = R.status;
      accepted[i] = R.accepted;
      rejected[i] = R.rejected;
    }
    return 0;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < n; ++i) {
    int64_t off = save_offsets[i], ns = save_offsets[i + 1] - save_offsets[i];
    SolveOut R = solve_group(P, *cfg, y0 + 6 * i, t0[i], t1[i], save_ts + off, ns, out + 6 * off, 1);
    status[i] = R.status;
    accepted[i] = R.accepted;
    rejected[i] = R.rejected;
  }
  return 0;
}

// Discrete adjoint of the constant-step RK map (diffrax ConstantStepSize time
// grid: t_{n+1} = t_n + dt, last step clipped onto t1) for the terminal loss
// L = sum_i |y_i(t1) - target_i|^2. Outputs the final states yT (n x 6), dL/dy0
// (n x 6) and, per component summed over orbits, dL/d(m, l1, l2) (ncomp x 3).
// With slopes (LinearParameter: p(t) = p + slope t, galax
// potential/_src/params/core.py:25-110) every stage evaluates the parameters
// at its own time, gparams holds the derivatives with respect to the values at
// t = 0, and gslopes (ncomp x 3) those with respect to the slopes: the
// stage-time derivative dL/dp(t_s), times 1 and times t_s.
int orc_adjoint_fixed(const Comp* comps, int ncomp, double G, const OrcSolverCfg* cfg, const double* y0,
                      double t0, double t1, const double* target, double* yT, double* gy,
                      double* gparams, int64_t n, int nthreads, const double* slopes, double* gslopes) {
  Pot P{comps, ncomp, G, slopes};
  const Tableau& TB = (cfg->method == 5) ? DOPRI5 : DOPRI8;
  const double dt = cfg->dt0;
  const int np = slopes ? 6 : 3;  // per component: values, then slopes
  std::vector<double> gp_all((size_t)n * ncomp * np, 0.0);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t o = 0; o < n; ++o) {
    System<double> S{&P, 1, 1.0};
    std::vector<double> ys, hs, taus;
    double y[6], y1[6], f0[6], F[13 * 6], Y[6];
    for (int j = 0; j < 6; ++j) y[j] = y0[6 * o + j];
    double tprev = t0, tnext = std::min(t0 + dt, t1);
    const double tol = 1e-10;
    while (tprev < t1) {
      double h = tnext - tprev;
      ys.insert(ys.end(), y, y + 6);
      hs.push_back(h);
      taus.push_back(tprev);
      S.f(tprev, y, f0);
      rk_step<double>(S, TB, tprev, y, f0, h, F, Y, y1, nullptr);
      for (int j = 0; j < 6; ++j) y[j] = y1[j];
      double nt0 = tnext, nt1 = tnext + dt;
      tprev = std::min(nt0, t1);
      if (nt1 > t1 - tol) nt1 = t1;
      tnext = nt1;
    }
    double lam[6];
    for (int j = 0; j < 6; ++j) {
      yT[6 * o + j] = y[j];
      lam[j] = 2.0 * (y[j] - target[6 * o + j]);
    }
    double* gpo = gp_all.data() + (size_t)o * ncomp * np;
    const int64_t N = (int64_t)hs.size();
    double Fb[13 * 6], Ys[13 * 6];
    for (int64_t st = N - 1; st >= 0; --st) {
      const double* yn = ys.data() + 6 * st;
      const double h = hs[st], tau = taus[st];
      // recompute the stages
      S.f(tau, yn, f0);
      for (int j = 0; j < 6; ++j) { F[j] = f0[j]; Ys[j] = yn[j]; }
      for (int i = 1; i < TB.s; ++i) {
        for (int j = 0; j < 6; ++j) {
          double acc = 0;
          bool first = true;
          for (int l = 0; l < i; ++l)
            if (TB.a[i][l] != 0.0) {
              double t = TB.a[i][l] * F[6 * l + j];
              acc = first ? t : acc + t;
              first = false;
            }
          Ys[6 * i + j] = yn[j] + h * acc;
        }
        S.f(tau + TB.c[i] * h, Ys + 6 * i, F + 6 * i);
      }
      double lam0[6];
      for (int j = 0; j < 6; ++j) lam0[j] = lam[j];
      for (int i = 0; i < TB.s; ++i)
        for (int j = 0; j < 6; ++j) Fb[6 * i + j] = h * TB.b[i] * lam[j];
      for (int i = TB.s - 1; i >= 0; --i) {
        const double* Yi = Ys + 6 * i;
        const double* fb = Fb + 6 * i;
        const double ti = tau + TB.c[i] * h;  // the stage's time (forward direction)
        // J^T fb with f = (p, -grad Phi(q)): (-H fb_p, fb_q)
        double H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int c = 0; c < ncomp; ++c) comp_hessian(comp_at(P, c, ti), G, Yi, H);
        double Yb[6];
        for (int r = 0; r < 3; ++r) Yb[r] = -(H[3 * r] * fb[3] + H[3 * r + 1] * fb[4] + H[3 * r + 2] * fb[5]);
        Yb[3] = fb[0]; Yb[4] = fb[1]; Yb[5] = fb[2];
        for (int c = 0; c < ncomp; ++c) {
          double d[3] = {0, 0, 0};
          comp_dgrad_dparams_dot(comp_at(P, c, ti), G, Yi, fb + 3, d);
          for (int k = 0; k < 3; ++k) gpo[np * c + k] -= d[k];
          if (slopes)
            for (int k = 0; k < 3; ++k) gpo[np * c + 3 + k] -= ti * d[k];
        }
        for (int j = 0; j < 6; ++j) lam0[j] += Yb[j];
        for (int l = 0; l < i; ++l)
          if (TB.a[i][l] != 0.0)
            for (int j = 0; j < 6; ++j) Fb[6 * l + j] += h * TB.a[i][l] * Yb[j];
      }
      for (int j = 0; j < 6; ++j) lam[j] = lam0[j];
    }
    for (int j = 0; j < 6; ++j) gy[6 * o + j] = lam[j];
  }
  for (int c = 0; c < ncomp * 3; ++c) gparams[c] = 0;
  if (slopes && gslopes)
    for (int c = 0; c < ncomp * 3; ++c) gslopes[c] = 0;
  for (int64_t o = 0; o < n; ++o) {
    const double* g = gp_all.data() + (size_t)o * ncomp * np;
    for (int c = 0; c < ncomp; ++c)
      for (int k = 0; k < 3; ++k) {
        gparams[3 * c + k] += g[np * c + k];
        if (slopes && gslopes) gslopes[3 * c + k] += g[np * c + 3 + k];
      }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Stream with a moving progenitor (test infrastructure for the stream row).
//
// Follows the reference's mock-stream pipeline
// (src/galax/dynamics/_src/experimental/stream.py:121-230 init: integrate the
// progenitor to the first release time, then along the release times;
// stream.py:380-446 run: every particle from its release time to the present;
// legacy/mockstream/mockstream_generator.py:160-275 with a progenitor potential
// moved along the progenitor's orbit, legacy/mockstream/_moving.py:20-42),
// with the release model of the King (1962) tidal radius
// (src/galax/dynamics/_src/cluster/radius.py:198-214:
// r_t = cbrt(G M / (Omega^2 - d2Phi/dr2)), Omega = |x x v| / r^2 from
// dynamics/_src/register_api.py:82-88, d2Phi/dr2 = rhat . H . rhat from
// potential/_src/register_funcs.py:444-457).
//
// Grid: constant steps dt. The progenitor is integrated backwards from
// (w_now, t_now) to t_now - n_rel dt, then forwards to t_now, recording its
// state at every grid time and its position at every stage of every forward
// step. Release r happens at grid time r; its two particles are integrated
// from there to t_now in the host potential plus a Plummer sphere (mass
// prog_m, radius prog_b) centred on the progenitor's stage positions, i.e.
// exactly the particle half of the coupled particle + progenitor system.
// Particle ICs (p = 2 r + side, side 0 = leading, 1 = trailing; s = -1 / +1)
// by one of three release models (see release_pair; df 2 is Chen 2024):
//   df 0 (offsets): x = x_prog + s r_t rhat + 0.1 r_t xi_p,
//                   v = v_prog + 0.1 Omega r_t eta_p, xi, eta given normal draws;
//   df 1 (Fardal 2015, legacy/mockstream/df/fardal15.py:62-94 and
//         experimental/df.py:148-177): four draws per release shared by both arms.
// ---------------------------------------------------------------------------
namespace orc {

static void stage_positions_step(const Pot& P, const Tableau& TB, const double* y, double h, double sign,
                                 double* ynew, double* Q /* s x 3 */) {
  double F[13 * 6], Y[6];
  field<double>(P, sign, y, F);
  for (int j = 0; j < 3; ++j) Q[j] = y[j];
  for (int i = 1; i < TB.s; ++i) {
    for (int j = 0; j < 6; ++j) {
      double acc = 0;
      bool first = true;
      for (int l = 0; l < i; ++l)
        if (TB.a[i][l] != 0.0) {
          double t = TB.a[i][l] * F[6 * l + j];
          acc = first ? t : acc + t;
          first = false;
        }
      Y[j] = y[j] + h * acc;
    }
    for (int j = 0; j < 3; ++j) Q[3 * i + j] = Y[j];
    field<double>(P, sign, Y, F + 6 * i);
  }
  for (int j = 0; j < 6; ++j) {
    double acc = 0;
    bool first = true;
    for (int l = 0; l < TB.s; ++l)
      if (TB.b[l] != 0.0) {
        double t = TB.b[l] * F[6 * l + j];
        acc = first ? t : acc + t;
        first = false;
      }
    ynew[j] = y[j] + h * acc;
  }
}

// field of a particle: host potential + Plummer(prog_m, prog_b) at Qi
static void particle_field(const Pot& P, double Gmp, double b2, const double* Qi, const double* y, double* dy) {
  double g[3];
  gradient<double>(P, y, g);
  double d[3] = {y[0] - Qi[0], y[1] - Qi[1], y[2] - Qi[2]};
  double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + TINY;
  double s2 = r2 + b2;
  double f = Gmp / (s2 * std::sqrt(s2));
  for (int j = 0; j < 3; ++j) g[j] += f * d[j];
  dy[0] = y[3]; dy[1] = y[4]; dy[2] = y[5];
  dy[3] = -g[0]; dy[4] = -g[1]; dy[5] = -g[2];
}

static void particle_step(const Pot& P, const Tableau& TB, double Gmp, double b2, const double* Qk, double* y,
                          double h) {
  double F[13 * 6], Y[6];
  particle_field(P, Gmp, b2, Qk, y, F);
  for (int i = 1; i < TB.s; ++i) {
    for (int j = 0; j < 6; ++j) {
      double acc = 0;
      bool first = true;
      for (int l = 0; l < i; ++l)
        if (TB.a[i][l] != 0.0) {
          double t = TB.a[i][l] * F[6 * l + j];
          acc = first ? t : acc + t;
          first = false;
        }
      Y[j] = y[j] + h * acc;
    }
    particle_field(P, Gmp, b2, Qk + 3 * i, Y, F + 6 * i);
  }
  double y1[6];
  for (int j = 0; j < 6; ++j) {
    double acc = 0;
    bool first = true;
    for (int l = 0; l < TB.s; ++l)
      if (TB.b[l] != 0.0) {
        double t = TB.b[l] * F[6 * l + j];
        acc = first ? t : acc + t;
        first = false;
      }
    y1[j] = y[j] + h * acc;
  }
  for (int j = 0; j < 6; ++j) y[j] = y1[j];
}

static double norm3(const double* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// King (1962) tidal radius and angular frequency at (x, v) for mass GM.
static void king_rt_om(const Pot& P, double GM, const double* x, const double* v, double& rt, double& om) {
  const double rr = norm3(x);
  const double rh[3] = {x[0] / rr, x[1] / rr, x[2] / rr};
  const double L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
  om = norm3(L) / (rr * rr);
  double H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int c = 0; c < P.n; ++c) comp_hessian(P.comps[c], P.G, x, H);
  double prr = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) prr += rh[i] * H[3 * i + j] * rh[j];
  rt = std::cbrt(GM / (om * om - prr));
}

// Release conditions of one release (out: lead[6], trail[6]). nz: the release's
// draws, 12 (offsets: xi_lead, eta_lead, xi_trail, eta_trail) or 4 (Fardal: kr,
// kvphi, kz, kvz). dfp: kr_bar, kvphi_bar, kz_bar, kvz_bar, sigma_kr,
// sigma_kvphi, sigma_kz, sigma_kvz.
static void release_pair(int df, const double* dfp, const double* nz, const double* x, const double* v, double rt,
                         double om, double GM, double* lead, double* trail) {
  const double rr = norm3(x);
  const double rh[3] = {x[0] / rr, x[1] / rr, x[2] / rr};
  double* out[2] = {lead, trail};
  if (df == 2) {
    // Chen et al. 2024 as galax samples it (legacy/mockstream/df/chen24.py):
    // posvel ~ N(mean, cov); here posvel = mean + A z with A the lower
    // triangular factor of cov and z = nz[0..5] standard normals.
    const double pv0 = 1.6 + 0.35 * nz[0];
    const double pv1 = -30.0 + 23.0 * nz[1];
    const double pv2 = 12.0 * nz[2];
    const double pv3 = 1.0;
    const double pv4 = 20.0 + 20.0 * (-0.7 * nz[0] + std::sqrt(1.0 - 0.49) * nz[4]);
    const double pv5 = 22.0 * nz[5];
    const double deg = 0.017453292519943295;
    const double Dr = pv0 * rt;
    const double Dv = pv3 * std::sqrt(2.0 * GM / Dr);
    const double cth = std::cos(pv2 * deg), sth = std::sin(pv2 * deg);
    const double cph = std::cos(pv1 * deg), sph = std::sin(pv1 * deg);
    const double cal = std::cos(pv4 * deg), sal = std::sin(pv4 * deg);
    const double cbe = std::cos(pv5 * deg), sbe = std::sin(pv5 * deg);
    const double L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
    const double Lm = norm3(L);
    const double vr = v[0] * rh[0] + v[1] * rh[1] + v[2] * rh[2];
    double yh[3] = {v[0] - vr * rh[0], v[1] - vr * rh[1], v[2] - vr * rh[2]};
    const double ym = norm3(yh);
    for (int j = 0; j < 3; ++j) {
      const double zh = L[j] / Lm;
      yh[j] /= ym;
      trail[j] = x[j] + Dr * cth * cph * rh[j] + Dr * cth * sph * yh[j] + Dr * sth * zh;
      trail[3 + j] = v[j] + Dv * cbe * cal * rh[j] + Dv * cbe * sal * yh[j] + Dv * sbe * zh;
      lead[j] = x[j] - Dr * cth * cph * rh[j] - Dr * cth * sph * yh[j] + Dr * sth * zh;
      lead[3 + j] = v[j] - Dv * cbe * cal * rh[j] - Dv * cbe * sal * yh[j] + Dv * sbe * zh;
    }
    return;
  }
  if (df == 1) {
    // Fardal et al. 2015 as galax samples it: k values from the four draws,
    // then the leading arm inside (-kr) and the trailing arm outside (+kr).
    const double kr = dfp[0] + nz[0] * dfp[4];
    const double kvphi = kr * (dfp[1] + nz[1] * dfp[5]);
    const double kz = dfp[2] + nz[2] * dfp[6];
    const double kvz = dfp[3] + nz[3] * dfp[7];
    const double L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
    const double Lm = norm3(L);
    const double zh[3] = {L[0] / Lm, L[1] / Lm, L[2] / Lm};
    const double vr = v[0] * rh[0] + v[1] * rh[1] + v[2] * rh[2];
    double ph[3] = {v[0] - vr * rh[0], v[1] - vr * rh[1], v[2] - vr * rh[2]};
    const double pm = norm3(ph);
    for (int j = 0; j < 3; ++j) ph[j] /= pm;
    const double vc = om * rt;
    for (int j = 0; j < 3; ++j) {
      lead[j] = x[j] - rt * (kr * rh[j] - kz * zh[j]);
      lead[3 + j] = v[j] - vc * (kvphi * ph[j] - kvz * zh[j]);
      trail[j] = x[j] + rt * (kr * rh[j] + kz * zh[j]);
      trail[3 + j] = v[j] + vc * (kvphi * ph[j] + kvz * zh[j]);
    }
    return;
  }
  for (int side = 0; side < 2; ++side) {
    const double s = side == 0 ? -1.0 : 1.0;
    const double* xi = nz + 6 * side;
    const double* eta = xi + 3;
    for (int j = 0; j < 3; ++j) {
      out[side][j] = x[j] + s * rt * rh[j] + 0.1 * rt * xi[j];
      out[side][3 + j] = v[j] + 0.1 * om * rt * eta[j];
    }
  }
}

}  // namespace orc

// Release conditions at n independent progenitor points w (n x 6) with masses
// mass (n): lead, trail (n x 6), r_tidal (n). noise: n x 12, n x 4 or n x 6 (df 0, 1, 2).
int orc_stream_df_sample(const Comp* comps, int ncomp, double G, int df, const double* dfp, const double* w,
                         const double* mass, const double* noise, int64_t n, double* lead, double* trail,
                         double* r_tidal) {
  Pot P{comps, ncomp, G};
  const int nq = df == 1 ? 4 : (df == 2 ? 6 : 12);
  for (int64_t r = 0; r < n; ++r) {
    double rt, om;
    orc::king_rt_om(P, G * mass[r], w + 6 * r, w + 6 * r + 3, rt, om);
    r_tidal[r] = rt;
    orc::release_pair(df, dfp, noise + nq * r, w + 6 * r, w + 6 * r + 3, rt, om, G * mass[r], lead + 6 * r,
                      trail + 6 * r);
  }
  return 0;
}

// prog_track: (n_rel + 1) x 6 forward states; ics, final_: 2 n_rel x 6;
// noise: n_rel x 12 (offsets), n_rel x 4 (Fardal) or n_rel x 6 (Chen); rt_om: n_rel x 2 (r_t, Omega).
int orc_stream_forward(const Comp* comps, int ncomp, double G, int method, double prog_m, double prog_b,
                       const double* w_now, double t_now, double dt, int64_t n_rel, int df, const double* dfp,
                       const double* noise, double* prog_track, double* rt_om, double* ics, double* final_,
                       int nthreads) {
  Pot P{comps, ncomp, G};
  const Tableau& TB = (method == 5) ? DOPRI5 : DOPRI8;
  const int S = TB.s;
  // backwards from t_now (reversed time, tau = -t, constant steps dt)
  double y[6], ynew[6];
  std::vector<double> Qb((size_t)S * 3);
  for (int j = 0; j < 6; ++j) y[j] = w_now[j];
  for (int64_t k = 0; k < n_rel; ++k) {
    stage_positions_step(P, TB, y, dt, -1.0, ynew, Qb.data());
    for (int j = 0; j < 6; ++j) y[j] = ynew[j];
  }
  // forwards, recording states and stage positions
  std::vector<double> Q((size_t)n_rel * S * 3);
  for (int j = 0; j < 6; ++j) prog_track[j] = y[j];
  for (int64_t k = 0; k < n_rel; ++k) {
    stage_positions_step(P, TB, y, dt, 1.0, ynew, Q.data() + (size_t)k * S * 3);
    for (int j = 0; j < 6; ++j) {
      y[j] = ynew[j];
      prog_track[6 * (k + 1) + j] = y[j];
    }
  }
  const double GM = G * prog_m, b2 = prog_b * prog_b;
  // release: King tidal radius and the particle ICs
  const int nq = df == 1 ? 4 : (df == 2 ? 6 : 12);
  for (int64_t r = 0; r < n_rel; ++r) {
    const double* w = prog_track + 6 * r;
    double rt, om;
    orc::king_rt_om(P, GM, w, w + 3, rt, om);
    rt_om[2 * r] = rt;
    rt_om[2 * r + 1] = om;
    orc::release_pair(df, dfp, noise + nq * r, w, w + 3, rt, om, GM, ics + 6 * (2 * r), ics + 6 * (2 * r + 1));
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t p = 0; p < 2 * n_rel; ++p) {
    const int64_t r = p / 2;
    double yp[6];
    for (int j = 0; j < 6; ++j) yp[j] = ics[6 * p + j];
    for (int64_t k = r; k < n_rel; ++k) particle_step(P, TB, GM, b2, Q.data() + (size_t)k * S * 3, yp, dt);
    for (int j = 0; j < 6; ++j) final_[6 * p + j] = yp[j];
  }
  return 0;
}

// Count algorithmic FP64 operations of one gradient evaluation and one RK step
// (without the controller). out: [add, mul, div, sqrt, log1p] for the
// gradient, then the same five for a full step of `method`.
void orc_count_ops(const Comp* comps, int ncomp, double G, int method, const double* y, int64_t* out) {
  Pot P{comps, ncomp, G};
  CD x[3] = {CD(y[0]), CD(y[1]), CD(y[2])}, g[3];
  g_ops = OpCount();
  gradient<CD>(P, x, g);
  out[0] = g_ops.add; out[1] = g_ops.mul; out[2] = g_ops.div; out[3] = g_ops.sqrt; out[4] = g_ops.log1p;
  System<CD> S{&P, 1, 1.0};
  CD yy[6], f0[6], y1[6], e[6];
  for (int j = 0; j < 6; ++j) yy[j] = CD(y[j]);
  const Tableau& TB = (method == 5) ? DOPRI5 : DOPRI8;
  g_ops = OpCount();
  if (!TB.fsal || true) S.f(0.0, yy, f0);  // the step's first evaluation
  std::vector<CD> Fb((size_t)TB.s * 6), Yb(6);
  rk_step<CD>(S, TB, 0.0, yy, f0, 1.0, Fb.data(), Yb.data(), y1, e);
  if (TB.fsal) {
    // FSAL: the last stage is the next step's first evaluation; do not count it twice.
    OpCount before = g_ops;
    g_ops = OpCount();
    S.f(0.0, yy, f0);
    OpCount one = g_ops;
    g_ops = before;
    g_ops.add -= one.add; g_ops.mul -= one.mul; g_ops.div -= one.div; g_ops.sqrt -= one.sqrt;
    g_ops.log1p -= one.log1p;
  }
  out[5] = g_ops.add; out[6] = g_ops.mul; out[7] = g_ops.div; out[8] = g_ops.sqrt; out[9] = g_ops.log1p;
}

}  // extern "C"
