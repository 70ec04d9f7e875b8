// Device side of the short-range Plummer sum (see split.cu): cell lookup and
// the tapered potential and gradient, shared by the evaluation kernel and the
// surrogate integrator's stage kernels.
#pragma once

#include <cstdint>

#include "potentials.cuh"

namespace gal {

struct SplitDev {
  const int64_t* start;  // [nx^3 + 1] CSR offsets per cell
  const double* items;   // [items][5]: cx, cy, cz, G m, b^2
  int nx;
  double lo, inv_h;      // cell (ix, iy, iz) covers lo + [ix, ix+1) / inv_h, ...
  double rc2, inv_rc2;   // r_cut^2 and its inverse
};

// Accumulates grad of sum_i Phi_i S(d_i / r_c) into g (and the potential into *phi).
// S(q) = (1 - q^2)^3: grad(Phi S) = d G m is (S is^2 + 6 t^2 / r_c^2), t = 1 - q^2,
// is = 1 / sqrt(d^2 + b^2).
__device__ __forceinline__ void split_short(const SplitDev& s, double x, double y, double z, double& gx, double& gy,
                                            double& gz, double* phi) {
  const double fx = (x - s.lo) * s.inv_h, fy = (y - s.lo) * s.inv_h, fz = (z - s.lo) * s.inv_h;
  if (!(fx >= 0.0 && fy >= 0.0 && fz >= 0.0)) return;
  const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  if (ix >= s.nx || iy >= s.nx || iz >= s.nx) return;
  const int64_t cell = ((int64_t)iz * s.nx + iy) * s.nx + ix;
  const int64_t b0 = s.start[cell], b1 = s.start[cell + 1];
  for (int64_t k = b0; k < b1; ++k) {
    const double* it = s.items + 5 * k;
    const double dx = x - it[0], dy = y - it[1], dz = z - it[2];
    const double d2 = fma(dx, dx, fma(dy, dy, dz * dz));
    if (d2 >= s.rc2) continue;
    const double t = fma(-d2, s.inv_rc2, 1.0);
    const double S = t * t * t;
    const double is = rsqrt(d2 + TINY + it[4]);
    const double Gmis = it[3] * is;
    const double f = Gmis * fma(S, is * is, 6.0 * t * t * s.inv_rc2);
    gx = fma(f, dx, gx);
    gy = fma(f, dy, gy);
    gz = fma(f, dz, gz);
    if (phi) *phi -= Gmis * S;
  }
}

}  // namespace gal

struct gal_split;
// Device view of a split (host pointer to a host-side struct; NULL for NULL).
extern "C" const gal::SplitDev* gal_split_device(const gal_split* sp);

namespace gal {

// A potential plus the short-range Plummer sum.
template <class Base>
struct WithShort {
  Base base;
  SplitDev sp;
  __device__ __forceinline__ void grad(double x, double y, double z, double& gx, double& gy, double& gz) const {
    base.grad(x, y, z, gx, gy, gz);
    split_short(sp, x, y, z, gx, gy, gz, nullptr);
  }
};

}  // namespace gal
