// Device side of the short-range Plummer sum (see split.cu): cell lookup and
// the tapered potential and gradient, shared by the evaluation kernel and the
// surrogate integrator's stage kernels.
#pragma once

#include <cstdint>

#include "potentials.cuh"

namespace gal {

struct SplitDev {
  const int64_t* start;  // [nx^3 + 1] CSR offsets per cell
  const float4* items;   // [items]: centre relative to its cell's low corner (x, y, z), G m
  const float* b2;       // [items]: b^2
  int nx;
  double lo, h, inv_h;   // cell (ix, iy, iz) covers lo + h [ix, ix+1) x ...
  double rc2, inv_rc2;   // r_cut^2 and its inverse
};

// Accumulates grad of sum_i Phi_i S(d_i / r_c) into g (and the potential into *phi).
// S(q) = (1 - q^2)^3: grad(Phi S) = d G m is (S is^2 + 6 t^2 / r_c^2), t = 1 - q^2,
// is = 1 / sqrt(d^2 + b^2). The point is placed relative to its cell's low
// corner once in FP64; the centres are stored relative to the same corner in
// FP32, so every term is FP32 work only (the FP32 pipe is 64x the FP64 one
// on this chip) and carries ~1e-7 relative error, far below the MLP's share of
// the surrogate's error; the terms are accumulated in FP64.
__device__ __forceinline__ void split_short(const SplitDev& s, double x, double y, double z, double& gx, double& gy,
                                            double& gz, double* phi) {
  const double fx = (x - s.lo) * s.inv_h, fy = (y - s.lo) * s.inv_h, fz = (z - s.lo) * s.inv_h;
  if (!(fx >= 0.0 && fy >= 0.0 && fz >= 0.0)) return;
  const int ix = (int)fx, iy = (int)fy, iz = (int)fz;
  if (ix >= s.nx || iy >= s.nx || iz >= s.nx) return;
  const int64_t cell = ((int64_t)iz * s.nx + iy) * s.nx + ix;
  const int64_t b0 = s.start[cell], b1 = s.start[cell + 1];
  if (b0 == b1) return;
  const float xr = (float)fma(-(double)ix, s.h, x - s.lo);
  const float yr = (float)fma(-(double)iy, s.h, y - s.lo);
  const float zr = (float)fma(-(double)iz, s.h, z - s.lo);
  const float rc2 = (float)s.rc2, inv_rc2 = (float)s.inv_rc2;
  float ax = 0.f, ay = 0.f, az = 0.f, ap = 0.f;
  for (int64_t k = b0; k < b1; ++k) {
    const float4 it = s.items[k];
    const float dx = xr - it.x, dy = yr - it.y, dz = zr - it.z;
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    if (d2 >= rc2) continue;
    const float t = fmaf(-d2, inv_rc2, 1.0f);
    const float S = t * t * t;
    const float is = rsqrtf(d2 + s.b2[k]);
    const float Gmis = it.w * is;
    const float f = Gmis * fmaf(S, is * is, 6.0f * t * t * inv_rc2);
    ax = fmaf(f, dx, ax);
    ay = fmaf(f, dy, ay);
    az = fmaf(f, dz, az);
    ap = fmaf(-Gmis, S, ap);
  }
  gx += (double)ax;
  gy += (double)ay;
  gz += (double)az;
  if (phi) *phi += (double)ap;
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
