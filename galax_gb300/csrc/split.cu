// Short-range part of a set of Plummer spheres, for the learned surrogate.
//
// Each Plummer sphere Phi_i = -G m_i / sqrt(d^2 + b_i^2) (d = |x - c_i|,
// src/galax/potential/_src/builtin/plummer.py:122-133, translated as
// xfm/translate.py:28-87) is split into a short-range part Phi_i S(d / r_c)
// and a long-range remainder Phi_i (1 - S), with the C2 taper
// S(q) = (1 - q^2)^3 for q < 1 and 0 beyond. The remainder is smooth on the
// scale r_c, which is what the MLP learns; the short-range part, non-zero only
// within r_c of a centre, is summed directly here (FP64 offsets and
// accumulation, FP32 terms: see split.cuh). A uniform grid of
// cells of side r_c over the centres' bounding box (grown by r_c) lists, for
// every cell, the spheres whose centre lies within r_c of some point of the
// cell, with their parameters copied into the list (centre relative to the
// cell's low corner and G m as a float4, b^2 beside it) so a lookup touches one
// contiguous run. Points outside the grid have no
// short-range neighbours.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "handle.h"
#include "split.cuh"

using namespace gal;

struct gal_split {
  SplitDev dev;
  int64_t* d_start;
  float4* d_items;
  float* d_b2;
  int32_t n;
};

namespace gal {

__global__ void k_split_eval(SplitDev s, const double* __restrict__ x, int64_t n, double* __restrict__ phi,
                             double* __restrict__ grad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double gx = 0.0, gy = 0.0, gz = 0.0, p = 0.0;
    split_short(s, x[i], x[n + i], x[2 * n + i], gx, gy, gz, phi ? &p : nullptr);
    if (grad) {
      grad[i] = gx;
      grad[n + i] = gy;
      grad[2 * n + i] = gz;
    }
    if (phi) phi[i] = p;
  }
}

}  // namespace gal

extern "C" {

gal_status gal_split_create(const gal_component* comps, int32_t n, double G, double r_cut, gal_split** out) {
  return no_throw([&]() -> gal_status {
    if (!comps || !out || n < 1 || !(r_cut > 0.0) || !(G > 0.0))
      return fail(GAL_ERR_INVALID_ARGUMENT, "bad gal_split_create arguments");
    *out = nullptr;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < n; ++i) {
      if (comps[i].kind != GAL_PLUMMER) return fail(GAL_ERR_UNSUPPORTED, "the split takes Plummer components only");
      if (!(comps[i].l1 > 0.0) || !std::isfinite(comps[i].l1) || !std::isfinite(comps[i].m))
        return fail(GAL_ERR_INVALID_ARGUMENT, "Plummer m must be finite and b finite and > 0");
      for (int d = 0; d < 3; ++d) {
        if (!std::isfinite(comps[i].origin[d])) return fail(GAL_ERR_INVALID_ARGUMENT, "non-finite Plummer centre");
        lo[d] = std::min(lo[d], comps[i].origin[d]);
        hi[d] = std::max(hi[d], comps[i].origin[d]);
      }
    }
    const double h = r_cut;
    double glo = 1e300, ghi = -1e300;
    for (int d = 0; d < 3; ++d) {
      glo = std::min(glo, lo[d] - r_cut);
      ghi = std::max(ghi, hi[d] + r_cut);
    }
    const double cells = std::ceil((ghi - glo) / h);  // per axis; checked before the integer conversion
    if (!(cells <= 406.0)) return fail(GAL_ERR_TOO_LARGE, "split grid above 2^26 cells");
    const int nx = std::max(1, (int)cells);
    const int64_t ncell = (int64_t)nx * nx * nx;
    std::vector<std::vector<int>> lists((size_t)ncell);
    for (int i = 0; i < n; ++i) {
      const double* c = comps[i].origin;
      int a[3], b[3];
      for (int d = 0; d < 3; ++d) {
        a[d] = std::max(0, (int)std::floor((c[d] - r_cut - glo) / h));
        b[d] = std::min(nx - 1, (int)std::floor((c[d] + r_cut - glo) / h));
      }
      for (int iz = a[2]; iz <= b[2]; ++iz)
        for (int iy = a[1]; iy <= b[1]; ++iy)
          for (int ix = a[0]; ix <= b[0]; ++ix) {
            // distance from the centre to the cell box
            const int idx[3] = {ix, iy, iz};
            double d2 = 0.0;
            for (int d = 0; d < 3; ++d) {
              const double blo = glo + idx[d] * h, bhi = blo + h;
              const double e = c[d] < blo ? blo - c[d] : (c[d] > bhi ? c[d] - bhi : 0.0);
              d2 += e * e;
            }
            if (d2 <= r_cut * r_cut) lists[((size_t)iz * nx + iy) * nx + ix].push_back(i);
          }
    }
    std::vector<int64_t> start((size_t)ncell + 1, 0);
    for (int64_t cidx = 0; cidx < ncell; ++cidx) start[cidx + 1] = start[cidx] + (int64_t)lists[cidx].size();
    std::vector<float4> items((size_t)start[ncell]);
    std::vector<float> b2s((size_t)start[ncell]);
    for (int64_t cidx = 0; cidx < ncell; ++cidx) {
      const int64_t ix = cidx % nx, iy = (cidx / nx) % nx, iz = cidx / ((int64_t)nx * nx);
      const double corner[3] = {glo + ix * h, glo + iy * h, glo + iz * h};
      for (size_t k = 0; k < lists[cidx].size(); ++k) {
        const gal_component& cc = comps[lists[cidx][k]];
        const size_t o = (size_t)start[cidx] + k;
        items[o] = make_float4((float)(cc.origin[0] - corner[0]), (float)(cc.origin[1] - corner[1]),
                               (float)(cc.origin[2] - corner[2]), (float)(G * cc.m));
        b2s[o] = (float)(cc.l1 * cc.l1);
      }
    }
    gal_split* sp = new gal_split();
    sp->n = n;
    sp->d_start = nullptr;
    sp->d_items = nullptr;
    sp->d_b2 = nullptr;
    const size_t ni = std::max<size_t>(items.size(), 1);
    cudaError_t e = cudaMalloc(&sp->d_start, sizeof(int64_t) * start.size());
    if (e == cudaSuccess) e = cudaMalloc(&sp->d_items, sizeof(float4) * ni);
    if (e == cudaSuccess) e = cudaMalloc(&sp->d_b2, sizeof(float) * ni);
    if (e == cudaSuccess)
      e = cudaMemcpy(sp->d_start, start.data(), sizeof(int64_t) * start.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !items.empty())
      e = cudaMemcpy(sp->d_items, items.data(), sizeof(float4) * items.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !b2s.empty())
      e = cudaMemcpy(sp->d_b2, b2s.data(), sizeof(float) * b2s.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(sp->d_start);
      cudaFree(sp->d_items);
      cudaFree(sp->d_b2);
      delete sp;
      return cuda_fail(e, "gal_split_create");
    }
    sp->dev.start = sp->d_start;
    sp->dev.items = sp->d_items;
    sp->dev.b2 = sp->d_b2;
    sp->dev.nx = nx;
    sp->dev.lo = glo;
    sp->dev.h = h;
    sp->dev.inv_h = 1.0 / h;
    sp->dev.rc2 = r_cut * r_cut;
    sp->dev.inv_rc2 = 1.0 / (r_cut * r_cut);
    *out = sp;
    return GAL_OK;
  });
}

gal_status gal_split_destroy(gal_split* sp) {
  if (!sp) return GAL_OK;
  cudaFree(sp->d_start);
  cudaFree(sp->d_items);
  cudaFree(sp->d_b2);
  delete sp;
  return GAL_OK;
}

gal_status gal_split_eval(const gal_split* sp, const double* x, int64_t n, double* phi, double* grad,
                          gal_stream_t stream) {
  if (!sp || n < 0 || (n > 0 && !x)) return fail(GAL_ERR_INVALID_ARGUMENT, "bad gal_split_eval arguments");
  if (n == 0) return GAL_OK;
  int64_t grid = (n + 255) / 256;
  const int64_t cap = (int64_t)device_sm_count() * 16;
  if (grid > cap) grid = cap;
  k_split_eval<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(sp->dev, x, n, phi, grad);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "short-range evaluation");
}

const SplitDev* gal_split_device(const gal_split* sp) { return sp ? &sp->dev : nullptr; }

}  // extern "C"
