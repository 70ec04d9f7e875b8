// Kernel entry points and launcher for one Runge-Kutta method (included once per
// method by integrate_dopri5.cu / integrate_dopri8.cu so the two compile in parallel).
#pragma once

#include "launch.h"

namespace gal {

constexpr int kMaxBlock = 256;

// Register variants of the Milky Way kernel (threads per block <= MAXT):
//   0: 128 threads, 3 blocks per SM  -> at most 168 registers, 12 warps per SM
//   1: 128 threads, 4 blocks per SM  -> at most 128 registers, 16 warps per SM (spills)
//   2: 256 threads, 1 block per SM   -> up to 255 registers
// The autotuner picks per workload; results do not depend on it.
template <class TB, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) k_integrate_mw(IntegrateArgs a, MWParams p) {
  const MWPot pot{p};
  integrate_loop<TB>(a, pot);
}

template <class TB>
cudaError_t mw_occupancy(int variant, int block, int* per_sm) {
  switch (variant) {
    case 1: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_integrate_mw<TB, 128, 4>, block, 0);
    case 2: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_integrate_mw<TB, 256, 1>, block, 0);
    default: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_integrate_mw<TB, 128, 3>, block, 0);
  }
}

template <class TB>
void mw_launch(int variant, unsigned grid, int block, cudaStream_t stream, const IntegrateArgs& a, const MWParams& p) {
  switch (variant) {
    case 1: k_integrate_mw<TB, 128, 4><<<grid, block, 0, stream>>>(a, p); break;
    case 2: k_integrate_mw<TB, 256, 1><<<grid, block, 0, stream>>>(a, p); break;
    default: k_integrate_mw<TB, 128, 3><<<grid, block, 0, stream>>>(a, p); break;
  }
}

// The Milky Way kernel on `grid` blocks with `smem` bytes of dynamic shared
// memory that it does not use: a request above half an SM's capacity keeps
// every other block that makes such a request off its SM.
template <class TB>
cudaError_t mw_launch_exclusive(int variant, unsigned grid, int block, size_t smem, cudaStream_t stream,
                                const IntegrateArgs& a, const MWParams& p) {
  cudaError_t e;
  switch (variant) {
    case 1:
      e = cudaFuncSetAttribute(k_integrate_mw<TB, 128, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) k_integrate_mw<TB, 128, 4><<<grid, block, smem, stream>>>(a, p);
      break;
    case 2:
      e = cudaFuncSetAttribute(k_integrate_mw<TB, 256, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) k_integrate_mw<TB, 256, 1><<<grid, block, smem, stream>>>(a, p);
      break;
    default:
      e = cudaFuncSetAttribute(k_integrate_mw<TB, 128, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e == cudaSuccess) k_integrate_mw<TB, 128, 3><<<grid, block, smem, stream>>>(a, p);
      break;
  }
  return e == cudaSuccess ? cudaGetLastError() : e;
}

template <class TB, bool TIMED>
__global__ void __launch_bounds__(kMaxBlock) k_integrate_table(IntegrateArgs a, const DevComp* comps, int ncomp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevComp* s_comps = reinterpret_cast<DevComp*>(smem_raw);
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) s_comps[i] = comps[i];
  __syncthreads();
  if constexpr (TIMED) {
    integrate_loop<TB>(a, TimedTablePot{s_comps, ncomp, a.lin});
  } else {
    integrate_loop<TB>(a, TablePot{s_comps, ncomp});
  }
}

// One warp per orbit (composites with many components): the lanes split the
// components and every lane ends each gradient with the same sum.
template <class TB, bool TIMED>
__global__ void __launch_bounds__(kMaxBlock) k_integrate_table_warp(IntegrateArgs a, const DevComp* comps, int ncomp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevComp* s_comps = reinterpret_cast<DevComp*>(smem_raw);
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) s_comps[i] = comps[i];
  __syncthreads();
  integrate_loop<TB, WarpTablePot<TIMED>, 32>(a, WarpTablePot<TIMED>{s_comps, ncomp, a.lin});
}

// Whether a component table runs one warp per orbit: always or never when
// asked (table_lanes 32 / 1); automatically when the table has many components
// and the batch is too small to give every SM sub-partition a warp of 32
// orbits, so that one thread per orbit would leave FP64 pipes idle.
inline bool use_warp_per_orbit(const LaunchShape& shape, int64_t n, int ncomp) {
  if (shape.table_lanes == 32) return true;
  if (shape.table_lanes == 1 || ncomp < kWarpMinComponents) return false;
  return (n + 31) / 32 < 4LL * device_sm_count();
}

// Four orbits per block of 128 threads and as many blocks per SM as fit (the
// launch shapes tuned for one thread per orbit do not apply).
template <class TB>
cudaError_t launch_integrate_warp(const IntegrateArgs& a, const DevComp* comps, int ncomp, cudaStream_t stream) {
  const int block = 128;
  const size_t smem = sizeof(DevComp) * (size_t)ncomp;
  auto kernel = a.lin ? k_integrate_table_warp<TB, true> : k_integrate_table_warp<TB, false>;
  cudaError_t err;
  if (smem > 48 * 1024) {
    err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
  }
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) per_sm = 1;
  const int warps = block / 32;
  int64_t grid = (int64_t)per_sm * device_sm_count();
  const int64_t need = (a.n + warps - 1) / warps;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  kernel<<<(unsigned)grid, block, smem, stream>>>(a, comps, ncomp);
  return cudaGetLastError();
}

template <class TB>
cudaError_t launch_integrate(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps, int ncomp,
                             LaunchShape shape, cudaStream_t stream) {
  if (!mw && use_warp_per_orbit(shape, a.n, ncomp)) return launch_integrate_warp<TB>(a, comps, ncomp, stream);
  const int block = shape.block_threads > 0 ? shape.block_threads : 128;
  if (block > kMaxBlock || block % 32 != 0) return cudaErrorInvalidValue;
  const size_t smem = mw ? 0 : sizeof(DevComp) * (size_t)ncomp;
  int per_sm = shape.blocks_per_sm;
  cudaError_t err;
  if (mw && shape.variant != 2 && block > 128) return cudaErrorInvalidValue;
  if (per_sm <= 0) {
    if (mw)
      err = mw_occupancy<TB>(shape.variant, block, &per_sm);
    else if (a.lin)
      err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrate_table<TB, true>, block, smem);
    else
      err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrate_table<TB, false>, block, smem);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) per_sm = 1;
  }
  int64_t grid = (int64_t)per_sm * device_sm_count();
  const int64_t need = (a.n + block - 1) / block;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  if (mw) {
    mw_launch<TB>(shape.variant, (unsigned)grid, block, stream, a, p);
  } else {
    auto kernel = a.lin ? k_integrate_table<TB, true> : k_integrate_table<TB, false>;
    if (smem > 48 * 1024) {
      err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (err != cudaSuccess) return err;
    }
    kernel<<<(unsigned)grid, block, smem, stream>>>(a, comps, ncomp);
  }
  return cudaGetLastError();
}

}  // namespace gal
