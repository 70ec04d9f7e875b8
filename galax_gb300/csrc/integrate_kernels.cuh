// Kernel entry points and launcher for one Runge-Kutta method (included once per
// method by integrate_dopri5.cu / integrate_dopri8.cu so the two compile in parallel).
#pragma once

#include "launch.h"

namespace gal {

constexpr int kMaxBlock = 256;

// MINB = 1: registers up to 255 (no spills); MINB = 2: at most 128 registers per
// thread for more resident warps (a few spills). The autotuner picks per workload.
template <class TB, int MINB>
__global__ void __launch_bounds__(kMaxBlock, MINB) k_integrate_mw(IntegrateArgs a, MWParams p) {
  const MWPot pot{p};
  integrate_loop<TB>(a, pot);
}

template <class TB>
__global__ void __launch_bounds__(kMaxBlock) k_integrate_table(IntegrateArgs a, const DevComp* comps, int ncomp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  DevComp* s_comps = reinterpret_cast<DevComp*>(smem_raw);
  for (int i = threadIdx.x; i < ncomp; i += blockDim.x) s_comps[i] = comps[i];
  __syncthreads();
  const TablePot pot{s_comps, ncomp};
  integrate_loop<TB>(a, pot);
}

template <class TB>
cudaError_t launch_integrate(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps, int ncomp,
                             LaunchShape shape, cudaStream_t stream) {
  const int block = shape.block_threads > 0 ? shape.block_threads : 128;
  if (block > kMaxBlock || block % 32 != 0) return cudaErrorInvalidValue;
  const size_t smem = mw ? 0 : sizeof(DevComp) * (size_t)ncomp;
  int per_sm = shape.blocks_per_sm;
  cudaError_t err;
  const bool dense = shape.variant == 1;
  if (per_sm <= 0) {
    if (mw)
      err = dense ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrate_mw<TB, 2>, block, 0)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrate_mw<TB, 1>, block, 0);
    else
      err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrate_table<TB>, block, smem);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) per_sm = 1;
  }
  int64_t grid = (int64_t)per_sm * device_sm_count();
  const int64_t need = (a.n + block - 1) / block;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  if (mw) {
    if (dense)
      k_integrate_mw<TB, 2><<<(unsigned)grid, block, 0, stream>>>(a, p);
    else
      k_integrate_mw<TB, 1><<<(unsigned)grid, block, 0, stream>>>(a, p);
  } else {
    if (smem > 48 * 1024) {
      err = cudaFuncSetAttribute(k_integrate_table<TB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (err != cudaSuccess) return err;
    }
    k_integrate_table<TB><<<(unsigned)grid, block, smem, stream>>>(a, comps, ncomp);
  }
  return cudaGetLastError();
}

}  // namespace gal
