// Dopri5 instantiation of the orbit-integration kernels, and the four-warp
// team kernel for the longest orbits of a two-pass Milky Way batch.
#include "integrate_kernels.cuh"
#include "integrate_team.cuh"

namespace gal {
cudaError_t launch_integrate_dopri5(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps,
                                    int ncomp, LaunchShape shape, cudaStream_t stream) {
  return launch_integrate<Dopri5>(a, mw, p, comps, ncomp, shape, stream);
}

cudaError_t launch_integrate_team(const IntegrateArgs& a, const MWParams& p, unsigned long long* tqueue,
                                  long long tcap, int blocks, size_t smem, cudaStream_t stream) {
  cudaError_t e =
      cudaFuncSetAttribute(k_integrate_mw_team<Dopri5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_integrate_mw_team<Dopri5><<<(unsigned)blocks, 128, smem, stream>>>(a, p, tqueue, tcap);
  return cudaGetLastError();
}

cudaError_t launch_integrate_dopri5_exclusive(const IntegrateArgs& a, const MWParams& p, int variant, int block,
                                              int grid, size_t smem, cudaStream_t stream) {
  if (variant != 2 && block > 128) block = 128;  // variants 0 and 1 are built for at most 128 threads
  return mw_launch_exclusive<Dopri5>(variant, (unsigned)grid, block, smem, stream, a, p);
}
}  // namespace gal
