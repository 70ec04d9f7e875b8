// Dopri5 instantiation of the orbit-integration kernels.
#include "integrate_kernels.cuh"

namespace gal {
cudaError_t launch_integrate_dopri5(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps,
                                    int ncomp, LaunchShape shape, cudaStream_t stream) {
  return launch_integrate<Dopri5>(a, mw, p, comps, ncomp, shape, stream);
}
}  // namespace gal
