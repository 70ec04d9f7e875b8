// Dopri8 instantiation of the orbit-integration kernels.
#include "integrate_kernels.cuh"

namespace gal {
cudaError_t launch_integrate_dopri8(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps,
                                    int ncomp, LaunchShape shape, cudaStream_t stream) {
  return launch_integrate<Dopri8>(a, mw, p, comps, ncomp, shape, stream);
}
}  // namespace gal
