// Host-side launchers shared between the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include "integrate.cuh"

namespace gal {

struct LaunchShape {
  int block_threads;  // 0 = default
  int blocks_per_sm;  // 0 = occupancy maximum
  int variant;        // Milky Way kernel: 0 = up to 255 registers, 1 = at most 128 (more warps)
};

cudaError_t launch_integrate_dopri5(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps,
                                    int ncomp, LaunchShape shape, cudaStream_t stream);
cudaError_t launch_integrate_dopri8(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps,
                                    int ncomp, LaunchShape shape, cudaStream_t stream);

int device_sm_count();

}  // namespace gal
