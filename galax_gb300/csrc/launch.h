// Host-side launchers shared between the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include "integrate.cuh"

namespace gal {

struct LaunchShape {
  int block_threads;  // 0 = default
  int blocks_per_sm;  // 0 = occupancy maximum
  int variant;        // Milky Way kernel: 0 = up to 255 registers, 1 = at most 128 (more warps)
  int table_lanes;    // component tables: 0 = automatic, 1 = one thread per orbit, 32 = one warp per orbit
};

// Component tables with at least this many components may run one warp per orbit.
constexpr int kWarpMinComponents = 32;

cudaError_t launch_integrate_dopri5(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps,
                                    int ncomp, LaunchShape shape, cudaStream_t stream);
cudaError_t launch_integrate_dopri8(const IntegrateArgs& a, bool mw, const MWParams& p, const DevComp* comps,
                                    int ncomp, LaunchShape shape, cudaStream_t stream);

// Four-warp teams (32 orbits per block) for queue positions [0, tcap) of a
// second-pass Milky Way Dopri5 batch; *tqueue must be zero. smem: dynamic
// shared memory requested (unused) to hold each team block's SM alone.
cudaError_t launch_integrate_team(const IntegrateArgs& a, const MWParams& p, unsigned long long* tqueue,
                                  long long tcap, int blocks, size_t smem, cudaStream_t stream);
// The one-thread Milky Way Dopri5 kernel, `block` threads per block, `grid`
// blocks, each requesting `smem` bytes (unused) so that blocks of this launch
// and of the team launch never share an SM.
cudaError_t launch_integrate_dopri5_exclusive(const IntegrateArgs& a, const MWParams& p, int variant, int block,
                                              int grid, size_t smem, cudaStream_t stream);
// The same two launches for a Dopri8 batch.
cudaError_t launch_integrate_team8(const IntegrateArgs& a, const MWParams& p, unsigned long long* tqueue,
                                   long long tcap, int blocks, size_t smem, cudaStream_t stream);
cudaError_t launch_integrate_dopri8_exclusive(const IntegrateArgs& a, const MWParams& p, int variant, int block,
                                              int grid, size_t smem, cudaStream_t stream);
constexpr size_t kExclusiveSmem = 120 * 1024;

int device_sm_count();

}  // namespace gal
