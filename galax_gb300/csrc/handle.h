// Internal definition of the opaque gal_potential handle and error helpers
// shared by the library's translation units.
#pragma once

#include <new>
#include <string>
#include <vector>

#include "../../include/galax_gb300.h"
#include "potentials.cuh"

struct gal_potential {
  std::vector<gal_component> comps;
  double G;
  gal::DevComp* d_comps;  // device copy of the folded table
  int n;
  bool is_mw;             // evaluated by the specialised Milky Way model
  gal::MWParams mw;
  gal::DevLinear* d_lin = nullptr;  // linear time dependence per component (NULL: static)
};

namespace gal {
// Entry points that evaluate the potential at fixed times only (adjoint,
// streams, surrogate) refuse time-dependent potentials with this.
inline bool time_dependent(const gal_potential* p) { return p && p->d_lin; }
}  // namespace gal

namespace gal {
gal_status fail(gal_status st, const std::string& msg);
gal_status cuda_fail(cudaError_t e, const char* where);
gal_status validate_cfg(const gal_solver_config* c);
int device_sm_count();

// Runs the body of an entry point that allocates host memory, so that no C++
// exception crosses the C ABI: a failed allocation becomes GAL_ERR_HOST_ALLOC.
template <class Body>
gal_status no_throw(Body&& body) noexcept {
  gal_status st = GAL_ERR_HOST_ALLOC;
  try {
    return body();
  } catch (const std::bad_alloc&) {
  } catch (...) {
    st = GAL_ERR_INVALID_ARGUMENT;
  }
  try {
    fail(st, st == GAL_ERR_HOST_ALLOC ? "host allocation failed" : "unexpected C++ exception");
  } catch (...) {
  }
  return st;
}
}  // namespace gal
