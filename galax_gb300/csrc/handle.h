// Internal definition of the opaque gal_potential handle and error helpers
// shared by the library's translation units.
#pragma once

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
// Entry points that evaluate the potential at fixed times only (adjoint, dense
// output, streams, surrogate) refuse time-dependent potentials with this.
inline bool time_dependent(const gal_potential* p) { return p && p->d_lin; }
}  // namespace gal

namespace gal {
gal_status fail(gal_status st, const std::string& msg);
gal_status cuda_fail(cudaError_t e, const char* where);
gal_status validate_cfg(const gal_solver_config* c);
int device_sm_count();
}  // namespace gal
