// XLA FFI handlers over the galax_gb300 C ABI, so that jax programs (galax's
// own orbit path runs under jax.jit) call the GB300 kernels as custom calls.
//
// Each handler is a thin forwarder: XLA owns every buffer (inputs, results and
// the scratch, which is one more result buffer sized by the matching
// *_workspace_size query on the host), and the work is queued on XLA's stream.
// The potential is a gal_potential built once on the host, outside the traced
// function, and passed as its address in the int64 attribute "pot".
//
// Replaces, under jax:
//   GalIntegrate : diffrax.diffeqsolve with SaveAt(ts) as driven by galax's
//                  Integrator / OrbitSolver (src/galax/dynamics/_src/fields.py:168-188,
//                  legacy/integrator.py:179-245), per-orbit controllers
//   GalGradient  : AbstractPotential._gradient = jax.grad(_potential)
//                  (src/galax/potential/_src/base.py:170-179)
//   GalAdjoint   : reverse-mode differentiation through diffeqsolve for a
//                  terminal cotangent (src/galax/dynamics/_src/orbit/solver.py:99-108,133)
//
// Built against the headers jaxlib ships (jax.ffi.include_dir()) by
// galax_gb300/xla/__init__.py::build, and linked to libgalax_gb300.so.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "galax_gb300.h"
#include "xla/ffi/api/ffi.h"

namespace ffi = xla::ffi;

namespace {

ffi::Error status_error(gal_status st, const char* what) {
  if (st == GAL_OK) return ffi::Error::Success();
  std::string msg = std::string(what) + ": " + gal_status_string(st) + ": " + gal_last_error();
  if (st == GAL_ERR_INVALID_ARGUMENT || st == GAL_ERR_UNSUPPORTED || st == GAL_ERR_TOO_LARGE ||
      st == GAL_ERR_WORKSPACE)
    return ffi::Error::InvalidArgument(msg);
  return ffi::Error::Internal(msg);
}

const gal_potential* as_potential(int64_t address) { return reinterpret_cast<const gal_potential*>(address); }

// The gal_solver_config of a custom call, from its attributes.
gal_solver_config solver_config(int32_t method, int32_t adaptive, int64_t max_steps, double dt0, double rtol,
                                double atol, double dtmin, double dtmax, double pcoeff, double icoeff, double dcoeff,
                                double safety, double factormin, double factormax, int32_t force_dtmin,
                                int32_t schedule) {
  gal_solver_config c{};
  c.method = method;
  c.adaptive = adaptive;
  c.max_steps = max_steps;
  c.dt0 = dt0;
  c.rtol = rtol;
  c.atol = atol;
  c.dtmin = dtmin;
  c.dtmax = dtmax;
  c.pcoeff = pcoeff;
  c.icoeff = icoeff;
  c.dcoeff = dcoeff;
  c.safety = safety;
  c.factormin = factormin;
  c.factormax = factormax;
  c.force_dtmin = force_dtmin;
  c.schedule = schedule;
  return c;
}

// y0 [6][n]; t0, t1 [n]; save_offsets [n+1] (CSR save grids) or [0] (one grid
// shared by every orbit); save_ts [T] -> out [6][T][n] (shared) or [6][T]
// (CSR), status [n], steps [n], workspace [bytes].
ffi::Error Integrate(cudaStream_t stream, ffi::Buffer<ffi::F64> y0, ffi::Buffer<ffi::F64> t0,
                     ffi::Buffer<ffi::F64> t1, ffi::Buffer<ffi::S64> save_offsets, ffi::Buffer<ffi::F64> save_ts,
                     ffi::ResultBuffer<ffi::F64> out, ffi::ResultBuffer<ffi::S32> status,
                     ffi::ResultBuffer<ffi::S64> steps, ffi::ResultBuffer<ffi::U8> workspace, int64_t pot,
                     int32_t method, int32_t adaptive, int64_t max_steps, double dt0, double rtol, double atol,
                     double dtmin, double dtmax, double pcoeff, double icoeff, double dcoeff, double safety,
                     double factormin, double factormax, int32_t force_dtmin, int32_t schedule) {
  const int64_t n = (int64_t)t0.element_count();
  if ((int64_t)y0.element_count() != 6 * n || (int64_t)t1.element_count() != n)
    return ffi::Error::InvalidArgument("GalIntegrate: y0 must be [6][n] and t0, t1 [n]");
  const bool csr = save_offsets.element_count() != 0;
  if (csr && (int64_t)save_offsets.element_count() != n + 1)
    return ffi::Error::InvalidArgument("GalIntegrate: save_offsets must be [n+1] or empty");
  const int64_t n_saves = (int64_t)save_ts.element_count();
  const int64_t want = csr ? 6 * n_saves : 6 * n_saves * n;
  if ((int64_t)out->element_count() != want)
    return ffi::Error::InvalidArgument("GalIntegrate: out must be [6][T][n] (shared grid) or [6][T] (CSR)");
  const gal_solver_config cfg = solver_config(method, adaptive, max_steps, dt0, rtol, atol, dtmin, dtmax, pcoeff,
                                              icoeff, dcoeff, safety, factormin, factormax, force_dtmin, schedule);
  const gal_status st = gal_integrate(
      as_potential(pot), &cfg, y0.typed_data(), t0.typed_data(), t1.typed_data(),
      csr ? save_offsets.typed_data() : nullptr, save_ts.typed_data(), n_saves, out->typed_data(),
      status->typed_data(), steps->typed_data(), nullptr, n, workspace->untyped_data(),
      (size_t)workspace->size_bytes(), reinterpret_cast<gal_stream_t>(stream));
  return status_error(st, "gal_integrate");
}

// x [3][n] -> grad [3][n] at time t.
ffi::Error Gradient(cudaStream_t stream, ffi::Buffer<ffi::F64> x, ffi::ResultBuffer<ffi::F64> grad, int64_t pot,
                    double t) {
  const int64_t n = (int64_t)x.element_count() / 3;
  if ((int64_t)x.element_count() != 3 * n || grad->element_count() != x.element_count())
    return ffi::Error::InvalidArgument("GalGradient: x and grad must be [3][n]");
  const gal_status st = gal_eval_gradient(as_potential(pot), x.typed_data(), t, n, grad->typed_data(),
                                          reinterpret_cast<gal_stream_t>(stream));
  return status_error(st, "gal_eval_gradient");
}

// y0 [6][n], lambda = dL/dy(t1) [6][n] -> yT [6][n], dL/dy0 [6][n],
// dL/d(m, l1, l2) [ncomp][3] (with the slopes, [ncomp][6], for a
// time-dependent potential), workspace [bytes]; constant step dt.
ffi::Error Adjoint(cudaStream_t stream, ffi::Buffer<ffi::F64> y0, ffi::Buffer<ffi::F64> lambda,
                   ffi::ResultBuffer<ffi::F64> yT, ffi::ResultBuffer<ffi::F64> grad_y0,
                   ffi::ResultBuffer<ffi::F64> grad_params, ffi::ResultBuffer<ffi::U8> workspace, int64_t pot,
                   int32_t method, double dt, double t0, double t1, int32_t k_ckpt) {
  const int64_t n = (int64_t)y0.element_count() / 6;
  if ((int64_t)y0.element_count() != 6 * n || lambda.element_count() != y0.element_count() ||
      yT->element_count() != y0.element_count() || grad_y0->element_count() != y0.element_count())
    return ffi::Error::InvalidArgument("GalAdjoint: y0, lambda, yT and grad_y0 must be [6][n]");
  const int64_t per = gal_potential_is_time_dependent(as_potential(pot)) ? 6 : 3;
  if ((int64_t)grad_params->element_count() != per * (int64_t)gal_potential_num_components(as_potential(pot)))
    return ffi::Error::InvalidArgument("GalAdjoint: grad_params must be [ncomp][3] ([ncomp][6] when time-dependent)");
  const gal_solver_config cfg =
      solver_config(method, 0, INT64_MAX, dt, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.9, 0.2, 10.0, 1, 0);
  const gal_status st = gal_adjoint(as_potential(pot), &cfg, y0.typed_data(), t0, t1, lambda.typed_data(), nullptr,
                                    yT->typed_data(), grad_y0->typed_data(), grad_params->typed_data(), k_ckpt, n,
                                    workspace->untyped_data(), (size_t)workspace->size_bytes(),
                                    reinterpret_cast<gal_stream_t>(stream));
  return status_error(st, "gal_adjoint");
}

}  // namespace

XLA_FFI_DEFINE_HANDLER_SYMBOL(GalIntegrate, Integrate,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()  // y0
                                  .Arg<ffi::Buffer<ffi::F64>>()  // t0
                                  .Arg<ffi::Buffer<ffi::F64>>()  // t1
                                  .Arg<ffi::Buffer<ffi::S64>>()  // save_offsets
                                  .Arg<ffi::Buffer<ffi::F64>>()  // save_ts
                                  .Ret<ffi::Buffer<ffi::F64>>()  // out
                                  .Ret<ffi::Buffer<ffi::S32>>()  // status
                                  .Ret<ffi::Buffer<ffi::S64>>()  // steps
                                  .Ret<ffi::Buffer<ffi::U8>>()   // workspace
                                  .Attr<int64_t>("pot")
                                  .Attr<int32_t>("method")
                                  .Attr<int32_t>("adaptive")
                                  .Attr<int64_t>("max_steps")
                                  .Attr<double>("dt0")
                                  .Attr<double>("rtol")
                                  .Attr<double>("atol")
                                  .Attr<double>("dtmin")
                                  .Attr<double>("dtmax")
                                  .Attr<double>("pcoeff")
                                  .Attr<double>("icoeff")
                                  .Attr<double>("dcoeff")
                                  .Attr<double>("safety")
                                  .Attr<double>("factormin")
                                  .Attr<double>("factormax")
                                  .Attr<int32_t>("force_dtmin")
                                  .Attr<int32_t>("schedule"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(GalGradient, Gradient,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()  // x
                                  .Ret<ffi::Buffer<ffi::F64>>()  // grad
                                  .Attr<int64_t>("pot")
                                  .Attr<double>("t"));

XLA_FFI_DEFINE_HANDLER_SYMBOL(GalAdjoint, Adjoint,
                              ffi::Ffi::Bind()
                                  .Ctx<ffi::PlatformStream<cudaStream_t>>()
                                  .Arg<ffi::Buffer<ffi::F64>>()  // y0
                                  .Arg<ffi::Buffer<ffi::F64>>()  // lambda
                                  .Ret<ffi::Buffer<ffi::F64>>()  // yT
                                  .Ret<ffi::Buffer<ffi::F64>>()  // grad_y0
                                  .Ret<ffi::Buffer<ffi::F64>>()  // grad_params
                                  .Ret<ffi::Buffer<ffi::U8>>()   // workspace
                                  .Attr<int64_t>("pot")
                                  .Attr<int32_t>("method")
                                  .Attr<double>("dt")
                                  .Attr<double>("t0")
                                  .Attr<double>("t1")
                                  .Attr<int32_t>("k_ckpt"));
