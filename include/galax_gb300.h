/*
 * galax_gb300 — C ABI of the GB300 (sm_103a) orbit-integration library.
 *
 * The library replaces, for static composites of Kepler / Hernquist /
 * Miyamoto-Nagai / NFW / Plummer components, the part of GalacticDynamics/galax
 * that runs below `gd.evaluate_orbit` and `gp.AbstractPotential.gradient`:
 * the field, potential-gradient, Runge-Kutta stepping, step-size control and
 * save-time interpolation that galax hands to diffrax.
 *
 * Conventions
 *   - Units are galax's "galactic" system: kpc, Myr, Msun (G passed in).
 *   - Arrays are caller-owned device memory, structure-of-arrays float64:
 *     positions x[3][n] (x[0..n) = all x, then y, then z); phase-space
 *     y[6][n] (x, y, z, vx, vy, vz).
 *   - Every call is asynchronous on the given stream (cudaStream_t; NULL = legacy
 *     default stream) and returns a gal_status. Nothing synchronises the device.
 *   - Scratch memory is caller-provided: size it with the matching
 *     *_workspace_size query. The library allocates device memory only inside
 *     gal_potential_create (its component table) and frees it in
 *     gal_potential_destroy.
 *   - No C++ exception crosses this boundary.
 */
#ifndef GALAX_GB300_H
#define GALAX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gal_stream_t; /* identical to cudaStream_t */

#if defined(__GNUC__)
#define GAL_API __attribute__((visibility("default")))
#else
#define GAL_API
#endif

/* ------------------------------------------------------------------ status */
typedef enum gal_status {
  GAL_OK = 0,
  GAL_ERR_INVALID_ARGUMENT = 1,
  GAL_ERR_UNSUPPORTED = 2,
  GAL_ERR_CUDA = 3,
  GAL_ERR_WORKSPACE = 4,
  GAL_ERR_TOO_LARGE = 5,
  GAL_ERR_HOST_ALLOC = 6 /* a host-side allocation failed; no C++ exception leaves the library */
} gal_status;

/* Per-orbit outcome; mirrors diffrax.RESULTS as raised by galax's solvers
 * (src/galax/dynamics/_src/solver.py:69-72). */
typedef enum gal_orbit_status {
  GAL_ORBIT_OK = 0,
  GAL_ORBIT_MAX_STEPS = 1, /* diffrax RESULTS.max_steps_reached */
  GAL_ORBIT_DT_MIN = 2,    /* diffrax RESULTS.dt_min_reached (force_dtmin = 0) */
  GAL_ORBIT_NONFINITE = 3  /* state became NaN/inf; integration stopped */
} gal_orbit_status;

/* ------------------------------------------------------------------ potential */
typedef enum gal_kind {
  GAL_KEPLER = 0,         /* Phi = -G m / r                src/galax/potential/_src/builtin/kepler.py */
  GAL_HERNQUIST = 1,      /* Phi = -G m / (r + r_s)        .../builtin/hernquist.py:80-82 */
  GAL_MIYAMOTO_NAGAI = 2, /* Phi = -G m / sqrt(R^2 + (sqrt(z^2+b^2)+a)^2)  .../miyamotonagai.py:73-78 */
  GAL_NFW = 3,            /* Phi = -G m log(1 + r/r_s) / r .../builtin/nfw/base.py:326-338 */
  GAL_PLUMMER = 4,        /* Phi = -G m / sqrt(r^2 + b^2)  .../builtin/plummer.py:122-133 */
  GAL_ISOCHRONE = 5,      /* Phi = -G m / (b + sqrt(r^2 + b^2))  .../builtin/isochrone.py:61-110 */
  GAL_LOGARITHMIC = 6,    /* Phi = v_c^2 / 2 log(r_s^2 + r^2)    .../builtin/logarithmic.py:45-53 */
  GAL_POWERLAW_CUTOFF = 7 /* rho ~ (r_c/r)^alpha exp(-(r/r_c)^2): Phi = -G m P(a1, s^2) / r
                           * - G m Gamma(a2, s^2) / (r_c Gamma(a1)), s = r / r_c, a1 = (3 - alpha)/2,
                           * a2 = 1 - alpha/2, P / Gamma(., .) the regularised lower / upper
                           * incomplete gamma functions  .../builtin/powerlawcutoff.py:21-120 */
} gal_kind;

/* One component of a composite potential (src/galax/potential/_src/base_multi.py:39-55).
 * m  : m_tot (Kepler, Hernquist, Miyamoto-Nagai, Plummer, isochrone), m (NFW) or
 *      v_c in kpc/Myr (logarithmic)
 * l1 : r_s (Hernquist, NFW, Plummer, isochrone b, logarithmic), a (Miyamoto-Nagai) or
 *      r_c (power law with cutoff); unused for Kepler
 * l2 : b (Miyamoto-Nagai) or alpha (power law with cutoff, 0 <= alpha < 2: galax's
 *      potential is not finite for alpha >= 2); unused otherwise
 * origin : constant translation of the component centre
 *          (src/galax/potential/_src/xfm/translate.py:28-87 with a constant shift). */
typedef struct gal_component {
  int32_t kind;
  int32_t flags; /* must be 0 */
  double m;
  double l1;
  double l2;
  double origin[3];
} gal_component;

typedef struct gal_potential gal_potential; /* opaque */

/* Build a device-resident composite. Replaces the construction of
 * gp.CompositePotential / gp.MilkyWayPotential (src/galax/potential/_src/composite.py:32-108,
 * builtin/milkyway.py:172-236). n in [1, GAL_MAX_COMPONENTS]. */
#define GAL_MAX_COMPONENTS 1024
GAL_API gal_status gal_potential_create(const gal_component* comps, int32_t n, double G, gal_potential** out);
GAL_API gal_status gal_potential_destroy(gal_potential* pot);
/* Linear time dependence of component parameters, galax's LinearParameter
 * (src/galax/potential/_src/params/core.py:25-110): with slopes [n][3] (host
 * array, d(m, l1, l2)/dt per component), component i is evaluated with
 * m + slopes[i][0] t, l1 + slopes[i][1] t, l2 + slopes[i][2] t, where the
 * component table holds the values at t = 0 (galax's point-slope form
 * p(t) = slope (t - t_i) + p(t_i) gives p(0) = p(t_i) - slope t_i). The
 * gal_eval_* functions evaluate at their t; gal_integrate,
 * gal_integrate_noalloc, the dense-output pair (gal_integrate_dense,
 * gal_dense_evaluate) and gal_adjoint evaluate every stage at its own time;
 * gal_adjoint also returns the derivatives with respect to the slopes. Stream
 * and surrogate entry points reject time-dependent potentials
 * (GAL_ERR_UNSUPPORTED). slopes = NULL makes the potential static again; any
 * other array, all zeros included, makes it time-dependent. */
GAL_API gal_status gal_potential_set_linear(gal_potential* pot, const double* slopes);
/* Replace the parameters (same count and kinds), e.g. between optimiser steps. */
GAL_API gal_status gal_potential_update(gal_potential* pot, const gal_component* comps, int32_t n, gal_stream_t stream);
GAL_API int32_t gal_potential_num_components(const gal_potential* pot);
/* 1 when the composite is evaluated by the specialised MilkyWayPotential kernel. */
GAL_API int32_t gal_potential_is_milky_way(const gal_potential* pot);
/* 1 when gal_potential_set_linear gave the composite time-dependent parameters. */
GAL_API int32_t gal_potential_is_time_dependent(const gal_potential* pot);

/* Batched evaluation at n positions x[3][n] at time t. t matters only for a
 * potential with LinearParameter slopes (gal_potential_set_linear), whose
 * parameters are evaluated at t; static potentials ignore it.
 *   gal_eval_potential    : phi[n]       replaces AbstractPotential._potential   (base.py:113-136)
 *   gal_eval_gradient     : out[3][n]    replaces AbstractPotential._gradient    (base.py:170-179)
 *   gal_eval_acceleration : out[3][n]    replaces api.acceleration = -gradient   (register_funcs.py:327-340)
 *   gal_eval_hessian      : out[9][n]    replaces AbstractPotential._hessian     (base.py:230-239) */
GAL_API gal_status gal_eval_potential(const gal_potential* pot, const double* x, double t, int64_t n, double* phi,
                              gal_stream_t stream);
GAL_API gal_status gal_eval_gradient(const gal_potential* pot, const double* x, double t, int64_t n, double* out,
                             gal_stream_t stream);
GAL_API gal_status gal_eval_acceleration(const gal_potential* pot, const double* x, double t, int64_t n, double* out,
                                 gal_stream_t stream);
GAL_API gal_status gal_eval_hessian(const gal_potential* pot, const double* x, double t, int64_t n, double* out,
                            gal_stream_t stream);

/* ------------------------------------------------------------------ integration */
/* Solver configuration; field meanings follow diffrax's Dopri5/Dopri8,
 * ConstantStepSize and PIDController as configured by galax
 * (src/galax/dynamics/_src/legacy/integrator.py:161-168, orbit/solver.py:121-141). */
typedef struct gal_solver_config {
  int32_t method;    /* 5 = Dopri5, 8 = Dopri8 */
  int32_t adaptive;  /* 0 = ConstantStepSize(dt0), 1 = PIDController */
  int64_t max_steps; /* bound on step attempts per orbit (accepted + rejected) */
  double dt0;        /* constant step; for PID the initial step (<= 0: automatic selection) */
  double rtol, atol;
  double dtmin, dtmax; /* <= 0 means None */
  double pcoeff, icoeff, dcoeff;
  double safety, factormin, factormax;
  int32_t force_dtmin;
  /* 0: one pass. 1: two passes over the batch with identical results: every
   * orbit first covers the first tenth of its time span, then the orbits are
   * resumed in order of decreasing estimated remaining work (steps so far x
   * remaining fraction), so the longest orbits start early instead of forming a
   * tail. Useful for adaptive batches with uneven lengths. */
  int32_t schedule;
} gal_solver_config;

/* Scratch bytes gal_integrate needs for n orbits (work-queue counters, and with
 * cfg->schedule = 1 a 128-byte resume record per orbit plus ordering arrays). */
GAL_API gal_status gal_integrate_workspace_size(const gal_solver_config* cfg, int64_t n, size_t* bytes);

/* Integrate n orbits from t0[i] to t1[i] (t1 < t0 integrates backwards) and
 * write the state at each orbit's save times. Replaces diffrax.diffeqsolve with
 * SaveAt(ts=...) as driven by galax's Integrator / OrbitSolver
 * (src/galax/dynamics/_src/legacy/integrator.py:179-245, orbit/solver.py:774-803),
 * one independent controller per orbit (the per-orbit dispatch of
 * legacy/integrator.py:449-527).
 *
 * y0        : [6][n] initial states at t0
 * t0, t1    : [n]
 * save_offsets : NULL  -> every orbit uses save_ts[0..n_saves) and out is [6][n_saves][n]
 *                !NULL -> [n+1] CSR offsets into save_ts; n_saves must equal save_offsets[n]
 *                         (the total) and out is [6][n_saves]
 * save_ts   : save times, increasing along the direction of integration, within [t0, t1]
 * out       : saved states; saves never reached (see status) are NaN
 * status    : [n] gal_orbit_status (may be NULL)
 * steps     : [n] accepted steps per orbit (may be NULL)
 * order     : optional [n] permutation: the work queue hands orbits out in this order
 * workspace : device scratch of at least gal_integrate_workspace_size bytes */
GAL_API gal_status gal_integrate(const gal_potential* pot, const gal_solver_config* cfg, const double* y0, const double* t0,
                         const double* t1, const int64_t* save_offsets, const double* save_ts, int64_t n_saves,
                         double* out, int32_t* status, int64_t* steps, const int32_t* order, int64_t n,
                         void* workspace, size_t workspace_bytes, gal_stream_t stream);

/* gal_integrate without a workspace. It has no counterpart in the reference:
 * galax runs under XLA, which manages all device memory.
 *
 * For callers that cannot allocate device memory: plug-ins that are handed
 * only their input and output buffers (an XLA custom call registered without a
 * scratch allocator, say), services that forbid device allocation after
 * start-up, and hosts with a fixed device-memory budget. The scratch that
 * gal_integrate takes from its workspace comes instead from a fixed array of
 * GAL_NOALLOC_SCRATCH_BYTES (4 MiB) in the library's own device memory, which
 * every GPU that loads the library holds until the process exits. Inputs and
 * outputs are the caller's, exactly as for gal_integrate, and the results are
 * bitwise the same. This function allocates and frees nothing.
 *  - Limit: a call whose gal_integrate_workspace_size exceeds the array is
 *    rejected with GAL_ERR_TOO_LARGE (with schedule = 1 that is about 30,000
 *    orbits per call; with schedule = 0 only 8 bytes are needed, so any n).
 *  - Set-up: the first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress) with that device current and keeps it for later
 *    calls; make that first call before any stream capture. cudaDeviceReset
 *    unloads the library's module and with it the array: do not call this
 *    function on a device after resetting it.
 *  - All calls share the one array and it keeps the previous call's contents
 *    (each call clears what must start at zero). Calls that overlap on the GPU,
 *    from different streams or threads, race on it: serialise them. */
#define GAL_NOALLOC_SCRATCH_BYTES (4 * 1024 * 1024)
GAL_API gal_status gal_integrate_noalloc(const gal_potential* pot, const gal_solver_config* cfg, const double* y0,
                                         const double* t0, const double* t1, const int64_t* save_offsets,
                                         const double* save_ts, int64_t n_saves, double* out, int32_t* status,
                                         int64_t* steps, const int32_t* order, int64_t n, gal_stream_t stream);

/* Dense output (dense=True): integrate n orbits from t0[i] to t1[i] like
 * gal_integrate (own controller per orbit) and record, for every accepted step,
 * what evaluates the orbit anywhere inside it afterwards. Replaces diffrax's
 * DenseInterpolation as wrapped by galax's PhaseSpaceInterpolation
 * (src/galax/dynamics/_src/orbit/interp.py:42-145).
 *   ts     : [n][cap+1] step boundaries (original time), ts[i][0] = t0[i]
 *   coef   : [n][cap][gal_dense_coef_per_step(method)] per step: Dopri5 the
 *            quartic of the save path in monomial form (5 x 6), Dopri8 the
 *            step's start state (6; evaluation takes a partial Dopri8 step)
 *   nsteps : [n] accepted steps recorded; status [n] (may be NULL): an orbit
 *            that needs more than cap steps stops with GAL_ORBIT_MAX_STEPS. */
GAL_API int32_t gal_dense_coef_per_step(int32_t method);
GAL_API gal_status gal_integrate_dense(const gal_potential* pot, const gal_solver_config* cfg, const double* y0,
                                       const double* t0, const double* t1, int64_t n, int64_t cap, double* ts,
                                       double* coef, int64_t* nsteps, int32_t* status, gal_stream_t stream);
/* Evaluate m queries (orbit[q], t[q]) of a dense result into out[6][m]; a query
 * outside its orbit's [t0, t1] gives NaN and adds 1 to *out_of_bounds (device
 * counter; galax raises "Time out of bounds", interp.py:60-64). */
GAL_API gal_status gal_dense_evaluate(const gal_potential* pot, int32_t method, const double* ts, const double* coef,
                                      const int64_t* nsteps, int64_t cap, int64_t n, const int64_t* orbit,
                                      const double* t, int64_t m, double* out, unsigned long long* out_of_bounds,
                                      gal_stream_t stream);

/* Launch shape used by gal_integrate for one (method, adaptive) pair: threads per
 * block (multiple of 32, <= 256; 0 = 128), blocks per SM (0 = occupancy maximum)
 * and register variant of the Milky Way kernel (0 = at most 168 registers per
 * thread, 3 blocks of 128 per SM; 1 = at most 128 registers, 4 blocks of 128;
 * 2 = up to 255 registers, blocks up to 256 threads; variants 0 and 1 need
 * block_threads <= 128). Process-wide setting, used by the autotuner; results
 * never depend on it. Defaults: adaptive runs use 128 threads, one block per SM,
 * variant 2 (one warp per SM sub-partition); constant-step runs use 128
 * threads at maximum occupancy (variant 0 for Dopri5, 2 for Dopri8). */
GAL_API gal_status gal_set_launch(int32_t method, int32_t adaptive, int32_t block_threads, int32_t blocks_per_sm,
                                  int32_t variant);
/* Second pass of a two-pass Dopri5 or Dopri8 batch in the Milky Way model: `blocks` > 0
 * (default 32, at most the SM count - 1) hands the 32 x blocks longest orbits to
 * four-warp team blocks, each on an SM of its own, on a library-owned stream
 * beside the one-thread-per-orbit kernel, which runs one block per remaining
 * SM; 0 keeps every orbit on the one-thread kernel with the launch shape of
 * gal_set_launch. Results are bitwise identical either way; the teams cut the
 * serial latency of the longest orbits. Process-wide. */
GAL_API gal_status gal_set_team(int32_t blocks);
/* Fraction of every orbit's span that the first pass of the two-pass schedule
 * (cfg->schedule = 1) covers before the orbits are ordered by their remaining
 * work (default 0.1, allowed [0.001, 0.9]). Results are bitwise identical for
 * any value; it only moves work between the passes. Process-wide. */
GAL_API gal_status gal_set_split_fraction(double fraction);
/* Orbits per thread or warp for component tables (composites other than the
 * specialised Milky Way kernel) in gal_integrate: 1 runs one thread per orbit;
 * 32 runs one warp per orbit, its lanes splitting the components and reducing
 * the gradient with warp shuffles; 0 (default) takes a warp per orbit when the
 * table has at least 32 components and the batch is too small to give every
 * SM sub-partition a warp of 32 orbits (fewer than 128 orbits per SM).
 * The two differ only in the order of the component sum (rounding).
 * Process-wide. galax evaluates a composite by summing its components
 * (src/galax/potential/_src/base_multi.py:48-55). */
GAL_API gal_status gal_set_table_lanes(int32_t lanes);

/* ------------------------------------------------------------------ adjoint */
/* Scratch bytes gal_adjoint needs for n orbits with checkpoints every k_ckpt steps. */
GAL_API gal_status gal_adjoint_workspace_size(const gal_potential* pot, const gal_solver_config* cfg, double t0, double t1,
                                      int32_t k_ckpt, int64_t n, size_t* bytes);

/* Discrete adjoint of the constant-step map y(t0) -> y(t1) (cfg->adaptive must be
 * 0; step cfg->dt0) for terminal cotangents: given lambda = dL/dy(t1) [6][n],
 * returns the final states yT [6][n], dL/dy0 [6][n] and dL/d(m, l1, l2) for
 * every component, summed over orbits, [ncomp][3]; for a time-dependent
 * potential (gal_potential_is_time_dependent) grad_params is [ncomp][6]:
 * d/d(m, l1, l2) of the values at t = 0, then d/d(their slopes), each stage
 * evaluated at its own time (galax's LinearParameter,
 * src/galax/potential/_src/params/core.py:25-110). The forward pass stores the
 * state every k_ckpt steps; the reverse pass recomputes each segment from its
 * checkpoint. Replaces reverse-mode differentiation through diffeqsolve with
 * RecursiveCheckpointAdjoint (src/galax/dynamics/_src/orbit/solver.py:99-108)
 * and the forward-mode jacfwd path (ForwardMode, orbit/solver.py:133).
 * If lambda is NULL, the loss L = sum |yT - target|^2 is used (target [6][n]). */
GAL_API gal_status gal_adjoint(const gal_potential* pot, const gal_solver_config* cfg, const double* y0, double t0,
                       double t1, const double* lambda, const double* target, double* yT, double* grad_y0,
                       double* grad_params, int32_t k_ckpt, int64_t n, void* workspace, size_t workspace_bytes,
                       gal_stream_t stream);

/* ------------------------------------------------------------------ mock stream */
/* A stream released by a Plummer progenitor that moves along its own orbit in
 * the host potential `pot` (at most 8 components). Replaces galax's
 * StreamSimulator.init/run (src/galax/dynamics/_src/experimental/stream.py:121-230,
 * 380-446) and MockStreamGenerator.run with a moving progenitor potential
 * (legacy/mockstream/mockstream_generator.py:160-275, legacy/mockstream/_moving.py:20-42)
 * for releases on a constant-step grid:
 *  - the progenitor starts at w_now (time t_now), is integrated n_release steps
 *    of dt backwards, then forwards again to t_now;
 *  - release r = 0..n_release-1 happens at t_now - (n_release - r) dt with the
 *    King (1962) tidal radius r_t = cbrt(G prog_m / (Omega^2 - d2Phi/dr2))
 *    (dynamics/_src/cluster/radius.py:198-214) and sends particle 2r (leading)
 *    and 2r+1 (trailing): x = x_prog -/+ r_t rhat + 0.1 r_t xi,
 *    v = v_prog + 0.1 Omega r_t eta (xi, eta from `noise`);
 *  - every particle is integrated to t_now in pot + Plummer(prog_m, prog_b)
 *    centred on the progenitor's position at every Runge-Kutta stage.
 * Constant steps (Dopri5 or Dopri8). noise: [12][n_release] device array, rows
 * xi_lead(3), eta_lead(3), xi_trail(3), eta_trail(3). */
typedef struct gal_stream_config {
  int32_t method;    /* 5 = Dopri5, 8 = Dopri8 */
  int32_t k_ckpt;    /* gradient: >= 1 keeps particle checkpoints every k_ckpt steps and recomputes
                      * (memory ~ 2 n_release (n_release / k_ckpt + k_ckpt) 48 bytes); 0 stores every
                      * particle stage position and Hessian instead, taking all potential evaluations
                      * off the reverse sweep (memory n_release (n_release + 1) S 144 bytes, S = 13
                      * for Dopri8) */
  int64_t n_release; /* releases (1 .. 2^18; GAL_ERR_TOO_LARGE above); particles = 2 n_release */
  double dt;         /* constant step (> 0) */
  double t_now;      /* present time (the potential is static: only labels times) */
  double prog_m;     /* progenitor Plummer mass */
  double prog_b;     /* progenitor Plummer scale radius */
  double w_now[6];   /* progenitor phase-space point at t_now (host values) */
  int32_t df;        /* release model: GAL_STREAM_DF_OFFSETS, _FARDAL2015 or _CHEN2024 */
  int32_t reserved;  /* 0 */
  double df_params[8]; /* Fardal 2015: kr_bar, kvphi_bar, kz_bar, kvz_bar, sigma_kr, sigma_kvphi,
                        * sigma_kz, sigma_kvz (galax's defaults 2, 0.3, 0, 0, 0.5, 0.5, 0.5, 0.5);
                        * unused by GAL_STREAM_DF_OFFSETS */
} gal_stream_config;

/* Release models. For release r with progenitor point (x, v), King tidal radius
 * r_t and angular frequency Omega = |x cross v| / |x|^2, particle 2r (leading,
 * s = -1) and 2r + 1 (trailing, s = +1) start at
 *   OFFSETS:     x + s r_t rhat + 0.1 r_t xi,  v + 0.1 Omega r_t eta;
 *                noise [12][n]: xi_lead, eta_lead, xi_trail, eta_trail (3 each);
 *   FARDAL2015:  x + r_t (s kr rhat + kz zhat),  v + Omega r_t (s kvphi phihat + kvz zhat),
 *                kr = kr_bar + sigma_kr n0, kvphi = kr (kvphi_bar + sigma_kvphi n1),
 *                kz = kz_bar + sigma_kz n2, kvz = kvz_bar + sigma_kvz n3, zhat along x cross v,
 *                phihat along v - (v . rhat) rhat; noise [4][n]: n0..n3, shared by both
 *                particles (legacy/mockstream/df/fardal15.py:49-94,
 *                experimental/df.py:136-177);
 *   CHEN2024:    posvel = mean + A z, z = noise [6][n] standard normals, A the
 *                lower-triangular factor of galax's covariance (posvel_0 and
 *                posvel_4 correlated at -0.7, posvel_3 fixed at 1); Dr = posvel_0 r_t,
 *                Dv = posvel_3 sqrt(2 G M / Dr), angles phi, theta, alpha, beta =
 *                posvel_1, 2, 4, 5 degrees; x -/+ Dr (cos th cos ph rhat + cos th sin ph
 *                phihat) + Dr sin th zhat, v -/+ Dv (cos b cos a rhat + cos b sin a phihat)
 *                + Dv sin b zhat (legacy/mockstream/df/chen24.py:21-137). */
#define GAL_STREAM_DF_OFFSETS 0
#define GAL_STREAM_DF_FARDAL2015 1
#define GAL_STREAM_DF_CHEN2024 2

/* Scratch bytes for gal_stream_run (with_grad = 0) or gal_stream_grad (1). */
GAL_API gal_status gal_stream_workspace_size(const gal_potential* pot, const gal_stream_config* cfg,
                                             int32_t with_grad, size_t* bytes);
/* Forward simulation: final_states [6][2 n_release] at t_now; optionally the
 * release conditions ics [6][2 n_release] and the progenitor's forwards track
 * prog_track [n_release + 1][6] (NULL to skip). */
GAL_API gal_status gal_stream_run(const gal_potential* pot, const gal_stream_config* cfg, const double* noise,
                                  double* final_states, double* ics, double* prog_track, void* workspace,
                                  size_t workspace_bytes, gal_stream_t stream);
/* Gradient of L = sum_p |y_p(t_now) - target_p|^2 (target [6][2 n_release])
 * with respect to (m, l1, l2) of every host component, grad_params [ncomp][3],
 * through the particle orbits, the release conditions (tidal radius included)
 * and the progenitor's orbit, by a hand-written discrete adjoint (galax takes
 * jax derivatives through the same pipeline; diffrax ForwardMode is the
 * stream solver's default, experimental/stream.py:35-43). Optional outputs:
 * final_states [6][2 n_release], grad_w_now [6] = dL/dw_now, loss [1] (device). */
GAL_API gal_status gal_stream_grad(const gal_potential* pot, const gal_stream_config* cfg, const double* noise,
                                   const double* target, double* final_states, double* grad_params,
                                   double* grad_w_now, double* loss, void* workspace, size_t workspace_bytes,
                                   gal_stream_t stream);

/* Release conditions sampled from a stream DF (the df and df_params fields of
 * gal_stream_config) at n progenitor points prog_w [6][n] with progenitor
 * masses prog_mass [n] (device arrays; df_params is a host array of 8 as in
 * gal_stream_config, NULL for the offsets model): lead and trail [6][n]
 * (device), and optionally the King (1962)
 * tidal radius r_tidal [n] (NULL to skip). Replaces FardalStreamDF._sample
 * (legacy/mockstream/df/fardal15.py:49-94) and Fardal2015DF.sample
 * (experimental/df.py:136-177) for a batch of release points, with
 * tidal_radius (dynamics/_src/cluster/radius.py:198-214) inside; the normal
 * draws come from the caller (noise [12][n], [4][n] or [6][n], see the release models
 * above) instead of a jax PRNG key. */
GAL_API gal_status gal_stream_df_sample(const gal_potential* pot, int32_t df, const double* df_params,
                                        const double* prog_w, const double* prog_mass, const double* noise, int64_t n,
                                        double* lead, double* trail, double* r_tidal, gal_stream_t stream);

/* ------------------------------------------------------------------ learned surrogate */
/* A small MLP, 3 -> 256 -> 256 -> 256 -> 256 -> 1 with SiLU activations, that
 * stands in for an expensive composite (a MilkyWayPotential plus hundreds of
 * Plummer subhalos; no counterpart class in galax). Input
 * u = x / length_scale, potential = phi_scale * out(u), gradient =
 * (phi_scale / length_scale) grad_u out. Parameters are one float32 vector of
 * gal_mlp_num_params() values: W1[256][3], b1, W2[256][256], b2, W3, b3, W4,
 * b4, w5[256], b5 (W rows are output units). */
typedef struct gal_mlp gal_mlp; /* opaque, device-resident inference weights */
GAL_API int64_t gal_mlp_num_params(void);
/* Training-side scratch for a batch of `batch` points. The 256 x 256 products
 * of the calls below run on the tensor cores (bf16 operands, FP32
 * accumulation); operands that the quantised passes do not round to bf16
 * enter as two bf16 parts (hi + lo), which keeps FP32-level accuracy. Zero a
 * new workspace before its first use: it holds a sticky error flag. */
GAL_API gal_status gal_mlp_workspace_size(int64_t batch, size_t* bytes);
/* The error flag of a training workspace (0 = none; non-zero = a tensor-core
 * product gave up waiting, so results since the last check are not valid);
 * synchronises `stream`, then clears the flag. */
GAL_API gal_status gal_mlp_workspace_error(void* workspace, int64_t batch, int32_t* code, gal_stream_t stream);
/* FP32 forward and input gradient of `batch` points u[batch][3] (network units):
 * phi[batch] = out(u), grad[batch][3] = grad_u out. quantize = 1 rounds weights
 * and the activations entering the 256x256 products to bfloat16, as inference does. */
GAL_API gal_status gal_mlp_forward_f32(const float* params, const float* u, int64_t batch, float* phi, float* grad,
                                       int32_t quantize, void* workspace, size_t workspace_bytes, gal_stream_t stream);
/* Loss L = 1/B sum_b w_b [alpha (out_b - phi_t,b)^2 + beta |grad_u out_b - g_t,b|^2]
 * (network units; weights[batch] = w_b, NULL for w_b = 1) and its exact gradient
 * with respect to every parameter (grad[num_params]). */
GAL_API gal_status gal_mlp_loss_grads(const float* params, const float* u, const float* phi_t, const float* g_t,
                                      const float* weights, int64_t batch, float alpha, float beta,
                                      int32_t quantize, float* grad, float* loss, void* workspace,
                                      size_t workspace_bytes, gal_stream_t stream);
/* One Adam step on that loss (step counts from 1). */
GAL_API gal_status gal_mlp_train_step(float* params, float* grad, float* adam_m, float* adam_v, const float* u,
                                      const float* phi_t, const float* g_t, const float* weights, int64_t batch,
                                      float alpha, float beta, float lr, float beta1, float beta2, float eps,
                                      int32_t step, int32_t quantize, float* loss, void* workspace,
                                      size_t workspace_bytes, gal_stream_t stream);
/* Train for `epochs` passes over n samples (u[n][3], phi_t[n], g_t[n][3],
 * weights[n] or NULL) in batches of `batch` (n / batch steps per epoch; the
 * remaining samples of a pass are left out), entirely on the device: each step
 * gathers its batch through a keyed pseudo-random permutation of the samples
 * (a new key every epoch, from `seed`), runs gal_mlp_loss_grads's kernels and
 * an Adam step with the cosine schedule lr_t = lr_final + (lr - lr_final)
 * (1 + cos(pi t / T)) / 2 (t = 1..T, T = all steps), and adds its loss / steps
 * per epoch to loss_per_epoch[epoch] (may be NULL). One step is captured as a
 * CUDA graph and replayed, so the host issues one launch per step. The
 * workspace (gal_mlp_train_workspace_size) starts with the error flag of
 * gal_mlp_workspace_error for `batch`; zero it before first use. */
GAL_API gal_status gal_mlp_train_workspace_size(int64_t batch, size_t* bytes);
GAL_API gal_status gal_mlp_train(float* params, float* adam_m, float* adam_v, const float* u, const float* phi_t,
                                 const float* g_t, const float* weights, int64_t n, int64_t batch, int32_t epochs,
                                 float alpha, float beta, float lr, float lr_final, float beta1, float beta2,
                                 float eps, uint64_t seed, int32_t quantize, float* loss_per_epoch, void* workspace,
                                 size_t workspace_bytes, gal_stream_t stream);
/* Build inference weights (bfloat16 operand images) from a host parameter vector. */
GAL_API gal_status gal_mlp_create(const float* params_host, double length_scale, double phi_scale, gal_mlp** out);
GAL_API gal_status gal_mlp_destroy(gal_mlp* mlp);
/* Tensor-core inference at n positions x[3][n] (physical units): grad[3][n]
 * (= or += grad_sign * grad Phi) and optionally phi[n]. */
GAL_API gal_status gal_mlp_eval(const gal_mlp* mlp, const double* x, int64_t n, double* grad, int32_t accumulate,
                                double grad_sign, double* phi, gal_stream_t stream);
/* Error code the inference kernel recorded (0 = none; non-zero = a bounded wait gave up). */
GAL_API gal_status gal_mlp_error(const gal_mlp* mlp, int32_t* code);

/* Short-range / long-range split of a set of Plummer spheres for the surrogate
 * (no counterpart in galax). Each sphere Phi_i = -G m_i / sqrt(d^2 + b_i^2)
 * (builtin/plummer.py:122-133, centred at its origin) is written as
 * Phi_i S(d / r_cut) + Phi_i (1 - S) with S(q) = (1 - q^2)^3 for q < 1, 0
 * beyond: the MLP learns the smooth remainder, the short-range part is summed
 * directly (FP64 offsets and accumulation, each term in FP32: ~1e-7 relative)
 * from per-cell neighbour lists built here (device memory allocated here,
 * freed by gal_split_destroy). comps must all be GAL_PLUMMER. */
typedef struct gal_split gal_split; /* opaque */
GAL_API gal_status gal_split_create(const gal_component* comps, int32_t n, double G, double r_cut, gal_split** out);
GAL_API gal_status gal_split_destroy(gal_split* split);
/* Short-range potential phi[n] and gradient grad[3][n] at x[3][n] (either output may be NULL). */
GAL_API gal_status gal_split_eval(const gal_split* split, const double* x, int64_t n, double* phi, double* grad,
                                  gal_stream_t stream);

/* Orbit integration with a surrogate: acceleration = -grad Phi_analytic (FP64,
 * `pot`) - grad Phi_short (FP64, `near`; NULL = none) - grad Phi_mlp (tensor
 * cores; NULL = none). Dopri5 with the constant step dt from t0 to t1 (the
 * last step clipped onto t1, as gal_integrate), advancing y[6][n] in place to
 * the final state. use_graph = 1 replays one captured CUDA graph per step.
 * Scratch from gal_surrogate_workspace_size (seven stage slopes and the stage
 * positions). */
GAL_API gal_status gal_surrogate_workspace_size(int64_t n, size_t* bytes);
GAL_API gal_status gal_integrate_surrogate(const gal_potential* pot, const gal_mlp* mlp, const gal_split* near,
                                           double dt, double t0, double t1, double* y, int64_t n, int32_t use_graph,
                                           void* workspace, size_t workspace_bytes, gal_stream_t stream);

/* ------------------------------------------------------------------ utilities */
/* Copy the library's Butcher tableau (c[13], a[13][13], b[13], e[13] = b - bhat);
 * returns the number of stages, or 0 for an unknown method. Host only. */
GAL_API int32_t gal_tableau(int32_t method, double* c, double* a, double* b, double* e);
/* FP64 FMA throughput probe: runs `iters` dependent-chain FMAs on every thread of
 * a full-device grid and writes the elapsed device time (ms) to *ms. Used to
 * measure the chip's FP64 peak for roofline reporting. */
GAL_API gal_status gal_fp64_peak_probe(int64_t iters, double* ms, double* flops, gal_stream_t stream);
GAL_API const char* gal_status_string(int32_t status);
GAL_API const char* gal_last_error(void);
GAL_API int32_t gal_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GALAX_GB300_H */
