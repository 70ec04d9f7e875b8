"""The CPU oracle against the reference's golden vectors and known-answer tests.

These pin the oracle before the CUDA library's tests trust it as their reference:
every potential / gradient / Hessian golden of the reference's unit tests, the
Dopri8 single-step doctest, the PID-controlled doctests, and self-consistency
(order conditions of both tableaux, finite differences of the Hessians, the
parameter derivatives and the discrete adjoint).
"""

from __future__ import annotations

import itertools

import numpy as np
import pytest

from oracle import oracle as O
from tests._helpers import golden_cfg, golden_comps, golden_save_ts


# ---------------------------------------------------------------- potentials
POTENTIAL_GOLDENS = ["hernquist", "miyamoto_nagai", "nfw", "plummer", "milky_way", "isochrone", "logarithmic",
                     "mn3_exponential", "mn3_sech2", "milky_way_2022", "powerlaw_cutoff", "bovy_mw_2014"]


@pytest.mark.parametrize("name", POTENTIAL_GOLDENS)
def test_potential_goldens(goldens, name):
    g = goldens["potentials"][name]
    c = golden_comps(g["params"])
    x = np.array([g["x"]])
    tol = g["tol"]
    np.testing.assert_allclose(O.potential(c, x)[0], g["potential"], **tol)
    np.testing.assert_allclose(O.gradient(c, x)[0], g["gradient"], **tol)
    np.testing.assert_allclose(O.hessian(c, x)[0].ravel(), g["hessian"], **tol)
    if not name.startswith(("milky_way", "bovy")):
        # single components match every printed digit (within one unit of the
        # last printed decimal: some goldens are truncated, e.g. the isochrone
        # potential -0.9231515 of -0.92315155), not just the reference's tolerance
        def half_ulp(v):
            digits = repr(float(v)).split("e")[0].split(".")[-1]
            return 10.0 ** -len(digits) + 1e-15

        np.testing.assert_allclose(O.potential(c, x)[0], g["potential"], rtol=0, atol=half_ulp(g["potential"]))
        for got, want in zip(O.gradient(c, x)[0], g["gradient"]):
            assert abs(got - want) <= half_ulp(want), (got, want)


@pytest.mark.parametrize("name", POTENTIAL_GOLDENS)
def test_density_and_tidal_tensor_goldens(goldens, name):
    """galax's density and tidal-tensor goldens follow from the oracle's Hessian:
    rho = tr(H) / (4 pi G) (Poisson) and T = H - tr(H) I / 3
    (register_funcs.py:347-378)."""
    g = goldens["potentials"][name]
    c = golden_comps(g["params"])
    H = O.hessian(c, np.array([g["x"]]))[0]
    tr = np.trace(H)
    np.testing.assert_allclose(tr / (4 * np.pi * O.G_GALACTIC), g["density"], rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose((H - np.eye(3) * tr / 3).ravel(), g["tidal_tensor"], rtol=1e-5, atol=1e-8)


def test_hamiltonian_field_doctest(goldens):
    """galax's HamiltonianField doctest: (dq/dt, dp/dt) = (p, -grad Phi) of a
    Kepler potential at 8 kpc, to every printed digit."""
    g = goldens["fields"]["hamiltonian_kepler"]
    c = golden_comps(g["potential"])
    acc = -O.gradient(c, np.array([g["x"]]))[0]
    half = 0.5 * 10.0 ** -g["decimals"]
    np.testing.assert_allclose(g["v"], g["dq_dt"], rtol=0, atol=half)
    np.testing.assert_allclose(acc, g["dp_dt"], rtol=0, atol=half)


def test_gradient_is_finite_at_origin():
    c = O.milky_way()
    g = O.gradient(c, np.zeros((1, 3)))
    assert np.all(np.isfinite(g)) and np.all(g == 0)


def _mixed_points(n=64, seed=5):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, 3)) * np.exp(rng.uniform(np.log(0.05), np.log(60), (n, 1)))


def _all_kinds():
    return O.comps([
        (O.KEPLER, 3e10, 0, 0, (0.3, -0.2, 0.1)),
        (O.HERNQUIST, 5e9, 1.0, 0),
        (O.MIYAMOTO_NAGAI, 6.8e10, 3.0, 0.28),
        (O.NFW, 5.4e11, 15.62, 0),
        (O.PLUMMER, 1e8, 0.5, 0, (4.0, 1.0, -2.0)),
        (O.ISOCHRONE, 2e10, 1.5, 0, (-1.0, 0.5, 0.2)),
        (O.LOGARITHMIC, 0.2, 2.0, 0),
        (O.POWERLAW_CUTOFF, 4.5e9, 1.9, 1.8, (0.5, -0.3, 0.2)),
    ])


def test_gradient_matches_finite_difference_of_potential():
    c = _all_kinds()
    x = _mixed_points()
    g = O.gradient(c, x)
    for k in range(3):
        h = 1e-6 * np.maximum(1.0, np.abs(x[:, k]))
        e = np.zeros(3); e[k] = 1
        fd = (O.potential(c, x + h[:, None] * e) - O.potential(c, x - h[:, None] * e)) / (2 * h)
        np.testing.assert_allclose(g[:, k], fd, rtol=1e-6, atol=1e-9)


def test_hessian_matches_finite_difference_of_gradient():
    c = _all_kinds()
    x = _mixed_points()
    H = O.hessian(c, x)
    for k in range(3):
        h = 1e-6 * np.maximum(1.0, np.abs(x[:, k]))
        e = np.zeros(3); e[k] = 1
        fd = (O.gradient(c, x + h[:, None] * e) - O.gradient(c, x - h[:, None] * e)) / (2 * h[:, None])
        np.testing.assert_allclose(H[:, :, k], fd, rtol=1e-5, atol=1e-10)
    np.testing.assert_allclose(H, np.swapaxes(H, 1, 2), rtol=1e-12, atol=1e-18)


def test_param_derivatives_match_finite_difference():
    c = _all_kinds()
    x = _mixed_points(32)
    v = np.random.default_rng(1).normal(size=x.shape)
    d = O.dgrad_dparams(c, x, v)
    for ci, field in itertools.product(range(len(c)), ("m", "l1", "l2")):
        if field == "l2" and c[ci]["kind"] not in (O.MIYAMOTO_NAGAI, O.POWERLAW_CUTOFF):
            continue
        if field == "l1" and c[ci]["kind"] == O.KEPLER:
            continue
        j = {"m": 0, "l1": 1, "l2": 2}[field]
        p0 = float(c[ci][field])
        h = 1e-5 * p0
        one = c[ci:ci + 1]  # difference the component alone (no cancellation against the others)
        cp, cm = one.copy(), one.copy()
        cp[0][field] = p0 + h
        cm[0][field] = p0 - h
        fd = ((O.gradient(cp, x) - O.gradient(cm, x)) / (2 * h) * v).sum(1)
        np.testing.assert_allclose(d[:, ci, j], fd, rtol=1e-6, atol=1e-6 * np.abs(fd).max())


# ---------------------------------------------------------------- tableaux
def _trees(n):
    if n == 1:
        return [()]
    out = set()

    def parts(m, mx):
        if m == 0:
            yield []
            return
        for p in range(min(m, mx), 0, -1):
            for rest in parts(m - p, p):
                yield [p] + rest

    for p in parts(n - 1, n - 1):
        for combo in itertools.product(*[_trees(k) for k in p]):
            out.add(tuple(sorted(combo)))
    return sorted(out)


def _size(t):
    return 1 + sum(_size(c) for c in t)


def _gamma(t):
    g = _size(t)
    for c in t:
        g *= _gamma(c)
    return g


def _phi(t, A):
    v = np.ones(A.shape[0], dtype=np.longdouble)
    for ch in t:
        v = v * (A @ _phi(ch, A))
    return v


@pytest.mark.parametrize("method,p,phat", [(5, 5, 4), (8, 8, 7)])
def test_tableau_order_conditions(method, p, phat):
    """Every rooted-tree condition up to the method's order holds for b, and up
    to the embedded order for b - e; the next order fails (so the count is exact)."""
    c, a, b, e = O.tableau(method)
    A = a.astype(np.longdouble)
    np.testing.assert_allclose(A.sum(1), c, atol=2e-15)
    for w, order in ((b, p), (b - e, phat)):
        w = w.astype(np.longdouble)
        worst = max(abs(float(w @ _phi(t, A) - 1 / np.longdouble(_gamma(t))))
                    for n in range(1, order + 1) for t in _trees(n))
        assert worst < 1e-14
        nxt = max(abs(float(w @ _phi(t, A) - 1 / np.longdouble(_gamma(t)))) for t in _trees(order + 1))
        assert nxt > 1e-7


def test_dopri5_midpoint_weights():
    """Shampine's midpoint weights are a 4th-order (or better) quadrature at 1/2."""
    c, a, b, e = O.tableau(5)
    w = O.dopri5_cmid()
    for k in range(4):
        assert abs(w @ c**k - 0.5 ** (k + 1) / (k + 1)) < 1e-15


# ---------------------------------------------------------------- integration KATs
EXACT = ["dopri8_single_step", "dopri8_pid_lockstep_run", "dopri8_pid_solve_220kms", "dopri8_pid_solve_array",
         "nfw_integrate_orbit", "legacy_integrator_1gyr"]


@pytest.mark.parametrize("name", EXACT)
def test_integration_kats_exact(goldens, name):
    """Doctest values reproduced to every printed digit (half a unit in the last
    place, plus 1e-9 of floating-point slack for the long PID runs)."""
    g = goldens["orbits"][name]
    c = golden_comps(g["potential"])
    cfg = golden_cfg(g["solver"])
    ts = golden_save_ts(g)
    saves, status, acc, rej = O.integrate(c, np.array(g["y0"], float), g["t0"], g["t1"], ts, cfg)
    assert np.all(status == 0)
    rows = g.get("rows", [-1])
    if cfg.lockstep:
        got = saves[-1]  # (n, 6)
    else:
        got = np.stack([saves[i][rows] for i in range(len(saves))]).reshape(-1, 6)
    want = np.concatenate([np.asarray(g["expect_q"]), np.asarray(g["expect_p"])], axis=-1).reshape(-1, 6)
    tol = 0.5 * 10.0 ** (-g["digits"]) + 1e-9
    np.testing.assert_allclose(got, want, rtol=0, atol=tol)


@pytest.mark.parametrize("name", ["kepler_integrate_field_array", "kepler_integrate_field_quantity"])
def test_kepler_integrate_field_within_ten_rtol(goldens, name):
    """integrate_field's Kepler doctest (PID 1e-7, dtmin 0.05).

    The final row is a step endpoint. With the initial-step rule that reproduces
    every Hernquist doctest digit, it agrees within 20 x rtol (the whole gap comes
    from the first step: starting at dt0 = dtmin reproduces all printed digits,
    so diffrax's first step here was <= dtmin). The t=10.1 Myr row lies inside a
    step, where diffrax's 7th-order Dopri8 interpolant carries ~3e-6 of its own
    error; the oracle's sub-step is checked against a converged solution."""
    g = goldens["orbits"][name]
    c = golden_comps(g["potential"])
    cfg = golden_cfg(g["solver"])
    ts = golden_save_ts(g)
    y0 = np.array(g["y0"], float)
    saves, status, acc, rej = O.integrate(c, y0, g["t0"], g["t1"], ts, cfg)
    got = saves[0][g["rows"]]
    want = np.concatenate([np.asarray(g["expect_q"]), np.asarray(g["expect_p"])], axis=-1)
    np.testing.assert_allclose(got[0], want[0], atol=1e-12)
    scale = np.abs(want[-1]).max()
    assert np.abs(got[-1] - want[-1]).max() <= 20 * 1e-7 * scale
    first_dtmin = golden_cfg(dict(g["solver"], dt0=0.05))
    s2, *_ = O.integrate(c, y0, g["t0"], g["t1"], ts, first_dtmin)
    np.testing.assert_allclose(s2[0][-1], want[-1], rtol=0, atol=0.5e-8 + 1e-9)
    # interpolated row: oracle within 1e-7 of the converged solution, reference within 5e-6
    fine, *_ = O.integrate(c, y0, g["t0"], ts[1], np.array([ts[1]]), O.solver_cfg(8, False, dt0=ts[1] / 2000))
    assert np.abs(got[1] - fine[0][0]).max() < 1e-7
    assert np.abs(want[1] - fine[0][0]).max() < 5e-6


def test_dopri8_substep_save_is_order_eight():
    """A save inside a step equals the Dopri8 step of the partial length: halving
    dt shrinks the save error ~2^8."""
    c = O.milky_way()
    y0 = np.array([[8.0, 0.5, 0.3, 0.02, 0.21, 0.01]])
    ts = np.array([37.3])
    ref, *_ = O.integrate(c, y0, 0.0, 40.0, ts, O.solver_cfg(8, False, dt0=0.05))
    errs = []
    for dt in (4.0, 2.0):
        s, *_ = O.integrate(c, y0, 0.0, 40.0, ts, O.solver_cfg(8, False, dt0=dt))
        errs.append(np.abs(s[0] - ref[0]).max())
    assert errs[1] < errs[0] / 100


def test_reverse_time_matches_forward():
    c = O.milky_way()
    y0 = np.array([[8.0, 0.5, 0.3, 0.02, 0.21, 0.01]])
    fwd, *_ = O.integrate(c, y0, 0.0, 200.0, np.array([200.0]), O.solver_cfg(8, False, dt0=0.5))
    back, *_ = O.integrate(c, fwd[0], 200.0, 0.0, np.array([0.0]), O.solver_cfg(8, False, dt0=0.5))
    np.testing.assert_allclose(back[0][0], y0[0], rtol=1e-10, atol=1e-12)


def test_max_steps_status():
    c = O.milky_way()
    y0 = np.array([[8.0, 0.0, 0.0, 0.0, 0.2, 0.0]])
    s, st, acc, rej = O.integrate(c, y0, 0.0, 100.0, np.array([50.0, 100.0]),
                                  O.solver_cfg(5, True, rtol=1e-8, atol=1e-10, max_steps=5))
    assert st[0] == 1 and acc[0] + rej[0] == 5
    assert np.all(np.isnan(s[0][-1]))


@pytest.mark.parametrize("t0, t1", [(0.0, np.inf), (0.0, -np.inf), (np.nan, 10.0)])
def test_non_finite_span_status(t0, t1):
    c = O.milky_way()
    y0 = np.array([[8.0, 0.0, 0.0, 0.0, 0.2, 0.0]])
    s, st, acc, rej = O.integrate(c, y0, t0, t1, np.array([0.0, 5.0]), O.solver_cfg(5, True, rtol=1e-8, atol=1e-10))
    assert st[0] == 3 and acc[0] + rej[0] == 0
    assert np.all(np.isnan(s[0]))


# ---------------------------------------------------------------- adjoint
def test_adjoint_matches_central_differences():
    c = O.milky_way()
    rng = np.random.default_rng(7)
    y0 = np.array([[8.0, 0.5, 0.3, 0.02, 0.21, 0.01], [12.0, -3.0, 1.0, 0.1, 0.15, -0.02]])
    cfg = O.solver_cfg(8, False, dt0=1.0)
    yT, *_ = O.integrate(c, y0, 0.0, 50.0, np.array([50.0]), cfg)
    target = np.stack([s[0] for s in yT]) + rng.normal(0, 0.1, (2, 6))
    yT2, gy, gp, L = O.adjoint_fixed(c, y0, 0.0, 50.0, target, cfg)

    def loss(cc, yy):
        s, *_ = O.integrate(cc, yy, 0.0, 50.0, np.array([50.0]), cfg)
        return float(sum(((s[i][0] - target[i]) ** 2).sum() for i in range(len(s))))

    assert abs(loss(c, y0) - L) < 1e-12 * max(1, L)
    for i, j in itertools.product(range(2), range(6)):
        h = 1e-6
        yp, ym = y0.copy(), y0.copy()
        yp[i, j] += h
        ym[i, j] -= h
        fd = (loss(c, yp) - loss(c, ym)) / (2 * h)
        assert abs(gy[i, j] - fd) <= 1e-5 * max(1.0, abs(fd))
    for ci in range(len(c)):
        for field, j in (("m", 0), ("l1", 1), ("l2", 2)):
            if field == "l2" and c[ci]["kind"] != O.MIYAMOTO_NAGAI:
                continue
            p0 = float(c[ci][field])
            h = 1e-6 * p0
            cp, cm = c.copy(), c.copy()
            cp[ci][field] = p0 + h
            cm[ci][field] = p0 - h
            fd = (loss(cp, y0) - loss(cm, y0)) / (2 * h)
            assert abs(gp[ci, j] - fd) <= 1e-5 * max(abs(fd), 1e-12 / p0), (ci, field, gp[ci, j], fd)


def test_adjoint_with_linear_parameters_matches_central_differences():
    """LinearParameter time dependence in the adjoint: d/d(value at t = 0) and
    d/d(slope) against central differences of the oracle's own integration, and
    zero slopes give the static adjoint bitwise."""
    c = O.milky_way()
    slopes = np.zeros((len(c), 3))
    slopes[0, 0] = -2e8    # disk mass (Msun / Myr)
    slopes[0, 1] = 1e-3    # disk a (kpc / Myr)
    slopes[1, 0] = 5e8     # halo mass
    slopes[1, 1] = -4e-3   # halo r_s
    y0 = np.array([[8.0, 0.5, 0.3, 0.02, 0.21, 0.01], [12.0, -3.0, 1.0, 0.1, 0.15, -0.02]])
    cfg = O.solver_cfg(8, False, dt0=1.0)
    t1 = 60.0
    yT, *_ = O.integrate(c, y0, 0.0, t1, np.array([t1]), cfg, slopes=slopes)
    target = np.stack([s[0] for s in yT]) + np.random.default_rng(8).normal(0, 0.1, (2, 6))
    _, gy, gp, L = O.adjoint_fixed(c, y0, 0.0, t1, target, cfg, slopes=slopes)
    assert gp.shape == (len(c), 6)

    def loss(cc, ss):
        s, *_ = O.integrate(cc, y0, 0.0, t1, np.array([t1]), cfg, slopes=ss)
        return float(sum(((s[i][0] - target[i]) ** 2).sum() for i in range(len(s))))

    assert abs(loss(c, slopes) - L) < 1e-12 * max(1, L)
    for ci, field, j in [(0, "m", 0), (0, "l1", 1), (0, "l2", 2), (1, "m", 0), (1, "l1", 1), (2, "m", 0)]:
        p0 = float(c[ci][field])
        h = 1e-6 * p0
        cp, cm = c.copy(), c.copy()
        cp[ci][field] = p0 + h
        cm[ci][field] = p0 - h
        fd = (loss(cp, slopes) - loss(cm, slopes)) / (2 * h)
        assert abs(gp[ci, j] - fd) <= 1e-5 * max(abs(fd), 1e-12 / p0), ("value", ci, field, gp[ci, j], fd)
        # the slope's scale: the value's, spread over the span
        hs = 1e-6 * p0 / t1
        sp, sm = slopes.copy(), slopes.copy()
        sp[ci, j] += hs
        sm[ci, j] -= hs
        fd = (loss(c, sp) - loss(c, sm)) / (2 * hs)
        assert abs(gp[ci, 3 + j] - fd) <= 1e-5 * max(abs(fd), 1e-12 * t1 / p0), ("slope", ci, field, gp[ci, 3 + j], fd)
    # static potential: the same values bitwise, slope derivatives = sum of t * d/dp(t)
    _, gy0, gp0, _ = O.adjoint_fixed(c, y0, 0.0, t1, target, cfg)
    _, gyz, gpz, _ = O.adjoint_fixed(c, y0, 0.0, t1, target, cfg, slopes=np.zeros_like(slopes))
    assert np.array_equal(gp0, gpz[:, :3]) and np.array_equal(gy0, gyz)
    assert np.all(np.isfinite(gpz[:, 3:]))


# ---------------------------------------------------------------- stream
def _stream_setup(n_release):
    from galax_gb300 import workloads as W

    c = O.milky_way()
    return c, W.stream_setup(lambda x: O.gradient(c, x), n_release=n_release)


def test_stream_release_map_is_the_king_tidal_radius():
    """Release conditions follow r_t = cbrt(G M / (Omega^2 - rhat.H.rhat))
    (galax dynamics/_src/cluster/radius.py:198-214) with Omega = |x x v|/r^2."""
    c, s = _stream_setup(40)
    out = O.stream_forward(c, s)
    P = out["track"][:-1]
    x, v = P[:, :3], P[:, 3:]
    r = np.linalg.norm(x, axis=1)
    rh = x / r[:, None]
    om = np.linalg.norm(np.cross(x, v), axis=1) / r**2
    H = O.hessian(c, x)
    prr = np.einsum("ni,nij,nj->n", rh, H, rh)
    rt = np.cbrt(O.G_GALACTIC * s.prog_m / (om**2 - prr))
    np.testing.assert_allclose(out["rt_om"][:, 0], rt, rtol=1e-13)
    np.testing.assert_allclose(out["rt_om"][:, 1], om, rtol=1e-13)
    nz = s.noise.reshape(-1, 2, 2, 3)  # release, side, (xi, eta), xyz
    for side, sgn in ((0, -1.0), (1, 1.0)):
        ics = out["ics"][side::2]
        np.testing.assert_allclose(ics[:, :3], x + sgn * rt[:, None] * rh + 0.1 * rt[:, None] * nz[:, side, 0],
                                   rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(ics[:, 3:], v + 0.1 * (om * rt)[:, None] * nz[:, side, 1], rtol=1e-13,
                                   atol=1e-15)


def test_stream_progenitor_track_round_trip():
    """The forwards track ends where the backwards integration started (Dopri8,
    dt = 1 Myr over 300 Myr: the round trip differs only by the method's
    truncation error, ~2e-9 kpc here)."""
    c, s = _stream_setup(300)
    tr = O.stream_forward(c, s)["track"]
    assert np.max(np.abs(tr[-1] - s.w_now) / np.maximum(np.abs(s.w_now), 1.0)) < 1e-8


def test_stream_particles_follow_the_coupled_system():
    """A particle released at the last grid point takes one step in the host
    potential plus the progenitor's Plummer sphere at the progenitor's stage
    positions; without the progenitor (mass -> 0) it is a plain orbit."""
    c, s = _stream_setup(5)
    s.prog_m = 1e-300  # negligible progenitor: particles move in the host alone
    out = O.stream_forward(c, s)
    for p in range(2 * s.n_release):
        r = p // 2
        nsteps = s.n_release - r
        y, st, _, _ = O.integrate(c, out["ics"][p:p + 1], 0.0, float(nsteps), np.array([float(nsteps)]),
                                  O.solver_cfg(8, False, dt0=1.0))
        np.testing.assert_allclose(out["final"][p], y[0][-1], rtol=1e-12, atol=1e-14)


def test_stream_finite_difference_gradient_converges():
    """The oracle's central differences (one Richardson step) agree across step
    sizes for the halo parameters, so they can check the GPU adjoint at 1e-6."""
    c, s = _stream_setup(100)
    target = O.stream_forward(c, s)["final"] + s.pert
    g1 = O.stream_fd_grad(c, s, target, [(1, "m"), (1, "l1")], rel_h=1e-4)
    g2 = O.stream_fd_grad(c, s, target, [(1, "m"), (1, "l1")], rel_h=1e-5)
    np.testing.assert_allclose(g1, g2, rtol=1e-6)


def test_king_tidal_radius_golden(goldens):
    """galax's tidal_radius doctest (King 1962): the oracle's release map gives
    the same r_t to the printed digits."""
    g = goldens["stream"]["king_tidal_radius"]
    c = golden_comps(g["potential"])
    w = np.array([g["x"] + g["v"]])
    _, _, rt = O.stream_df_sample(c, w, g["mass"], np.zeros((1, 4)))
    assert abs(rt[0] - g["r_tidal"]) <= 1e-8


def _fardal_reference(c, w, mass, nz, p=O.FARDAL2015_DEFAULTS):
    """Fardal 2015 written out as in galax (experimental/df.py:148-177,
    legacy/mockstream/df/fardal15.py:62-94), with numpy."""
    x, v = w[:, :3], w[:, 3:]
    r = np.linalg.norm(x, axis=1, keepdims=True)
    rh = x / r
    om = np.linalg.norm(np.cross(x, v), axis=1, keepdims=True) / r**2
    H = O.hessian(c, x)
    d2 = np.einsum("ni,nij,nj->n", rh, H, rh)[:, None]
    rt = np.cbrt(O.G_GALACTIC * mass / (om**2 - d2))
    vc = om * rt
    L = np.cross(x, v)
    zh = L / np.linalg.norm(L, axis=1, keepdims=True)
    ph = v - np.sum(v * rh, axis=1, keepdims=True) * rh
    ph = ph / np.linalg.norm(ph, axis=1, keepdims=True)
    kr = p[0] + nz[:, 0:1] * p[4]
    kvphi = kr * (p[1] + nz[:, 1:2] * p[5])
    kz = p[2] + nz[:, 2:3] * p[6]
    kvz = p[3] + nz[:, 3:4] * p[7]
    lead = np.concatenate([x - rt * (kr * rh - kz * zh), v - vc * (kvphi * ph - kvz * zh)], axis=1)
    trail = np.concatenate([x + rt * (kr * rh + kz * zh), v + vc * (kvphi * ph + kvz * zh)], axis=1)
    return lead, trail, rt[:, 0]


def test_fardal2015_sample_matches_the_written_out_formula():
    c = O.milky_way()
    rng = np.random.default_rng(3)
    x = rng.uniform(-30, 30, (50, 3))
    v = rng.normal(0, 0.2, (50, 3))
    w = np.concatenate([x, v], axis=1)
    nz = rng.normal(size=(50, 4))
    mass = rng.uniform(1e4, 1e6, 50)
    lead, trail, rt = O.stream_df_sample(c, w, mass, nz)
    el, et, ert = _fardal_reference(c, w, mass[:, None], nz)
    np.testing.assert_allclose(rt, ert, rtol=1e-12)
    np.testing.assert_allclose(lead, el, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(trail, et, rtol=1e-12, atol=1e-14)
    # other DF parameters
    p = (1.5, 0.2, 0.1, -0.1, 0.3, 0.4, 0.2, 0.1)
    lead, trail, _ = O.stream_df_sample(c, w, mass, nz, df_params=p)
    el, et, _ = _fardal_reference(c, w, mass[:, None], nz, p)
    np.testing.assert_allclose(lead, el, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(trail, et, rtol=1e-12, atol=1e-14)


def test_fardal2015_doctest_structure(goldens):
    """galax's Fardal2015DF.sample doctest draws from a jax key, so its numbers
    pin the arm geometry, not the draws: the arms are symmetric about the
    progenitor along rhat and phihat and shifted together along zhat. Taking
    the draws the printed values imply, the oracle reproduces every printed
    digit, and the implied draws are ordinary standard-normal values."""
    g = goldens["stream"]["fardal2015_sample"]
    c = golden_comps(g["potential"])
    x, v = np.array(g["x"]), np.array(g["v"])
    xl, vl, xt, vt = (np.array(g[k]) for k in ("x_lead", "v_lead", "x_trail", "v_trail"))
    w = np.concatenate([x, v])[None]
    _, _, rt = O.stream_df_sample(c, w, g["mass"], np.zeros((1, 4)))
    rt = rt[0]
    om = np.linalg.norm(np.cross(x, v)) / np.dot(x, x)
    rh, zh, ph = x / np.linalg.norm(x), np.array([0, 0, 1.0]), np.array([0, 1.0, 0])
    kr = np.dot((xt - xl) / 2, rh) / rt
    kz = np.dot((xt + xl) / 2 - x, zh) / rt
    kvphi = np.dot((vt - vl) / 2, ph) / (om * rt)
    kvz = np.dot((vt + vl) / 2 - v, zh) / (om * rt)
    p = O.FARDAL2015_DEFAULTS
    nz = np.array([[(kr - p[0]) / p[4], (kvphi / kr - p[1]) / p[5], (kz - p[2]) / p[6], (kvz - p[3]) / p[7]]])
    assert np.all(np.abs(nz) < 4.0), nz
    lead, trail, _ = O.stream_df_sample(c, w, g["mass"], nz)
    for got, want in ((lead[0, :3], xl), (lead[0, 3:], vl), (trail[0, :3], xt), (trail[0, 3:], vt)):
        np.testing.assert_allclose(got, want, rtol=2e-8, atol=1e-12)


def test_stream_forward_with_fardal_release():
    """The stream pipeline with Fardal release conditions: the ICs are the DF
    sample at the progenitor track's release points."""
    from galax_gb300 import workloads as W

    c = O.milky_way()
    s = W.stream_setup(lambda x: O.gradient(c, x), n_release=30, df=1)
    out = O.stream_forward(c, s)
    lead, trail, rt = O.stream_df_sample(c, out["track"][:-1], s.prog_m, s.noise)
    np.testing.assert_array_equal(out["ics"][0::2], lead)
    np.testing.assert_array_equal(out["ics"][1::2], trail)
    np.testing.assert_array_equal(out["rt_om"][:, 0], rt)


CHEN_MEAN = np.array([1.6, -30, 0, 1, 20, 0])
CHEN_COV = np.array([[0.1225, 0, 0, 0, -4.9, 0], [0, 529, 0, 0, 0, 0], [0, 0, 144, 0, 0, 0], [0, 0, 0, 0, 0, 0],
                     [-4.9, 0, 0, 0, 400, 0], [0, 0, 0, 0, 0, 484]])  # legacy/mockstream/df/chen24.py:21-32


def _chen_factor():
    A = np.diag([0.35, 23.0, 12.0, 0.0, 20.0 * np.sqrt(1 - 0.49), 22.0])
    A[4, 0] = -14.0
    return A


def test_chen_factor_reproduces_galax_covariance():
    np.testing.assert_allclose(_chen_factor() @ _chen_factor().T, CHEN_COV, rtol=1e-14, atol=1e-12)


def test_chen2024_sample_matches_the_written_out_formula():
    """Chen 2024 written out as in galax (legacy/mockstream/df/chen24.py:58-137),
    with posvel = mean + A z."""
    c = O.milky_way()
    rng = np.random.default_rng(8)
    n = 60
    x = rng.uniform(-30, 30, (n, 3))
    v = rng.normal(0, 0.2, (n, 3))
    w = np.concatenate([x, v], axis=1)
    z = rng.normal(size=(n, 6))
    mass = rng.uniform(1e4, 1e6, n)
    lead, trail, rt = O.stream_df_sample(c, w, mass, z, df=O.STREAM_DF_CHEN2024)
    _, _, ert = _fardal_reference(c, w, mass[:, None], np.zeros((n, 4)))
    np.testing.assert_allclose(rt, ert, rtol=1e-12)
    pv = CHEN_MEAN + z @ _chen_factor().T
    xh = x / np.linalg.norm(x, axis=1, keepdims=True)
    L = np.cross(x, v)
    zh = L / np.linalg.norm(L, axis=1, keepdims=True)
    yh = v - np.sum(v * xh, axis=1, keepdims=True) * xh
    yh = yh / np.linalg.norm(yh, axis=1, keepdims=True)
    Dr = pv[:, 0] * ert
    Dv = pv[:, 3] * np.sqrt(2 * O.G_GALACTIC * mass / Dr)
    ph, th, al, be = (np.deg2rad(pv[:, k]) for k in (1, 2, 4, 5))
    dx_in = (Dr * np.cos(th) * np.cos(ph))[:, None] * xh + (Dr * np.cos(th) * np.sin(ph))[:, None] * yh
    dx_z = (Dr * np.sin(th))[:, None] * zh
    dv_in = (Dv * np.cos(be) * np.cos(al))[:, None] * xh + (Dv * np.cos(be) * np.sin(al))[:, None] * yh
    dv_z = (Dv * np.sin(be))[:, None] * zh
    np.testing.assert_allclose(trail, np.concatenate([x + dx_in + dx_z, v + dv_in + dv_z], axis=1), rtol=1e-12,
                               atol=1e-14)
    np.testing.assert_allclose(lead, np.concatenate([x - dx_in + dx_z, v - dv_in + dv_z], axis=1), rtol=1e-12,
                               atol=1e-14)


def test_incomplete_gamma_matches_scipy():
    """The oracle's P(a, x), dP/da and Gamma(a, x) (power law with cutoff)
    against scipy's independent implementation (Cephes) over the range the
    potential uses (a = 3/2 - alpha/2 and 1 - alpha/2, 0 <= alpha < 2)."""
    sp = pytest.importorskip("scipy.special")
    for a in (0.05, 0.1, 0.35, 0.6, 1.0, 1.05, 1.5):
        for x in (1e-8, 1e-3, 0.3, 1.0, a + 0.999, a + 1.001, 2.5, 7.0, 30.0, 100.0, 700.0):
            P, dP, U = O.gamma_p(a, x)
            assert abs(P - sp.gammainc(a, x)) <= 2e-14 * sp.gammainc(a, x) + 1e-300, (a, x)
            Uref = sp.gammaincc(a, x) * sp.gamma(a)
            assert abs(U - Uref) <= 1e-13 * Uref + 1e-300, (a, x)
            h = 1e-6
            fd = (sp.gammainc(a + h, x) - sp.gammainc(a - h, x)) / (2 * h)
            assert abs(dP - fd) <= 1e-6 * abs(fd) + 1e-9, (a, x, dP, fd)  # FD resolves ~1e-10


def test_linear_parameter_doctest(goldens):
    """galax's LinearParameter doctest (params/core.py:52-74): a Kepler mass
    falling linearly to zero over 1 Gyr; the orbit's cylindrical radius at ten
    save times to the printed 3 decimals."""
    g = goldens["orbits"]["kepler_linear_mass"]
    c = golden_comps(g["potential"])
    saves, status, _, _ = O.integrate(c, np.array(g["y0"]), g["t0"], g["t1"], golden_save_ts(g),
                                      golden_cfg(g["solver"]), slopes=np.array(g["slopes"]))
    assert status[0] == 0
    rho = np.hypot(saves[0][:, 0], saves[0][:, 1])
    np.testing.assert_allclose(rho, g["expect_rho"], rtol=0, atol=0.5 * 10.0 ** -g["rho_decimals"] + 1e-9)


def test_linear_parameters_evaluate_at_time():
    """With slopes, every component is evaluated with p(t) = p(0) + slope t."""
    c = _all_kinds()
    rng = np.random.default_rng(4)
    sl = rng.normal(size=(len(c), 3)) * np.stack([np.abs(c["m"]) * 1e-4, np.full(len(c), 1e-4),
                                                   np.full(len(c), 1e-4)], axis=1)
    sl[c["kind"] == O.KEPLER, 1:] = 0.0
    sl[c["kind"] == O.POWERLAW_CUTOFF, 2] = 0.0
    x = _mixed_points(16)
    t = 37.5
    moved = c.copy()
    moved["m"] += sl[:, 0] * t
    moved["l1"] += sl[:, 1] * t
    moved["l2"] += sl[:, 2] * t
    np.testing.assert_array_equal(O.gradient(c, x, slopes=sl, t=t), O.gradient(moved, x))
    np.testing.assert_array_equal(O.potential(c, x, slopes=sl, t=t), O.potential(moved, x))
    np.testing.assert_array_equal(O.hessian(c, x, slopes=sl, t=t), O.hessian(moved, x))
