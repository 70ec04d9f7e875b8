"""Parity of the CUDA library with the CPU oracle (needs a GB300).

Every case runs the same seeded inputs through the C ABI (via the package's
ctypes front end) and through the oracle, and compares with the tolerances the
orbit path promises: 1e-9 relative in position and velocity for fixed steps,
10 x rtol for adaptive runs (per-orbit controllers on both sides, so most
orbits agree far tighter), rounding level for potential evaluation.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests._helpers import golden_cfg, golden_comps, golden_save_ts

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from galax_gb300.build import build

    build()
    import galax_gb300

    return galax_gb300


def _pot(gx, comps):
    from galax_gb300.potential import from_component_array

    return from_component_array(comps)


def _rel(a, b):
    """max over points of |a-b| / |b| per 3-vector block (position, velocity)."""
    a = np.asarray(a).reshape(-1, 6)
    b = np.asarray(b).reshape(-1, 6)
    out = 0.0
    for sl in (slice(0, 3), slice(3, 6)):
        d = np.linalg.norm(a[:, sl] - b[:, sl], axis=1)
        s = np.linalg.norm(b[:, sl], axis=1)
        out = max(out, float(np.max(d / np.maximum(s, 1e-300))))
    return out


def _rel_each(a, b):
    a = np.asarray(a).reshape(-1, 6)
    b = np.asarray(b).reshape(-1, 6)
    r = []
    for sl in (slice(0, 3), slice(3, 6)):
        r.append(np.linalg.norm(a[:, sl] - b[:, sl], axis=1) / np.maximum(np.linalg.norm(b[:, sl], axis=1), 1e-300))
    return np.maximum(*r)


def _mixed_points(n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, 3)) * np.exp(rng.uniform(np.log(0.02), np.log(150), (n, 1)))


def _kinds():
    return O.comps([
        (O.KEPLER, 3e10, 0, 0, (0.3, -0.2, 0.1)),
        (O.HERNQUIST, 5e9, 1.0, 0),
        (O.MIYAMOTO_NAGAI, 6.8e10, 3.0, 0.28),
        (O.NFW, 5.4e11, 15.62, 0),
        (O.PLUMMER, 1e8, 0.5, 0, (4.0, 1.0, -2.0)),
        (O.ISOCHRONE, 2e10, 1.5, 0, (-1.0, 0.5, 0.2)),
        (O.LOGARITHMIC, 0.2, 2.0, 0),
        (O.POWERLAW_CUTOFF, 4.5e9, 1.9, 1.8, (0.5, -0.3, 0.2)),
        (O.POWERLAW_CUTOFF, 2e9, 0.7, 0.4),
    ])


def _subhalos(n=512, seed=3):
    from galax_gb300 import workloads as W

    m, b, c = W.subhalo_table(seed, n)
    return np.concatenate([O.milky_way(), O.comps([(O.PLUMMER, m[i], b[i], 0, tuple(c[i])) for i in range(n)])])


# ------------------------------------------------------------------ evaluation
@pytest.mark.parametrize("which", ["kinds", "milky_way", "subhalos"])
def test_potential_gradient_hessian_match_oracle(gx, which):
    comps = {"kinds": _kinds, "milky_way": O.milky_way, "subhalos": _subhalos}[which]()
    pot = _pot(gx, comps)
    x = _mixed_points(4096, 11)
    phi_ref = O.potential(comps, x)  # (components of both signs cancel: absolute floor at the field's scale)
    np.testing.assert_allclose(pot.potential(x), phi_ref, rtol=1e-13, atol=1e-14 * np.abs(phi_ref).max())
    g_ref = O.gradient(comps, x)
    g = pot.gradient(x)
    scale = np.linalg.norm(g_ref, axis=1, keepdims=True)
    assert np.max(np.abs(g - g_ref) / scale) < 1e-13
    np.testing.assert_array_equal(pot.acceleration(x), -g)
    H_ref = O.hessian(comps, x)
    Hs = np.abs(H_ref).max(axis=(1, 2), keepdims=True)
    assert np.max(np.abs(pot.hessian(x) - H_ref) / Hs) < 1e-12


def test_reference_potential_goldens_on_gpu(gx, goldens):
    for name, g in goldens["potentials"].items():
        pot = _pot(gx, golden_comps(g["params"]))
        x = np.array([g["x"]])
        np.testing.assert_allclose(pot.potential(x)[0], g["potential"], **g["tol"])
        np.testing.assert_allclose(pot.gradient(x)[0], g["gradient"], **g["tol"])
        np.testing.assert_allclose(pot.hessian(x)[0].ravel(), g["hessian"], **g["tol"])
        np.testing.assert_allclose(pot.density(x)[0], g["density"], rtol=1e-5, atol=1e-8)
        np.testing.assert_allclose(pot.tidal_tensor(x)[0].ravel(), g["tidal_tensor"], rtol=1e-5, atol=1e-8)


def test_catalogue_classes_on_gpu(gx, goldens):
    """The front-end classes themselves (not the oracle's component tables)
    against galax's goldens."""
    cases = {
        "mn3_exponential": gx.MN3ExponentialPotential(m_tot=1e12, h_R=1.0, h_z=1.0),
        "mn3_sech2": gx.MN3Sech2Potential(m_tot=1e12, h_R=1.0, h_z=1.0),
        "milky_way_2022": gx.MilkyWayPotential2022(),
        "powerlaw_cutoff": gx.PowerLawCutoffPotential(m_tot=1e12, alpha=0.9, r_c=1.0),
        "bovy_mw_2014": gx.BovyMWPotential2014(),
    }
    for name, pot in cases.items():
        g = goldens["potentials"][name]
        x = np.array([g["x"]])
        np.testing.assert_allclose(pot.potential(x)[0], g["potential"], **g["tol"])
        np.testing.assert_allclose(pot.gradient(x)[0], g["gradient"], **g["tol"])
        np.testing.assert_allclose(pot.hessian(x)[0].ravel(), g["hessian"], **g["tol"])
        np.testing.assert_allclose(pot.density(x)[0], g["density"], rtol=1e-5, atol=1e-8)


def test_radial_derivatives_circular_velocity_and_enclosed_mass(gx):
    """dPhi/dr, d2Phi/dr2, v_circ and M(<r) (register_funcs.py:384-489) against
    the oracle's gradient and Hessian."""
    mw = gx.MilkyWayPotential()
    x = _mixed_points(2048, 21)
    g = O.gradient(O.milky_way(), x)
    H = O.hessian(O.milky_way(), x)
    r = np.linalg.norm(x, axis=1)
    rh = x / r[:, None]
    dr = np.sum(g * rh, axis=1)
    np.testing.assert_allclose(mw.dpotential_dr(x), dr, rtol=1e-12, atol=1e-18)
    np.testing.assert_allclose(mw.d2potential_dr2(x), np.einsum("ni,nij,nj->n", rh, H, rh), rtol=1e-10, atol=1e-16)
    np.testing.assert_allclose(mw.local_circular_velocity(x), np.sqrt(r * np.abs(dr)), rtol=1e-12)
    np.testing.assert_allclose(mw.spherical_mass_enclosed(x), r**2 * np.abs(dr) / O.G_GALACTIC, rtol=1e-12)


def test_milky_way_kernel_matches_general_table(gx):
    mw = gx.MilkyWayPotential()
    assert mw.is_milky_way_kernel()
    arr = O.milky_way()[[1, 0, 2, 3]]  # same components, order the specialised kernel does not take
    other = _pot(gx, arr)
    assert not other.is_milky_way_kernel()
    x = _mixed_points(8192, 12)
    g1, g2 = mw.gradient(x), other.gradient(x)
    assert np.max(np.abs(g1 - g2) / np.linalg.norm(g2, axis=1, keepdims=True)) < 1e-14


def test_gradient_at_origin_is_zero(gx):
    mw = gx.MilkyWayPotential()
    g = mw.gradient(np.zeros((3, 3)))
    assert np.all(g == 0)


def test_hamiltonian_field_doctest_on_gpu(gx, goldens):
    """The front end's HamiltonianField on galax's doctest point (Kepler 1e11 at
    8 kpc, 220 km/s): the printed field to every digit."""
    g = goldens["fields"]["hamiltonian_kepler"]
    field = gx.HamiltonianField(gx.KeplerPotential(m_tot=g["potential"]["m"]))
    w = np.concatenate([g["x"], g["v"]])
    f = np.asarray(field(0.0, w)).reshape(6)
    half = 0.5 * 10.0 ** -g["decimals"]
    np.testing.assert_allclose(f, np.concatenate([g["dq_dt"], g["dp_dt"]]), rtol=0, atol=half)


def test_batch_equals_rows_and_orbit_shapes(gx):
    """galax's AbstractPotential_Test (tests/unit/potential/test_base.py:120-131,
    177-201): a batch [[1,2,3],[4,5,6],[7,8,9]] evaluates to its rows evaluated
    one at a time (galax: atol 1e-15; here bitwise), and evaluate_orbit of one
    point with 100 saves over 1 Myr returns (100, 3) positions at those times."""
    xs = np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0], [7.0, 8.0, 9.0]])
    pots = [gx.MilkyWayPotential(), gx.HernquistPotential(m_tot=1e12, r_s=1.0),
            gx.MiyamotoNagaiPotential(m_tot=1e12, a=1.0, b=1.0), gx.NFWPotential(m=1e12, r_s=1.0),
            gx.PlummerPotential(m_tot=1e12, r_s=1.0)]
    for pot in pots:
        for fn in ("potential", "gradient", "hessian"):
            batch = getattr(pot, fn)(xs)
            for i in range(len(xs)):
                one = getattr(pot, fn)(xs[i])
                assert one.shape == batch[i].shape
                np.testing.assert_array_equal(one, batch[i])
    t = np.linspace(0.0, 1.0, 100)
    orb = gx.MilkyWayPotential().evaluate_orbit(np.array([8.0, 0.0, 0.0, 0.0, 0.2, 0.0]), t)
    assert orb.q.shape == (100, 3) and orb.p.shape == (100, 3)
    np.testing.assert_array_equal(orb.t, t)


# ------------------------------------------------------------------ fixed step
def _ics(n, seed):
    from galax_gb300 import workloads as W

    return W.disk_like_ics(lambda x: O.gradient(O.milky_way(), x), n, seed)


@pytest.mark.parametrize("method,dt", [(8, 1.0), (5, 0.5)])
def test_fixed_step_matches_oracle_within_1e9(gx, method, dt):
    """The small plain workload: MW, 1,024 orbits, 1 Gyr, 100 uniform saves."""
    y0 = _ics(1024, 0)
    ts = np.linspace(0.0, 1000.0, 100)
    integ = gx.Integrator(solver=gx.Dopri8() if method == 8 else gx.Dopri5(),
                          stepsize_controller=gx.ConstantStepSize(), dt0=dt)
    orb = gx.evaluate_orbit(gx.MilkyWayPotential(), y0, ts, integrator=integ)
    assert orb.q.shape == (1024, 100, 3)
    assert np.all(orb.steps == int(round(1000 / dt)))
    ref, st, acc, rej = O.integrate(O.milky_way(), y0, 0.0, 1000.0, ts, O.solver_cfg(method, False, dt0=dt))
    assert np.all(st == 0)
    got = orb.w.reshape(-1, 6)
    want = np.stack(ref).reshape(-1, 6)
    assert _rel(got, want) < 1e-9
    np.testing.assert_array_equal(orb.w[:, 0], y0)  # the first save is t0 itself


def test_fixed_step_general_table_matches_oracle(gx):
    comps = _kinds()
    y0 = _ics(256, 5)
    y0[:, :3] += 0.7  # keep clear of the Kepler point mass
    ts = np.linspace(0.0, 300.0, 37)
    integ = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=0.5)
    orb = gx.evaluate_orbit(_pot(gx, comps), y0, ts, integrator=integ)
    ref, st, *_ = O.integrate(comps, y0, 0.0, 300.0, ts, O.solver_cfg(8, False, dt0=0.5))
    assert _rel(orb.w.reshape(-1, 6), np.stack(ref).reshape(-1, 6)) < 1e-9


def _table_lanes(lanes):
    from galax_gb300 import _lib

    _lib.check(_lib.load().gal_set_table_lanes(lanes), "gal_set_table_lanes")


@pytest.mark.parametrize("method,adaptive", [(8, False), (5, True), (8, True)])
def test_warp_per_orbit_composite_matches_oracle(gx, method, adaptive):
    """One warp per orbit for a composite with many components (the Milky Way
    plus 512 Plummer subhalos): chosen automatically for a small batch, forced
    on and off; against the oracle, and the two modes against each other (they
    differ only in the order of the component sum)."""
    from galax_gb300.dynamics import integrate

    comps = _subhalos()
    pot = _pot(gx, comps)
    y0 = _ics(300, 23)
    ts = np.linspace(0.0, 200.0, 21)
    ctrl = gx.PIDController(rtol=1e-8, atol=1e-10) if adaptive else gx.ConstantStepSize()
    cfg = gx.Integrator(solver=gx.Dopri8() if method == 8 else gx.Dopri5(), stepsize_controller=ctrl,
                        dt0=None if adaptive else 0.5, max_steps=2**16).config()
    ocfg = (O.solver_cfg(method, True, rtol=1e-8, atol=1e-10, max_steps=2**16) if adaptive
            else O.solver_cfg(method, False, dt0=0.5))
    ref, rst, acc, _ = O.integrate(comps, y0, 0.0, 200.0, ts, ocfg)
    want = np.stack(ref).reshape(-1, 6)
    got = {}
    try:
        for lanes in (0, 32, 1):
            _table_lanes(lanes)
            out, st, steps = integrate(pot, y0, 0.0, 200.0, ts, cfg)
            assert np.all(st.cpu().numpy() == 0)
            got[lanes] = (out.permute(2, 1, 0).cpu().numpy().reshape(-1, 6), steps.cpu().numpy())
    finally:
        _table_lanes(0)
    np.testing.assert_array_equal(got[0][0], got[32][0])  # 300 orbits: the automatic choice is a warp each
    for lanes in (32, 1):
        rel = _rel_each(got[lanes][0], want)
        if adaptive:  # 516 components summed in another order than the oracle's: rounding-level medians
            assert rel.max() <= 10 * 1e-8 and np.median(rel) < 1e-10
            # rounding differences in the 516-term sums move some accept/reject decisions
            assert np.mean(got[lanes][1] == acc) > 0.9
        else:
            assert rel.max() < 1e-9
    assert _rel(got[32][0], got[1][0]) < (1e-7 if adaptive else 1e-11)


def test_warp_per_orbit_time_dependent_composite(gx):
    """The warp-per-orbit kernel with LinearParameter slopes, against the oracle."""
    from galax_gb300.dynamics import integrate
    from galax_gb300.potential import from_component_array

    comps = _subhalos(n=60, seed=8)
    sl = np.zeros((len(comps), 3))
    sl[0, 0] = -2e7
    sl[4:, 0] = -1e3 * comps["m"][4:] / 1e6  # subhalos losing mass
    y0 = _ics(128, 29)
    ts = np.linspace(0.0, 300.0, 16)
    cfg = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0).config()
    try:
        _table_lanes(32)
        out, st, _ = integrate(from_component_array(comps, slopes=sl), y0, 0.0, 300.0, ts, cfg)
    finally:
        _table_lanes(0)
    ref, rst, _, _ = O.integrate(comps, y0, 0.0, 300.0, ts, O.solver_cfg(8, False, dt0=1.0), slopes=sl)
    assert np.all(st.cpu().numpy() == 0)
    assert _rel(out.permute(2, 1, 0).cpu().numpy().reshape(-1, 6), np.stack(ref).reshape(-1, 6)) < 1e-9


# ------------------------------------------------------------------ adaptive
@pytest.mark.parametrize("method,rtol,atol", [(8, 1e-7, 1e-7), (5, 1e-8, 1e-10)])
def test_adaptive_matches_oracle(gx, method, rtol, atol):
    y0 = _ics(512, 7)
    ts = np.linspace(0.0, 500.0, 51)
    integ = gx.Integrator(solver=gx.Dopri8() if method == 8 else gx.Dopri5(),
                          stepsize_controller=gx.PIDController(rtol=rtol, atol=atol), max_steps=2**16)
    orb = gx.evaluate_orbit(gx.MilkyWayPotential(), y0, ts, integrator=integ)
    ref, st, acc, rej = O.integrate(O.milky_way(), y0, 0.0, 500.0, ts,
                                    O.solver_cfg(method, True, rtol=rtol, atol=atol, max_steps=2**16))
    assert np.all(st == 0)
    rel = _rel_each(orb.w.reshape(-1, 6), np.stack(ref).reshape(-1, 6))
    assert rel.max() <= 10 * rtol
    assert np.median(rel) < 1e-11  # identical step sequences: rounding-level agreement
    same_steps = np.mean(np.asarray(orb.steps) == acc)
    assert same_steps > 0.95


def test_uneven_batch_csr_matches_oracle(gx):
    """The batched uneven workload at reduced size: ragged save grids, per-orbit
    durations, Dopri5 PID rtol=1e-8 atol=1e-10, one persistent launch."""
    from galax_gb300 import workloads as W

    b = W.uneven_ics(lambda x: O.gradient(O.milky_way(), x), 384, seed=1, tmax=800.0, smax=200)
    integ = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                          max_steps=2**16)
    grids = [b.save_ts[b.save_offsets[i]:b.save_offsets[i + 1]] for i in range(len(b.t1))]
    res, status, steps = gx.integrate_orbit(gx.MilkyWayPotential(), b.y0, b.t0, b.t1, grids, integrator=integ,
                                            throw=False)
    ref, st, acc, rej = O.integrate(O.milky_way(), b.y0, b.t0, b.t1, grids,
                                    O.solver_cfg(5, True, rtol=1e-8, atol=1e-10, max_steps=2**16))
    st_gpu = status.cpu().numpy()
    np.testing.assert_array_equal(st_gpu, st)
    ok = st == 0
    rel = np.array([_rel_each(res[i].cpu().numpy(), ref[i]).max() if ok[i] else 0.0 for i in range(len(ok))])
    same = ok & (rel < 1e-10)
    # nearly every orbit takes the identical step sequence: rounding-level agreement
    assert same.sum() >= 0.95 * ok.sum()
    # a borderline accept/reject that rounds the other way changes the step
    # sequence; such an orbit must then agree within its own integration error
    diff = np.nonzero(ok & ~same)[0]
    if len(diff):
        fine, *_ = O.integrate(O.milky_way(), b.y0[diff], b.t0[diff], b.t1[diff], [grids[i] for i in diff],
                               O.solver_cfg(5, True, rtol=1e-11, atol=1e-13, max_steps=2**20))
        for k, i in enumerate(diff):
            err_ref = np.abs(ref[i] - fine[k]).max()
            assert np.abs(res[i].cpu().numpy() - ref[i]).max() <= 10 * max(err_ref, 1e-8 * np.abs(ref[i]).max())
    # orbits that ran out of steps report it and leave unreached saves NaN
    for i in np.nonzero(~ok)[0]:
        assert np.isnan(res[i].cpu().numpy()[-1]).all()


# ------------------------------------------------------------------ reference KATs on the GPU
@pytest.mark.parametrize("name", ["dopri8_single_step", "dopri8_pid_solve_220kms", "dopri8_pid_solve_array",
                                  "nfw_integrate_orbit", "legacy_integrator_1gyr"])
def test_reference_kats_on_gpu(gx, goldens, name):
    g = goldens["orbits"][name]
    comps = golden_comps(g["potential"])
    cfgd = dict(g["solver"])
    method = cfgd.pop("method")
    adaptive = cfgd.pop("adaptive")
    if adaptive:
        ctrl = gx.PIDController(rtol=cfgd["rtol"], atol=cfgd["atol"], dtmin=cfgd.get("dtmin"))
        integ = gx.Integrator(solver=gx.Dopri8() if method == 8 else gx.Dopri5(), stepsize_controller=ctrl)
    else:
        integ = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=cfgd["dt0"])
    ts = golden_save_ts(g)
    rows = g.get("rows", [-1])
    if "save_ts" in g:  # a single end time: evaluate_orbit starts from t[0], so prepend t0
        ts = np.concatenate([[g["t0"]], ts])
    orb = gx.evaluate_orbit(_pot(gx, comps), np.array(g["y0"], float), ts, integrator=integ)
    got = orb.w[:, rows].reshape(-1, 6)
    want = np.concatenate([np.asarray(g["expect_q"]), np.asarray(g["expect_p"])], axis=-1).reshape(-1, 6)
    np.testing.assert_allclose(got, want, rtol=0, atol=0.5 * 10.0 ** (-g["digits"]) + 1e-9)


# ------------------------------------------------------------------ semantics and edge cases
def test_reverse_time_round_trip(gx):
    y0 = _ics(128, 9)
    integ = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=0.5)
    mw = gx.MilkyWayPotential()
    fwd = gx.evaluate_orbit(mw, y0, np.array([0.0, 200.0]), integrator=integ).w[:, -1]
    back = gx.evaluate_orbit(mw, fwd, np.array([200.0, 0.0]), integrator=integ).w[:, -1]
    assert _rel(back, y0) < 1e-8  # Dopri8 truncation error over 2 x 200 Myr
    ref, *_ = O.integrate(O.milky_way(), fwd, 200.0, 0.0, np.array([0.0]), O.solver_cfg(8, False, dt0=0.5))
    assert _rel(back, np.stack(ref).reshape(-1, 6)) < 1e-12


def test_two_phase_evaluate_orbit(gx):
    """w0 carrying its own time is first moved to t[0] (galax legacy/funcs.py:186-213)."""
    y0 = _ics(64, 13)
    tw = np.linspace(-150.0, -50.0, 64)
    ts = np.linspace(0.0, 300.0, 31)
    integ = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-8))
    w0 = gx.PhaseSpaceCoordinate(q=y0[:, :3], p=y0[:, 3:], t=tw)
    orb = gx.evaluate_orbit(gx.MilkyWayPotential(), w0, ts, integrator=integ)
    cfg = O.solver_cfg(8, True, rtol=1e-8, atol=1e-8)
    mid, *_ = O.integrate(O.milky_way(), y0, tw, 0.0, np.array([0.0]), cfg)
    ref, *_ = O.integrate(O.milky_way(), np.stack(mid).reshape(-1, 6), 0.0, 300.0, ts, cfg)
    assert _rel_each(orb.w.reshape(-1, 6), np.stack(ref).reshape(-1, 6)).max() < 1e-7


def test_edge_cases(gx):
    import torch

    mw = gx.MilkyWayPotential()
    y0 = _ics(8, 21)
    # t0 == t1: every save is the initial state
    integ = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0)
    orb = gx.evaluate_orbit(mw, y0, np.array([5.0, 5.0]), integrator=integ)
    np.testing.assert_array_equal(orb.w[:, 1], y0)
    # max_steps: status, unreached saves NaN, no exception with throw=False
    integ = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                          max_steps=5)
    orb = gx.evaluate_orbit(mw, y0, np.linspace(0, 500, 5), integrator=integ, throw=False)
    assert np.all(orb.status == 1) and np.all(np.isnan(orb.w[:, -1]))
    with pytest.raises(gx.GalaxGB300Error, match="max_steps_reached"):
        gx.evaluate_orbit(mw, y0, np.linspace(0, 500, 5), integrator=integ)
    # a non-finite start stops with status 3
    bad = y0.copy()
    bad[3, 0] = np.nan
    integ = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0)
    orb = gx.evaluate_orbit(mw, bad, np.linspace(0, 50, 3), integrator=integ, throw=False)
    assert orb.status[3] == 3 and np.all(orb.status[[0, 1, 2, 4, 5, 6, 7]] == 0)
    # empty batch
    from galax_gb300.dynamics import integrate

    out, st, steps = integrate(mw, np.zeros((0, 6)), 0.0, 1.0, np.array([1.0]),
                               gx.Integrator(stepsize_controller=gx.ConstantStepSize(), dt0=0.5).config())
    assert out.shape == (6, 1, 0)
    torch.cuda.synchronize()


def test_launch_shapes_give_identical_results(gx):
    """The work queue makes results independent of block size and grid."""
    from galax_gb300 import _lib
    from galax_gb300.dynamics import integrate

    L = _lib.load()
    mw = gx.MilkyWayPotential()
    y0 = _ics(3000, 23)
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10)).config()
    outs = []
    for block, per_sm, variant in ((128, 0, 0), (64, 1, 1), (256, 2, 2), (32, 3, 1), (128, 0, 2)):
        _lib.check(L.gal_set_launch(5, 1, block, per_sm, variant), "gal_set_launch")
        out, st, steps = integrate(mw, y0, 0.0, 300.0, np.linspace(0, 300, 11), cfg)
        outs.append(out.cpu().numpy())
    _lib.check(L.gal_set_launch(5, 1, 0, 0, 0), "gal_set_launch")
    for o in outs[1:]:
        np.testing.assert_array_equal(o, outs[0])


# ------------------------------------------------------------------ adjoint
@pytest.mark.parametrize("which", ["milky_way", "table", "isochrone_logarithmic", "powerlaw_cutoff"])
def test_adjoint_matches_oracle(gx, which):
    import torch

    from galax_gb300.adjoint import orbit_adjoint

    extra = {"milky_way": [], "table": [(O.PLUMMER, 1e9, 0.8, 0, (6.0, 2.0, 0.5))],
             "isochrone_logarithmic": [(O.ISOCHRONE, 3e10, 1.2, 0, (1.0, -0.5, 0.3)), (O.LOGARITHMIC, 0.05, 4.0, 0)],
             "powerlaw_cutoff": [(O.POWERLAW_CUTOFF, 4.5e9, 1.9, 1.8, (0.3, 0.2, -0.1))]}
    comps = np.concatenate([O.milky_way(), O.comps(extra[which])]) if extra[which] else O.milky_way()
    pot = _pot(gx, comps)
    y0 = _ics(96, 31)
    rng = np.random.default_rng(20)
    cfg = O.solver_cfg(8, False, dt0=1.0)
    yT_ref, *_ = O.integrate(comps, y0, 0.0, 150.0, np.array([150.0]), cfg)
    target = np.stack(yT_ref).reshape(-1, 6) + np.concatenate(
        [rng.normal(0, 0.1, (96, 3)), rng.normal(0, 2 * 0.001022712165045695, (96, 3))], axis=1)
    yT_o, gy_o, gp_o, L_o = O.adjoint_fixed(comps, y0, 0.0, 150.0, target, cfg)
    res = orbit_adjoint(pot, y0, 0.0, 150.0, dt=1.0, target=target, method=8, k_ckpt=16)
    torch.cuda.synchronize()
    assert _rel(res.yT, yT_o) < 1e-12
    np.testing.assert_allclose(res.grad_y0, gy_o, rtol=1e-8, atol=1e-12 * np.abs(gy_o).max())
    mask = gp_o != 0
    np.testing.assert_allclose(res.grad_params[mask], gp_o[mask], rtol=1e-8)
    assert abs(res.loss - L_o) <= 1e-10 * L_o


@pytest.mark.parametrize("method", [8, 5])
def test_adjoint_matches_oracle_at_the_differentiation_shape(gx, method):
    """The differentiation workload's shape: dt = 0.5 Myr, checkpoints every 256
    steps, 1,200 steps (four full segments and a partial fifth), Milky Way, the
    workload's initial conditions; both tableaux."""
    import torch

    from galax_gb300 import workloads as W
    from galax_gb300.adjoint import orbit_adjoint

    comps = O.milky_way()
    n, dt, t1 = 128, 0.5, 600.0
    y0 = W.disk_like_ics(lambda x: O.gradient(comps, x), n, seed=2)
    cfg = O.solver_cfg(method, False, dt0=dt)
    yT_ref, *_ = O.integrate(comps, y0, 0.0, t1, np.array([t1]), cfg)
    rng = np.random.default_rng(20)
    target = np.stack(yT_ref).reshape(-1, 6) + np.concatenate(
        [rng.normal(0, 0.1, (n, 3)), rng.normal(0, 2 * 0.001022712165045695, (n, 3))], axis=1)
    yT_o, gy_o, gp_o, L_o = O.adjoint_fixed(comps, y0, 0.0, t1, target, cfg)
    res = orbit_adjoint(gx.MilkyWayPotential(), y0, 0.0, t1, dt=dt, target=target, method=method, k_ckpt=256)
    torch.cuda.synchronize()
    assert _rel(res.yT, yT_o) < 1e-9
    np.testing.assert_allclose(res.grad_y0, gy_o, rtol=1e-7, atol=1e-10 * np.abs(gy_o).max())
    mask = gp_o != 0
    np.testing.assert_allclose(res.grad_params[mask], gp_o[mask], rtol=1e-7)
    assert abs(res.loss - L_o) <= 1e-9 * L_o
    # the checkpoint interval changes only where the forward states come from
    res16 = orbit_adjoint(gx.MilkyWayPotential(), y0, 0.0, t1, dt=dt, target=target, method=method, k_ckpt=16)
    np.testing.assert_array_equal(res16.grad_y0, res.grad_y0)
    np.testing.assert_array_equal(res16.grad_params, res.grad_params)


def test_orbit_map_backward_matches_oracle_adjoint(gx):
    """The torch.autograd.Function: loss.backward() through OrbitMap gives the
    oracle's discrete-adjoint gradients with respect to the initial conditions
    and the (m, l1, l2) of every component."""
    import torch

    from galax_gb300 import workloads as W
    from galax_gb300.adjoint import OrbitMap, params_of

    comps = O.milky_way()
    n, dt, t1 = 64, 0.5, 300.0
    y0h = W.disk_like_ics(lambda x: O.gradient(comps, x), n, seed=5)
    cfg = O.solver_cfg(8, False, dt0=dt)
    yT_ref, *_ = O.integrate(comps, y0h, 0.0, t1, np.array([t1]), cfg)
    rng = np.random.default_rng(6)
    target = np.stack(yT_ref).reshape(-1, 6) + rng.normal(0, 0.05, (n, 6))
    _, gy_o, gp_o, L_o = O.adjoint_fixed(comps, y0h, 0.0, t1, target, cfg)

    mw = gx.MilkyWayPotential()
    y0 = torch.tensor(y0h, dtype=torch.float64, device="cuda", requires_grad=True)
    params = params_of(mw).requires_grad_()
    yT = OrbitMap.apply(mw, y0, params, 0.0, t1, dt, 8, 64)
    loss = ((yT - torch.as_tensor(target, device="cuda")) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    assert abs(float(loss) - L_o) <= 1e-9 * L_o
    np.testing.assert_allclose(y0.grad.cpu().numpy(), gy_o, rtol=1e-8, atol=1e-12 * np.abs(gy_o).max())
    gp = params.grad.cpu().numpy()
    mask = gp_o != 0
    np.testing.assert_allclose(gp[mask], gp_o[mask], rtol=1e-8)
    np.testing.assert_array_equal(gp[~mask], 0.0)


@pytest.mark.parametrize("method", [5, 8])
def test_two_pass_schedule_is_bitwise_identical(gx, method):
    """Longest-remaining-first rescheduling parks and resumes orbits from their
    exact state, so every save and step count is unchanged."""
    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import integrate

    b = W.uneven_ics(lambda x: O.gradient(O.milky_way(), x), 2000, seed=4, tmax=600.0, smax=60)
    mw = gx.MilkyWayPotential()
    res = []
    for sched in (False, True):
        cfg = gx.Integrator(solver=gx.Dopri8() if method == 8 else gx.Dopri5(),
                            stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10), max_steps=2**16,
                            schedule=sched).config()
        out, st, steps = integrate(mw, b.y0, b.t0, b.t1, b.save_ts, cfg, save_offsets=b.save_offsets)
        res.append((out.cpu().numpy(), st.cpu().numpy(), steps.cpu().numpy()))
    np.testing.assert_array_equal(res[0][1], res[1][1])
    np.testing.assert_array_equal(res[0][2], res[1][2])
    np.testing.assert_array_equal(res[0][0], res[1][0])


# ------------------------------------------------------------------ time-dependent (linear) parameters
def test_linear_parameter_doctest_on_gpu(gx, goldens):
    """galax's LinearParameter doctest (params/core.py:52-74) through the front
    end: KeplerPotential(m_tot=LinearParameter(...)) and compute_orbit's
    default solver, radii to the printed 3 decimals."""
    g = goldens["orbits"]["kepler_linear_mass"]
    lp = gx.LinearParameter(slope=g["slopes"][0][0], point_time=0.0, point_value=g["potential"]["m"])
    pot = gx.KeplerPotential(m_tot=lp)
    y0 = np.array(g["y0"][0])
    w0 = gx.PhaseSpaceCoordinate(q=y0[:3], p=y0[3:], t=g["t0"])
    for orb in (gx.compute_orbit(pot, w0, golden_save_ts(g)),  # the doctest's own call
                gx.evaluate_orbit(pot, y0, golden_save_ts(g), integrator=gx.OrbitSolver())):
        rho = np.hypot(orb.q[:, 0], orb.q[:, 1])
        np.testing.assert_allclose(rho, g["expect_rho"], rtol=0, atol=0.5 * 10.0 ** -g["rho_decimals"] + 1e-9)
    assert not pot.is_milky_way_kernel()
    # the Hamiltonian field at t = 500 Myr sees half the mass
    f = gx.HamiltonianField(pot)(500.0, np.array([[5.0, 0, 0, 0, 0.2, 0]]))
    np.testing.assert_allclose(f[0, 3], -O.G_GALACTIC * 5e11 / 25.0, rtol=1e-14)


def _timed_kinds(seed=4):
    c = _kinds()
    rng = np.random.default_rng(seed)
    sl = rng.normal(size=(len(c), 3)) * np.stack([np.abs(c["m"]) * 1e-4, np.full(len(c), 1e-4),
                                                   np.full(len(c), 1e-4)], axis=1)
    sl[c["kind"] == O.KEPLER, 1:] = 0.0
    sl[~np.isin(c["kind"], (O.MIYAMOTO_NAGAI, O.POWERLAW_CUTOFF)), 2] = 0.0  # l2 is no parameter there
    return c, sl


def test_linear_parameters_evaluate_at_time(gx):
    from galax_gb300.potential import from_component_array

    c, sl = _timed_kinds()
    pot = from_component_array(c, slopes=sl)
    np.testing.assert_array_equal(pot.slopes(), sl)
    x = _mixed_points(2048, 12)
    for t in (0.0, 37.5, -120.0):
        np.testing.assert_allclose(pot.potential(x, t), O.potential(c, x, slopes=sl, t=t), rtol=1e-13,
                                   atol=1e-14 * np.abs(O.potential(c, x, slopes=sl, t=t)).max())
        g_ref = O.gradient(c, x, slopes=sl, t=t)
        assert np.max(np.abs(pot.gradient(x, t) - g_ref) / np.linalg.norm(g_ref, axis=1, keepdims=True)) < 1e-13
        H_ref = O.hessian(c, x, slopes=sl, t=t)
        assert np.max(np.abs(pot.hessian(x, t) - H_ref) / np.abs(H_ref).max(axis=(1, 2), keepdims=True)) < 1e-12


@pytest.mark.parametrize("method", [8, 5])
def test_linear_parameters_integrate_like_oracle(gx, method):
    """Adaptive integration with time-dependent parameters, forwards and
    backwards in time, with saves, against the oracle evaluating every stage at
    its own time."""
    from galax_gb300.dynamics import integrate

    c = O.milky_way()
    sl = np.zeros((len(c), 3))
    sl[0, 0] = -2e7   # disk mass falling 2e7 Msun / Myr
    sl[1, 1] = 5e-3   # halo scale radius growing 5 pc / Myr
    y0 = _ics(256, 17)
    ts = np.linspace(0.0, 400.0, 21)
    ocfg = O.solver_cfg(method, True, rtol=1e-9, atol=1e-9)
    cfg = gx.Integrator(solver=gx.Dopri8() if method == 8 else gx.Dopri5(),
                        stepsize_controller=gx.PIDController(rtol=1e-9, atol=1e-9)).config()
    from galax_gb300.potential import from_component_array

    pot = from_component_array(c, slopes=sl)
    for t0, t1, grid in ((0.0, 400.0, ts), (400.0, 0.0, ts[::-1].copy())):
        out, st, _ = integrate(pot, y0, t0, t1, grid, cfg)
        ref, rst, _, _ = O.integrate(c, y0, t0, t1, grid, ocfg, slopes=sl)
        assert np.all(st.cpu().numpy() == 0) and np.all(rst == 0)
        got = out.permute(2, 1, 0).cpu().numpy()  # (n, T, 6)
        assert _rel(got.reshape(-1, 6), np.stack(ref).reshape(-1, 6)) < 1e-8
    # the slopes matter: the same table held static gives different orbits
    static = integrate(from_component_array(c), y0, 0.0, 400.0, ts, cfg)[0].cpu().numpy()
    assert not np.allclose(static, integrate(pot, y0, 0.0, 400.0, ts, cfg)[0].cpu().numpy())


def test_time_dependent_potentials_are_refused_where_unsupported(gx):
    from galax_gb300 import surrogate as S
    from galax_gb300._lib import GalaxGB300Error

    pot = gx.KeplerPotential(m_tot=gx.LinearParameter(slope=-1e8, point_time=0.0, point_value=1e11))
    y0 = _ics(4, 1)
    with pytest.raises(GalaxGB300Error):
        S.integrate(pot, None, y0, 0.0, 10.0, 1.0)


def _linear_mw():
    c = O.milky_way()
    slopes = np.zeros((len(c), 3))
    slopes[0, 0] = -2e8    # disk mass (Msun / Myr)
    slopes[0, 1] = 1e-3    # disk a (kpc / Myr)
    slopes[1, 0] = 5e8     # halo mass
    slopes[1, 1] = -4e-3   # halo r_s
    return c, slopes


@pytest.mark.parametrize("method", [8, 5])
def test_adjoint_with_linear_parameters_matches_oracle(gx, method):
    """The GPU adjoint through LinearParameter time dependence (every stage at
    its own time) against the oracle's, which central differences pin:
    d/d(values at t = 0) and d/d(slopes) of every component."""
    import torch

    from galax_gb300.adjoint import orbit_adjoint
    from galax_gb300.potential import from_component_array

    c, slopes = _linear_mw()
    n, dt, t1 = 64, 0.5, 300.0
    y0 = _ics(n, 41)
    cfg = O.solver_cfg(method, False, dt0=dt)
    yT_ref, *_ = O.integrate(c, y0, 0.0, t1, np.array([t1]), cfg, slopes=slopes)
    target = np.stack(yT_ref).reshape(-1, 6) + np.random.default_rng(42).normal(0, 0.05, (n, 6))
    yT_o, gy_o, gp_o, L_o = O.adjoint_fixed(c, y0, 0.0, t1, target, cfg, slopes=slopes)
    assert gp_o.shape == (len(c), 6)
    res = orbit_adjoint(from_component_array(c, slopes=slopes), y0, 0.0, t1, dt=dt, target=target,
                        method=method, k_ckpt=64)
    torch.cuda.synchronize()
    assert res.grad_params.shape == (len(c), 6)
    assert _rel(res.yT, yT_o) < 1e-9
    np.testing.assert_allclose(res.grad_y0, gy_o, rtol=1e-7, atol=1e-10 * np.abs(gy_o).max())
    mask = gp_o != 0
    np.testing.assert_allclose(res.grad_params[mask], gp_o[mask], rtol=1e-7)
    assert abs(res.loss - L_o) <= 1e-9 * L_o


@pytest.mark.parametrize("zero_slopes", [False, True])
def test_orbit_map_through_linear_parameters(gx, zero_slopes):
    """OrbitMap with (ncomp, 6) parameters: values at t = 0 and slopes; with
    every slope zero the potential stays time-dependent, so the slope
    derivatives are still returned (and equal the oracle's at zero slope)."""
    import torch

    from galax_gb300.adjoint import OrbitMap, params_of
    from galax_gb300.potential import from_component_array

    c, slopes = _linear_mw()
    if zero_slopes:
        slopes = np.zeros_like(slopes)
    n, dt, t1 = 32, 1.0, 200.0
    y0h = _ics(n, 43)
    cfg = O.solver_cfg(8, False, dt0=dt)
    yT_ref, *_ = O.integrate(c, y0h, 0.0, t1, np.array([t1]), cfg, slopes=slopes)
    target = np.stack(yT_ref).reshape(-1, 6) + np.random.default_rng(44).normal(0, 0.05, (n, 6))
    _, gy_o, gp_o, L_o = O.adjoint_fixed(c, y0h, 0.0, t1, target, cfg, slopes=slopes)
    base = from_component_array(c)
    params = torch.tensor(np.concatenate([np.stack([c["m"], c["l1"], c["l2"]], 1), slopes], 1),
                          dtype=torch.float64, device="cuda", requires_grad=True)
    if not zero_slopes:
        np.testing.assert_array_equal(params_of(from_component_array(c, slopes=slopes)).cpu().numpy(),
                                      params.detach().cpu().numpy())
    y0 = torch.tensor(y0h, dtype=torch.float64, device="cuda", requires_grad=True)
    yT = OrbitMap.apply(base, y0, params, 0.0, t1, dt, 8, 50)
    loss = ((yT - torch.as_tensor(target, device="cuda")) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    assert abs(float(loss) - L_o) <= 1e-9 * L_o
    np.testing.assert_allclose(y0.grad.cpu().numpy(), gy_o, rtol=1e-8, atol=1e-12 * np.abs(gy_o).max())
    gp = params.grad.cpu().numpy()
    mask = gp_o != 0
    np.testing.assert_allclose(gp[mask], gp_o[mask], rtol=1e-8)
    assert np.count_nonzero(gp[:, 3:]) > 0  # slope derivatives, also at zero slope


# ------------------------------------------------------------------ four-warp teams for the longest orbits
def _set_team(blocks):
    from galax_gb300 import _lib

    _lib.check(_lib.load().gal_set_team(int(blocks)), "gal_set_team")


@pytest.mark.parametrize("method", [5, 8])
@pytest.mark.parametrize("case", ["csr_forward", "shared_grid_backward", "few_orbits", "max_steps",
                                  "constant_step_scheduled"])
def test_team_kernel_is_bitwise_identical(gx, case, method):
    """The second pass with the longest orbits on four-warp teams gives the
    same saves, statuses and step counts, bit for bit, as the one-thread
    kernel alone; Dopri5 (FSAL, quartic saves) and Dopri8 (a slope round after
    every accepted step, saves by partial sub-steps)."""
    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import integrate

    mw = gx.MilkyWayPotential()
    n = {"csr_forward": 12000, "shared_grid_backward": 6000, "few_orbits": 300, "max_steps": 3000,
         "constant_step_scheduled": 4000}[case]
    if method == 8:
        n //= 2
    b = W.uneven_ics(lambda x: O.gradient(O.milky_way(), x), n, seed=8, tmax=1500.0, smax=40)
    max_steps = 2000 if case == "max_steps" else 2**16
    solver = gx.Dopri5() if method == 5 else gx.Dopri8()
    if case == "constant_step_scheduled":
        cfg = gx.Integrator(solver=solver, stepsize_controller=gx.ConstantStepSize(), dt0=0.7,
                            schedule=True).config()
    else:
        cfg = gx.Integrator(solver=solver, stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                            max_steps=max_steps).config()
    res = []
    try:
        for team in (0, 8, 100):
            _set_team(team)
            if case == "shared_grid_backward":
                ts = np.linspace(0.0, -400.0, 17)
                out, st, steps = integrate(mw, b.y0, 0.0, -400.0, ts, cfg)
            else:
                out, st, steps = integrate(mw, b.y0, b.t0, b.t1, b.save_ts, cfg, save_offsets=b.save_offsets)
            res.append((out.cpu().numpy(), st.cpu().numpy(), steps.cpu().numpy()))
    finally:
        _set_team(32)
    for other in res[1:]:
        np.testing.assert_array_equal(res[0][1], other[1])
        np.testing.assert_array_equal(res[0][2], other[2])
        np.testing.assert_array_equal(res[0][0], other[0])
    if case == "max_steps":
        assert (res[1][1] == 1).any()  # some orbits ran out of steps, on the team path too


def test_results_written_straight_into_pinned_host_memory(gx):
    """``out``/``status`` may be pinned host tensors: the kernels write them
    directly (device-visible host memory), with the same bits as device outputs."""
    import torch

    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import integrate

    mw = gx.MilkyWayPotential()
    b = W.uneven_ics(lambda x: O.gradient(O.milky_way(), x), 3000, seed=12, tmax=800.0, smax=30)
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10)).config()
    out_d, st_d, steps_d = integrate(mw, b.y0, b.t0, b.t1, b.save_ts, cfg, save_offsets=b.save_offsets)
    h_out = torch.empty(tuple(out_d.shape), dtype=torch.float64).pin_memory()
    h_st = torch.empty(tuple(st_d.shape), dtype=torch.int32).pin_memory()
    o, s, steps = integrate(mw, b.y0, b.t0, b.t1, b.save_ts, cfg, save_offsets=b.save_offsets, out=h_out,
                            status=h_st)
    torch.cuda.synchronize()
    assert o is h_out and s is h_st
    np.testing.assert_array_equal(h_out.numpy(), out_d.cpu().numpy())
    np.testing.assert_array_equal(h_st.numpy(), st_d.cpu().numpy())
    # the save grid read in place from pinned host memory, too
    h_ts = torch.as_tensor(b.save_ts).pin_memory()
    h_offs = torch.as_tensor(b.save_offsets).pin_memory()
    o2, s2, steps2 = integrate(mw, b.y0, b.t0, b.t1, h_ts, cfg, save_offsets=h_offs, out=h_out, status=h_st)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(h_out.numpy(), out_d.cpu().numpy())
    np.testing.assert_array_equal(steps2.cpu().numpy(), steps_d.cpu().numpy())
    with pytest.raises(ValueError):
        integrate(mw, b.y0, b.t0, b.t1, b.save_ts, cfg, save_offsets=b.save_offsets,
                  out=torch.empty(3, dtype=torch.float64))


def test_team_path_replays_from_a_cuda_graph(gx):
    """gal_integrate with the team fork/join (library stream, events) captured
    into a CUDA graph replays to the eager result."""
    import torch

    from galax_gb300 import workloads as W
    from galax_gb300.dynamics import Workspace, integrate

    mw = gx.MilkyWayPotential()
    y0 = torch.as_tensor(W.disk_like_ics(lambda x: O.gradient(O.milky_way(), x), 2000, seed=21),
                         device="cuda").t().contiguous()
    t0 = torch.zeros(2000, dtype=torch.float64, device="cuda")
    t1 = torch.full((2000,), 300.0, dtype=torch.float64, device="cuda")
    ts = torch.linspace(0.0, 300.0, 11, dtype=torch.float64, device="cuda")
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10),
                        schedule=True).config()
    ws = Workspace()
    eager, st_e, _ = integrate(mw, y0, t0, t1, ts, cfg, soa=True, workspace=ws)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        out_g, st_g, _ = integrate(mw, y0, t0, t1, ts, cfg, soa=True, workspace=ws)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out_g, eager) and torch.equal(st_g, st_e)
