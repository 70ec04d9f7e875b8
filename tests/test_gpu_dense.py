"""Dense output (evaluate_orbit(..., dense=True), galax's PhaseSpaceInterpolation)
on a GB300: the interpolant evaluated at save times reproduces the save path
(bitwise for Dopri8, whose saves are the same partial step; to rounding for the
Dopri5 quartic, stored in monomial form) and the oracle's saves."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O

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


def _ics(n, seed):
    from galax_gb300 import workloads as W

    return W.disk_like_ics(lambda x: O.gradient(O.milky_way(), x), n, seed=seed)


def _rel(a, b):
    a = np.asarray(a).reshape(-1, 6)
    b = np.asarray(b).reshape(-1, 6)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)))


@pytest.mark.parametrize("t1", [300.0, -300.0])
def test_dopri8_dense_equals_saves_bitwise(gx, t1):
    from galax_gb300.dynamics import integrate, integrate_dense

    mw = gx.MilkyWayPotential()
    y0 = _ics(200, 1)
    cfg = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0).config()
    ts = np.linspace(0.0, t1, 37)  # off the step grid
    out, st, _ = integrate(mw, y0, 0.0, t1, ts, cfg)
    interp = integrate_dense(mw, y0, 0.0, t1, cfg)
    q, p = interp.evaluate(ts)
    w = np.concatenate([q.cpu().numpy(), p.cpu().numpy()], axis=-1)  # (n, T, 6)
    ref = out.permute(2, 1, 0).cpu().numpy()
    assert np.array_equal(w, ref)


def test_dopri5_adaptive_dense_matches_saves_and_oracle(gx):
    from galax_gb300.dynamics import integrate, integrate_dense

    mw = gx.MilkyWayPotential()
    y0 = _ics(150, 2)
    integ = gx.Integrator(gx.Dopri5(), gx.PIDController(rtol=1e-8, atol=1e-10))
    cfg = integ.config()
    ts = np.linspace(0.0, 500.0, 41)
    out, st, _ = integrate(mw, y0, 0.0, 500.0, ts, cfg)
    interp = integrate_dense(mw, y0, 0.0, 500.0, cfg)
    q, p = interp.evaluate(ts)
    w = np.concatenate([q.cpu().numpy(), p.cpu().numpy()], axis=-1)
    ref = out.permute(2, 1, 0).cpu().numpy()
    assert _rel(w, ref) < 1e-12
    oref, *_ = O.integrate(O.milky_way(), y0, 0.0, 500.0, ts, O.solver_cfg(5, True, rtol=1e-8, atol=1e-10))
    assert _rel(w, np.stack(oref)) < 1e-7
    # the recorded steps are the controller's accepted steps
    assert np.all(interp.nsteps.cpu().numpy() > 10)
    np.testing.assert_allclose(interp.t1.cpu().numpy(), 500.0)


def test_evaluate_orbit_dense_returns_the_saves_and_an_interpolant(gx):
    mw = gx.MilkyWayPotential()
    y0 = _ics(64, 3)
    integ = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=0.5)
    ts = np.linspace(0.0, 200.0, 11)
    a = gx.evaluate_orbit(mw, y0, ts, integrator=integ)
    b = gx.evaluate_orbit(mw, y0, ts, integrator=integ, dense=True)
    assert np.array_equal(a.w, b.w)
    q, p = b.interpolant.evaluate(np.array([13.3, 157.25]))
    ref = gx.evaluate_orbit(mw, y0, np.array([0.0, 13.3, 157.25]), integrator=integ)
    assert _rel(np.concatenate([q.cpu().numpy(), p.cpu().numpy()], -1), ref.w[:, 1:]) < 1e-12


def test_out_of_bounds_raises_and_capacity_grows(gx):
    from galax_gb300.dynamics import integrate, integrate_dense

    mw = gx.MilkyWayPotential()
    y0 = _ics(16, 4)
    cfg = gx.Integrator(gx.Dopri5(), gx.PIDController(rtol=1e-8, atol=1e-10)).config()
    interp = integrate_dense(mw, y0, 0.0, 100.0, cfg, cap=2)  # far too small: doubled until it fits
    assert interp.cap > 2
    with pytest.raises(ValueError, match="out of bounds"):
        interp.evaluate(np.array([50.0, 100.5]))
    ts = np.array([0.0, 100.0])
    q, p = interp.evaluate(ts)
    out, *_ = integrate(mw, y0, 0.0, 100.0, ts, cfg)
    ref = out.permute(2, 1, 0).cpu().numpy()
    assert _rel(np.concatenate([q.cpu().numpy(), p.cpu().numpy()], -1), ref) < 1e-12


def test_table_potential_dense(gx):
    from galax_gb300.dynamics import integrate, integrate_dense
    from galax_gb300.potential import from_component_array

    comps = O.comps([(O.NFW, 8e11, 16.0, 0.0), (O.PLUMMER, 2e9, 0.5, 0.0, (6.0, 1.0, -0.5))])
    pot = from_component_array(comps)
    y0 = _ics(40, 5)
    cfg = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0).config()
    ts = np.linspace(0.0, 80.0, 9) + 0.25
    ts[-1] = 80.0
    out, *_ = integrate(pot, y0, 0.0, 80.0, ts, cfg)
    q, p = integrate_dense(pot, y0, 0.0, 80.0, cfg).evaluate(ts)
    assert np.array_equal(np.concatenate([q.cpu().numpy(), p.cpu().numpy()], -1), out.permute(2, 1, 0).cpu().numpy())


@pytest.mark.parametrize("method,adaptive", [(8, False), (5, True), (8, True)])
def test_linear_parameters_dense_matches_saves(gx, method, adaptive):
    """LinearParameter potentials in dense output: every stage, and every
    Dopri8 re-evaluation, at its own time, so the interpolant at the save times
    reproduces the save path (constant-step Dopri8 bitwise, otherwise to
    rounding), and the time dependence is visible against the static values."""
    from galax_gb300.dynamics import integrate, integrate_dense

    def pot(lin):
        L = gx.LinearParameter
        return gx.CompositePotential(
            disk=gx.MiyamotoNagaiPotential(m_tot=L(5e7, 0.0, 6.8e10) if lin else 6.8e10, a=3.0, b=0.28),
            halo=gx.NFWPotential(m=L(2e8, 0.0, 5.4e11) if lin else 5.4e11,
                                 r_s=L(-2e-3, 0.0, 15.62) if lin else 15.62))

    solver = gx.Dopri8() if method == 8 else gx.Dopri5()
    if adaptive:
        integ = gx.Integrator(solver=solver, stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-10))
    else:
        integ = gx.Integrator(solver=solver, stepsize_controller=gx.ConstantStepSize(), dt0=1.0)
    cfg = integ.config()
    y0 = _ics(64, 7)
    ts = np.linspace(0.0, 400.0, 29)
    out, st, _ = integrate(pot(True), y0, 0.0, 400.0, ts, cfg)
    interp = integrate_dense(pot(True), y0, 0.0, 400.0, cfg)
    q, p = interp.evaluate(ts)
    w = np.concatenate([q.cpu().numpy(), p.cpu().numpy()], axis=-1)
    ref = out.permute(2, 1, 0).cpu().numpy()
    assert np.all(st.cpu().numpy() == 0)
    if method == 8 and not adaptive:
        assert np.array_equal(w, ref)
    else:
        assert _rel(w, ref) < 1e-12
    static, _, _ = integrate(pot(False), y0, 0.0, 400.0, ts, cfg)
    assert _rel(ref, static.permute(2, 1, 0).cpu().numpy()) > 1e-6
