"""Spans that would never end on a GB300: an orbit whose start or end time is
not finite finishes at once with the non-finite status (saves NaN) while the
other orbits of the batch are unchanged bitwise, and the host-side constant-step
grids (adjoint, surrogate) reject such spans, and steps too small to move the
time, with an error instead of looping."""

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


@pytest.mark.parametrize("adaptive", [True, False])
def test_non_finite_span_ends_the_orbit_at_once(gx, adaptive):
    import torch
    from galax_gb300.dynamics import integrate

    mw = gx.MilkyWayPotential()
    n = 64
    y0 = _ics(n, 3)
    if adaptive:
        cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-8)).config()
    else:
        cfg = gx.Integrator(solver=gx.Dopri8(), stepsize_controller=gx.ConstantStepSize(), dt0=1.0).config()
    t0 = np.zeros(n)
    t1 = np.full(n, 200.0)
    ts = np.linspace(0.0, 200.0, 9)
    out_ok, st_ok, _ = integrate(mw, y0, t0, t1, ts, cfg)
    t0b, t1b = t0.copy(), t1.copy()
    t1b[5] = np.inf
    t1b[17] = -np.inf
    t0b[40] = np.nan
    out, st, _ = integrate(mw, y0, t0b, t1b, ts, cfg)
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    bad = [5, 17, 40]
    assert list(st[bad]) == [3, 3, 3]
    good = np.setdiff1d(np.arange(n), bad)
    assert (st[good] == 0).all()
    o = out.cpu().numpy()
    assert np.isnan(o[:, :, bad]).all()
    assert np.array_equal(o[:, :, good], out_ok.cpu().numpy()[:, :, good])


def test_dense_non_finite_span(gx):
    from galax_gb300.dynamics import integrate_dense

    mw = gx.MilkyWayPotential()
    y0 = _ics(16, 4)
    cfg = gx.Integrator(solver=gx.Dopri5(), stepsize_controller=gx.PIDController(rtol=1e-8, atol=1e-8)).config()
    t1 = np.full(16, 100.0)
    t1[3] = np.inf
    interp = integrate_dense(mw, y0, 0.0, t1, cfg, throw=False)
    assert int(interp.nsteps[3]) == 0
    with pytest.raises(gx.GalaxGB300Error):
        integrate_dense(mw, y0, 0.0, t1, cfg)


def test_adjoint_rejects_unbounded_grids(gx):
    from galax_gb300.adjoint import orbit_adjoint

    mw = gx.MilkyWayPotential()
    y0 = _ics(8, 5)
    for t0, t1, dt in [(0.0, np.inf, 1.0), (np.nan, 10.0, 1.0), (1e20, 1e20 + 1e6, 1.0)]:
        with pytest.raises(gx.GalaxGB300Error):
            orbit_adjoint(mw, y0, t0, t1, dt=dt, target=np.zeros_like(y0))


def test_surrogate_rejects_unbounded_grids(gx):
    from galax_gb300 import surrogate as S

    mw = gx.MilkyWayPotential()
    y0 = _ics(8, 6)
    for t0, t1, dt in [(0.0, np.inf, 1.0), (1e20, 1e20 + 1e6, 1.0)]:
        with pytest.raises(gx.GalaxGB300Error):
            S.integrate(mw, None, y0, t0, t1, dt)
