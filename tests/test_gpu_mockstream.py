"""Stream release models and galax's mock-stream front ends on the GPU (needs
a GB300).

- ``gal_stream_df_sample`` (King tidal radius + Fardal 2015 or offsets)
  against the oracle, galax's tidal-radius doctest and the arm geometry of
  galax's Fardal2015DF doctest;
- ``MockStreamGenerator.run`` and ``StreamSimulator.init/run`` against the
  same pipeline composed from the oracle's integrator and DF sampler (galax's
  Dopri8 + PID defaults, so both sides take the same steps; 10 x rtol).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests._helpers import golden_comps

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from galax_gb300.build import build

    build()
    from galax_gb300 import mockstream

    return mockstream


def _pot(comps):
    from galax_gb300.potential import from_component_array

    return from_component_array(comps)


def _points(n, seed=3):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-30, 30, (n, 3))
    v = rng.normal(0, 0.2, (n, 3))
    return np.concatenate([x, v], axis=1), rng


@pytest.mark.parametrize("df", [1, 0, 2])
def test_df_sample_matches_oracle(M, df):
    from galax_gb300 import stream

    c = O.milky_way()
    w, rng = _points(1000)
    mass = rng.uniform(1e4, 1e6, len(w))
    nz = rng.normal(size=(len(w), O.NOISE_COLUMNS[df]))
    p = (1.5, 0.2, 0.1, -0.1, 0.3, 0.4, 0.2, 0.1)
    lead, trail, rt = stream.df_sample(_pot(c), w, mass, nz, df=df, df_params=p)
    el, et, ert = O.stream_df_sample(c, w, mass, nz, df=df, df_params=p)
    np.testing.assert_allclose(rt, ert, rtol=1e-13)
    np.testing.assert_allclose(lead, el, rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(trail, et, rtol=1e-13, atol=1e-14)


def test_king_tidal_radius_golden(M, goldens):
    from galax_gb300 import stream

    g = goldens["stream"]["king_tidal_radius"]
    _, _, rt = stream.df_sample(_pot(golden_comps(g["potential"])), np.array([g["x"] + g["v"]]), g["mass"],
                                np.zeros((1, 4)))
    assert abs(rt[0] - g["r_tidal"]) <= 1e-8


def test_fardal2015_doctest_geometry(M, goldens):
    """With the draws galax's printed sample implies, Fardal2015DF.sample on the
    GPU reproduces every printed digit."""
    g = goldens["stream"]["fardal2015_sample"]
    c = golden_comps(g["potential"])
    x, v = np.array(g["x"]), np.array(g["v"])
    xl, vl, xt, vt = (np.array(g[k]) for k in ("x_lead", "v_lead", "x_trail", "v_trail"))
    _, _, rt = O.stream_df_sample(c, np.concatenate([x, v])[None], g["mass"], np.zeros((1, 4)))
    om = np.linalg.norm(np.cross(x, v)) / np.dot(x, x)
    kr = (xt - xl)[0] / 2 / rt[0]
    kz = ((xt + xl) / 2 - x)[2] / rt[0]
    kvphi = (vt - vl)[1] / 2 / (om * rt[0])
    kvz = ((vt + vl) / 2 - v)[2] / (om * rt[0])
    draws = np.array([[(kr - 2.0) / 0.5, (kvphi / kr - 0.3) / 0.5, kz / 0.5, kvz / 0.5]])
    df = M.Fardal2015DF()
    got = df.sample(None, _pot(c), 0.0, x, v, g["mass"], draws=draws)
    for a, b in zip(got, (xl, vl, xt, vt)):
        np.testing.assert_allclose(a, b, rtol=2e-8, atol=1e-12)


def test_mock_stream_generator_with_chen_df(M):
    c = O.milky_way()
    ts = np.linspace(0.0, 500.0, 51)
    w0 = np.array([12.0, 0.0, 4.0, 0.0, 0.2, 0.02])
    draws = np.random.default_rng(5).normal(size=(len(ts), 6))
    gen = M.MockStreamGenerator(M.ChenStreamDF(), _pot(c))
    arms, _ = gen.run(None, ts, w0, 2e4, draws=draws)
    lead, trail, _ = _oracle_generator(c, ts, w0, 2e4, draws, df=O.STREAM_DF_CHEN2024)
    assert _rel(arms["lead"].q, lead[:, :3]) < 1e-6
    assert _rel(arms["trail"].p, trail[:, 3:]) < 1e-6


def _oracle_generator(c, ts, w0, mass, draws, rtol=1e-7, df=O.STREAM_DF_FARDAL2015):
    cfg = O.solver_cfg(8, True, rtol=rtol, atol=rtol)
    saves, st, _, _ = O.integrate(c, w0[None], ts[0], ts[-1], ts, cfg)
    assert st[0] == 0
    track = saves[0]
    lead, trail, _ = O.stream_df_sample(c, track, mass, draws, df=df)
    t_f = ts[-1] + 1e-3
    ics = np.concatenate([lead, trail])
    t0 = np.concatenate([ts, ts])
    out, st, _, _ = O.integrate(c, ics, t0, t_f, [np.array([t_f])] * len(ics), cfg)
    assert np.all(st == 0)
    fin = np.array([o[-1] for o in out])
    n = len(ts)
    return fin[:n], fin[n:], track[-1]


def _rel(a, b):
    a, b = np.asarray(a).reshape(-1, 3), np.asarray(b).reshape(-1, 3)
    return float(np.max(np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)))


def test_mock_stream_generator_matches_oracle(M):
    """galax's functional mock-stream setup (tests/functional/
    test_mockstreamgenerator.py: MilkyWay with a 5e10 disk, progenitor at
    (30, 10, 20) kpc, (10, -150, -20) km/s, 1e4 Msun), on a shorter grid of
    stripping times."""
    c = O.milky_way()
    ts = np.linspace(0.0, 1000.0, 101)
    kms = 0.001022712165045695
    w0 = np.array([30.0, 10.0, 20.0, 10.0 * kms, -150.0 * kms, -20.0 * kms])
    rng = np.random.default_rng(12)
    draws = rng.normal(size=(len(ts), 4))
    gen = M.MockStreamGenerator(M.FardalStreamDF(), _pot(c))
    arms, prog = gen.run(None, ts, w0, 1e4, draws=draws)
    lead, trail, prog_ref = _oracle_generator(c, ts, w0, 1e4, draws)
    assert _rel(arms["lead"].q, lead[:, :3]) < 1e-6
    assert _rel(arms["trail"].q, trail[:, :3]) < 1e-6
    assert _rel(arms["lead"].p, lead[:, 3:]) < 1e-6
    assert _rel(arms["trail"].p, trail[:, 3:]) < 1e-6
    np.testing.assert_allclose(prog, prog_ref, rtol=1e-6)
    np.testing.assert_array_equal(arms["lead"].release_time, ts)
    assert np.all(arms["trail"].t == ts[-1])
    # same draws from a seeded generator give the same stream
    a2, _ = gen.run(np.random.default_rng(12), ts, w0, 1e4)
    np.testing.assert_array_equal(a2["lead"].q, arms["lead"].q)
    # a decreasing grid is reversed first, as in galax
    a3, _ = gen.run(None, ts[::-1], w0, 1e4, draws=draws)
    np.testing.assert_array_equal(a3["trail"].p, arms["trail"].p)


def test_stream_simulator_matches_oracle(M):
    """galax's StreamSimulator doctest setup (experimental/stream.py:244-262):
    NFW(8.73951152e11, 15), progenitor at (10, 0, 0) kpc with 0.17386107
    kpc/Myr, release times 0..1000 Myr, run back to t1 = t0."""
    c = O.comps([(O.NFW, 8.73951152e11, 15.0, 0.0)])
    pot = _pot(c)
    rts = np.linspace(0.0, 1000.0, 200)
    qp0 = (np.array([10.0, 0.0, 0.0]), np.array([0.0, 0.17386107, 0.0]))
    draws = np.random.default_rng(0).normal(size=(len(rts), 4))
    sim = M.StreamSimulator()
    ics = sim.init(pot, qp0, 0.0, release_times=rts, Msat=1e5, key=None, draws=draws)
    (ql, vl), (qt, vt) = sim.run(pot, ics, t1=0.0)
    cfg = O.solver_cfg(8, True, rtol=1e-7, atol=1e-7)
    w0 = np.concatenate(qp0)
    saves, _, _, _ = O.integrate(c, w0[None], 0.0, rts[-1], rts, cfg)
    lead, trail, _ = O.stream_df_sample(c, saves[0], 1e5, draws)
    np.testing.assert_allclose(np.concatenate(ics.qp_lead, axis=1), lead, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(np.concatenate(ics.qp_trail, axis=1), trail, rtol=1e-6, atol=1e-9)
    icsr = np.concatenate([lead, trail])
    out, st, _, _ = O.integrate(c, icsr, np.concatenate([rts, rts]), 0.0, [np.array([0.0])] * len(icsr), cfg)
    fin = np.array([o[-1] for o in out])
    n = len(rts)
    assert _rel(ql, fin[:n, :3]) < 1e-6
    assert _rel(qt, fin[n:, :3]) < 1e-6
    # the particle released at t0 is already there: it comes back unchanged
    np.testing.assert_allclose(ql[0], ics.qp_lead[0][0], rtol=1e-14)
    # dense=True: one interpolant over both arms, valid from each release time to t1
    interp = sim.run(pot, ics, t1=0.0, dense=True)
    q, p = (x.cpu().numpy() for x in interp.evaluate(np.array([0.0])))
    assert q.shape == (2, n, 1, 3) and p.shape == (2, n, 1, 3)
    assert _rel(q[0, :, 0], ql) < 1e-12 and _rel(q[1, :, 0], qt) < 1e-12
    assert _rel(p[0, :, 0], vl) < 1e-12 and _rel(p[1, :, 0], vt) < 1e-12
