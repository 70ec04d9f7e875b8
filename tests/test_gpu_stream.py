"""Mock stream with a moving progenitor: the CUDA pipeline against the oracle
(needs a GB300).

Forward: progenitor track, release conditions and final particle states agree
with the oracle to 1e-9 relative (constant steps on both sides), for both
release models (Gaussian offsets, galax's Fardal 2015 and Chen 2024 DFs), for
the Milky Way, a table and BovyMWPotential2014 (with its power law with
cutoff). Gradient: the
discrete adjoint of the whole pipeline (particles, tidal-radius release map,
progenitor orbit) against central finite differences of the oracle with one
Richardson extrapolation, 1e-6 relative for the halo mass and scale radius,
and within the finite differences' own spread for the other parameters.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

N_REL = 200


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from galax_gb300.build import build

    build()
    from galax_gb300 import stream

    return stream


def _setup(comps, n_release=N_REL, **kw):
    from galax_gb300 import workloads as W

    return W.stream_setup(lambda x: O.gradient(comps, x), n_release=n_release, **kw)


def _cfg(S, s, method=8, k_ckpt=64):
    return S.config(n_release=s.n_release, dt=s.dt, w_now=s.w_now, prog_m=s.prog_m, prog_b=s.prog_b,
                    t_now=s.t_now, method=method, k_ckpt=k_ckpt, df=s.df)


def _pot(comps):
    from galax_gb300.potential import from_component_array

    return from_component_array(comps)


def _relmax(a, b):
    a = np.asarray(a).reshape(-1, 6)
    b = np.asarray(b).reshape(-1, 6)
    out = 0.0
    for sl in (slice(0, 3), slice(3, 6)):
        d = np.linalg.norm(a[:, sl] - b[:, sl], axis=1)
        n = np.linalg.norm(b[:, sl], axis=1)
        out = max(out, float(np.max(d / np.maximum(n, 1e-300))))
    return out


HOSTS = {
    "milky_way": O.milky_way(),
    "table": O.comps([(O.NFW, 8e11, 16.0, 0.0), (O.HERNQUIST, 3e10, 0.8, 0.0), (O.MIYAMOTO_NAGAI, 5e10, 2.5, 0.3)]),
    # BovyMWPotential2014: Miyamoto-Nagai disk, power law with cutoff bulge, NFW halo
    "bovy2014": O.bovy_mw_2014(),
}
SHAPED = (O.MIYAMOTO_NAGAI, O.POWERLAW_CUTOFF)  # components with a second shape parameter (l2)


@pytest.mark.parametrize("df", [0, 1, 2])
@pytest.mark.parametrize("host", list(HOSTS))
@pytest.mark.parametrize("method", [8, 5])
def test_forward_matches_oracle(S, host, method, df):
    comps = HOSTS[host]
    s = _setup(comps, df=df)
    got = S.simulate(_pot(comps), _cfg(S, s, method), s.noise)
    ref = O.stream_forward(comps, s, method=method)
    assert _relmax(got.track, ref["track"]) < 1e-9
    assert _relmax(got.ics, ref["ics"]) < 1e-9
    assert _relmax(got.final, ref["final"]) < 1e-9


@pytest.mark.parametrize("host,k_ckpt,df", [(h, k, d) for h in ("milky_way", "table")
                                             for k, d in [(64, 0), (0, 0), (0, 1), (64, 2)]]
                         + [("bovy2014", 64, 0), ("bovy2014", 0, 1)])
def test_gradient_matches_finite_differences(S, host, k_ckpt, df):
    comps = HOSTS[host]
    s = _setup(comps, df=df)
    ref = O.stream_forward(comps, s)
    target = ref["final"] + s.pert
    g = S.gradient(_pot(comps), _cfg(S, s, k_ckpt=k_ckpt), s.noise, target)
    assert _relmax(g.final, ref["final"]) < 1e-9
    assert g.loss == pytest.approx(float(np.sum((ref["final"] - target) ** 2)), rel=1e-7)
    fields = ("m", "l1", "l2")
    params = [(c, f) for c in range(len(comps)) for f in fields
              if not (f == "l2" and comps[c]["kind"] not in SHAPED)]
    fd1 = O.stream_fd_grad(comps, s, target, params, rel_h=1e-4)
    fd2 = O.stream_fd_grad(comps, s, target, params, rel_h=1e-5)
    for (c, f), a, b in zip(params, fd1, fd2):
        got = g.grad_params[c][fields.index(f)]
        spread = abs(a - b)
        halo = comps[c]["kind"] == O.NFW
        tol = 1e-6 * abs(a) + (0.0 if halo else 10 * spread)
        assert abs(got - a) <= tol, (c, f, got, a, b)
    # parameters that do not exist (l2 of the other spherical components) get exactly zero
    for c in range(len(comps)):
        if comps[c]["kind"] not in SHAPED:
            assert g.grad_params[c][2] == 0.0


@pytest.mark.parametrize("df", [0, 1, 2])
def test_gradient_with_respect_to_the_present_progenitor_point(S, df):
    comps = HOSTS["milky_way"]
    s = _setup(comps, n_release=60, df=df)
    ref = O.stream_forward(comps, s)
    target = ref["final"] + s.pert
    g = S.gradient(_pot(comps), _cfg(S, s), s.noise, target)
    for j in range(6):
        def loss(h):
            s2 = _setup(comps, n_release=60, df=df)
            s2.w_now = s.w_now.copy()
            s2.w_now[j] += h
            return O.stream_loss(comps, s2, target)
        h = 1e-6 * max(abs(s.w_now[j]), 0.1)
        d1 = (loss(h) - loss(-h)) / (2 * h)
        d2 = (loss(h / 2) - loss(-h / 2)) / h
        fd = (4 * d2 - d1) / 3
        assert abs(g.grad_w_now[j] - fd) <= 1e-5 * max(abs(fd), 1e-3 * np.max(np.abs(g.grad_w_now))), (j, fd)


def test_checkpoint_interval_does_not_change_results(S):
    """Checkpointed sweeps agree bitwise for every interval; the stored-stage
    sweep (k_ckpt = 0, Hessians computed ahead) agrees to rounding."""
    comps = HOSTS["milky_way"]
    s = _setup(comps, n_release=70)
    target = O.stream_forward(comps, s)["final"] + s.pert
    outs = [S.gradient(_pot(comps), _cfg(S, s, k_ckpt=k), s.noise, target) for k in (1, 16, 256)]
    for o in outs[1:]:
        assert np.array_equal(o.grad_params, outs[0].grad_params)
        assert np.array_equal(o.grad_w_now, outs[0].grad_w_now)
        assert np.array_equal(o.final, outs[0].final)
    st = S.gradient(_pot(comps), _cfg(S, s, k_ckpt=0), s.noise, target)
    assert np.array_equal(st.final, outs[0].final)
    np.testing.assert_allclose(st.grad_params, outs[0].grad_params, rtol=1e-10, atol=1e-300)
    np.testing.assert_allclose(st.grad_w_now, outs[0].grad_w_now, rtol=1e-10, atol=1e-14)


def test_single_release_and_repeatability(S):
    comps = HOSTS["milky_way"]
    s = _setup(comps, n_release=1)
    ref = O.stream_forward(comps, s)
    got = S.simulate(_pot(comps), _cfg(S, s), s.noise)
    assert _relmax(got.final, ref["final"]) < 1e-9
    s = _setup(comps, n_release=33)  # a partial last warp
    target = O.stream_forward(comps, s)["final"] + s.pert
    a = S.gradient(_pot(comps), _cfg(S, s), s.noise, target)
    b = S.gradient(_pot(comps), _cfg(S, s), s.noise, target)
    assert np.array_equal(a.grad_params, b.grad_params)
    fd = O.stream_fd_grad(comps, s, target, [(1, "m"), (1, "l1")], rel_h=1e-4)
    assert abs(a.grad_params[1][0] - fd[0]) <= 1e-6 * abs(fd[0])
    assert abs(a.grad_params[1][1] - fd[1]) <= 1e-6 * abs(fd[1])


def test_invalid_configurations_raise(S):
    from galax_gb300._lib import GalaxGB300Error

    comps = HOSTS["milky_way"]
    s = _setup(comps, n_release=4)
    for bad in (dict(method=6), dict(k_ckpt=-1)):
        cfg = _cfg(S, s, **bad)
        with pytest.raises(GalaxGB300Error):
            S.simulate(_pot(comps), cfg, s.noise)
    cfg = _cfg(S, s)
    cfg.df = 7
    with pytest.raises(GalaxGB300Error):
        S.simulate(_pot(comps), cfg, s.noise)
    cfg.df = 1
    cfg.df_params[0] = float("nan")
    with pytest.raises(GalaxGB300Error):
        S.simulate(_pot(comps), cfg, s.noise[:, :4])
    cfg = _cfg(S, s)
    cfg.dt = 0.0
    with pytest.raises(GalaxGB300Error):
        S.simulate(_pot(comps), cfg, s.noise)
