"""Mock stellar streams built from a release DF and batched orbits on the GPU.

galax's two stream front ends, with the same arguments and results:

- ``MockStreamGenerator(df, potential).run(rng, ts, prog_w0, prog_mass)``
  (legacy/mockstream/mockstream_generator.py:160-275): the progenitor orbit
  is saved at the stripping times ``ts``; ``df.sample`` draws a leading and a
  trailing particle at each of those points; every particle is integrated in
  the host potential from its release time to ``ts[-1] + 1e-3``. The
  progenitor's own potential is not included. It returns the two arms at the
  final time and the progenitor's last point.
- ``StreamSimulator().init(pot, prog_w0, prog_t0, release_times=..., Msat=...,
  key=...)`` and ``.run(pot, ics, t1=...)`` (experimental/stream.py:121-446).
  These do the same on sorted release times. ``init`` first integrates the
  progenitor from ``prog_t0`` to the first release time.

The release points are sampled by ``gal_stream_df_sample``: the King (1962)
tidal radius and the Fardal (2015) or Chen (2024) model, one thread per
release. The particle
orbits run through the uneven-span integrator (``gal_integrate`` with
per-orbit start and end times). The progenitor is one ``evaluate_orbit``
call.

galax draws the DF's normals from a jax PRNG key. Here ``rng`` is a
``numpy.random.Generator`` or an integer seed: four draws per release point
for Fardal (kr, kvphi, kz, kvz), six for Chen. ``draws=`` passes them
explicitly. For streams with the progenitor's own moving potential, and for
their gradients, see ``galax_gb300.stream``.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import stream as _stream
from .dynamics import Dopri8, Integrator, PIDController, evaluate_orbit, integrate_dense, integrate_orbit
from .potential import AbstractPotential


def _torch():
    import torch

    return torch


def _draws(rng, n: int, draws=None, k: int = 4) -> np.ndarray:
    if draws is not None:
        return np.asarray(draws, np.float64).reshape(n, k)
    g = rng if isinstance(rng, np.random.Generator) else np.random.default_rng(rng)
    return g.normal(size=(n, k))


def _np(x) -> np.ndarray:
    torch = _torch()
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x, np.float64)


@dataclass
class MockStreamArm:
    """One arm: positions q (n, 3), velocities p (n, 3) at times t (n,),
    released at release_time (n,) (galax mockstream/arm.py)."""

    q: np.ndarray
    p: np.ndarray
    t: np.ndarray
    release_time: np.ndarray

    def w(self) -> np.ndarray:
        return np.concatenate([self.q, self.p], axis=-1)


@dataclass
class ConstantMassProgenitor:
    """A progenitor mass that does not change (legacy/mockstream/df/progenitor.py)."""

    m_tot: float

    def __call__(self, t):
        return np.full(np.shape(t), float(self.m_tot))


@dataclass(frozen=True)
class Fardal2015DF:
    """Fardal et al. (2015) release model with galax's parameters
    (experimental/df.py:57-177): ``sample(rng, pot, t, x, v, Msat)`` returns
    (x_lead, v_lead, x_trail, v_trail) for one or many release points."""

    kr_bar: float = 2.0
    kvphi_bar: float = 0.3
    kz_bar: float = 0.0
    kvz_bar: float = 0.0
    sigma_kr: float = 0.5
    sigma_kvphi: float = 0.5
    sigma_kz: float = 0.5
    sigma_kvz: float = 0.5

    @property
    def params(self) -> tuple:
        return (self.kr_bar, self.kvphi_bar, self.kz_bar, self.kvz_bar, self.sigma_kr, self.sigma_kvphi,
                self.sigma_kz, self.sigma_kvz)

    def sample(self, rng, pot: AbstractPotential, t, x, v, Msat, *, draws=None):
        del t  # static potentials: the release time only labels the point
        x = np.asarray(x, np.float64)
        v = np.asarray(v, np.float64)
        batch = x.shape[:-1]
        w = np.concatenate([x.reshape(-1, 3), v.reshape(-1, 3)], axis=1)
        n = w.shape[0]
        lead, trail, _ = _stream.df_sample(pot, w, np.broadcast_to(np.asarray(Msat, np.float64), (n,)),
                                           _draws(rng, n, draws), df="fardal2015", df_params=self.params)
        return (lead[:, :3].reshape(*batch, 3), lead[:, 3:].reshape(*batch, 3), trail[:, :3].reshape(*batch, 3),
                trail[:, 3:].reshape(*batch, 3))


@dataclass(frozen=True)
class FardalStreamDF:
    """galax's legacy Fardal DF (legacy/mockstream/df/fardal15.py:40-94), with
    the fixed constants kr_bar = 2, kvphi_bar = 0.3, kz_bar = kvz_bar = 0 and
    all sigmas 0.5. ``sample(rng, pot, prog_orbit, prog_mass)`` returns
    {"lead": MockStreamArm, "trail": MockStreamArm} at the orbit's times."""

    params: tuple = (2.0, 0.3, 0.0, 0.0, 0.5, 0.5, 0.5, 0.5)

    def sample(self, rng, pot: AbstractPotential, prog_orbit, prog_mass, *, draws=None) -> dict:
        q = _np(prog_orbit.q).reshape(-1, 3)
        p = _np(prog_orbit.p).reshape(-1, 3)
        ts = _np(prog_orbit.t).reshape(-1)
        n = q.shape[0]
        mprog = prog_mass if callable(prog_mass) else ConstantMassProgenitor(prog_mass)
        m = np.broadcast_to(np.asarray(mprog(ts), np.float64), (n,))
        lead, trail, _ = _stream.df_sample(pot, np.concatenate([q, p], axis=1), m, _draws(rng, n, draws),
                                           df="fardal2015", df_params=self.params)
        return {"lead": MockStreamArm(lead[:, :3], lead[:, 3:], ts.copy(), ts.copy()),
                "trail": MockStreamArm(trail[:, :3], trail[:, 3:], ts.copy(), ts.copy())}


@dataclass(frozen=True)
class ChenStreamDF:
    """galax's Chen et al. (2024) DF, "no progenitor" version
    (legacy/mockstream/df/chen24.py:21-137): six correlated draws per release
    point, posvel = mean + A z from six standard normals z (A: the
    lower-triangular factor of galax's covariance). ``sample`` has the same
    signature and result as FardalStreamDF.sample."""

    def sample(self, rng, pot: AbstractPotential, prog_orbit, prog_mass, *, draws=None) -> dict:
        q = _np(prog_orbit.q).reshape(-1, 3)
        p = _np(prog_orbit.p).reshape(-1, 3)
        ts = _np(prog_orbit.t).reshape(-1)
        n = q.shape[0]
        mprog = prog_mass if callable(prog_mass) else ConstantMassProgenitor(prog_mass)
        m = np.broadcast_to(np.asarray(mprog(ts), np.float64), (n,))
        lead, trail, _ = _stream.df_sample(pot, np.concatenate([q, p], axis=1), m, _draws(rng, n, draws, 6),
                                           df="chen2024")
        return {"lead": MockStreamArm(lead[:, :3], lead[:, 3:], ts.copy(), ts.copy()),
                "trail": MockStreamArm(trail[:, :3], trail[:, 3:], ts.copy(), ts.copy())}


def _default_integrator() -> Integrator:
    return Integrator()


@dataclass
class MockStreamGenerator:
    """galax's MockStreamGenerator (legacy/mockstream/mockstream_generator.py:33-275)."""

    df: FardalStreamDF | ChenStreamDF
    potential: AbstractPotential
    progenitor_integrator: Integrator = field(default_factory=_default_integrator)
    stream_integrator: Integrator = field(default_factory=_default_integrator)

    def run(self, rng, ts, prog_w0, prog_mass, *, vmapped=None, draws=None):
        """Returns ({"lead": arm, "trail": arm}, progenitor's final point (6,)).

        ``prog_w0``: the progenitor's (6,) phase-space point at ``ts[0]``. As in
        galax, a decreasing ``ts`` is reversed first. ``vmapped`` is accepted
        for signature parity: the GPU integrates all particles in one batch
        either way."""
        del vmapped
        ts = np.asarray(ts, np.float64).reshape(-1)
        if ts.size > 1 and ts[1] < ts[0]:
            ts = ts[::-1].copy()
        w0 = np.asarray(prog_w0, np.float64).reshape(6)
        orbit = evaluate_orbit(self.potential, w0, ts, integrator=self.progenitor_integrator)
        mock0 = self.df.sample(rng, self.potential, orbit, prog_mass, draws=draws)
        t_f = ts[-1] + 1e-3  # galax bumps the final time by 1e-3 (mockstream_generator.py:95, 136)
        n = ts.size
        ics = np.concatenate([mock0["lead"].w(), mock0["trail"].w()], axis=0)
        t0 = np.concatenate([ts, ts])
        fin, _, _ = integrate_orbit(self.potential, ics, t0, np.full(2 * n, t_f), None,
                                    integrator=self.stream_integrator)
        fin = _np(fin)
        t = np.full(n, ts[-1])
        arms = {"lead": MockStreamArm(fin[:n, :3], fin[:n, 3:], t, ts.copy()),
                "trail": MockStreamArm(fin[n:, :3], fin[n:, 3:], t.copy(), ts.copy())}
        prog_final = np.concatenate([np.asarray(orbit.q)[-1], np.asarray(orbit.p)[-1]])
        return arms, prog_final


@dataclass
class StreamICs:
    """Release times, progenitor masses and the two arms' release conditions
    (experimental/stream.py StreamICs)."""

    release_times: np.ndarray
    prog_mass: np.ndarray
    qp_lead: tuple
    qp_trail: tuple


def _experimental_integrator(solver_kwargs) -> Integrator:
    # galax's experimental default solver: Dopri8 with PID rtol = atol = 1e-7
    # (experimental/integrate.py:28-35)
    kw = dict(rtol=1e-7, atol=1e-7)
    kw.update(solver_kwargs or {})
    return Integrator(solver=Dopri8(), stepsize_controller=PIDController(**kw))


class StreamSimulator:
    """galax's experimental StreamSimulator (experimental/stream.py:52-446)."""

    def init(self, pot: AbstractPotential, prog_w0, prog_t0, /, release_times, Msat, kinematic_df=None, *, key,
             solver_kwargs=None, draws=None) -> StreamICs:
        rts = np.sort(np.asarray(release_times, np.float64).reshape(-1))
        x0, v0 = (np.asarray(a, np.float64).reshape(3) for a in prog_w0)
        integ = _experimental_integrator(solver_kwargs)
        w0 = np.concatenate([x0, v0])
        # progenitor: prog_t0 -> first release time, then saved at every release time
        start, _, _ = integrate_orbit(pot, w0[None], np.array([float(prog_t0)]), np.array([rts[0]]), None,
                                      integrator=integ)
        orbit = evaluate_orbit(pot, _np(start)[0], rts, integrator=integ)
        q, p = np.asarray(orbit.q), np.asarray(orbit.p)
        m = np.broadcast_to(np.asarray(Msat, np.float64), rts.shape).copy()
        df = Fardal2015DF() if kinematic_df is None else kinematic_df
        xl, vl, xt, vt = df.sample(key, pot, rts, q, p, m, draws=draws)
        return StreamICs(rts, m, (xl, vl), (xt, vt))

    def run(self, pot: AbstractPotential, prog: StreamICs, /, *, t1, dense: bool = False, solver_kwargs=None):
        """Each arm integrated from its release time to ``t1``: returns
        ((q_lead, v_lead), (q_trail, v_trail)).

        With ``dense=True`` it returns instead one dense interpolant over every
        particle (galax returns one dense diffrax solution per particle,
        experimental/stream.py:393-399, 436-441): a ``PhaseSpaceInterpolation``
        with batch (2, n), leading arm first, each particle valid from its
        release time to ``t1``."""
        n = prog.release_times.size
        ics = np.concatenate([np.concatenate(prog.qp_lead, axis=1), np.concatenate(prog.qp_trail, axis=1)], axis=0)
        t0 = np.concatenate([prog.release_times, prog.release_times])
        integ = _experimental_integrator(solver_kwargs)
        if dense:
            return integrate_dense(pot, ics, t0, np.full(2 * n, float(t1)), integ.config(), batch=(2, n))
        fin, _, _ = integrate_orbit(pot, ics, t0, np.full(2 * n, float(t1)), None, integrator=integ)
        fin = _np(fin)
        return (fin[:n, :3], fin[:n, 3:]), (fin[n:, :3], fin[n:, 3:])
