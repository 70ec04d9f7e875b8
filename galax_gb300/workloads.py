"""Seeded synthetic workloads with the shapes and distributions of the
benchmark configurations (there is no dataset: galax benchmarks synthetic
orbits). Everything is drawn with ``numpy.random.default_rng(seed)`` in float64
galactic units; velocities use the local circular speed sqrt(r |dPhi/dr|)
(galax's local_circular_velocity, src/galax/potential/_src/register_funcs.py:384-400)
computed from a caller-supplied gradient function ``grad(x (n,3)) -> (n,3)``.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

KMS = 0.001022712165045695  # kpc/Myr per km/s


def isotropic(rng: np.random.Generator, n: int) -> np.ndarray:
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def circular_speed(grad, x: np.ndarray) -> np.ndarray:
    g = np.asarray(grad(x))
    r = np.linalg.norm(x, axis=1)
    dphidr = np.sum(g * x / r[:, None], axis=1)
    return np.sqrt(r * np.abs(dphidr))


def disk_like_ics(grad, n: int, seed: int, rmin: float = 4.0, rmax: float = 20.0) -> np.ndarray:
    """Orbits of the small plain workload: r ~ U(rmin, rmax), isotropic direction,
    v = v_c(r) phi_hat * N(1, 0.1) per component + z_hat * N(0, 20 km/s). Returns (n, 6)."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(rmin, rmax, n)
    x = isotropic(rng, n) * r[:, None]
    vc = circular_speed(grad, x)
    R = np.hypot(x[:, 0], x[:, 1])
    phi_hat = np.stack([-x[:, 1] / R, x[:, 0] / R, np.zeros(n)], axis=1)
    v = vc[:, None] * phi_hat * rng.normal(1.0, 0.1, (n, 3))
    v[:, 2] += rng.normal(0.0, 20.0 * KMS, n)
    return np.concatenate([x, v], axis=1)


@dataclass
class UnevenBatch:
    y0: np.ndarray          # (n, 6)
    t0: np.ndarray          # (n,)
    t1: np.ndarray          # (n,)
    save_offsets: np.ndarray  # (n+1,) int64
    save_ts: np.ndarray     # (total,)


def uneven_ics(grad, n: int, seed: int = 1, rmin: float = 0.5, rmax: float = 100.0, tmin: float = 100.0,
               tmax: float = 5000.0, smin: int = 10, smax: int = 1000) -> UnevenBatch:
    """The batched uneven workload: r log-uniform [rmin, rmax], isotropic
    direction, v = v_c * U(0.3, 1.1) along a random tangential direction,
    duration log-uniform [tmin, tmax] Myr, save count uniform in [smin, smax],
    saves evenly spaced over each orbit's span."""
    rng = np.random.default_rng(seed)
    r = np.exp(rng.uniform(np.log(rmin), np.log(rmax), n))
    rhat = isotropic(rng, n)
    x = rhat * r[:, None]
    vc = circular_speed(grad, x)
    a = isotropic(rng, n)
    tang = a - np.sum(a * rhat, axis=1, keepdims=True) * rhat
    tang /= np.linalg.norm(tang, axis=1, keepdims=True)
    v = tang * (vc * rng.uniform(0.3, 1.1, n))[:, None]
    dur = np.exp(rng.uniform(np.log(tmin), np.log(tmax), n))
    ns = rng.integers(smin, smax + 1, n)
    offs = np.zeros(n + 1, np.int64)
    offs[1:] = np.cumsum(ns)
    # evenly spaced saves over [0, dur_i] for every orbit, vectorised
    orbit_of = np.repeat(np.arange(n), ns)
    k = np.arange(offs[-1]) - offs[orbit_of]
    save_ts = dur[orbit_of] * (k / (ns[orbit_of] - 1))
    last = offs[1:] - 1
    save_ts[last] = dur  # exact end times
    return UnevenBatch(np.concatenate([x, v], axis=1), np.zeros(n), dur, offs, save_ts)


def subhalo_table(seed: int = 3, n: int = 512):
    """Plummer subhalos: m log-uniform [1e6, 1e8] Msun, r_s ~ U(0.1, 1) kpc,
    centres isotropic at radius U(5, 50) kpc. Returns (m, r_s, centres (n,3))."""
    rng = np.random.default_rng(seed)
    m = np.exp(rng.uniform(np.log(1e6), np.log(1e8), n))
    b = rng.uniform(0.1, 1.0, n)
    c = isotropic(rng, n) * rng.uniform(5.0, 50.0, n)[:, None]
    return m, b, c


def training_points(n: int, seed: int = 30, rmin: float = 0.1, rmax: float = 200.0) -> np.ndarray:
    """Positions log-uniform in radius over [rmin, rmax] kpc with isotropic directions."""
    rng = np.random.default_rng(seed)
    r = np.exp(rng.uniform(np.log(rmin), np.log(rmax), n))
    return isotropic(rng, n) * r[:, None]


@dataclass
class StreamSetup:
    w_now: np.ndarray     # (6,) progenitor phase-space point at t_now
    t_now: float
    dt: float
    n_release: int        # release times t_now - (n_release - r) dt, r = 0..n_release-1
    prog_m: float
    prog_b: float
    noise: np.ndarray     # (n_release, 12 | 4 | 6) draws of the offsets / Fardal / Chen model, N(0, 1)
    pert: np.ndarray      # (2 n_release, 6): target offsets (N(0, 0.1 kpc), N(0, 2 km/s))
    df: int = 0           # release model: 0 offsets, 1 Fardal 2015, 2 Chen 2024
    df_params: tuple = (2.0, 0.3, 0.0, 0.0, 0.5, 0.5, 0.5, 0.5)


def stream_setup(grad, n_release: int = 3000, dt: float = 1.0, seed: int = 4, apocentre: float = 20.0,
                 speed_frac: float = 0.6, incl_deg: float = 30.0, prog_m: float = 1e5,
                 prog_b: float = 0.02, df: int = 0) -> StreamSetup:
    """The stream-like batched-gradient workload: a Plummer progenitor (1e5 Msun,
    b = 20 pc) at apocentre (x = apocentre kpc, velocity speed_frac v_c
    tangential, inclined incl_deg to the x-y plane) at t_now = 0, released
    over n_release dt before the present, two particles per release with
    seeded release draws (df 0: Gaussian offsets, 12 per release; df 1:
    Fardal 2015, 4; df 2: Chen 2024, 6), and seeded target perturbations for
    the loss."""
    rng = np.random.default_rng(seed)
    x = np.array([[apocentre, 0.0, 0.0]])
    vc = float(circular_speed(grad, x)[0])
    inc = np.deg2rad(incl_deg)
    w_now = np.array([apocentre, 0.0, 0.0, 0.0, speed_frac * vc * np.cos(inc), speed_frac * vc * np.sin(inc)])
    noise = rng.normal(size=(n_release, {1: 4, 2: 6}.get(df, 12)))
    pert = np.concatenate([rng.normal(0.0, 0.1, (2 * n_release, 3)), rng.normal(0.0, 2 * KMS, (2 * n_release, 3))],
                          axis=1)
    return StreamSetup(w_now, 0.0, dt, n_release, prog_m, prog_b, noise, pert, int(df))
