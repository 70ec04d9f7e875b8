"""ctypes front end of the CPU FP64 oracle (test infrastructure only).

The oracle restates galax's potentials, Hamiltonian field and the diffrax
Runge-Kutta / PID-controller arithmetic in C++ (``galax_oracle.cpp``). Only the
test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, to check and to time the CUDA library against; the
``galax_gb300`` package never does.

Component records use the same 56-byte layout as the CUDA library's
``gal_component`` (kind, flags, mass, l1, l2, origin[3]).
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

KEPLER, HERNQUIST, MIYAMOTO_NAGAI, NFW, PLUMMER, ISOCHRONE, LOGARITHMIC, POWERLAW_CUTOFF = range(8)

G_GALACTIC = 4.498502151469553e-12  # kpc^3 / (Msun Myr^2), astropy CODATA-2018 G

COMP_DTYPE = np.dtype(
    [("kind", "<i4"), ("flags", "<i4"), ("m", "<f8"), ("l1", "<f8"), ("l2", "<f8"), ("origin", "<f8", (3,))],
    align=True,
)
assert COMP_DTYPE.itemsize == 56


class SolverCfg(C.Structure):
    _fields_ = [
        ("method", C.c_int32),
        ("adaptive", C.c_int32),
        ("max_steps", C.c_int64),
        ("dt0", C.c_double),
        ("rtol", C.c_double),
        ("atol", C.c_double),
        ("dtmin", C.c_double),
        ("dtmax", C.c_double),
        ("pcoeff", C.c_double),
        ("icoeff", C.c_double),
        ("dcoeff", C.c_double),
        ("safety", C.c_double),
        ("factormin", C.c_double),
        ("factormax", C.c_double),
        ("force_dtmin", C.c_int32),
        ("lockstep", C.c_int32),
    ]


def solver_cfg(
    method: int = 8,
    adaptive: bool = True,
    *,
    dt0: float = 0.0,
    rtol: float = 1e-7,
    atol: float = 1e-7,
    dtmin: float = 0.0,
    dtmax: float = 0.0,
    pcoeff: float = 0.0,
    icoeff: float = 1.0,
    dcoeff: float = 0.0,
    safety: float = 0.9,
    factormin: float = 0.2,
    factormax: float = 10.0,
    force_dtmin: bool = True,
    max_steps: int = 2**62,
    lockstep: bool = False,
) -> SolverCfg:
    return SolverCfg(
        method, int(adaptive), max_steps, dt0, rtol, atol, dtmin, dtmax, pcoeff, icoeff, dcoeff, safety,
        factormin, factormax, int(force_dtmin), int(lockstep),
    )


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(str(path))
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        cp = np.ctypeslib.ndpointer(COMP_DTYPE, flags="C_CONTIGUOUS")
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        for name in ("orc_potential", "orc_gradient", "orc_hessian"):
            getattr(L, name).argtypes = [cp, C.c_int, C.c_double, dp, C.c_int64, dp, C.c_void_p, C.c_double]
            getattr(L, name).restype = None
        L.orc_dgrad_dparams.argtypes = [cp, C.c_int, C.c_double, dp, dp, C.c_int64, dp]
        L.orc_tableau.argtypes = [C.c_int, dp, dp, dp, dp]
        L.orc_tableau.restype = C.c_int
        L.orc_dopri5_cmid.argtypes = [dp]
        L.orc_integrate.argtypes = [
            cp, C.c_int, C.c_double, C.POINTER(SolverCfg), dp, dp, dp, i64p, dp, dp, i32p, i64p, i64p,
            C.c_int64, C.c_int, C.c_void_p,
        ]
        L.orc_integrate.restype = C.c_int
        L.orc_count_ops.argtypes = [cp, C.c_int, C.c_double, C.c_int, dp, i64p]
        L.orc_adjoint_fixed.argtypes = [
            cp, C.c_int, C.c_double, C.POINTER(SolverCfg), dp, C.c_double, C.c_double, dp, dp, dp, dp,
            C.c_int64, C.c_int, C.c_void_p, C.c_void_p,
        ]
        L.orc_adjoint_fixed.restype = C.c_int
        _lib = L
    return _lib


def comps(records) -> np.ndarray:
    """Build a component array from (kind, m, l1, l2, origin) tuples."""
    a = np.zeros(len(records), COMP_DTYPE)
    for i, r in enumerate(records):
        kind, m, l1, l2 = r[:4]
        origin = r[4] if len(r) > 4 else (0.0, 0.0, 0.0)
        a[i]["kind"] = kind
        a[i]["m"] = m
        a[i]["l1"] = l1
        a[i]["l2"] = l2
        a[i]["origin"] = origin
    return a


# Smith et al. (2015) three-Miyamoto-Nagai fits as galax tabulates them
# (src/galax/potential/_src/builtin/mn3.py:27-51): mass fractions and a / h_R
# as quartics in b / h_R, which is a cubic in h_z / h_R.
MN3_K = {
    True: np.array([[0.0036, -0.0330, 0.1117, -0.1335, 0.1749], [-0.0131, 0.1090, -0.3035, 0.2921, -5.7976],
                    [-0.0048, 0.0454, -0.1425, 0.1012, 6.7120], [-0.0158, 0.0993, -0.2070, -0.7089, 0.6445],
                    [-0.0319, 0.1514, -0.1279, -0.9325, 2.6836], [-0.0326, 0.1816, -0.2943, -0.6329, 2.3193]]),
    False: np.array([[-0.0090, 0.0640, -0.1653, 0.1164, 1.9487], [0.0173, -0.0903, 0.0877, 0.2029, -1.3077],
                     [-0.0051, 0.0287, -0.0361, -0.0544, 0.2242], [-0.0358, 0.2610, -0.6987, -0.1193, 2.0074],
                     [-0.0830, 0.4992, -0.7967, -1.2966, 4.4441], [-0.0247, 0.1718, -0.4124, -0.5944, 0.7333]]),
}
MN3_B = {"exponential": np.array([-0.269, 1.08, 1.092]), "sech2": np.array([-0.033, 0.262, 0.659])}


def mn3(m_tot: float, h_R: float, h_z: float, profile: str = "sech2", positive_density: bool = False):  # noqa: N803
    """Component records of galax's MN3ExponentialPotential / MN3Sech2Potential
    (builtin/mn3.py:54-133): three Miyamoto-Nagai disks."""
    q = h_z / h_R
    b_hR = MN3_B[profile] @ np.array([q**3, q**2, q])
    pv = MN3_K[bool(positive_density)] @ np.vander([b_hR], N=5)[0]
    return [(MIYAMOTO_NAGAI, pv[i] * m_tot, pv[3 + i] * h_R, b_hR * h_R) for i in range(3)]


def milky_way_2022() -> np.ndarray:
    """galax MilkyWayPotential2022 defaults (builtin/milkyway.py:239-313): MN3Sech2
    disk (positive density), NFW halo, Hernquist bulge and nucleus."""
    return comps(mn3(4.7717e10, 2.6, 0.3, "sech2", True) + [
        (NFW, 5.5427e11, 15.626, 0.0),
        (HERNQUIST, 5e9, 1.0, 0.0),
        (HERNQUIST, 1.8142e9, 0.0688867, 0.0),
    ])


def gamma_p(a: float, x: float):
    """(P(a, x), dP/da, Gamma(a, x)) from the oracle's incomplete gamma."""
    L = lib()
    out = np.zeros(3)
    L.orc_gamma_p.argtypes = [C.c_double, C.c_double, np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")]
    L.orc_gamma_p(float(a), float(x), out)
    return out


def bovy_mw_2014() -> np.ndarray:
    """galax BovyMWPotential2014 defaults (builtin/milkyway.py:33-98): Miyamoto-Nagai
    disk, power law with cutoff bulge (alpha 1.8, r_c 1.9 kpc), NFW halo."""
    return comps([
        (MIYAMOTO_NAGAI, 68_193_902_782.346756, 3.0, 0.28),
        (POWERLAW_CUTOFF, 4501365375.06545, 1.9, 1.8),
        (NFW, 4.3683325e11, 16.0, 0.0),
    ])


def milky_way(**over) -> np.ndarray:
    """galax MilkyWayPotential defaults, component order disk, halo, bulge, nucleus
    (src/galax/potential/_src/builtin/milkyway.py:203-229)."""
    d = dict(disk=(6.8e10, 3.0, 0.28), halo=(5.4e11, 15.62), bulge=(5e9, 1.0), nucleus=(1.71e9, 0.07))
    d.update(over)
    return comps([
        (MIYAMOTO_NAGAI, d["disk"][0], d["disk"][1], d["disk"][2]),
        (NFW, d["halo"][0], d["halo"][1], 0.0),
        (HERNQUIST, d["bulge"][0], d["bulge"][1], 0.0),
        (HERNQUIST, d["nucleus"][0], d["nucleus"][1], 0.0),
    ])


def _xyz(x):
    x = np.ascontiguousarray(np.atleast_2d(np.asarray(x, np.float64)))
    assert x.shape[-1] == 3
    return x.reshape(-1, 3)


def _slopes_ptr(c: np.ndarray, slopes):
    """(keep-alive array, pointer) for per-component d(m, l1, l2)/dt, or (None, None)."""
    if slopes is None:
        return None, None
    a = np.ascontiguousarray(slopes, np.float64).reshape(len(c), 3)
    return a, a.ctypes.data


def potential(c: np.ndarray, x, G: float = G_GALACTIC, *, slopes=None, t: float = 0.0) -> np.ndarray:
    """Phi at x (n, 3) and time t; ``slopes`` (ncomp, 3) makes (m, l1, l2)
    linear in time with the table holding their values at t = 0."""
    x = _xyz(x)
    out = np.empty(len(x))
    keep, sp = _slopes_ptr(c, slopes)
    lib().orc_potential(np.ascontiguousarray(c), len(c), G, x, len(x), out, sp, float(t))
    return out


def gradient(c: np.ndarray, x, G: float = G_GALACTIC, *, slopes=None, t: float = 0.0) -> np.ndarray:
    x = _xyz(x)
    out = np.empty((len(x), 3))
    keep, sp = _slopes_ptr(c, slopes)
    lib().orc_gradient(np.ascontiguousarray(c), len(c), G, x, len(x), out, sp, float(t))
    return out


def hessian(c: np.ndarray, x, G: float = G_GALACTIC, *, slopes=None, t: float = 0.0) -> np.ndarray:
    x = _xyz(x)
    out = np.empty((len(x), 3, 3))
    keep, sp = _slopes_ptr(c, slopes)
    lib().orc_hessian(np.ascontiguousarray(c), len(c), G, x, len(x), out, sp, float(t))
    return out


def dgrad_dparams(c: np.ndarray, x, v, G: float = G_GALACTIC) -> np.ndarray:
    """d(grad Phi(x) . v)/d(m, l1, l2) per component: shape (n, ncomp, 3)."""
    x = _xyz(x)
    v = _xyz(v)
    out = np.empty((len(x), len(c), 3))
    lib().orc_dgrad_dparams(np.ascontiguousarray(c), len(c), G, x, v, len(x), out)
    return out


def tableau(method: int):
    c = np.zeros(13); a = np.zeros(169); b = np.zeros(13); e = np.zeros(13)
    s = lib().orc_tableau(method, c, a, b, e)
    return c[:s], a.reshape(13, 13)[:s, :s], b[:s], e[:s]


def dopri5_cmid() -> np.ndarray:
    out = np.zeros(7)
    lib().orc_dopri5_cmid(out)
    return out


def integrate(
    c: np.ndarray,
    y0,
    t0,
    t1,
    save_ts,
    cfg: SolverCfg,
    *,
    G: float = G_GALACTIC,
    nthreads: int = 0,
    slopes=None,
    flat: bool = False,
):
    """Integrate orbits. ``save_ts`` is a list of per-orbit 1-D arrays or a
    single 1-D array shared by all orbits. Returns (saves list of (T_i, 6),
    status, accepted, rejected); in lockstep mode saves is (T, n, 6).
    ``slopes`` (ncomp, 3): linear time dependence of (m, l1, l2).
    ``flat``: return the saves as one (sum T_i, 6) array in orbit order instead
    of a list."""
    y0 = np.ascontiguousarray(np.atleast_2d(np.asarray(y0, np.float64)))
    n = len(y0)
    t0 = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, np.float64), (n,)))
    t1 = np.ascontiguousarray(np.broadcast_to(np.asarray(t1, np.float64), (n,)))
    if isinstance(save_ts, np.ndarray) and save_ts.ndim == 1:
        save_list = [save_ts] * n
    else:
        save_list = [np.asarray(s, np.float64).ravel() for s in save_ts]
    offs = np.zeros(n + 1, np.int64)
    offs[1:] = np.cumsum([len(s) for s in save_list])
    ts_flat = np.ascontiguousarray(np.concatenate(save_list) if n else np.zeros(0))
    status = np.zeros(n, np.int32)
    acc = np.zeros(n, np.int64)
    rej = np.zeros(n, np.int64)
    if cfg.lockstep:
        ns = len(save_list[0])
        out = np.empty((ns, n, 6))
    else:
        out = np.empty((int(offs[-1]), 6))
    keep, sp = _slopes_ptr(c, slopes)
    lib().orc_integrate(
        np.ascontiguousarray(c), len(c), G, C.byref(cfg), y0, t0, t1, offs, ts_flat, out, status, acc, rej, n,
        nthreads, sp,
    )
    if cfg.lockstep or flat:
        return out, status, acc, rej
    return [out[offs[i]:offs[i + 1]] for i in range(n)], status, acc, rej


def adjoint_fixed(
    c: np.ndarray,
    y0,
    t0: float,
    t1: float,
    target,
    cfg: SolverCfg,
    *,
    G: float = G_GALACTIC,
    nthreads: int = 0,
    slopes=None,
):
    """Discrete adjoint of constant steps ``cfg.dt0`` from t0 to t1 for the loss
    L = sum_i |y_i(t1) - target_i|^2. Returns (yT (n,6), dL/dy0 (n,6),
    dL/dparams, L). dL/dparams is (ncomp, 3), d/d(m, l1, l2); with ``slopes``
    (ncomp, 3) of LinearParameter time dependence it is (ncomp, 6): d/d(m, l1,
    l2) at t = 0, then d/d(slopes)."""
    y0 = np.ascontiguousarray(np.atleast_2d(np.asarray(y0, np.float64)))
    target = np.ascontiguousarray(np.asarray(target, np.float64).reshape(y0.shape))
    n = len(y0)
    yT = np.empty_like(y0)
    gy = np.empty_like(y0)
    gp = np.zeros((len(c), 3))
    gs = np.zeros((len(c), 3))
    keep, sp = _slopes_ptr(c, slopes)
    lib().orc_adjoint_fixed(
        np.ascontiguousarray(c), len(c), G, C.byref(cfg), y0, float(t0), float(t1), target, yT, gy,
        gp.reshape(-1), n, nthreads, sp, gs.ctypes.data if sp else None,
    )
    del keep
    L = float(np.sum((yT - target) ** 2))
    return yT, gy, (np.concatenate([gp, gs], axis=1) if sp else gp), L


def count_ops(c: np.ndarray, method: int, y=(8.0, 1.0, 0.5, 0.0, 0.2, 0.01), G: float = G_GALACTIC):
    """Algorithmic FP64 operation counts: dict for one gradient and one step."""
    out = np.zeros(10, np.int64)
    lib().orc_count_ops(np.ascontiguousarray(c), len(c), G, method, np.asarray(y, np.float64), out)
    keys = ("add", "mul", "div", "sqrt", "log1p")
    return dict(zip(keys, out[:5].tolist())), dict(zip(keys, out[5:].tolist()))


def nthreads_default() -> int:
    return os.cpu_count() or 1


def stream_forward(c: np.ndarray, setup, *, method: int = 8, G: float = G_GALACTIC, nthreads: int = 0):
    """The stream pipeline with a moving progenitor on the CPU (see
    orc_stream_forward). ``setup`` carries w_now, t_now, dt, n_release,
    prog_m, prog_b, noise. Returns dict(track (n_rel+1, 6), rt_om (n_rel, 2),
    ics (2 n_rel, 6), final (2 n_rel, 6))."""
    L = lib()
    if not hasattr(L, "_stream_bound"):
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        cp = np.ctypeslib.ndpointer(COMP_DTYPE, flags="C_CONTIGUOUS")
        L.orc_stream_forward.argtypes = [cp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double, dp, C.c_double,
                                         C.c_double, C.c_int64, C.c_int, dp, dp, dp, dp, dp, dp, C.c_int]
        L.orc_stream_forward.restype = C.c_int
        L._stream_bound = True
    n = int(setup.n_release)
    df, dfp = _df_of(setup)
    track = np.empty((n + 1, 6))
    rt_om = np.empty((n, 2))
    ics = np.empty((2 * n, 6))
    final = np.empty((2 * n, 6))
    noise = np.ascontiguousarray(setup.noise, np.float64).reshape(n, NOISE_COLUMNS.get(df, 12))
    L.orc_stream_forward(np.ascontiguousarray(c), len(c), G, method, float(setup.prog_m), float(setup.prog_b),
                         np.ascontiguousarray(setup.w_now, np.float64), float(setup.t_now), float(setup.dt), n, df,
                         dfp, noise, track, rt_om, ics, final, nthreads)
    return dict(track=track, rt_om=rt_om, ics=ics, final=final)


STREAM_DF_OFFSETS, STREAM_DF_FARDAL2015, STREAM_DF_CHEN2024 = 0, 1, 2
NOISE_COLUMNS = {STREAM_DF_OFFSETS: 12, STREAM_DF_FARDAL2015: 4, STREAM_DF_CHEN2024: 6}
FARDAL2015_DEFAULTS = (2.0, 0.3, 0.0, 0.0, 0.5, 0.5, 0.5, 0.5)


def _df_of(setup):
    df = int(getattr(setup, "df", STREAM_DF_OFFSETS))
    p = getattr(setup, "df_params", None)
    p = FARDAL2015_DEFAULTS if p is None else p
    return df, np.ascontiguousarray(p, np.float64).reshape(8)


def stream_df_sample(c: np.ndarray, w, mass, noise, *, df: int = STREAM_DF_FARDAL2015, df_params=None,
                     G: float = G_GALACTIC):
    """Release conditions at n progenitor points w (n, 6) with masses (n,):
    returns (lead (n, 6), trail (n, 6), r_tidal (n,)) (see orc_stream_df_sample)."""
    L = lib()
    if not hasattr(L, "_df_bound"):
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        cp = np.ctypeslib.ndpointer(COMP_DTYPE, flags="C_CONTIGUOUS")
        L.orc_stream_df_sample.argtypes = [cp, C.c_int, C.c_double, C.c_int, dp, dp, dp, dp, C.c_int64, dp, dp, dp]
        L.orc_stream_df_sample.restype = C.c_int
        L._df_bound = True
    w = np.ascontiguousarray(w, np.float64).reshape(-1, 6)
    n = len(w)
    mass = np.ascontiguousarray(np.broadcast_to(np.asarray(mass, np.float64), (n,)))
    noise = np.ascontiguousarray(noise, np.float64).reshape(n, NOISE_COLUMNS.get(df, 12))
    p = np.ascontiguousarray(FARDAL2015_DEFAULTS if df_params is None else df_params, np.float64).reshape(8)
    lead, trail, rt = np.empty((n, 6)), np.empty((n, 6)), np.empty(n)
    L.orc_stream_df_sample(np.ascontiguousarray(c), len(c), G, int(df), p, w, mass, noise, n, lead, trail, rt)
    return lead, trail, rt


def stream_loss(c: np.ndarray, setup, target, **kw) -> float:
    f = stream_forward(c, setup, **kw)["final"]
    return float(np.sum((f - target) ** 2))


def stream_fd_grad(c: np.ndarray, setup, target, params, *, rel_h: float = 1e-5, **kw) -> np.ndarray:
    """Central finite differences of the stream loss with one Richardson
    extrapolation, for parameters given as (component, field) pairs with field
    in ("m", "l1", "l2"). Returns an array of len(params)."""
    out = []
    for ci, fld in params:
        x0 = float(c[ci][fld])

        def d(h):
            cp_, cm_ = c.copy(), c.copy()
            cp_[ci][fld] = x0 + h
            cm_[ci][fld] = x0 - h
            return (stream_loss(cp_, setup, target, **kw) - stream_loss(cm_, setup, target, **kw)) / (2 * h)

        h = rel_h * abs(x0)
        out.append((4.0 * d(h / 2) - d(h)) / 3.0)
    return np.array(out)


def plummer_short_range(c: np.ndarray, x, r_cut: float, G: float = G_GALACTIC, *, magnitudes: bool = False):
    """Short-range part sum_i Phi_i S(d_i / r_cut), S(q) = (1 - q^2)^3 for q < 1,
    of Plummer components (direct sum over all of them, no cell lists): returns
    (phi (n,), grad (n, 3)), and with magnitudes=True also, over the spheres
    within r_cut, the sums of the untapered scales |Phi_i| and
    |grad Phi_i| + |Phi_i| 6 |d| / r_cut^2 (the scales of each term's rounding:
    near the taper's edge t = 1 - q^2 cancels, so S itself carries a large
    relative but tiny absolute error). Restates the surrogate's split of
    Phi_i = -G m_i / sqrt(d^2 + b_i^2) (galax builtin/plummer.py:122-133)."""
    x = _xyz(x)
    phi = np.zeros(len(x))
    g = np.zeros((len(x), 3))
    mphi = np.zeros(len(x))
    mg = np.zeros(len(x))
    for comp in c:
        d = x - np.asarray(comp["origin"])
        d2 = np.sum(d * d, axis=1)
        q2 = d2 / r_cut**2
        inside = q2 < 1.0
        t = np.where(inside, 1.0 - q2, 0.0)
        S = t**3
        s2 = d2 + np.finfo(float).tiny + comp["l1"] ** 2
        Gm = G * comp["m"]
        ph = -Gm / np.sqrt(s2)
        phi += ph * S
        # grad(Phi S) = S grad Phi + Phi grad S, grad S = -6 t^2 d / r_cut^2
        gi = (S * Gm / s2**1.5)[:, None] * d + (ph * (-6.0 * t**2 / r_cut**2))[:, None] * d
        g += gi
        dn = np.sqrt(d2)
        mphi += np.where(inside, np.abs(ph), 0.0)
        mg += np.where(inside, Gm * dn / s2**1.5 + np.abs(ph) * 6.0 * dn / r_cut**2, 0.0)
    return (phi, g, mphi, mg) if magnitudes else (phi, g)
