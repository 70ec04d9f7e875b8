"""Mock streams with a moving progenitor, and their gradients, on the GPU.

Mirrors the pipeline of galax's ``StreamSimulator`` (init: progenitor orbit to
the release times, release conditions; run: every particle to the present;
src/galax/dynamics/_src/experimental/stream.py:121-446) with the progenitor's
own Plummer potential moved along its orbit (legacy/mockstream/_moving.py and
``MockStreamGenerator``), on a constant-step grid of release times. Release
conditions use the King (1962) tidal radius
(dynamics/_src/cluster/radius.py:198-214) and one of three release models for
particles 2r (leading) and 2r + 1 (trailing) of release r:

- "offsets": ``x_prog -/+ r_t rhat + 0.1 r_t xi`` with velocity
  ``v_prog + 0.1 Omega r_t eta``;
- "fardal2015": galax's Fardal (2015) DF (legacy/mockstream/df/fardal15.py,
  experimental/df.py);
- "chen2024": galax's Chen (2024) DF (legacy/mockstream/df/chen24.py).

``df_sample`` evaluates a release model alone at any batch of progenitor
points.

``simulate`` runs the forward pipeline (``gal_stream_run``); ``gradient``
returns dL/d(component parameters) of L = sum_p |y_p(t_now) - target_p|^2
through particles, release conditions and the progenitor orbit
(``gal_stream_grad``, a hand-written discrete adjoint; galax would take jax
derivatives, ForwardMode by default).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .dynamics import Workspace, _as_cuda
from .potential import AbstractPotential


def _torch():
    import torch

    return torch


DFS = {"offsets": _lib.STREAM_DF_OFFSETS, "fardal2015": _lib.STREAM_DF_FARDAL2015,
       "chen2024": _lib.STREAM_DF_CHEN2024}
# kr_bar, kvphi_bar, kz_bar, kvz_bar, sigma_kr, sigma_kvphi, sigma_kz, sigma_kvz
# (galax's defaults, legacy/mockstream/df/fardal15.py:26-35, experimental/df.py:57-64)
FARDAL2015_DEFAULTS = (2.0, 0.3, 0.0, 0.0, 0.5, 0.5, 0.5, 0.5)
NOISE_COLUMNS = {_lib.STREAM_DF_OFFSETS: 12, _lib.STREAM_DF_FARDAL2015: 4, _lib.STREAM_DF_CHEN2024: 6}


def _df_code(df) -> int:
    if isinstance(df, str):
        if df not in DFS:
            raise ValueError(f"unknown stream DF {df!r}; expected one of {sorted(DFS)}")
        return DFS[df]
    return int(df)


def config(*, n_release: int, dt: float, w_now, prog_m: float, prog_b: float, t_now: float = 0.0,
           method: int = 8, k_ckpt: int = 256, df="offsets", df_params=None) -> _lib.StreamConfig:
    """``gal_stream_config``. ``df``: "offsets" (noise (n_release, 12)),
    "fardal2015" (noise (n_release, 4); ``df_params`` defaults to galax's
    Fardal values) or "chen2024" (noise (n_release, 6))."""
    w = np.asarray(w_now, np.float64).reshape(6)
    code = _df_code(df)
    p = FARDAL2015_DEFAULTS if df_params is None else tuple(float(v) for v in df_params)
    if len(p) != 8:
        raise ValueError("df_params has 8 values")
    return _lib.StreamConfig(int(method), int(k_ckpt), int(n_release), float(dt), float(t_now), float(prog_m),
                             float(prog_b), (C.c_double * 6)(*w.tolist()), code, 0, (C.c_double * 8)(*p))


@dataclass
class StreamResult:
    final: object        # (2 n_release, 6): particle states at t_now (leading, trailing interleaved)
    ics: object          # (2 n_release, 6): release conditions
    track: object        # (n_release + 1, 6): the progenitor's forwards track on the grid


@dataclass
class StreamGradient:
    final: object        # (2 n_release, 6)
    grad_params: object  # (ncomp, 3): dL/d(m, l1, l2) per host component
    grad_w_now: object   # (6,): dL/d(progenitor phase-space point at t_now)
    loss: float


_WS = Workspace()


def _noise_soa(noise, n_release: int, df: int):
    torch = _torch()
    nz = _as_cuda(noise, torch.float64).reshape(n_release, NOISE_COLUMNS.get(int(df), 12))
    return nz.t().contiguous()


def simulate(pot: AbstractPotential, cfg: _lib.StreamConfig, noise) -> StreamResult:
    """Forward stream: ``noise`` holds standard-normal draws per release,
    (n_release, 12) for the offsets model (xi_lead, eta_lead, xi_trail,
    eta_trail), (n_release, 4) for Fardal 2015 (kr, kvphi, kz, kvz) or
    (n_release, 6) for Chen 2024 (standard normals behind posvel). NumPy
    in, NumPy out; CUDA tensors stay on the device."""
    torch = _torch()
    is_np = not isinstance(noise, torch.Tensor)
    n = int(cfg.n_release)
    L = _lib.load()
    h = pot.handle()
    nb = C.c_size_t()
    _lib.check(L.gal_stream_workspace_size(h, C.byref(cfg), 0, C.byref(nb)), "gal_stream_workspace_size")
    ws = _WS.get(nb.value)
    nz = _noise_soa(noise, n, cfg.df)
    fin = torch.empty((6, 2 * n), dtype=torch.float64, device="cuda")
    ics = torch.empty((6, 2 * n), dtype=torch.float64, device="cuda")
    track = torch.empty((n + 1, 6), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.gal_stream_run(h, C.byref(cfg), nz.data_ptr(), fin.data_ptr(), ics.data_ptr(), track.data_ptr(),
                                ws.data_ptr(), ws.numel(), st), "gal_stream_run")
    res = StreamResult(fin.t(), ics.t(), track)
    if is_np:
        res = StreamResult(res.final.cpu().numpy(), res.ics.cpu().numpy(), track.cpu().numpy())
    return res


def gradient(pot: AbstractPotential, cfg: _lib.StreamConfig, noise, target) -> StreamGradient:
    """Loss sum |y_p(t_now) - target_p|^2 over all 2 n_release particles and its
    gradient with respect to every host component's (m, l1, l2) and to the
    progenitor's present phase-space point."""
    torch = _torch()
    is_np = not isinstance(noise, torch.Tensor)
    n = int(cfg.n_release)
    L = _lib.load()
    h = pot.handle()
    nb = C.c_size_t()
    _lib.check(L.gal_stream_workspace_size(h, C.byref(cfg), 1, C.byref(nb)), "gal_stream_workspace_size")
    ws = _WS.get(nb.value)
    nz = _noise_soa(noise, n, cfg.df)
    tg = _as_cuda(target, torch.float64).reshape(2 * n, 6).t().contiguous()
    fin = torch.empty((6, 2 * n), dtype=torch.float64, device="cuda")
    ncomp = len(pot.components())
    gp = torch.empty((ncomp, 3), dtype=torch.float64, device="cuda")
    gw = torch.empty(6, dtype=torch.float64, device="cuda")
    loss = torch.empty(1, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.gal_stream_grad(h, C.byref(cfg), nz.data_ptr(), tg.data_ptr(), fin.data_ptr(), gp.data_ptr(),
                                 gw.data_ptr(), loss.data_ptr(), ws.data_ptr(), ws.numel(), st), "gal_stream_grad")
    if is_np:
        return StreamGradient(fin.t().cpu().numpy(), gp.cpu().numpy(), gw.cpu().numpy(), float(loss))
    return StreamGradient(fin.t(), gp, gw, loss)


def df_sample(pot: AbstractPotential, prog_w, prog_mass, noise, *, df="fardal2015", df_params=None):
    """Release conditions at n progenitor points ``prog_w`` (n, 6) with masses
    ``prog_mass`` (scalar or (n,)) from standard-normal ``noise`` ((n, 4) for
    Fardal 2015, (n, 6) for Chen 2024, (n, 12) for the offsets model): returns (lead (n, 6), trail
    (n, 6), r_tidal (n,)) (``gal_stream_df_sample``; FardalStreamDF._sample,
    legacy/mockstream/df/fardal15.py:49-94). NumPy in, NumPy out; CUDA
    tensors stay on the device."""
    torch = _torch()
    is_np = not isinstance(prog_w, torch.Tensor)
    code = _df_code(df)
    w = _as_cuda(prog_w, torch.float64).reshape(-1, 6)
    n = w.shape[0]
    ws = w.t().contiguous()
    m = _as_cuda(prog_mass, torch.float64).reshape(-1).expand(n).contiguous()
    nz = _as_cuda(noise, torch.float64).reshape(n, NOISE_COLUMNS.get(code, 12)).t().contiguous()
    p = FARDAL2015_DEFAULTS if df_params is None else tuple(float(v) for v in df_params)
    if len(p) != 8:
        raise ValueError("df_params has 8 values")
    pa = (C.c_double * 8)(*p)
    lead = torch.empty((6, n), dtype=torch.float64, device="cuda")
    trail = torch.empty((6, n), dtype=torch.float64, device="cuda")
    rt = torch.empty(n, dtype=torch.float64, device="cuda")
    L = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(L.gal_stream_df_sample(pot.handle(), code, C.addressof(pa), ws.data_ptr(), m.data_ptr(),
                                      nz.data_ptr(), n, lead.data_ptr(), trail.data_ptr(), rt.data_ptr(), st),
               "gal_stream_df_sample")
    lead, trail = lead.t(), trail.t()
    if is_np:
        return lead.cpu().numpy(), trail.cpu().numpy(), rt.cpu().numpy()
    return lead, trail, rt
