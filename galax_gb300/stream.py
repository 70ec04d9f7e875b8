"""Mock streams with a moving progenitor, and their gradients, on the GPU.

Mirrors the pipeline of galax's ``StreamSimulator`` (init: progenitor orbit to
the release times, release conditions; run: every particle to the present;
src/galax/dynamics/_src/experimental/stream.py:121-446) with the progenitor's
own Plummer potential moved along its orbit (legacy/mockstream/_moving.py and
``MockStreamGenerator``), on a constant-step grid of release times. Release
conditions use the King (1962) tidal radius
(dynamics/_src/cluster/radius.py:198-214): for release r, particles 2r
(leading) and 2r + 1 (trailing) start at
``x_prog -/+ r_t rhat + 0.1 r_t xi`` with velocity ``v_prog + 0.1 Omega r_t eta``.

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


def config(*, n_release: int, dt: float, w_now, prog_m: float, prog_b: float, t_now: float = 0.0,
           method: int = 8, k_ckpt: int = 256) -> _lib.StreamConfig:
    w = np.asarray(w_now, np.float64).reshape(6)
    return _lib.StreamConfig(int(method), int(k_ckpt), int(n_release), float(dt), float(t_now), float(prog_m),
                             float(prog_b), (C.c_double * 6)(*w.tolist()))


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


def _noise_soa(noise, n_release: int):
    torch = _torch()
    nz = _as_cuda(noise, torch.float64).reshape(n_release, 12)
    return nz.t().contiguous()


def simulate(pot: AbstractPotential, cfg: _lib.StreamConfig, noise) -> StreamResult:
    """Forward stream: ``noise`` (n_release, 12) standard-normal draws (xi_lead,
    eta_lead, xi_trail, eta_trail). NumPy in, NumPy out; CUDA tensors stay on
    the device."""
    torch = _torch()
    is_np = not isinstance(noise, torch.Tensor)
    n = int(cfg.n_release)
    L = _lib.load()
    h = pot.handle()
    nb = C.c_size_t()
    _lib.check(L.gal_stream_workspace_size(h, C.byref(cfg), 0, C.byref(nb)), "gal_stream_workspace_size")
    ws = _WS.get(nb.value)
    nz = _noise_soa(noise, n)
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
    nz = _noise_soa(noise, n)
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
