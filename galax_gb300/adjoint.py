"""Gradients through orbits: the hand-written discrete adjoint of the CUDA library.

Two entry points:

* ``orbit_adjoint`` — one call that integrates forward with checkpoints and runs
  the reverse sweep, for a terminal loss sum |y(t1) - target|^2 (or any given
  cotangent dL/dy(t1)); returns the final states, dL/dy0 and dL/d(parameters).
* ``OrbitMap`` — a ``torch.autograd.Function`` y0, params -> y(t1) whose backward
  calls the same adjoint kernel, so orbits sit inside torch losses and
  optimisers.

Parameters are the component table's (m, l1, l2) per component, in the order
of ``pot.components()``; for a potential with LinearParameter slopes they are
(m, l1, l2) at t = 0 followed by the three slopes, six per component, and
every stage is evaluated at its own time. galax differentiates through diffrax
instead (ForwardMode by default, src/galax/dynamics/_src/orbit/solver.py:133).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .dynamics import Workspace, _as_cuda, on_stream
from .potential import AbstractPotential, CompositePotential, from_component_array


def _torch():
    import torch

    return torch


@dataclass
class AdjointResult:
    yT: object          # (n, 6)
    grad_y0: object     # (n, 6)
    grad_params: object  # (ncomp, 3): d/d(m, l1, l2); (ncomp, 6) with d/d(slopes) for time-dependent potentials
    loss: float | None


_WS = Workspace()


def _run(pot, y0_soa, t0, t1, dt, method, k_ckpt, lam_soa=None, target_soa=None, stream=None):
    torch = _torch()
    if stream is not None and stream != torch.cuda.current_stream().cuda_stream:
        with on_stream(stream):
            return _run(pot, y0_soa, t0, t1, dt, method, k_ckpt, lam_soa, target_soa)
    n = y0_soa.shape[1]
    cfg = _lib.solver_config(method, False, dt0=dt)
    L = _lib.load()
    h = pot.handle()
    nb = C.c_size_t()
    _lib.check(L.gal_adjoint_workspace_size(h, C.byref(cfg), float(t0), float(t1), int(k_ckpt), n, C.byref(nb)),
               "gal_adjoint_workspace_size")
    ws = _WS.get(nb.value)
    yT = torch.empty((6, n), dtype=torch.float64, device="cuda")
    gy = torch.empty((6, n), dtype=torch.float64, device="cuda")
    ncomp = len(pot.components())
    gp = torch.empty((ncomp, 6 if L.gal_potential_is_time_dependent(h) else 3), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(
        L.gal_adjoint(
            h, C.byref(cfg), y0_soa.data_ptr(), float(t0), float(t1),
            lam_soa.data_ptr() if lam_soa is not None else None,
            target_soa.data_ptr() if target_soa is not None else None,
            yT.data_ptr(), gy.data_ptr(), gp.data_ptr(), int(k_ckpt), n, ws.data_ptr(), ws.numel(), st,
        ),
        "gal_adjoint",
    )
    return yT, gy, gp


def orbit_adjoint(pot: AbstractPotential, y0, t0: float, t1: float, *, dt: float, target=None, cotangent=None,
                  method: int = 8, k_ckpt: int = 256) -> AdjointResult:
    """Forward + reverse sweep for n orbits with constant step ``dt``.

    Give ``target`` (n, 6) for the loss sum |y(t1) - target|^2, or ``cotangent``
    (n, 6) = dL/dy(t1) for any other loss. NumPy in, NumPy out; CUDA tensors stay
    on the device.
    """
    torch = _torch()
    is_np = not isinstance(y0, torch.Tensor)
    y = _as_cuda(y0, torch.float64).reshape(-1, 6).t().contiguous()
    lam = tgt = None
    if cotangent is not None:
        lam = _as_cuda(cotangent, torch.float64).reshape(-1, 6).t().contiguous()
    elif target is not None:
        tgt = _as_cuda(target, torch.float64).reshape(-1, 6).t().contiguous()
    else:
        raise ValueError("give target or cotangent")
    yT, gy, gp = _run(pot, y, t0, t1, dt, method, k_ckpt, lam, tgt)
    loss = float(((yT - tgt) ** 2).sum()) if tgt is not None else None
    res = AdjointResult(yT.t(), gy.t(), gp, loss)
    if is_np:
        res = AdjointResult(res.yT.cpu().numpy(), res.grad_y0.cpu().numpy(), gp.cpu().numpy(), loss)
    return res


class OrbitMap:
    """y(t1) = Phi(y0; params) as a differentiable torch op (constant step).
    ``params`` is ``params_of(pot)``: (ncomp, 3), or (ncomp, 6) with the
    LinearParameter slopes of a time-dependent potential."""

    @staticmethod
    def apply(pot: AbstractPotential, y0, params, t0: float, t1: float, dt: float, method: int = 8,
              k_ckpt: int = 256):
        torch = _torch()

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, y0_, params_):
                p = _with_params(pot, params_)
                y = y0_.detach().to(torch.float64).reshape(-1, 6).t().contiguous()
                from .dynamics import integrate

                cfg = _lib.solver_config(method, False, dt0=dt)
                out, status, _ = integrate(p, y, t0, t1, torch.tensor([float(t1)], dtype=torch.float64), cfg,
                                           soa=True)
                ctx.save_for_backward(y0_, params_)
                ctx.pot = p
                return out[:, 0, :].t().contiguous()

            @staticmethod
            def backward(ctx, gout):
                y0_, params_ = ctx.saved_tensors
                y = y0_.detach().to(torch.float64).reshape(-1, 6).t().contiguous()
                lam = gout.detach().to(torch.float64).reshape(-1, 6).t().contiguous()
                _, gy, gp = _run(ctx.pot, y, t0, t1, dt, method, k_ckpt, lam_soa=lam)
                return gy.t().reshape(y0_.shape), gp.reshape(params_.shape)

        return _Fn.apply(y0, params)


def _with_params(pot: AbstractPotential, params) -> AbstractPotential:
    """A potential with the same component kinds and origins but parameters
    ``params``: (ncomp, 3) values, or (ncomp, 6) values at t = 0 and slopes."""
    arr = pot.component_array().copy()
    p = params.detach().cpu().numpy() if hasattr(params, "detach") else np.asarray(params)
    p = p.reshape(len(arr), -1)
    arr["m"], arr["l1"], arr["l2"] = p[:, 0], p[:, 1], p[:, 2]
    if p.shape[1] != 6:
        return from_component_array(arr, G=pot.G)
    return _WithSlopes(from_component_array(arr, G=pot.G, slopes=p[:, 3:6]), p[:, 3:6])


class _WithSlopes(CompositePotential):
    """A component table with explicit LinearParameter slopes, kept even when
    they are all zero, so that the adjoint differentiates with respect to them."""

    def __init__(self, table: AbstractPotential, slopes):
        super().__init__({"table": table}, constants=table.constants)
        self._sl = np.ascontiguousarray(slopes, np.float64).reshape(-1, 3)

    def slopes(self):
        return self._sl


def params_of(pot: AbstractPotential):
    """The parameter tensor of ``pot`` on the GPU: (ncomp, 3) = (m, l1, l2), or
    (ncomp, 6) = (m, l1, l2) at t = 0 and their slopes when ``pot`` has
    LinearParameter time dependence."""
    torch = _torch()
    arr = pot.component_array()
    vals = np.stack([arr["m"], arr["l1"], arr["l2"]], axis=1)
    sl = pot.slopes()
    if sl is not None:
        vals = np.concatenate([vals, np.asarray(sl, np.float64).reshape(len(arr), 3)], axis=1)
    return torch.tensor(vals, dtype=torch.float64, device="cuda")
