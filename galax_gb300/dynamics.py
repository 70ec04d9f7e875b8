"""Orbit integration with galax's public interface, run by the CUDA library.

Mirrors ``galax.dynamics.evaluate_orbit`` (src/galax/dynamics/_src/legacy/funcs.py:42-213),
the legacy ``Integrator`` (legacy/integrator.py:42-245), ``OrbitSolver``'s
defaults (orbit/solver.py:121-141) and the per-orbit save grids of
``experimental.integrate_orbit`` (experimental/integrate.py:301-575). The
solver and step-size-controller objects carry diffrax's names and fields
(``Dopri5``, ``Dopri8``, ``ConstantStepSize``, ``PIDController``).

Every orbit gets its own step-size controller (galax's per-orbit dispatch,
legacy/integrator.py:449-527); galax's batched ``evaluate_orbit`` with shared
start and end times instead advances the whole batch with one step size, so
adaptive results agree per orbit within the controller tolerance, not bitwise.
Fixed-step results agree to rounding.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Any, Sequence

import numpy as np

from . import _lib
from .potential import KMS_TO_KPC_MYR, AbstractPotential

# galax's legacy Integrator passes max_steps=None (unbounded); a GPU loop must end,
# so "unbounded" becomes this per-orbit bound on step attempts.
UNBOUNDED_MAX_STEPS = 2**20


def _torch():
    import torch

    return torch


# ---------------------------------------------------------------- solver objects
@dataclass(frozen=True)
class Dopri5:
    """Dormand-Prince 5(4), 7 stages, FSAL (diffrax.Dopri5)."""

    order: int = 5


@dataclass(frozen=True)
class Dopri8:
    """Prince-Dormand 8(7) 13-stage pair (diffrax.Dopri8)."""

    order: int = 8


@dataclass(frozen=True)
class ConstantStepSize:
    """Fixed step dt0 (diffrax.ConstantStepSize)."""


@dataclass(frozen=True)
class PIDController:
    """diffrax.PIDController fields, with diffrax's defaults."""

    rtol: float
    atol: float
    pcoeff: float = 0.0
    icoeff: float = 1.0
    dcoeff: float = 0.0
    dtmin: float | None = None
    dtmax: float | None = None
    force_dtmin: bool = True
    safety: float = 0.9
    factormin: float = 0.2
    factormax: float = 10.0
    step_ts: Any = None
    jump_ts: Any = None

    def __post_init__(self):
        if self.step_ts is not None or self.jump_ts is not None:
            raise NotImplementedError("step_ts / jump_ts are not supported on the GPU path")


def _method(solver) -> int:
    if isinstance(solver, (Dopri5, Dopri8)):
        return solver.order
    name = type(solver).__name__ if not isinstance(solver, str) else solver
    if name in ("Dopri5", "dopri5", "5"):
        return 5
    if name in ("Dopri8", "dopri8", "8"):
        return 8
    raise NotImplementedError(f"solver {name!r}: only Dopri5 and Dopri8 are implemented")


@dataclass
class Integrator:
    """galax's legacy Integrator (src/galax/dynamics/_src/legacy/integrator.py:161-168):
    Dopri8 with PIDController(rtol=1e-7, atol=1e-7) and no step limit by default."""

    solver: Any = field(default_factory=Dopri8)
    stepsize_controller: Any = field(default_factory=lambda: PIDController(rtol=1e-7, atol=1e-7))
    dt0: float | None = None
    max_steps: int | None = None
    # two-pass longest-remaining-first scheduling (identical results); None = on for adaptive runs
    schedule: bool | None = None

    def config(self) -> _lib.SolverConfig:
        method = _method(self.solver)
        max_steps = UNBOUNDED_MAX_STEPS if self.max_steps is None else int(self.max_steps)
        c = self.stepsize_controller
        if isinstance(c, ConstantStepSize):
            if not self.dt0 or self.dt0 <= 0:
                raise ValueError("ConstantStepSize needs dt0 > 0")
            return _lib.solver_config(method, False, dt0=self.dt0, max_steps=max_steps,
                                      schedule=bool(self.schedule))
        if isinstance(c, PIDController):
            return _lib.solver_config(
                method, True, dt0=self.dt0 or 0.0, rtol=c.rtol, atol=c.atol, dtmin=c.dtmin, dtmax=c.dtmax,
                pcoeff=c.pcoeff, icoeff=c.icoeff, dcoeff=c.dcoeff, safety=c.safety, factormin=c.factormin,
                factormax=c.factormax, force_dtmin=c.force_dtmin, max_steps=max_steps,
                schedule=True if self.schedule is None else self.schedule,
            )
        raise NotImplementedError(f"step-size controller {type(c).__name__} is not supported")


def OrbitSolver(solver=None, stepsize_controller=None, *, max_steps: int = 2**16, dt0=None) -> Integrator:
    """galax's OrbitSolver defaults (src/galax/dynamics/_src/orbit/solver.py:121-141):
    Dopri8, PIDController(rtol=1e-8, atol=1e-8), max_steps=2**16."""
    return Integrator(
        solver=solver or Dopri8(),
        stepsize_controller=stepsize_controller or PIDController(rtol=1e-8, atol=1e-8),
        dt0=dt0,
        max_steps=max_steps,
    )


# ---------------------------------------------------------------- containers
@dataclass
class PhaseSpaceCoordinate:
    """Host-side stand-in for gc.PhaseSpaceCoordinate: q (...,3) kpc, p (...,3) kpc/Myr, t (...) Myr."""

    q: Any
    p: Any
    t: Any = None


@dataclass
class Orbit:
    """Result of evaluate_orbit: q, p of shape (B, T, 3) (or (T, 3) for one orbit), times t (T,)."""

    q: Any
    p: Any
    t: Any
    status: Any = None
    steps: Any = None
    interpolant: Any = None

    @property
    def shape(self):
        return tuple(self.q.shape[:-1])

    @property
    def w(self):
        torch = _torch()
        if isinstance(self.q, torch.Tensor):
            return torch.cat([self.q, self.p], dim=-1)
        return np.concatenate([self.q, self.p], axis=-1)


def kms(v):
    """km/s -> kpc/Myr."""
    return np.asarray(v, np.float64) * KMS_TO_KPC_MYR


# ---------------------------------------------------------------- low level
class Workspace:
    """Device scratch reused across calls, grown on demand.

    One buffer per (device, current stream): calls queued on different streams
    never share scratch, and torch's caching allocator only hands a replaced
    buffer's memory to later work on the stream it was allocated on. The work
    using it must run on torch's current stream (``on_stream`` below makes an
    explicit stream current). The 16 most recently used streams keep theirs."""

    MAX_STREAMS = 16

    def __init__(self):
        self._bufs: dict = {}

    def get(self, nbytes: int):
        torch = _torch()
        key = (torch.cuda.current_device(), torch.cuda.current_stream().cuda_stream)
        buf = self._bufs.pop(key, None)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device="cuda")
        self._bufs[key] = buf  # most recently used last
        while len(self._bufs) > self.MAX_STREAMS:
            self._bufs.pop(next(iter(self._bufs)))
        return buf


def on_stream(stream):
    """Context in which torch's current stream is ``stream`` (a cudaStream_t
    handle as int, or None for no change), so that every temporary a call
    allocates is ordered with the kernels it launches there."""
    import contextlib

    torch = _torch()
    if stream is None or stream == torch.cuda.current_stream().cuda_stream:
        return contextlib.nullcontext()
    return torch.cuda.stream(torch.cuda.ExternalStream(stream))


_WS = Workspace()


def _as_cuda(x, dtype):
    torch = _torch()
    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=dtype)
    a = np.asarray(x)
    if not a.flags.writeable:  # broadcast views: torch wants writable memory
        a = a.copy()
    return torch.as_tensor(a, dtype=dtype, device="cuda")


def _in_place_or_cuda(x, dtype):
    """A contiguous pinned host tensor of the right dtype as it is (the kernels
    read it through unified addressing), anything else as a contiguous CUDA tensor."""
    torch = _torch()
    if isinstance(x, torch.Tensor) and not x.is_cuda and x.dtype == dtype and x.is_contiguous() and x.is_pinned():
        return x
    return _as_cuda(x, dtype).contiguous()


def _result_buffer(buf, shape, dtype, name):
    """A caller-given output (CUDA or pinned host, contiguous, right shape and
    dtype) or a new CUDA tensor."""
    torch = _torch()
    if buf is None:
        return torch.empty(shape, dtype=dtype, device="cuda")
    if not isinstance(buf, torch.Tensor) or buf.dtype != dtype or tuple(buf.shape) != tuple(shape):
        raise ValueError(f"{name} must be a {dtype} tensor of shape {tuple(shape)}")
    if not buf.is_contiguous() or not (buf.is_cuda or buf.is_pinned()):
        raise ValueError(f"{name} must be contiguous, on the GPU or in pinned host memory")
    return buf


def integrate(
    pot: AbstractPotential,
    y0,
    t0,
    t1,
    save_ts,
    cfg: _lib.SolverConfig,
    *,
    save_offsets=None,
    order=None,
    soa: bool = False,
    stream=None,
    workspace: Workspace | None = None,
    out=None,
    status=None,
):
    """Integrate n orbits on the current CUDA device.

    y0: (n, 6) (or (6, n) with ``soa=True``); t0, t1: scalars or (n,);
    save_ts: (T,) shared by all orbits, or the flat CSR values with
    ``save_offsets`` (n+1,). Returns (out, status, steps) with out of shape
    (6, T, n) for a shared grid or (6, total) for CSR saves. Asynchronous.

    ``out`` (float64) and ``status`` (int32), if given, receive the results in
    place: contiguous CUDA tensors of those shapes, or pinned host tensors,
    which the kernels then write directly (device-visible host memory under
    unified addressing), overlapping the transfer with the integration.
    Likewise ``save_ts`` (float64) and ``save_offsets`` (int64) may be
    contiguous pinned host tensors, which the kernels read in place: the save
    grid, usually the largest input, then crosses to the GPU while the orbits
    run instead of in a copy before them.

    ``stream`` (a cudaStream_t handle) runs the call on that stream instead of
    torch's current one; its temporaries are then allocated there too.
    """
    torch = _torch()
    if stream is not None and stream != torch.cuda.current_stream().cuda_stream:
        with on_stream(stream):
            return integrate(pot, y0, t0, t1, save_ts, cfg, save_offsets=save_offsets, order=order, soa=soa,
                             workspace=workspace, out=out, status=status)
    y = _as_cuda(y0, torch.float64)
    if not soa:
        y = y.reshape(-1, 6).t()
    y = y.contiguous()
    n = y.shape[1]
    t0v = _as_cuda(t0, torch.float64).reshape(-1).expand(n).contiguous()
    t1v = _as_cuda(t1, torch.float64).reshape(-1).expand(n).contiguous()
    ts = _in_place_or_cuda(save_ts, torch.float64).reshape(-1)
    if save_offsets is not None:
        offs = _in_place_or_cuda(save_offsets, torch.int64).reshape(-1)
        if offs.numel() != n + 1:
            raise ValueError("save_offsets must have n + 1 entries")
        total = int(ts.numel())
        # the kernel indexes saves through these offsets: reject inconsistent ones before launch
        if int(offs[0]) != 0 or int(offs[-1]) != total or bool((offs[1:] < offs[:-1]).any()):
            raise ValueError("save_offsets must start at 0, be non-decreasing and end at len(save_ts)")
        shape = (6, total)
        offs_ptr, n_saves = offs.data_ptr(), total
    else:
        shape = (6, ts.numel(), n)
        offs_ptr, n_saves = None, ts.numel()
    out = _result_buffer(out, shape, torch.float64, "out")
    status = _result_buffer(status, (n,), torch.int32, "status")
    steps = torch.empty(n, dtype=torch.int64, device="cuda")
    ordp = None
    if order is not None:
        ordt = _as_cuda(order, torch.int32).reshape(-1).contiguous()
        if ordt.numel() != n or (n and (int(ordt.min()) < 0 or int(ordt.max()) >= n)):
            raise ValueError("order must be a permutation of range(n)")
        ordp = ordt.data_ptr()
    L = _lib.load()
    nbytes = C.c_size_t()
    _lib.check(L.gal_integrate_workspace_size(C.byref(cfg), n, C.byref(nbytes)), "gal_integrate_workspace_size")
    ws = (workspace or _WS).get(nbytes.value)
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(
        L.gal_integrate(
            pot.handle(), C.byref(cfg), y.data_ptr(), t0v.data_ptr(), t1v.data_ptr(), offs_ptr, ts.data_ptr(),
            n_saves, out.data_ptr(), status.data_ptr(), steps.data_ptr(), ordp, n, ws.data_ptr(), ws.numel(), st,
        ),
        "gal_integrate",
    )
    return out, status, steps


def _raise_on_status(status, what: str) -> None:
    torch = _torch()
    bad = status != 0
    if bool(bad.any()):
        s = status.cpu().numpy()
        idx = np.nonzero(s)[0]
        first = int(idx[0])
        raise _lib.GalaxGB300Error(
            f"{what}: {len(idx)} orbit(s) did not finish; orbit {first}: {_lib.ORBIT_STATUS.get(int(s[first]), s[first])}"
        )
    del torch


def _split_w0(w0):
    torch = _torch()
    if isinstance(w0, PhaseSpaceCoordinate) or (hasattr(w0, "q") and hasattr(w0, "p")):
        q = _as_cuda(w0.q, torch.float64)
        p = _as_cuda(w0.p, torch.float64)
        q, p = torch.broadcast_tensors(q, p)
        t = getattr(w0, "t", None)
        return torch.cat([q, p], dim=-1), t
    w = _as_cuda(w0, torch.float64)
    if w.shape[-1] != 6:
        raise ValueError("w0 must be (..., 6) phase-space points or have q and p")
    return w, None


# ---------------------------------------------------------------- dense output
class PhaseSpaceInterpolation:
    """Dense orbits on the GPU (galax's PhaseSpaceInterpolation,
    src/galax/dynamics/_src/orbit/interp.py:42-145): per accepted step the
    library keeps the step boundaries and its interpolation data
    (``gal_integrate_dense``); ``evaluate(ts)`` returns every orbit at the
    times ``ts`` (``gal_dense_evaluate``). Times outside an orbit's [t0, t1]
    raise, as galax's ``eqx.error_if(..., "Time out of bounds.")`` does."""

    def __init__(self, pot: AbstractPotential, method: int, ts, coef, nsteps, cap: int, batch: tuple):
        self.pot = pot
        self.method = int(method)
        self.ts = ts            # (n, cap + 1)
        self.coef = coef        # (n, cap, per_step)
        self.nsteps = nsteps    # (n,)
        self.cap = int(cap)
        self.batch = tuple(batch)

    @property
    def t0(self):
        return self.ts[:, 0]

    @property
    def t1(self):
        torch = _torch()
        return torch.gather(self.ts, 1, self.nsteps.reshape(-1, 1)).reshape(-1)

    def evaluate(self, t):
        """(q, p) of every orbit at times t: shapes (*batch, T, 3)."""
        torch = _torch()
        tq = _as_cuda(t, torch.float64).reshape(-1)
        T = tq.numel()
        n = self.nsteps.numel()
        orbit = torch.arange(n, dtype=torch.int64, device="cuda").repeat_interleave(T)
        times = tq.repeat(n).contiguous()
        m = orbit.numel()
        out = torch.empty((6, m), dtype=torch.float64, device="cuda")
        oob = torch.zeros(1, dtype=torch.int64, device="cuda")
        L = _lib.load()
        _lib.check(L.gal_dense_evaluate(self.pot.handle(), self.method, self.ts.data_ptr(), self.coef.data_ptr(),
                                        self.nsteps.data_ptr(), self.cap, n, orbit.data_ptr(), times.data_ptr(), m,
                                        out.data_ptr(), oob.data_ptr(), torch.cuda.current_stream().cuda_stream),
                   "gal_dense_evaluate")
        if int(oob) != 0:
            raise ValueError("Time out of bounds.")
        w = out.t().reshape(*self.batch, T, 6)
        return w[..., :3], w[..., 3:]

    __call__ = evaluate


def integrate_dense(pot: AbstractPotential, y0, t0, t1, cfg: _lib.SolverConfig, *, cap: int | None = None,
                    batch: tuple | None = None, throw: bool = True) -> PhaseSpaceInterpolation:
    """Integrate orbits y0 (n, 6) from t0 to t1 keeping a dense interpolant. The
    step capacity per orbit grows (doubling) until every orbit fits or
    cfg.max_steps is reached."""
    torch = _torch()
    y = _as_cuda(y0, torch.float64).reshape(-1, 6)
    n = y.shape[0]
    t0v = _as_cuda(t0, torch.float64).reshape(-1).expand(n).contiguous()
    t1v = _as_cuda(t1, torch.float64).reshape(-1).expand(n).contiguous()
    y_soa = y.t().contiguous()
    L = _lib.load()
    per = int(L.gal_dense_coef_per_step(cfg.method))
    if cap is None:
        if not cfg.adaptive and cfg.dt0 > 0:
            cap = int(float((t1v - t0v).abs().max()) / cfg.dt0) + 2
        else:
            cap = 1024
    cap = max(1, min(int(cap), int(cfg.max_steps)))
    while True:
        ts = torch.empty((n, cap + 1), dtype=torch.float64, device="cuda")
        coef = torch.empty((n, cap, per), dtype=torch.float64, device="cuda")
        nsteps = torch.empty(n, dtype=torch.int64, device="cuda")
        status = torch.empty(n, dtype=torch.int32, device="cuda")
        _lib.check(L.gal_integrate_dense(pot.handle(), C.byref(cfg), y_soa.data_ptr(), t0v.data_ptr(),
                                         t1v.data_ptr(), n, cap, ts.data_ptr(), coef.data_ptr(), nsteps.data_ptr(),
                                         status.data_ptr(), torch.cuda.current_stream().cuda_stream),
                   "gal_integrate_dense")
        full = bool(((status == 1) & (nsteps == cap)).any())
        if full and cap < cfg.max_steps:
            cap = min(2 * cap, int(cfg.max_steps))
            continue
        break
    if throw:
        _raise_on_status(status, "dense integration")
    return PhaseSpaceInterpolation(pot, cfg.method, ts, coef, nsteps, cap, batch if batch is not None else (n,))


# ---------------------------------------------------------------- front doors
def evaluate_orbit(pot: AbstractPotential, w0, t, /, *, integrator: Integrator | None = None, dense: bool = False,
                   throw: bool = True) -> Orbit:
    """Compute orbits in ``pot`` saved at times ``t`` (galax legacy/funcs.py:42-213).

    As in galax, a ``w0`` that carries its own time is first integrated from
    ``w0.t`` to ``t[0]``, then from ``t[0]`` to ``t[-1]`` with saves at every
    ``t``; without a time, ``w0`` is taken to be at ``t[0]``.
    """
    torch = _torch()
    integrator = integrator or Integrator()
    cfg = integrator.config()
    is_np = not isinstance(t, torch.Tensor) and not isinstance(w0, torch.Tensor)
    ts = _as_cuda(t, torch.float64).reshape(-1)
    if ts.numel() == 0:
        raise ValueError("t must hold at least one time")
    w, tw0 = _split_w0(w0)
    batch = w.shape[:-1]
    y = w.reshape(-1, 6)
    n = y.shape[0]
    t_first, t_last = ts[0], ts[-1]
    if tw0 is not None:
        tw = _as_cuda(tw0, torch.float64).reshape(-1).expand(n).contiguous()
        out0, st0, _ = integrate(pot, y, tw, t_first.reshape(1), t_first.reshape(1), cfg)
        if throw:
            _raise_on_status(st0, "evaluate_orbit (w0.t -> t[0])")
        y = out0[:, 0, :].t()
    if dense:
        # galax returns the saves plus an interpolant over [t[0], t[-1]]
        interp = integrate_dense(pot, y, t_first.reshape(1), t_last.reshape(1), cfg, batch=tuple(batch),
                                 throw=throw)
        q, p = interp.evaluate(ts)
        orb = Orbit(q=q, p=p, t=ts, interpolant=interp)
        if is_np:
            orb = Orbit(q=q.cpu().numpy(), p=p.cpu().numpy(), t=ts.cpu().numpy(), interpolant=interp)
        return orb
    out, status, steps = integrate(pot, y, t_first.reshape(1), t_last.reshape(1), ts, cfg)
    if throw:
        _raise_on_status(status, "evaluate_orbit")
    w_btk = out.permute(2, 1, 0)  # (n, T, 6)
    q = w_btk[..., :3].reshape(*batch, ts.numel(), 3)
    p = w_btk[..., 3:].reshape(*batch, ts.numel(), 3)
    orb = Orbit(q=q, p=p, t=ts, status=status.reshape(batch), steps=steps.reshape(batch))
    if is_np:
        orb = Orbit(q=q.cpu().numpy(), p=p.cpu().numpy(), t=ts.cpu().numpy(), status=orb.status.cpu().numpy(),
                    steps=orb.steps.cpu().numpy())
    return orb


@dataclass(frozen=True)
class HamiltonianField:
    """galax's HamiltonianField over a potential (orbit/field_hamiltonian.py:21-249):
    (dq/dt, dp/dt) = (p, -grad Phi(q, t))."""

    potential: AbstractPotential

    def __call__(self, t, w):
        """The field at time t for phase-space points w (..., 6), on the GPU."""
        torch = _torch()
        ww = _as_cuda(w, torch.float64).reshape(-1, 6)
        acc = self.potential.acceleration(ww[:, :3].cpu().numpy(), t)
        out = np.concatenate([ww[:, 3:].cpu().numpy(), np.asarray(acc).reshape(-1, 3)], axis=1)
        return out.reshape(np.shape(w))


def compute_orbit(field, w0, ts, /, *, solver: Integrator | None = None, dense: bool = False) -> Orbit:
    """galax's ``compute_orbit`` (orbit/compute.py:28-66): ``evaluate_orbit``'s
    two phases (``w0.t`` to ``ts[0]``, then saves at ``ts``) with the
    ``OrbitSolver`` defaults (Dopri8, PID rtol = atol = 1e-8, 2**16 steps).
    ``field`` is a potential or a HamiltonianField."""
    pot = field.potential if isinstance(field, HamiltonianField) else field
    return evaluate_orbit(pot, w0, ts, integrator=solver if solver is not None else OrbitSolver(), dense=dense)


def integrate_orbit(pot: AbstractPotential, w0, t0, t1, saveat: Sequence | None = None, *,
                    integrator: Integrator | None = None, throw: bool = True):
    """Per-orbit start/end times and save grids (galax experimental/integrate.py:301-575).

    ``saveat`` is a list of 1-D arrays, one per orbit (ragged allowed), or None
    for the final state only. Returns (list of (T_i, 6) arrays or a (n, 6)
    array, status, steps).
    """
    torch = _torch()
    integrator = integrator or Integrator(solver=Dopri8(), stepsize_controller=PIDController(rtol=1e-7, atol=1e-7))
    cfg = integrator.config()
    w, _ = _split_w0(w0)
    y = w.reshape(-1, 6)
    n = y.shape[0]
    t0v = _as_cuda(t0, torch.float64).reshape(-1).expand(n)
    t1v = _as_cuda(t1, torch.float64).reshape(-1).expand(n)
    if saveat is None:
        offs = torch.arange(n + 1, dtype=torch.int64, device="cuda")
        flat = t1v.contiguous()
    else:
        lens = [len(s) for s in saveat]
        if len(lens) != n:
            raise ValueError("saveat needs one grid per orbit")
        offs = torch.zeros(n + 1, dtype=torch.int64)
        offs[1:] = torch.cumsum(torch.as_tensor(lens, dtype=torch.int64), 0)
        flat = torch.cat([_as_cuda(s, torch.float64).reshape(-1) for s in saveat])
    out, status, steps = integrate(pot, y, t0v, t1v, flat, cfg, save_offsets=offs)
    if throw:
        _raise_on_status(status, "integrate_orbit")
    res = out.t()
    if saveat is None:
        return res, status, steps
    o = offs.cpu().numpy()
    return [res[o[i]:o[i + 1]] for i in range(n)], status, steps
