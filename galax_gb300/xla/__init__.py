"""jax.ffi binding of the GB300 library: orbit integration, potential gradients
and the discrete adjoint as XLA custom calls, so jax programs (galax's orbit
path is jax) run the same kernels inside ``jax.jit``.

``gb300_xla.cc`` holds the XLA FFI handlers (``GalIntegrate``, ``GalGradient``,
``GalAdjoint``); ``build()`` compiles them against the headers jaxlib ships
(``jax.ffi.include_dir()``) and links them to ``libgalax_gb300.so``;
``register()`` registers them with XLA for the CUDA platform. The functions
below take jax arrays in galactic units, as galax's ``gd.evaluate_orbit``
(src/galax/dynamics/_src/legacy/funcs.py:42-213) and
``gp.gradient`` (src/galax/potential/_src/register_funcs.py:86-98) do after
stripping units.

Every buffer belongs to XLA: the kernels' scratch is one more result buffer of
the custom call, sized on the host with the library's ``*_workspace_size``
queries. The potential is built once outside the traced function; its handle
enters the custom call as a static attribute. Attributes are passed with the
widths the handlers bind (np.int32 / np.int64 / np.float64), and jax must run
with 64-bit types enabled (``jax_enable_x64``), as galax requires.
"""

from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

from .. import _lib

HERE = Path(__file__).resolve().parent
PKG = HERE.parent
SOURCE = HERE / "gb300_xla.cc"
LIB = PKG / "_lib" / "libgalax_gb300_xla.so"
INCLUDE = PKG.parent / "include"
TARGETS = {"gal_integrate": "GalIntegrate", "gal_gradient": "GalGradient", "gal_adjoint": "GalAdjoint"}

_registered = False


def _jax():
    import jax

    return jax


def _cuda_include() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "include" / "cuda_runtime.h").exists():
            return str(Path(cand) / "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        return str(Path(nvcc).resolve().parents[1] / "include")
    raise RuntimeError("CUDA headers not found")


def build(force: bool = False) -> Path:
    """Compile the FFI handlers (needs jaxlib's FFI headers and the built library)."""
    jax = _jax()
    from ..build import build as build_lib

    core = build_lib()
    if not force and LIB.exists() and LIB.stat().st_mtime > max(SOURCE.stat().st_mtime, core.stat().st_mtime):
        return LIB
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    cmd = [cxx, "-std=c++17", "-O2", "-shared", "-fPIC", "-I", jax.ffi.include_dir(), "-I", str(INCLUDE),
           "-I", _cuda_include(), str(SOURCE), "-L", str(core.parent), "-lgalax_gb300",
           "-Wl,-rpath,$ORIGIN", "-o", str(LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the XLA FFI handlers failed:\n{r.stderr}")
    return LIB


def register() -> None:
    """Register the handlers with XLA (CUDA platform); builds them if needed."""
    global _registered
    if _registered:
        return
    jax = _jax()
    _lib.load()  # the core library first, so the handlers resolve against it
    lib = C.CDLL(str(build()))
    for target, symbol in TARGETS.items():
        jax.ffi.register_ffi_target(target, jax.ffi.pycapsule(getattr(lib, symbol)), platform="CUDA")
    _registered = True


def _ws_integrate(cfg, n: int) -> int:
    nb = C.c_size_t()
    _lib.check(_lib.load().gal_integrate_workspace_size(C.byref(cfg), n, C.byref(nb)), "gal_integrate_workspace_size")
    return max(int(nb.value), 1)


def integrate(pot, y0, t0, t1, save_ts, cfg, save_offsets=None):
    """Orbits under jax: y0 (n, 6), t0 and t1 (n,) or scalars, save_ts (T,)
    shared by all orbits (out (n, T, 6)) or, with CSR ``save_offsets`` (n+1,),
    the concatenated per-orbit grids (out (total, 6)). ``cfg`` is a
    ``gal_solver_config`` (``galax_gb300.Integrator(...).config()``).
    Returns (out, status (n,), accepted steps (n,))."""
    jax = _jax()
    jnp = jax.numpy
    register()
    y0 = jnp.asarray(y0, jnp.float64).reshape(-1, 6)
    n = y0.shape[0]
    t0 = jnp.broadcast_to(jnp.asarray(t0, jnp.float64), (n,))
    t1 = jnp.broadcast_to(jnp.asarray(t1, jnp.float64), (n,))
    save_ts = jnp.asarray(save_ts, jnp.float64).reshape(-1)
    T = save_ts.shape[0]
    offs = jnp.zeros((0,), jnp.int64) if save_offsets is None else jnp.asarray(save_offsets, jnp.int64)
    out_shape = (6, T) if save_offsets is not None else (6, T, n)
    call = jax.ffi.ffi_call(
        "gal_integrate",
        (jax.ShapeDtypeStruct(out_shape, jnp.float64), jax.ShapeDtypeStruct((n,), jnp.int32),
         jax.ShapeDtypeStruct((n,), jnp.int64), jax.ShapeDtypeStruct((_ws_integrate(cfg, n),), jnp.uint8)))
    out, status, steps, _ = call(
        y0.T, t0, t1, offs, save_ts, pot=np.int64(pot.handle()), method=np.int32(cfg.method),
        adaptive=np.int32(cfg.adaptive), max_steps=np.int64(cfg.max_steps), dt0=np.float64(cfg.dt0),
        rtol=np.float64(cfg.rtol), atol=np.float64(cfg.atol), dtmin=np.float64(cfg.dtmin),
        dtmax=np.float64(cfg.dtmax), pcoeff=np.float64(cfg.pcoeff), icoeff=np.float64(cfg.icoeff),
        dcoeff=np.float64(cfg.dcoeff), safety=np.float64(cfg.safety), factormin=np.float64(cfg.factormin),
        factormax=np.float64(cfg.factormax), force_dtmin=np.int32(cfg.force_dtmin), schedule=np.int32(cfg.schedule))
    out = out.T if save_offsets is not None else jnp.transpose(out, (2, 1, 0))
    return out, status, steps


def gradient(pot, x, t: float = 0.0):
    """grad Phi at positions x (..., 3) and time t, under jax."""
    jax = _jax()
    jnp = jax.numpy
    register()
    x = jnp.asarray(x, jnp.float64)
    xs = x.reshape(-1, 3).T
    g = jax.ffi.ffi_call("gal_gradient", jax.ShapeDtypeStruct(xs.shape, jnp.float64))(
        xs, pot=np.int64(pot.handle()), t=np.float64(t))
    return g.T.reshape(x.shape)


def _ws_adjoint(pot, cfg, t0, t1, k_ckpt, n) -> int:
    nb = C.c_size_t()
    _lib.check(_lib.load().gal_adjoint_workspace_size(pot.handle(), C.byref(cfg), float(t0), float(t1), int(k_ckpt),
                                                      n, C.byref(nb)), "gal_adjoint_workspace_size")
    return max(int(nb.value), 1)


def adjoint(pot, y0, lam, t0: float, t1: float, dt: float, method: int = 8, k_ckpt: int = 256):
    """Discrete adjoint of the constant-step map y0 -> y(t1) for the cotangent
    lam = dL/dy(t1) (n, 6): returns (y(t1), dL/dy0, dL/d(m, l1, l2) per component,
    followed by d/d(slopes) for a time-dependent potential)."""
    jax = _jax()
    jnp = jax.numpy
    register()
    y0 = jnp.asarray(y0, jnp.float64).reshape(-1, 6)
    lam = jnp.asarray(lam, jnp.float64).reshape(-1, 6)
    n = y0.shape[0]
    cfg = _lib.solver_config(method, False, dt0=dt)
    ncomp = len(pot.components())
    per = 6 if _lib.load().gal_potential_is_time_dependent(pot.handle()) else 3
    call = jax.ffi.ffi_call(
        "gal_adjoint",
        (jax.ShapeDtypeStruct((6, n), jnp.float64), jax.ShapeDtypeStruct((6, n), jnp.float64),
         jax.ShapeDtypeStruct((ncomp, per), jnp.float64),
         jax.ShapeDtypeStruct((_ws_adjoint(pot, cfg, t0, t1, k_ckpt, n),), jnp.uint8)))
    yT, gy, gp, _ = call(y0.T, lam.T, pot=np.int64(pot.handle()), method=np.int32(method), dt=np.float64(dt),
                         t0=np.float64(t0), t1=np.float64(t1), k_ckpt=np.int32(k_ckpt))
    return yT.T, gy.T, gp


def orbit_map(pot, t0: float, t1: float, dt: float, method: int = 8, k_ckpt: int = 256):
    """y0 (n, 6) -> y(t1) (n, 6) with constant steps, as a jax function whose
    reverse-mode derivative (jax.grad, jax.vjp) runs the adjoint kernel."""
    jax = _jax()
    jnp = jax.numpy
    cfg = _lib.solver_config(method, False, dt0=dt)

    @jax.custom_vjp
    def f(y0):
        out, _, _ = integrate(pot, y0, t0, t1, jnp.asarray([t1]), cfg)
        return out[:, 0, :]

    def fwd(y0):
        return f(y0), y0

    def bwd(y0, g):
        _, gy, _ = adjoint(pot, y0, g, t0, t1, dt, method, k_ckpt)
        return (gy,)

    f.defvjp(fwd, bwd)
    return f
