"""plum plug-in: galax calls the GB300 library through its own API.

galax loads this module through the entry-point groups ``galax.potential.interop``
and ``galax.dynamics.interop`` (declared in this project's ``pyproject.toml``;
galax's groups are ``pyproject.toml:87-99`` and its loader
``load_interop_plugins``, src/galax/dynamics/setup_package.py:61-84, imports
every registered module). Importing the module performs the registrations;
galax itself is not modified. Requires galax (with jax, unxt, plum) in the same
environment, so it is only ever imported by galax's loader or by a user.

Two ways in:

* ``GB300Integrator`` — pass it as ``integrator=`` to galax's own
  ``gd.evaluate_orbit(pot, w0, t, integrator=GB300Integrator())``
  (src/galax/dynamics/_src/legacy/funcs.py:42-213) with an ordinary galax
  potential. galax calls its integrator as ``integrator(field, w0, t0, t1, *,
  saveat=None, dense=False)`` (funcs.py:197-210, the convention of
  ``Integrator.__call__``, src/galax/dynamics/_src/legacy/integrator.py:269-355);
  this one converts ``field.potential`` into a component table, integrates on
  the GPU and returns a ``gc.PhaseSpaceCoordinate`` as galax's integrator does
  (integrator.py:231-245).
* dispatches of ``gd.evaluate_orbit``, ``gp.potential``, ``gp.gradient`` and
  ``gp.acceleration`` on ``galax_gb300`` potentials, so galax's functions accept
  the library's potential objects (the plum pattern of funcs.py:42-51 and
  src/galax/potential/_src/register_funcs.py:33-155).

Units: galax quantities are converted to galactic units (kpc, Myr, Msun) with
unxt; results come back as unxt quantities in galactic units.
"""

from __future__ import annotations

from typing import Any

import jax.numpy as jnp
import numpy as np
import unxt as u

import galax.coordinates as gc
import galax.dynamics as gd
import galax.potential as gp

from .. import dynamics as D
from .. import potential as P
from .convert import to_gb300


def _strip(unit: str, q: Any):
    """q in ``unit`` as a NumPy value; bare arrays are taken to be in galactic units already."""
    if hasattr(q, "unit"):
        return np.asarray(u.ustrip(unit, q), np.float64)
    return np.asarray(q, np.float64)


def _w_galactic(w0: Any) -> tuple[np.ndarray, np.ndarray | None]:
    """(phase-space array (..., 6) in kpc, kpc/Myr; its time in Myr or None)."""
    t = getattr(w0, "t", None)
    if hasattr(w0, "w"):
        w = np.asarray(w0.w(units="galactic"), np.float64)
    elif isinstance(w0, tuple):
        w = np.concatenate([_strip("kpc", w0[0]), _strip("kpc / Myr", w0[1])], axis=-1)
    else:
        w = _strip("", w0)
    return w, (None if t is None else _strip("Myr", t))


class GB300Integrator:
    """galax-callable integrator running on the GB300 library.

    ``integrator`` is a ``galax_gb300.Integrator`` (solver, step-size controller,
    max_steps); the default is galax's legacy default, Dopri8 with
    PIDController(rtol=1e-7, atol=1e-7)."""

    def __init__(self, integrator: D.Integrator | None = None):
        self.integrator = integrator or D.Integrator()

    def __call__(self, field: Any, w0: Any, t0: Any, t1: Any, /, *, saveat: Any = None, dense: bool = False):
        if dense:
            raise NotImplementedError("dense=True with galax's interpolant objects is not on the GPU path; "
                                      "use galax_gb300.evaluate_orbit(..., dense=True)")
        pot = to_gb300(field.potential, _strip)
        w, _ = _w_galactic(w0)
        batch = w.shape[:-1]
        y = w.reshape(-1, 6)
        n = y.shape[0]
        t0v = np.broadcast_to(_strip("Myr", t0), batch).reshape(-1)
        t1v = np.broadcast_to(_strip("Myr", t1), batch).reshape(-1)
        cfg = self.integrator.config()
        if saveat is None:
            # the state at each orbit's own t1: one save per orbit (CSR grid)
            offs = np.arange(n + 1, dtype=np.int64)
            out, status, _ = D.integrate(pot, y, t0v, t1v, t1v.copy(), cfg, save_offsets=offs)
            D._raise_on_status(status, "GB300Integrator")
            ww = out.t().cpu().numpy().reshape(*batch, 6)
            t_out = t1v.reshape(batch)
        else:
            ts = _strip("Myr", saveat).reshape(-1)
            out, status, _ = D.integrate(pot, y, t0v, t1v, ts, cfg)
            D._raise_on_status(status, "GB300Integrator")
            ww = out.permute(2, 1, 0).cpu().numpy().reshape(*batch, ts.size, 6)
            t_out = ts
        return gc.PhaseSpaceCoordinate(q=u.Q(jnp.asarray(ww[..., :3]), "kpc"),
                                       p=u.Q(jnp.asarray(ww[..., 3:]), "kpc / Myr"),
                                       t=u.Q(jnp.asarray(t_out), "Myr"), frame=gc.frames.simulation_frame)


def _gx_integrator(integrator: Any) -> D.Integrator | None:
    if integrator is None or isinstance(integrator, D.Integrator):
        return integrator
    if isinstance(integrator, GB300Integrator):
        return integrator.integrator
    raise NotImplementedError(f"{type(integrator).__name__}: pass a galax_gb300 integrator for a GB300 potential")


@gd.evaluate_orbit.dispatch
def evaluate_orbit(pot: P.AbstractPotential, w0: Any, t: Any, /, *, integrator: Any = None,
                   dense: bool = False) -> D.Orbit:
    """galax's evaluate_orbit for a galax_gb300 potential (same two phases)."""
    w, tw = _w_galactic(w0)
    start = D.PhaseSpaceCoordinate(q=w[..., :3], p=w[..., 3:], t=tw) if tw is not None else w
    return D.evaluate_orbit(pot, start, _strip("Myr", t), integrator=_gx_integrator(integrator), dense=dense)


@gp.potential.dispatch
def potential(pot: P.AbstractPotential, xyz: Any, t: Any, /) -> Any:
    return u.Q(jnp.asarray(pot.potential(_strip("kpc", xyz), float(_strip("Myr", t)))), "kpc2 / Myr2")


@gp.gradient.dispatch
def gradient(pot: P.AbstractPotential, xyz: Any, t: Any, /) -> Any:
    return u.Q(jnp.asarray(pot.gradient(_strip("kpc", xyz), float(_strip("Myr", t)))), "kpc / Myr2")


@gp.acceleration.dispatch
def acceleration(pot: P.AbstractPotential, xyz: Any, t: Any, /) -> Any:
    return u.Q(jnp.asarray(pot.acceleration(_strip("kpc", xyz), float(_strip("Myr", t)))), "kpc / Myr2")
