"""galax potential objects -> galax_gb300 potentials.

galax potentials are equinox modules whose parameters are ``AbstractParameter``
fields (src/galax/potential/_src/params/core.py:25-157): a
``ConstantParameter`` holds a unit-carrying ``value``; a ``LinearParameter``
holds ``slope``, ``point_time`` and ``point_value``. Composites
(``AbstractCompositePotential``, src/galax/potential/_src/base_multi.py:32-303)
are mappings name -> potential; ``TranslatedPotential``
(src/galax/potential/_src/xfm/translate.py:29-160) wraps ``base_potential``
with a ``translation``.

The conversion reads those attributes by name and strips units with the
``strip(unit, quantity) -> value`` function it is given (unxt's ``ustrip`` in
the plug-in), so it needs neither galax nor jax to be imported here and can be
checked with stand-in objects. Everything the GPU path cannot evaluate raises
``NotImplementedError``, as galax_gb300's own constructors do.
"""

from __future__ import annotations

from typing import Any, Callable

import numpy as np

from .. import potential as P

MASS, LENGTH, SPEED, TIME, ONE = "Msun", "kpc", "kpc / Myr", "Myr", ""
G_UNIT = "kpc3 / (Msun Myr2)"

# galax class name -> (galax_gb300 class, {parameter: unit})
SINGLE = {
    "KeplerPotential": (P.KeplerPotential, {"m_tot": MASS}),
    "HernquistPotential": (P.HernquistPotential, {"m_tot": MASS, "r_s": LENGTH}),
    "MiyamotoNagaiPotential": (P.MiyamotoNagaiPotential, {"m_tot": MASS, "a": LENGTH, "b": LENGTH}),
    "NFWPotential": (P.NFWPotential, {"m": MASS, "r_s": LENGTH}),
    "PlummerPotential": (P.PlummerPotential, {"m_tot": MASS, "r_s": LENGTH}),
    "IsochronePotential": (P.IsochronePotential, {"m_tot": MASS, "r_s": LENGTH}),
    "LogarithmicPotential": (P.LogarithmicPotential, {"v_c": SPEED, "r_s": LENGTH}),
    "PowerLawCutoffPotential": (P.PowerLawCutoffPotential, {"m_tot": MASS, "alpha": ONE, "r_c": LENGTH}),
    "MN3ExponentialPotential": (P.MN3ExponentialPotential, {"m_tot": MASS, "h_R": LENGTH, "h_z": LENGTH}),
    "MN3Sech2Potential": (P.MN3Sech2Potential, {"m_tot": MASS, "h_R": LENGTH, "h_z": LENGTH}),
}


def _mro_names(obj: Any) -> set[str]:
    return {c.__name__ for c in type(obj).__mro__}


def _scalar(x) -> float:
    a = np.asarray(x, np.float64)
    if a.size != 1:
        raise NotImplementedError("array-valued parameters are not supported on the GPU path")
    return float(a.reshape(()))


def parameter(p: Any, unit: str, strip: Callable[[str, Any], Any], name: str = "parameter"):
    """A galax parameter in galactic units: a float for constants, a
    galax_gb300 LinearParameter for linear ones; other callables raise."""
    kind = type(p).__name__
    if kind == "ConstantParameter":
        return _scalar(strip(unit, p.value))
    if kind == "LinearParameter":
        slope_unit = f"{unit} / {TIME}" if unit else f"1 / {TIME}"
        return P.LinearParameter(slope=_scalar(strip(slope_unit, p.slope)),
                                 point_time=_scalar(strip(TIME, p.point_time)),
                                 point_value=_scalar(strip(unit, p.point_value)))
    if "AbstractParameter" in _mro_names(p) or kind.endswith("Parameter"):
        raise NotImplementedError(f"{name}: {kind} is not on the GPU path (constant and LinearParameter only)")
    return _scalar(strip(unit, p))  # a bare quantity


def _constants(pot: Any, strip) -> dict:
    consts = getattr(pot, "constants", None)
    if consts is None or "G" not in consts:
        return {}
    return {"G": _scalar(strip(G_UNIT, consts["G"]))}


def to_gb300(pot: Any, strip: Callable[[str, Any], Any]) -> P.AbstractPotential:
    """The galax_gb300 potential equal to the galax potential ``pot``."""
    if isinstance(pot, P.AbstractPotential):
        return pot
    names = _mro_names(pot)
    consts = _constants(pot, strip)
    if "AbstractCompositePotential" in names:
        return P.CompositePotential({k: to_gb300(v, strip) for k, v in pot.items()}, constants=consts or None)
    if "TranslatedPotential" in names:
        shift = np.asarray(strip(LENGTH, _translation_value(pot.translation)), np.float64).reshape(-1)
        if shift.size != 3:
            raise NotImplementedError("TranslatedPotential: the translation must be one 3-vector")
        return P.TranslatedPotential(to_gb300(pot.base_potential, strip), tuple(shift))
    entry = SINGLE.get(type(pot).__name__)
    if entry is None:
        raise NotImplementedError(f"{type(pot).__name__} is not on the GPU path")
    cls, units = entry
    kw = {k: parameter(getattr(pot, k), u, strip, k) for k, u in units.items()}
    if issubclass(cls, (P.MN3ExponentialPotential, P.MN3Sech2Potential)):
        kw["positive_density"] = bool(getattr(pot, "positive_density", False))
    return cls(**kw, constants=consts or None)


def _translation_value(t: Any):
    kind = type(t).__name__
    if kind == "ConstantParameter":
        return t.value
    if "AbstractParameter" in _mro_names(t) or kind.endswith("Parameter") or callable(t):
        raise NotImplementedError("TranslatedPotential: only constant translations are on the GPU path")
    return t
