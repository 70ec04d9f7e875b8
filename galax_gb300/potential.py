"""Potentials with galax's public interface, evaluated by the CUDA library.

Mirrors the part of ``galax.potential`` on the orbit path:
``HernquistPotential``, ``MiyamotoNagaiPotential``, ``NFWPotential``,
``PlummerPotential``, ``KeplerPotential``, ``MilkyWayPotential`` and
``CompositePotential`` (src/galax/potential/_src/builtin/*.py,
composite.py:32-108, builtin/milkyway.py:172-236) with the methods
``potential``, ``gradient``, ``acceleration``, ``hessian``,
``local_circular_velocity`` and ``evaluate_orbit``
(src/galax/potential/_src/base.py:138-143, 181-186, 250-255, 384-456;
register_funcs.py:327-340, 384-400).

Inputs are arrays in galax's "galactic" unit system (kpc, Myr, Msun; velocities
in kpc/Myr) with positions on the last axis, as galax accepts bare arrays. NumPy
inputs give NumPy outputs; CUDA torch tensors stay on the device. Parameters
are constants (galax's ConstantParameter) or galax's LinearParameter; other
callable parameters are rejected, as are unit systems other than "galactic".
"""

from __future__ import annotations

import ctypes as C
import math
from collections.abc import Mapping
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _lib

G_GALACTIC = 4.498502151469553e-12  # kpc^3 / (Msun Myr^2): astropy's CODATA-2018 G in galactic units
KMS_TO_KPC_MYR = 0.001022712165045695


def _torch():
    import torch

    return torch


@dataclass(frozen=True)
class LinearParameter:
    """galax's LinearParameter (src/galax/potential/_src/params/core.py:25-110),
    in galactic units: p(t) = slope (t - point_time) + point_value."""

    slope: float
    point_time: float
    point_value: float

    def __call__(self, t):
        return self.slope * (np.asarray(t, np.float64) - self.point_time) + self.point_value

    @property
    def value_at_zero(self) -> float:
        return float(self.point_value - self.slope * self.point_time)


def _param(name: str, v: Any) -> float:
    if isinstance(v, LinearParameter):
        raise NotImplementedError(f"{name}: a LinearParameter is not supported for this parameter on the GPU path")
    if callable(v):
        raise NotImplementedError(f"{name}: only constant and LinearParameter parameters are supported on the "
                                  "GPU path")
    try:
        f = float(v)
    except Exception as e:  # noqa: BLE001
        raise TypeError(f"{name} must be a number in galactic units, got {type(v).__name__}") from e
    if not math.isfinite(f):
        raise ValueError(f"{name} must be finite")
    return f


def _check_units(units: Any) -> None:
    if units not in (None, "galactic"):
        raise NotImplementedError("only the 'galactic' unit system (kpc, Myr, Msun) is supported")


class AbstractPotential:
    """Base class: a sum of closed-form components evaluated on the GPU."""

    units = "galactic"

    def __init__(self, *, units: Any = "galactic", constants: Mapping[str, float] | None = None):
        _check_units(units)
        self.constants = {"G": G_GALACTIC}
        if constants:
            self.constants.update({k: float(v) for k, v in constants.items()})
        self._handle = None
        self._handle_device = None
        self._handle_key = None

    # ---- component table -------------------------------------------------
    def components(self) -> list[tuple[int, float, float, float, tuple[float, float, float]]]:
        raise NotImplementedError

    def component_array(self) -> np.ndarray:
        recs = self.components()
        a = np.zeros(len(recs), _lib.COMPONENT_DTYPE)
        for i, (kind, m, l1, l2, origin) in enumerate(recs):
            a[i]["kind"], a[i]["m"], a[i]["l1"], a[i]["l2"] = kind, m, l1, l2
            a[i]["origin"] = origin
        return a

    def slopes(self):
        """d(m, l1, l2)/dt per component (ncomp, 3), or None for a static potential."""
        return None

    def parameter_names(self) -> list[tuple[str, str, str]]:
        """(component, mass-name, length names) per component, for gradients."""
        return [(f"c{i}", "m", "l1", "l2") for i in range(len(self.components()))]

    @property
    def G(self) -> float:
        return self.constants["G"]

    def handle(self) -> int:
        """The device-side ``gal_potential`` for the current CUDA device."""
        torch = _torch()
        if not torch.cuda.is_available():
            raise _lib.GalaxGB300Error("no CUDA device: the galax_gb300 path has no CPU fallback")
        dev = torch.cuda.current_device()
        arr = self.component_array()
        slopes = self.slopes()
        key = arr.tobytes() + np.float64(self.G).tobytes() + (b"" if slopes is None else slopes.tobytes())
        if self._handle is not None and self._handle_device == dev and self._handle_key == key:
            return self._handle
        self._release()
        L = _lib.load()
        h = C.c_void_p()
        _lib.check(L.gal_potential_create(arr.ctypes.data, len(arr), self.G, C.byref(h)), "gal_potential_create")
        if slopes is not None:
            sl = np.ascontiguousarray(slopes, np.float64)
            st = L.gal_potential_set_linear(h, sl.ctypes.data)
            if st != 0:
                L.gal_potential_destroy(h)
                _lib.check(st, "gal_potential_set_linear")
        self._handle, self._handle_device, self._handle_key, self._arr = h.value, dev, key, arr
        return self._handle

    def _release(self) -> None:
        if getattr(self, "_handle", None):
            try:
                torch = _torch()
                with torch.cuda.device(self._handle_device):
                    _lib.load().gal_potential_destroy(self._handle)
            except Exception:  # noqa: BLE001  (interpreter shutdown)
                pass
        self._handle = None

    def __del__(self):
        self._release()

    def is_milky_way_kernel(self) -> bool:
        return bool(_lib.load().gal_potential_is_milky_way(self.handle()))

    # ---- evaluation --------------------------------------------------------
    def _positions(self, x):
        torch = _torch()
        is_np = not isinstance(x, torch.Tensor)
        xt = torch.as_tensor(np.asarray(x, dtype=np.float64) if is_np else x)
        if xt.shape[-1] != 3:
            raise ValueError(f"positions must have a last axis of size 3, got shape {tuple(xt.shape)}")
        batch = xt.shape[:-1]
        soa = xt.reshape(-1, 3).to(device="cuda", dtype=torch.float64).t().contiguous()
        return soa, batch, is_np

    @staticmethod
    def _out(t, is_np):
        return t.cpu().numpy() if is_np else t

    def _eval(self, fn: str, x, t, ncomp_out: int):
        torch = _torch()
        soa, batch, is_np = self._positions(x)
        n = soa.shape[1]
        out = torch.empty((ncomp_out, n), dtype=torch.float64, device="cuda")
        L = _lib.load()
        stream = torch.cuda.current_stream().cuda_stream
        _lib.check(getattr(L, fn)(self.handle(), soa.data_ptr(), float(t or 0.0), n, out.data_ptr(), stream), fn)
        return out, batch, is_np

    def potential(self, x, t=0.0):
        out, batch, is_np = self._eval("gal_eval_potential", x, t, 1)
        return self._out(out.reshape(batch), is_np)

    def gradient(self, x, t=0.0):
        out, batch, is_np = self._eval("gal_eval_gradient", x, t, 3)
        return self._out(out.t().reshape(*batch, 3), is_np)

    def acceleration(self, x, t=0.0):
        out, batch, is_np = self._eval("gal_eval_acceleration", x, t, 3)
        return self._out(out.t().reshape(*batch, 3), is_np)

    def hessian(self, x, t=0.0):
        out, batch, is_np = self._eval("gal_eval_hessian", x, t, 9)
        return self._out(out.t().reshape(*batch, 3, 3), is_np)

    def local_circular_velocity(self, x, t=0.0):
        """sqrt(r |dPhi/dr|) at x (src/galax/potential/_src/register_funcs.py:384-400)."""
        torch = _torch()
        is_np = not isinstance(x, torch.Tensor)
        xt = torch.as_tensor(np.asarray(x, np.float64) if is_np else x).to("cuda", torch.float64)
        g = self.gradient(xt, t)
        r = torch.linalg.vector_norm(xt, dim=-1)
        dphidr = (g * xt / r[..., None]).sum(-1)
        return self._out(torch.sqrt(r * dphidr.abs()), is_np)

    def dpotential_dr(self, x, t=0.0):
        """rhat . grad Phi (src/galax/potential/_src/register_funcs.py:415-427)."""
        torch = _torch()
        is_np = not isinstance(x, torch.Tensor)
        xt = torch.as_tensor(np.asarray(x, np.float64) if is_np else x).to("cuda", torch.float64)
        g = self.gradient(xt, t)
        rhat = xt / torch.linalg.vector_norm(xt, dim=-1, keepdim=True)
        return self._out((g * rhat).sum(-1), is_np)

    def d2potential_dr2(self, x, t=0.0):
        """rhat . H . rhat (src/galax/potential/_src/register_funcs.py:444-457)."""
        torch = _torch()
        is_np = not isinstance(x, torch.Tensor)
        xt = torch.as_tensor(np.asarray(x, np.float64) if is_np else x).to("cuda", torch.float64)
        H = self.hessian(xt, t)
        rhat = xt / torch.linalg.vector_norm(xt, dim=-1, keepdim=True)
        return self._out(torch.einsum("...i,...ij,...j->...", rhat, H, rhat), is_np)

    def tidal_tensor(self, x, t=0.0):
        """H - tr(H) I / 3 (src/galax/potential/_src/register_funcs.py:347-378)."""
        torch = _torch()
        is_np = not isinstance(x, torch.Tensor)
        xt = torch.as_tensor(np.asarray(x, np.float64) if is_np else x).to("cuda", torch.float64)
        H = self.hessian(xt, t)
        tr = torch.diagonal(H, dim1=-2, dim2=-1).sum(-1)
        eye = torch.eye(3, dtype=torch.float64, device="cuda")
        return self._out(H - eye * (tr / 3.0)[..., None, None], is_np)

    def density(self, x, t=0.0):
        """Mass density from Poisson's equation, tr(H) / (4 pi G): equal to galax's
        closed-form densities of these components (base.py:208-228)."""
        torch = _torch()
        is_np = not isinstance(x, torch.Tensor)
        xt = torch.as_tensor(np.asarray(x, np.float64) if is_np else x).to("cuda", torch.float64)
        H = self.hessian(xt, t)
        tr = torch.diagonal(H, dim1=-2, dim2=-1).sum(-1)
        return self._out(tr / (4.0 * np.pi * self.G), is_np)

    def spherical_mass_enclosed(self, x, t=0.0):
        """r^2 |dPhi/dr| / G (src/galax/potential/_src/register_funcs.py:473-489)."""
        torch = _torch()
        is_np = not isinstance(x, torch.Tensor)
        xt = torch.as_tensor(np.asarray(x, np.float64) if is_np else x).to("cuda", torch.float64)
        r2 = (xt * xt).sum(-1)
        dr = self.dpotential_dr(xt, t)
        return self._out(r2 * dr.abs() / self.G, is_np)

    def evaluate_orbit(self, w0, t, *, integrator=None, dense: bool = False):
        from .dynamics import evaluate_orbit

        return evaluate_orbit(self, w0, t, integrator=integrator, dense=dense)

    def compute_orbit(self, w0, t, *, solver=None, dense: bool = False):
        """galax's ``AbstractPotential.compute_orbit`` (potential/_src/base.py):
        ``dynamics.compute_orbit`` on this potential."""
        from .dynamics import compute_orbit

        return compute_orbit(self, w0, t, solver=solver, dense=dense)

    def __or__(self, other: "AbstractPotential") -> "CompositePotential":
        return CompositePotential(_flatten(self) + _flatten(other))

    def __repr__(self) -> str:
        return f"{type(self).__name__}({self._repr_params()})"

    def _repr_params(self) -> str:
        return ""


class AbstractSinglePotential(AbstractPotential):
    kind: int
    _names: tuple[str, ...]

    def __init__(self, *, origin=(0.0, 0.0, 0.0), units: Any = "galactic", constants=None, **params):
        super().__init__(units=units, constants=constants)
        self._slopes = {}
        for name in self._names:
            if name not in params:
                raise TypeError(f"{type(self).__name__} needs parameter {name!r}")
            v = params.pop(name)
            if isinstance(v, LinearParameter):  # stored as its value at t = 0 plus a slope
                self._slopes[name] = _param(f"{name}.slope", v.slope)
                v = v.value_at_zero
            setattr(self, name, _param(name, v))
        if params:
            raise TypeError(f"unexpected parameters {sorted(params)}")
        self.origin = tuple(float(v) for v in origin)
        if len(self.origin) != 3:
            raise ValueError("origin must have 3 entries")

    def _repr_params(self) -> str:
        return ", ".join(f"{k}={getattr(self, k)!r}" for k in self._names)

    def slopes(self):
        if not any(self._slopes.values()):
            return None
        order = getattr(self, "_record", self._names)
        row = [self._slopes.get(order[j], 0.0) if j < len(order) else 0.0 for j in range(3)]
        return np.array([row], np.float64)


class KeplerPotential(AbstractSinglePotential):
    """Point mass: Phi = -G m_tot / r."""

    kind = _lib.GAL_KEPLER
    _names = ("m_tot",)

    def components(self):
        return [(self.kind, self.m_tot, 0.0, 0.0, self.origin)]


class HernquistPotential(AbstractSinglePotential):
    """Phi = -G m_tot / (r + r_s) (src/galax/potential/_src/builtin/hernquist.py:80-82)."""

    kind = _lib.GAL_HERNQUIST
    _names = ("m_tot", "r_s")

    def components(self):
        return [(self.kind, self.m_tot, self.r_s, 0.0, self.origin)]


class MiyamotoNagaiPotential(AbstractSinglePotential):
    """Phi = -G m_tot / sqrt(R^2 + (sqrt(z^2 + b^2) + a)^2) (builtin/miyamotonagai.py:73-78)."""

    kind = _lib.GAL_MIYAMOTO_NAGAI
    _names = ("m_tot", "a", "b")

    def components(self):
        return [(self.kind, self.m_tot, self.a, self.b, self.origin)]


class NFWPotential(AbstractSinglePotential):
    """Phi = -G m log(1 + r/r_s) / r (builtin/nfw/base.py:326-338)."""

    kind = _lib.GAL_NFW
    _names = ("m", "r_s")

    def components(self):
        return [(self.kind, self.m, self.r_s, 0.0, self.origin)]


class PlummerPotential(AbstractSinglePotential):
    """Phi = -G m_tot / sqrt(r^2 + r_s^2) (builtin/plummer.py:122-133)."""

    kind = _lib.GAL_PLUMMER
    _names = ("m_tot", "r_s")

    def components(self):
        return [(self.kind, self.m_tot, self.r_s, 0.0, self.origin)]


class IsochronePotential(AbstractSinglePotential):
    """Phi = -G m_tot / (r_s + sqrt(r^2 + r_s^2)) (builtin/isochrone.py:61-110)."""

    kind = _lib.GAL_ISOCHRONE
    _names = ("m_tot", "r_s")

    def components(self):
        return [(self.kind, self.m_tot, self.r_s, 0.0, self.origin)]


class LogarithmicPotential(AbstractSinglePotential):
    """Phi = v_c^2 / 2 log(r_s^2 + r^2) (builtin/logarithmic.py:45-53); v_c in kpc/Myr."""

    kind = _lib.GAL_LOGARITHMIC
    _names = ("v_c", "r_s")

    def components(self):
        return [(self.kind, self.v_c, self.r_s, 0.0, self.origin)]


# Smith et al. (2015) fits of a double-exponential / exponential-sech^2 disk by
# three Miyamoto-Nagai disks, as tabulated in galax (builtin/mn3.py:27-51).
# Rows: the three mass fractions, then the three a / h_R; columns: coefficients
# of (b/h_R)^4 ... (b/h_R)^0. b/h_R itself is a cubic in h_z/h_R without a
# constant term.
_MN3_K_POSITIVE_DENSITY = (
    (0.0036, -0.0330, 0.1117, -0.1335, 0.1749),
    (-0.0131, 0.1090, -0.3035, 0.2921, -5.7976),
    (-0.0048, 0.0454, -0.1425, 0.1012, 6.7120),
    (-0.0158, 0.0993, -0.2070, -0.7089, 0.6445),
    (-0.0319, 0.1514, -0.1279, -0.9325, 2.6836),
    (-0.0326, 0.1816, -0.2943, -0.6329, 2.3193),
)
_MN3_K_NEGATIVE_DENSITY = (
    (-0.0090, 0.0640, -0.1653, 0.1164, 1.9487),
    (0.0173, -0.0903, 0.0877, 0.2029, -1.3077),
    (-0.0051, 0.0287, -0.0361, -0.0544, 0.2242),
    (-0.0358, 0.2610, -0.6987, -0.1193, 2.0074),
    (-0.0830, 0.4992, -0.7967, -1.2966, 4.4441),
    (-0.0247, 0.1718, -0.4124, -0.5944, 0.7333),
)
_MN3_B_EXPONENTIAL = (-0.269, 1.08, 1.092)  # (h_z/h_R)^3, ^2, ^1
_MN3_B_SECH2 = (-0.033, 0.262, 0.659)


class _AbstractMN3Potential(AbstractPotential):
    """Three Miyamoto-Nagai disks standing in for an exponential disk (galax
    builtin/mn3.py:54-133): the component table holds the three disks, so the
    GPU evaluates exactly galax's sum."""

    _b_coeffs: tuple = ()

    def __init__(self, *, m_tot, h_R, h_z, positive_density: bool = False, origin=(0.0, 0.0, 0.0),  # noqa: N803
                 units: Any = "galactic", constants=None):
        super().__init__(units=units, constants=constants)
        # each disk's mass is a fixed multiple of m_tot, so a LinearParameter
        # m_tot is exact as per-disk slopes; the scale lengths enter the disks
        # non-linearly and must be constant
        self._m_tot_slope = 0.0
        if isinstance(m_tot, LinearParameter):
            self._m_tot_slope = _param("m_tot.slope", m_tot.slope)
            m_tot = m_tot.value_at_zero
        self.m_tot = _param("m_tot", m_tot)
        self.h_R = _param("h_R", h_R)
        self.h_z = _param("h_z", h_z)
        self.positive_density = bool(positive_density)
        self.origin = tuple(float(v) for v in origin)

    def _coefficients(self) -> tuple[list[float], float]:
        """The six mass / scale-length factors of the three disks, and b."""
        q = self.h_z / self.h_R
        c3, c2, c1 = self._b_coeffs
        b_over_hR = ((c3 * q + c2) * q + c1) * q
        powers = (b_over_hR**4, b_over_hR**3, b_over_hR**2, b_over_hR, 1.0)
        K = _MN3_K_POSITIVE_DENSITY if self.positive_density else _MN3_K_NEGATIVE_DENSITY
        return [sum(k * x for k, x in zip(row, powers)) for row in K], b_over_hR * self.h_R

    def disks(self) -> list[tuple[float, float, float]]:
        """(m_tot, a, b) of the three Miyamoto-Nagai disks (at t = 0)."""
        coef, b = self._coefficients()
        return [(coef[i] * self.m_tot, coef[3 + i] * self.h_R, b) for i in range(3)]

    def components(self):
        return [(_lib.GAL_MIYAMOTO_NAGAI, m, a, b, self.origin) for (m, a, b) in self.disks()]

    def slopes(self):
        if not self._m_tot_slope:
            return None
        coef, _ = self._coefficients()
        return np.array([[coef[i] * self._m_tot_slope, 0.0, 0.0] for i in range(3)], np.float64)

    def _repr_params(self) -> str:
        return (f"m_tot={self.m_tot!r}, h_R={self.h_R!r}, h_z={self.h_z!r}, "
                f"positive_density={self.positive_density!r}")


class MN3ExponentialPotential(_AbstractMN3Potential):
    """Double-exponential disk as three Miyamoto-Nagai disks (galax builtin/mn3.py:136-165)."""

    _b_coeffs = _MN3_B_EXPONENTIAL


class MN3Sech2Potential(_AbstractMN3Potential):
    """Exponential disk with a sech^2 vertical profile as three Miyamoto-Nagai
    disks (galax builtin/mn3.py:168-197)."""

    _b_coeffs = _MN3_B_SECH2


class PowerLawCutoffPotential(AbstractSinglePotential):
    """Spherical power law with an exponential cutoff, rho ~ (r_c / r)^alpha
    exp(-(r / r_c)^2) (galax builtin/powerlawcutoff.py:26-120). Supported for
    0 <= alpha < 2, where galax's potential is finite."""

    kind = _lib.GAL_POWERLAW_CUTOFF
    _names = ("m_tot", "alpha", "r_c")
    _record = ("m_tot", "r_c", "alpha")  # order of (m, l1, l2) in the component table

    def __init__(self, **kw):
        super().__init__(**kw)
        if not (0.0 <= self.alpha < 2.0):
            raise ValueError("alpha must satisfy 0 <= alpha < 2 (galax's potential is not finite beyond)")

    def components(self):
        return [(self.kind, self.m_tot, self.r_c, self.alpha, self.origin)]


def _flatten(p: AbstractPotential) -> list[AbstractPotential]:
    if isinstance(p, CompositePotential):
        out = []
        for v in p.values():
            out += _flatten(v)
        return out
    return [p]


class CompositePotential(AbstractPotential):
    """Sum of potentials (src/galax/potential/_src/composite.py:32-108): a mapping
    name -> potential whose Phi, gradient and Hessian are the component sums."""

    def __init__(self, potentials=None, /, *, units: Any = "galactic", constants=None, **kw):
        super().__init__(units=units, constants=constants)
        if potentials is None:
            items = list(kw.items())
        elif isinstance(potentials, Mapping):
            items = list(potentials.items()) + list(kw.items())
        else:
            items = [(f"p{i}", p) for i, p in enumerate(potentials)] + list(kw.items())
        for k, v in items:
            if not isinstance(v, AbstractPotential):
                raise TypeError(f"component {k!r} is not a potential")
        self._items = dict(items)

    def keys(self):
        return self._items.keys()

    def values(self):
        return self._items.values()

    def items(self):
        return self._items.items()

    def __getitem__(self, k):
        return self._items[k]

    def __len__(self):
        return len(self._items)

    def __iter__(self):
        return iter(self._items)

    def components(self):
        out = []
        for v in self._items.values():
            out += v.components()
        return out

    def slopes(self):
        parts = [(v.slopes(), len(v.components())) for v in self._items.values()]
        if all(sl is None for sl, _ in parts):
            return None
        return np.concatenate([np.zeros((k, 3)) if sl is None else sl for sl, k in parts], axis=0)

    def _repr_params(self) -> str:
        return ", ".join(f"{k}={v!r}" for k, v in self._items.items())


class MilkyWayPotential(CompositePotential):
    """galax's MilkyWayPotential (src/galax/potential/_src/builtin/milkyway.py:172-236):
    Miyamoto-Nagai disk, NFW halo, Hernquist bulge and nucleus, in that order."""

    DEFAULTS = {
        "disk": {"m_tot": 6.8e10, "a": 3.0, "b": 0.28},
        "halo": {"m": 5.4e11, "r_s": 15.62},
        "bulge": {"m_tot": 5e9, "r_s": 1.0},
        "nucleus": {"m_tot": 1.71e9, "r_s": 0.07},
    }

    def __init__(self, disk=None, halo=None, bulge=None, nucleus=None, *, units: Any = "galactic", constants=None):
        def part(name, cls, given):
            if isinstance(given, AbstractPotential):
                return given
            kw = dict(self.DEFAULTS[name])
            kw.update(given or {})
            return cls(**kw, units=units, constants=constants)

        super().__init__(
            {
                "disk": part("disk", MiyamotoNagaiPotential, disk),
                "halo": part("halo", NFWPotential, halo),
                "bulge": part("bulge", HernquistPotential, bulge),
                "nucleus": part("nucleus", HernquistPotential, nucleus),
            },
            units=units,
            constants=constants,
        )


class BovyMWPotential2014(CompositePotential):
    """galax's BovyMWPotential2014 (src/galax/potential/_src/builtin/milkyway.py:33-98):
    Miyamoto-Nagai disk, power law with cutoff bulge, NFW halo, in that order."""

    DEFAULTS = {
        "disk": {"m_tot": 68_193_902_782.346756, "a": 3.0, "b": 0.28},
        "bulge": {"m_tot": 4501365375.06545, "alpha": 1.8, "r_c": 1.9},
        "halo": {"m": 4.3683325e11, "r_s": 16.0},
    }

    def __init__(self, disk=None, bulge=None, halo=None, *, units: Any = "galactic", constants=None):
        def part(name, cls, given):
            if isinstance(given, AbstractPotential):
                return given
            kw = dict(self.DEFAULTS[name])
            kw.update(given or {})
            return cls(**kw, units=units, constants=constants)

        super().__init__(
            {
                "disk": part("disk", MiyamotoNagaiPotential, disk),
                "bulge": part("bulge", PowerLawCutoffPotential, bulge),
                "halo": part("halo", NFWPotential, halo),
            },
            units=units,
            constants=constants,
        )


class MilkyWayPotential2022(CompositePotential):
    """galax's MilkyWayPotential2022 (src/galax/potential/_src/builtin/milkyway.py:239-313):
    an MN3Sech2 disk (positive density), NFW halo, Hernquist bulge and nucleus,
    in that order (six table components)."""

    DEFAULTS = {
        "disk": {"m_tot": 4.7717e10, "h_R": 2.6, "h_z": 0.3, "positive_density": True},
        "halo": {"m": 5.5427e11, "r_s": 15.626},
        "bulge": {"m_tot": 5e9, "r_s": 1.0},
        "nucleus": {"m_tot": 1.8142e9, "r_s": 0.0688867},
    }

    def __init__(self, disk=None, halo=None, bulge=None, nucleus=None, *, units: Any = "galactic", constants=None):
        def part(name, cls, given):
            if isinstance(given, AbstractPotential):
                return given
            kw = dict(self.DEFAULTS[name])
            kw.update(given or {})
            return cls(**kw, units=units, constants=constants)

        super().__init__(
            {
                "disk": part("disk", MN3Sech2Potential, disk),
                "halo": part("halo", NFWPotential, halo),
                "bulge": part("bulge", HernquistPotential, bulge),
                "nucleus": part("nucleus", HernquistPotential, nucleus),
            },
            units=units,
            constants=constants,
        )


class TranslatedPotential(CompositePotential):
    """A potential shifted by a constant translation (src/galax/potential/_src/xfm/translate.py:28-87,
    constant translations only)."""

    def __init__(self, original: AbstractPotential, translation, *, units: Any = "galactic"):
        super().__init__({"original": original}, units=units, constants=original.constants)
        self.translation = tuple(float(v) for v in translation)
        if callable(translation):
            raise NotImplementedError("time-dependent translations are not supported on the GPU path")

    def components(self):
        tx, ty, tz = self.translation
        return [(k, m, l1, l2, (o[0] + tx, o[1] + ty, o[2] + tz))
                for (k, m, l1, l2, o) in self["original"].components()]


def from_component_array(arr: np.ndarray, G: float = G_GALACTIC, slopes=None) -> CompositePotential:
    """Composite built from a ``gal_component`` record array; ``slopes``
    (ncomp, 3), if given, makes (m, l1, l2) LinearParameters through their
    table values at t = 0."""
    cls = {_lib.GAL_KEPLER: KeplerPotential, _lib.GAL_HERNQUIST: HernquistPotential,
           _lib.GAL_MIYAMOTO_NAGAI: MiyamotoNagaiPotential, _lib.GAL_NFW: NFWPotential,
           _lib.GAL_PLUMMER: PlummerPotential, _lib.GAL_ISOCHRONE: IsochronePotential,
           _lib.GAL_LOGARITHMIC: LogarithmicPotential, _lib.GAL_POWERLAW_CUTOFF: PowerLawCutoffPotential}
    parts = {}
    for i, rec in enumerate(arr):
        k = int(rec["kind"])
        names = getattr(cls[k], "_record", cls[k]._names)
        vals = [float(rec["m"]), float(rec["l1"]), float(rec["l2"])][: len(names)]
        if slopes is not None:
            vals = [LinearParameter(float(slopes[i][j]), 0.0, v) if slopes[i][j] != 0.0 else v
                    for j, v in enumerate(vals)]
        parts[f"c{i}"] = cls[k](**dict(zip(names, vals)), origin=tuple(rec["origin"]), constants={"G": G})
    return CompositePotential(parts, constants={"G": G})
