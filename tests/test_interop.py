"""The two reference-side bindings, checked without jax or galax (neither is
installed on the test machines):

* the XLA FFI handlers (galax_gb300/xla/gb300_xla.cc) compile against
  include/galax_gb300.h, their parameters are exactly what their bindings
  declare, they export the handler symbols, and the Python side passes the
  attributes each binding declares, with the declared widths;
* the plum plug-in's conversion of galax potential objects into component
  tables (galax_gb300/interop/convert.py), on stand-ins that carry galax's
  class names and attributes; and the entry-point declaration galax loads.
"""

from __future__ import annotations

import ast
import re
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "galax_gb300" / "xla" / "gb300_xla.cc"
STUB = ROOT / "tests" / "xla_ffi_stub"
CUDA_INC = Path("/usr/local/cuda/include")


def _cxx():
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx or not (CUDA_INC / "cuda_runtime.h").exists():
        pytest.skip("needs g++ and the CUDA headers")
    return cxx


def test_xla_handlers_compile_against_the_header(tmp_path):
    cxx = _cxx()
    obj = tmp_path / "gb300_xla.o"
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-c", "-fPIC", "-I", str(STUB),
                        "-I", str(ROOT / "include"), "-I", str(CUDA_INC), str(SRC), "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-g", "--defined-only", str(obj)], capture_output=True, text=True).stdout
    for sym in ("GalIntegrate", "GalGradient", "GalAdjoint"):
        assert re.search(rf"\bT {sym}$", nm, re.M), sym


def test_the_stub_rejects_a_handler_that_differs_from_its_binding(tmp_path):
    """The binding check is real: one attribute's width changed must not compile."""
    cxx = _cxx()
    bad = tmp_path / "bad.cc"
    bad.write_text(SRC.read_text().replace('.Attr<int32_t>("k_ckpt")', '.Attr<int64_t>("k_ckpt")'))
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-I", str(STUB), "-I", str(ROOT / "include"),
                        "-I", str(CUDA_INC), str(bad)], capture_output=True, text=True)
    assert r.returncode != 0 and "differ from its binding" in r.stderr


def _bindings():
    """handler symbol -> (number of Arg, number of Ret, [(attr name, C type)])."""
    text = SRC.read_text()
    out = {}
    for m in re.finditer(r"XLA_FFI_DEFINE_HANDLER_SYMBOL\((\w+),\s*\w+,(.*?)\);", text, re.S):
        body = m.group(2)
        out[m.group(1)] = (len(re.findall(r"\.Arg<", body)), len(re.findall(r"\.Ret<", body)),
                           re.findall(r'\.Attr<(\w+)>\("(\w+)"\)', body))
    return out


def test_python_calls_pass_what_each_binding_declares():
    binds = _bindings()
    assert set(binds) == {"GalIntegrate", "GalGradient", "GalAdjoint"}
    mod = ast.parse((ROOT / "galax_gb300" / "xla" / "__init__.py").read_text())
    targets = {}
    for node in ast.walk(mod):
        if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name) and node.targets[0].id == "TARGETS":
            targets = ast.literal_eval(node.value)
    widths = {"int32": "int32_t", "int64": "int64_t", "float64": "double"}
    seen = set()
    for fn in [n for n in mod.body if isinstance(n, ast.FunctionDef)]:
        calls = [n for n in ast.walk(fn) if isinstance(n, ast.Call) and isinstance(n.func, ast.Attribute)
                 and n.func.attr == "ffi_call"]
        if not calls:
            continue
        target = calls[0].args[0].value
        n_ret = len(calls[0].args[1].elts) if isinstance(calls[0].args[1], ast.Tuple) else 1
        invoke = [n for n in ast.walk(fn) if isinstance(n, ast.Call) and any(k.arg == "pot" for k in n.keywords)]
        assert len(invoke) == 1, fn.name
        kws = [(k.arg, k.value.func.attr) for k in invoke[0].keywords]
        n_arg, n_ret_c, attrs = binds[targets[target]]
        assert len(invoke[0].args) == n_arg, fn.name
        assert n_ret == n_ret_c, fn.name
        assert [(name, widths[w]) for name, w in kws] == [(name, ty) for ty, name in attrs], fn.name
        seen.add(target)
    assert seen == set(targets)


# ---------------------------------------------------------------- plug-in conversion
class Q:
    """A unit-carrying value standing in for an unxt quantity."""

    TO = {"pc": ("kpc", 1e-3), "Gyr": ("Myr", 1e3), "km / s": ("kpc / Myr", 0.001022712165045695)}

    def __init__(self, value, unit):
        self.value, self.unit = np.asarray(value, np.float64), unit


def strip(unit, q):
    if not isinstance(q, Q):
        raise TypeError("expected a quantity")
    if q.unit == unit:
        return q.value
    to, f = Q.TO.get(q.unit, (None, None))
    if to != unit:
        raise ValueError(f"cannot strip {q.unit} to {unit}")
    return q.value * f


def _classes():
    class AbstractParameter:
        pass

    class ConstantParameter(AbstractParameter):
        def __init__(self, value):
            self.value = value

        def __call__(self, t):
            return self.value

    class LinearParameter(AbstractParameter):
        def __init__(self, slope, point_time, point_value):
            self.slope, self.point_time, self.point_value = slope, point_time, point_value

        def __call__(self, t):
            raise AssertionError("not evaluated by the conversion")

    class CustomParameter(AbstractParameter):
        def __call__(self, t):
            return 0.0

    class AbstractPotential:
        def __init__(self, **kw):
            for k, v in kw.items():
                setattr(self, k, v if isinstance(v, AbstractParameter) else ConstantParameter(v))

    class AbstractCompositePotential(AbstractPotential, dict):
        def __init__(self, **parts):
            dict.__init__(self, parts)

    ns = {c.__name__: c for c in (AbstractParameter, ConstantParameter, LinearParameter, CustomParameter,
                                  AbstractPotential, AbstractCompositePotential)}
    for name in ("HernquistPotential", "MiyamotoNagaiPotential", "NFWPotential", "PlummerPotential",
                 "MN3Sech2Potential", "PowerLawCutoffPotential", "GaussianPotential"):
        ns[name] = type(name, (AbstractPotential,), {})
    ns["MilkyWayPotential"] = type("MilkyWayPotential", (AbstractCompositePotential,), {})

    class TranslatedPotential(AbstractPotential):
        def __init__(self, base_potential, translation):
            self.base_potential, self.translation = base_potential, ConstantParameter(translation)

    ns["TranslatedPotential"] = TranslatedPotential
    return ns


def test_galax_milky_way_converts_to_the_same_component_table():
    import galax_gb300 as gx
    from galax_gb300.interop.convert import to_gb300

    g = _classes()
    mw = g["MilkyWayPotential"](
        disk=g["MiyamotoNagaiPotential"](m_tot=Q(6.8e10, "Msun"), a=Q(3000.0, "pc"), b=Q(0.28, "kpc")),
        halo=g["NFWPotential"](m=Q(5.4e11, "Msun"), r_s=Q(15.62, "kpc")),
        bulge=g["HernquistPotential"](m_tot=Q(5e9, "Msun"), r_s=Q(1.0, "kpc")),
        nucleus=g["HernquistPotential"](m_tot=Q(1.71e9, "Msun"), r_s=Q(70.0, "pc")))
    got = to_gb300(mw, strip).component_array()
    want = gx.MilkyWayPotential().component_array()
    for f in ("kind", "m", "l1", "l2", "origin"):
        np.testing.assert_allclose(got[f], want[f], rtol=1e-15, atol=0)


def test_linear_parameter_translation_and_mn3_convert():
    import galax_gb300 as gx
    from galax_gb300.interop.convert import to_gb300

    g = _classes()
    lin = g["LinearParameter"](Q(-1e9, "Msun / Myr"), Q(0.5, "Gyr"), Q(1e12, "Msun"))
    kep = g["PlummerPotential"](m_tot=lin, r_s=Q(2.0, "kpc"))
    got = to_gb300(g["TranslatedPotential"](kep, Q([1.0, -2.0, 3.0], "kpc")), strip)
    arr = got.component_array()
    assert np.allclose(arr["origin"][0], [1.0, -2.0, 3.0])
    assert arr["m"][0] == pytest.approx(1e12 + 1e9 * 500.0)  # the value at t = 0
    np.testing.assert_allclose(got.slopes(), [[-1e9, 0.0, 0.0]])
    disk = g["MN3Sech2Potential"](m_tot=Q(4.7717e10, "Msun"), h_R=Q(2.6, "kpc"), h_z=Q(0.3, "kpc"))
    disk.positive_density = True
    want = gx.MN3Sech2Potential(m_tot=4.7717e10, h_R=2.6, h_z=0.3, positive_density=True).component_array()
    np.testing.assert_allclose(to_gb300(disk, strip).component_array()["m"], want["m"], rtol=1e-15)


def test_unsupported_galax_objects_raise_not_implemented():
    from galax_gb300.interop.convert import to_gb300

    g = _classes()
    with pytest.raises(NotImplementedError):
        to_gb300(g["GaussianPotential"](m_tot=Q(1.0, "Msun")), strip)
    with pytest.raises(NotImplementedError):
        to_gb300(g["HernquistPotential"](m_tot=g["CustomParameter"](), r_s=Q(1.0, "kpc")), strip)


def test_entry_points_name_the_plugin_module():
    if sys.version_info < (3, 11):
        pytest.skip("tomllib")
    import tomllib

    meta = tomllib.loads((ROOT / "pyproject.toml").read_text())
    eps = meta["project"]["entry-points"]
    for group in ("galax.potential.interop", "galax.dynamics.interop"):
        assert eps[group]["gb300"] == "galax_gb300.interop.galax_plugin"
    src = (ROOT / "galax_gb300" / "interop" / "galax_plugin.py").read_text()
    for fn in ("gd.evaluate_orbit", "gp.potential", "gp.gradient", "gp.acceleration"):
        assert f"@{fn}.dispatch" in src
    ast.parse(src)
