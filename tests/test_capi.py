"""The C-ABI library without a GPU: it loads, exports every symbol the header
declares, and carries the same tableaux as the oracle (host-only calls)."""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "galax_gb300.h"


@pytest.fixture(scope="module")
def lib():
    from galax_gb300 import _lib
    from galax_gb300.build import build

    build()
    return _lib.load()


def declared_symbols() -> list[str]:
    text = HEADER.read_text()
    return re.findall(r"^GAL_API\s+[\w\s\*]+?\b(gal_\w+)\(", text, flags=re.M)


def test_header_declares_the_api():
    syms = declared_symbols()
    assert len(syms) >= 19
    for s in ("gal_potential_create", "gal_eval_gradient", "gal_integrate", "gal_adjoint"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    from galax_gb300 import _lib

    for s in declared_symbols():
        assert hasattr(lib, s), s
        assert s in _lib.SIGNATURES, f"{s} has no ctypes signature"


def test_abi_version_and_status_strings(lib):
    assert lib.gal_abi_version() == 1
    assert lib.gal_status_string(0) == b"ok"
    assert lib.gal_status_string(4) == b"workspace too small"
    assert lib.gal_status_string(6) == b"host allocation failed"
    # every status the header declares has its own message
    codes = [int(v) for v in re.findall(r"GAL_(?:OK|ERR_[A-Z_]+) = (\d+)", HEADER.read_text())]
    assert sorted(codes) == list(range(len(codes)))
    msgs = [lib.gal_status_string(c) for c in codes]
    assert len(set(msgs)) == len(codes) and b"unknown status" not in msgs
    assert lib.gal_status_string(len(codes)) == b"unknown status"


@pytest.mark.parametrize("method", [5, 8])
def test_tableau_matches_oracle_bitwise(lib, method):
    c = np.zeros(13); a = np.zeros(169); b = np.zeros(13); e = np.zeros(13)
    s = lib.gal_tableau(method, c.ctypes.data, a.ctypes.data, b.ctypes.data, e.ctypes.data)
    oc, oa, ob, oe = O.tableau(method)
    assert s == len(oc)
    assert np.array_equal(c[:s], oc)
    assert np.array_equal(a.reshape(13, 13)[:s, :s], oa)
    assert np.array_equal(b[:s], ob)
    assert np.array_equal(e[:s], oe)
    assert lib.gal_tableau(7, c.ctypes.data, a.ctypes.data, b.ctypes.data, e.ctypes.data) == 0


def test_struct_layouts_match_oracle():
    from galax_gb300 import _lib

    assert _lib.COMPONENT_DTYPE == O.COMP_DTYPE
    assert C.sizeof(_lib.SolverConfig) == C.sizeof(O.SolverCfg)


def test_validation_without_gpu(lib):
    """Argument checks run on the host and fail before any device work."""
    from galax_gb300 import _lib

    h = C.c_void_p()
    bad = np.zeros(1, _lib.COMPONENT_DTYPE)
    bad[0]["kind"] = 9
    assert lib.gal_potential_create(bad.ctypes.data, 1, 1.0, C.byref(h)) == 2
    assert b"unsupported" in lib.gal_last_error()
    bad[0]["kind"] = _lib.GAL_NFW
    bad[0]["m"] = 1.0
    bad[0]["l1"] = 0.0
    assert lib.gal_potential_create(bad.ctypes.data, 1, 1.0, C.byref(h)) == 1
    assert lib.gal_potential_create(bad.ctypes.data, 0, 1.0, C.byref(h)) == 1
    bad[0]["kind"] = _lib.GAL_MIYAMOTO_NAGAI  # a <= -b would let sqrt(z^2 + b^2) + a vanish
    bad[0]["l1"], bad[0]["l2"] = -1.0, 1.0
    assert lib.gal_potential_create(bad.ctypes.data, 1, 1.0, C.byref(h)) == 1
    bad[0]["kind"] = _lib.GAL_POWERLAW_CUTOFF  # alpha >= 2 or r_c <= 0: galax's potential is not finite
    bad[0]["l1"], bad[0]["l2"] = 1.0, 2.0
    assert lib.gal_potential_create(bad.ctypes.data, 1, 1.0, C.byref(h)) == 1
    bad[0]["l1"], bad[0]["l2"] = 0.0, 1.0
    assert lib.gal_potential_create(bad.ctypes.data, 1, 1.0, C.byref(h)) == 1
    nbytes = C.c_size_t()
    cfg = _lib.solver_config(8, False, dt0=1.0)
    assert lib.gal_integrate_workspace_size(C.byref(cfg), 10, C.byref(nbytes)) == 0 and nbytes.value >= 8
    assert lib.gal_set_launch(8, 0, 100, 0, 0) == 1  # not a multiple of 32
    assert lib.gal_set_launch(8, 0, 128, 0, 3) == 1  # unknown register variant
    assert lib.gal_set_launch(8, 0, 256, 0, 0) == 1  # variant 0 takes at most 128 threads
    assert lib.gal_set_split_fraction(C.c_double(0.0)) == 1 and lib.gal_set_split_fraction(C.c_double(0.95)) == 1
    assert lib.gal_set_split_fraction(C.c_double(0.1)) == 0


def test_python_api_rejects_unsupported_inputs():
    import galax_gb300 as gx

    with pytest.raises(NotImplementedError):
        gx.HernquistPotential(m_tot=1e12, r_s=5.0, units="solarsystem")
    with pytest.raises(NotImplementedError):
        gx.HernquistPotential(m_tot=lambda t: 1e12, r_s=5.0)
    with pytest.raises(NotImplementedError):
        gx.Integrator(solver="Tsit5").config()
    with pytest.raises(NotImplementedError):
        gx.PIDController(rtol=1e-7, atol=1e-7, jump_ts=[1.0])
    mw = gx.MilkyWayPotential()
    arr = mw.component_array()
    assert list(arr["kind"]) == [2, 3, 1, 1]
    np.testing.assert_array_equal(arr, O.milky_way())


def test_workloads_follow_their_distributions():
    from galax_gb300 import workloads as W

    grad = lambda x: O.gradient(O.milky_way(), x)  # noqa: E731
    y = W.disk_like_ics(grad, 2000, seed=0)
    r = np.linalg.norm(y[:, :3], axis=1)
    assert r.min() >= 4 and r.max() <= 20
    vz_kms = y[:, 5] / W.KMS
    assert 10 < np.std(vz_kms) < 40
    b = W.uneven_ics(grad, 3000, seed=1)
    ns = np.diff(b.save_offsets)
    assert ns.min() >= 10 and ns.max() <= 1000
    assert np.all(b.t1 >= 100 - 1e-9) and np.all(b.t1 <= 5000 + 1e-9)
    assert np.allclose(b.save_ts[b.save_offsets[1:] - 1], b.t1)
    assert np.all(b.save_ts[b.save_offsets[:-1]] == 0)
    r = np.linalg.norm(b.y0[:, :3], axis=1)
    assert np.allclose(np.sum(b.y0[:, :3] * b.y0[:, 3:], axis=1) / r, 0, atol=1e-12)  # tangential


def test_flop_constants_match_counted_oracle():
    from galax_gb300 import flops

    for method in (5, 8):
        g, s = O.count_ops(O.milky_way(), method)
        assert sum(g.values()) == flops.GRADIENT_FLOPS_MW
        assert sum(s.values()) == flops.STEP_FLOPS_MW[method]
        c = np.concatenate([O.milky_way(), O.comps([(O.PLUMMER, 1e5, 0.02, 0.0, (1.0, 2.0, 3.0))])])
        _, s = O.count_ops(c, method)
        assert sum(s.values()) == flops.STEP_FLOPS_MW_PLUMMER[method]
    from galax_gb300 import workloads as W

    m, b, c = W.subhalo_table(3, 512)
    sub = O.comps([(O.PLUMMER, float(m[i]), float(b[i]), 0.0, tuple(c[i])) for i in range(512)])
    for method in (5, 8):
        _, s = O.count_ops(np.concatenate([O.milky_way(), sub]), method)
        assert sum(s.values()) == flops.STEP_FLOPS_MW_SUBHALOS[method]


def test_mn3_and_milky_way_2022_component_tables():
    """The front end expands MN3 disks into the same three Miyamoto-Nagai
    components as the oracle's restatement of galax's fit (whose potentials
    match galax's goldens), and MilkyWayPotential2022 into six components."""
    from galax_gb300 import potential as P

    for cls, profile in ((P.MN3ExponentialPotential, "exponential"), (P.MN3Sech2Potential, "sech2")):
        for pos in (False, True):
            got = cls(m_tot=3e10, h_R=2.5, h_z=0.4, positive_density=pos).component_array()
            want = O.comps(O.mn3(3e10, 2.5, 0.4, profile, pos))
            for f in ("kind", "m", "l1", "l2"):
                np.testing.assert_allclose(got[f], want[f], rtol=1e-14)
    got = P.MilkyWayPotential2022().component_array()
    want = O.milky_way_2022()
    for f in ("kind", "m", "l1", "l2"):
        np.testing.assert_allclose(got[f], want[f], rtol=1e-14)


def test_linear_parameters_on_the_host():
    """LinearParameter semantics and the slope table the front end hands to
    gal_potential_set_linear (no GPU needed)."""
    import galax_gb300 as gx

    lp = gx.LinearParameter(slope=-1e9, point_time=100.0, point_value=1e12)
    assert lp(100.0) == 1e12 and lp(0.0) == lp.value_at_zero == 1e12 + 1e11
    pot = gx.CompositePotential(a=gx.KeplerPotential(m_tot=lp),
                                b=gx.PowerLawCutoffPotential(m_tot=1e10, alpha=gx.LinearParameter(1e-4, 0.0, 1.0),
                                                             r_c=2.0),
                                c=gx.NFWPotential(m=1e11, r_s=10.0))
    np.testing.assert_array_equal(pot.slopes(), [[-1e9, 0, 0], [0, 0, 1e-4], [0, 0, 0]])
    assert pot.component_array()["m"][0] == 1.1e12  # the table holds the values at t = 0
    assert gx.MilkyWayPotential().slopes() is None
    with pytest.raises(NotImplementedError):
        gx.KeplerPotential(m_tot=lambda t: 1e12)  # other callables stay unsupported
    # MN3: a linear m_tot is exact as per-disk slopes; the scale lengths must be constant
    mn3 = gx.MN3Sech2Potential(m_tot=gx.LinearParameter(2e8, 0.0, 5e10), h_R=3.0, h_z=0.3)
    ref = gx.MN3Sech2Potential(m_tot=5e10, h_R=3.0, h_z=0.3)
    np.testing.assert_array_equal(mn3.component_array(), ref.component_array())
    masses = ref.component_array()["m"]
    np.testing.assert_allclose(mn3.slopes()[:, 0], masses / 5e10 * 2e8, rtol=1e-15)
    assert not mn3.slopes()[:, 1:].any() and ref.slopes() is None
    with pytest.raises(NotImplementedError, match="h_R"):
        gx.MN3ExponentialPotential(m_tot=5e10, h_R=gx.LinearParameter(1e-3, 0.0, 3.0), h_z=0.3)


def test_set_linear_validates_on_the_host(lib):
    assert lib.gal_potential_set_linear(None, None) == 1


def test_struct_layouts_match_the_header(tmp_path):
    """Every field of the header's structs sits at the offset the ctypes and
    NumPy layouts use (the header compiled as C99 by the host compiler)."""
    import shutil
    import subprocess

    from galax_gb300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    layouts = {
        "gal_component": {n: (_lib.COMPONENT_DTYPE.fields[n][1]) for n in _lib.COMPONENT_DTYPE.names},
        "gal_solver_config": {n: getattr(_lib.SolverConfig, n).offset for n, _ in _lib.SolverConfig._fields_},
        "gal_stream_config": {n: getattr(_lib.StreamConfig, n).offset for n, _ in _lib.StreamConfig._fields_},
    }
    sizes = {"gal_component": _lib.COMPONENT_DTYPE.itemsize, "gal_solver_config": C.sizeof(_lib.SolverConfig),
             "gal_stream_config": C.sizeof(_lib.StreamConfig)}
    lines = ['#include "galax_gb300.h"', "#include <stdio.h>", "#include <stddef.h>", "int main(void) {"]
    for st, fields in layouts.items():
        lines.append(f'  printf("{st} size %zu\\n", sizeof({st}));')
        for f in fields:
            lines.append(f'  printf("{st} {f} %zu\\n", offsetof({st}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", str(HEADER.parent), "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for ln in filter(None, out):
        st, f, v = ln.split()
        got[(st, f)] = int(v)
    for st, fields in layouts.items():
        assert got[(st, "size")] == sizes[st], st
        for f, off in fields.items():
            assert got[(st, f)] == off, (st, f)


def test_ctypes_signatures_match_the_header_arity():
    """Each ctypes binding passes as many arguments as the header's prototype
    declares (a missing or extra argument would shift every later one)."""
    from galax_gb300 import _lib

    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    protos = re.findall(r"GAL_API\s+[\w\s\*]+?\b(gal_\w+)\((.*?)\);", text, flags=re.S)
    assert len(protos) == len(declared_symbols())
    for name, params in protos:
        params = params.strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        assert len(_lib.SIGNATURES[name][1]) == n, (name, n, len(_lib.SIGNATURES[name][1]))


def test_ctypes_argument_types_match_the_header():
    """Scalars are bound with the header's width and kind (an int32 passed
    where an int64 is declared leaves the upper half of the register
    undefined); pointers and streams are bound as pointers."""
    from galax_gb300 import _lib

    scalar = {"int32_t": C.c_int32, "int64_t": C.c_int64, "uint64_t": C.c_uint64, "double": C.c_double,
              "float": C.c_float,
              "size_t": C.c_size_t}
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    for name, params in re.findall(r"GAL_API\s+[\w\s\*]+?\b(gal_\w+)\((.*?)\);", text, flags=re.S):
        decl = [p.strip() for p in params.split(",") if p.strip() and p.strip() != "void"]
        for i, (p, t) in enumerate(zip(decl, _lib.SIGNATURES[name][1])):
            ctype = " ".join(p.split()[:-1])
            if "*" in p or ctype == "gal_stream_t":
                is_ptr = t is C.c_void_p or t is C.c_char_p or issubclass(t, C._Pointer) or hasattr(t, "_dtype_")
                assert is_ptr, (name, i, p, t)
            else:
                assert C.sizeof(t) == C.sizeof(scalar[ctype]) and (t._type_ in "fd") == (ctype in ("float", "double")), \
                    (name, i, p, t)


def test_ctypes_return_types_match_the_header():
    from galax_gb300 import _lib

    want = {"gal_status": C.c_int32, "int32_t": C.c_int32, "int64_t": C.c_int64, "const char*": C.c_char_p}
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    for ret, name in re.findall(r"GAL_API\s+([\w\s\*]+?)\b(gal_\w+)\(", text):
        r, w = _lib.SIGNATURES[name][0], want[" ".join(ret.split())]
        assert r is w or (w is not C.c_char_p and C.sizeof(r) == C.sizeof(w) and r._type_ in "ilq"), (name, r)
