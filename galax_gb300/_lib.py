"""ctypes binding of the C ABI in ``include/galax_gb300.h``.

The shared library is built in-tree by ``galax_gb300.build``. There is no CPU
fallback: if the library is missing or no CUDA device is present, the calls
that need it raise.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgalax_gb300.so"

(GAL_KEPLER, GAL_HERNQUIST, GAL_MIYAMOTO_NAGAI, GAL_NFW, GAL_PLUMMER, GAL_ISOCHRONE, GAL_LOGARITHMIC,
 GAL_POWERLAW_CUTOFF) = range(8)
ORBIT_STATUS = {0: "successful", 1: "max_steps_reached", 2: "dt_min_reached", 3: "non_finite"}

COMPONENT_DTYPE = np.dtype(
    [("kind", "<i4"), ("flags", "<i4"), ("m", "<f8"), ("l1", "<f8"), ("l2", "<f8"), ("origin", "<f8", (3,))],
    align=True,
)
assert COMPONENT_DTYPE.itemsize == 56


class SolverConfig(C.Structure):
    """``gal_solver_config``."""

    _fields_ = [
        ("method", C.c_int32),
        ("adaptive", C.c_int32),
        ("max_steps", C.c_int64),
        ("dt0", C.c_double),
        ("rtol", C.c_double),
        ("atol", C.c_double),
        ("dtmin", C.c_double),
        ("dtmax", C.c_double),
        ("pcoeff", C.c_double),
        ("icoeff", C.c_double),
        ("dcoeff", C.c_double),
        ("safety", C.c_double),
        ("factormin", C.c_double),
        ("factormax", C.c_double),
        ("force_dtmin", C.c_int32),
        ("schedule", C.c_int32),
    ]


class StreamConfig(C.Structure):
    """``gal_stream_config``."""

    _fields_ = [
        ("method", C.c_int32),
        ("k_ckpt", C.c_int32),
        ("n_release", C.c_int64),
        ("dt", C.c_double),
        ("t_now", C.c_double),
        ("prog_m", C.c_double),
        ("prog_b", C.c_double),
        ("w_now", C.c_double * 6),
        ("df", C.c_int32),
        ("reserved", C.c_int32),
        ("df_params", C.c_double * 8),
    ]


STREAM_DF_OFFSETS = 0
STREAM_DF_FARDAL2015 = 1
STREAM_DF_CHEN2024 = 2


class GalaxGB300Error(RuntimeError):
    """A call into the CUDA library failed."""


# name -> (restype, argtypes); every symbol the header declares
_VP, _DP, _I64P, _I32P = C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p
SIGNATURES = {
    "gal_potential_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_void_p)]),
    "gal_potential_destroy": (C.c_int, [C.c_void_p]),
    "gal_potential_update": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    "gal_potential_num_components": (C.c_int32, [C.c_void_p]),
    "gal_potential_is_milky_way": (C.c_int32, [C.c_void_p]),
    "gal_potential_is_time_dependent": (C.c_int32, [C.c_void_p]),
    "gal_eval_potential": (C.c_int, [C.c_void_p, _DP, C.c_double, C.c_int64, _DP, C.c_void_p]),
    "gal_eval_gradient": (C.c_int, [C.c_void_p, _DP, C.c_double, C.c_int64, _DP, C.c_void_p]),
    "gal_eval_acceleration": (C.c_int, [C.c_void_p, _DP, C.c_double, C.c_int64, _DP, C.c_void_p]),
    "gal_eval_hessian": (C.c_int, [C.c_void_p, _DP, C.c_double, C.c_int64, _DP, C.c_void_p]),
    "gal_integrate_workspace_size": (C.c_int, [C.POINTER(SolverConfig), C.c_int64, C.POINTER(C.c_size_t)]),
    "gal_integrate": (C.c_int, [C.c_void_p, C.POINTER(SolverConfig), _DP, _DP, _DP, _I64P, _DP, C.c_int64, _DP,
                                _I32P, _I64P, _I32P, C.c_int64, _VP, C.c_size_t, C.c_void_p]),
    "gal_integrate_noalloc": (C.c_int, [C.c_void_p, C.POINTER(SolverConfig), _DP, _DP, _DP, _I64P, _DP, C.c_int64,
                                        _DP, _I32P, _I64P, _I32P, C.c_int64, C.c_void_p]),
    "gal_set_launch": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "gal_set_team": (C.c_int, [C.c_int32]),
    "gal_set_split_fraction": (C.c_int, [C.c_double]),
    "gal_set_table_lanes": (C.c_int, [C.c_int32]),
    "gal_dense_coef_per_step": (C.c_int32, [C.c_int32]),
    "gal_integrate_dense": (C.c_int, [C.c_void_p, C.POINTER(SolverConfig), _DP, _DP, _DP, C.c_int64, C.c_int64, _DP,
                                      _DP, _I64P, _I32P, C.c_void_p]),
    "gal_dense_evaluate": (C.c_int, [C.c_void_p, C.c_int32, _DP, _DP, _I64P, C.c_int64, C.c_int64, _I64P, _DP,
                                     C.c_int64, _DP, C.c_void_p, C.c_void_p]),
    "gal_adjoint_workspace_size": (C.c_int, [C.c_void_p, C.POINTER(SolverConfig), C.c_double, C.c_double,
                                             C.c_int32, C.c_int64, C.POINTER(C.c_size_t)]),
    "gal_adjoint": (C.c_int, [C.c_void_p, C.POINTER(SolverConfig), _DP, C.c_double, C.c_double, _DP, _DP, _DP, _DP,
                              _DP, C.c_int32, C.c_int64, _VP, C.c_size_t, C.c_void_p]),
    "gal_stream_workspace_size": (C.c_int, [C.c_void_p, C.POINTER(StreamConfig), C.c_int32,
                                            C.POINTER(C.c_size_t)]),
    "gal_stream_run": (C.c_int, [C.c_void_p, C.POINTER(StreamConfig), _DP, _DP, _DP, _DP, _VP, C.c_size_t,
                                 C.c_void_p]),
    "gal_stream_grad": (C.c_int, [C.c_void_p, C.POINTER(StreamConfig), _DP, _DP, _DP, _DP, _DP, _DP, _VP,
                                  C.c_size_t, C.c_void_p]),
    "gal_potential_set_linear": (C.c_int, [C.c_void_p, _DP]),
    "gal_stream_df_sample": (C.c_int, [C.c_void_p, C.c_int32, _DP, _DP, _DP, _DP, C.c_int64, _DP, _DP, _DP,
                                       C.c_void_p]),
    "gal_mlp_num_params": (C.c_int64, []),
    "gal_mlp_workspace_size": (C.c_int, [C.c_int64, C.POINTER(C.c_size_t)]),
    "gal_mlp_workspace_error": (C.c_int, [_VP, C.c_int64, C.POINTER(C.c_int32), C.c_void_p]),
    "gal_mlp_forward_f32": (C.c_int, [_VP, _VP, C.c_int64, _VP, _VP, C.c_int32, _VP, C.c_size_t, C.c_void_p]),
    "gal_mlp_loss_grads": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_int64, C.c_float, C.c_float, C.c_int32, _VP,
                                     _VP, _VP, C.c_size_t, C.c_void_p]),
    "gal_mlp_train_step": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, C.c_int64, C.c_float, C.c_float,
                                     C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32, C.c_int32, _VP, _VP,
                                     C.c_size_t, C.c_void_p]),
    "gal_mlp_train_workspace_size": (C.c_int, [C.c_int64, C.POINTER(C.c_size_t)]),
    "gal_mlp_train": (C.c_int, [_VP, _VP, _VP, _VP, _VP, _VP, _VP, C.c_int64, C.c_int64, C.c_int32, C.c_float,
                                C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_uint64,
                                C.c_int32, _VP, _VP, C.c_size_t, C.c_void_p]),
    "gal_mlp_create": (C.c_int, [_VP, C.c_double, C.c_double, C.POINTER(C.c_void_p)]),
    "gal_mlp_destroy": (C.c_int, [_VP]),
    "gal_mlp_eval": (C.c_int, [_VP, _DP, C.c_int64, _DP, C.c_int32, C.c_double, _DP, C.c_void_p]),
    "gal_mlp_error": (C.c_int, [_VP, C.POINTER(C.c_int32)]),
    "gal_surrogate_workspace_size": (C.c_int, [C.c_int64, C.POINTER(C.c_size_t)]),
    "gal_split_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.POINTER(C.c_void_p)]),
    "gal_split_destroy": (C.c_int, [_VP]),
    "gal_split_eval": (C.c_int, [_VP, _DP, C.c_int64, _DP, _DP, C.c_void_p]),
    "gal_integrate_surrogate": (C.c_int, [_VP, _VP, _VP, C.c_double, C.c_double, C.c_double, _DP, C.c_int64,
                                          C.c_int32, _VP, C.c_size_t, C.c_void_p]),
    "gal_tableau": (C.c_int32, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gal_fp64_peak_probe": (C.c_int, [C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p]),
    "gal_status_string": (C.c_char_p, [C.c_int32]),
    "gal_last_error": (C.c_char_p, []),
    "gal_abi_version": (C.c_int32, []),
}

_lib = None
_lock = threading.Lock()


def load() -> C.CDLL:
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise GalaxGB300Error(
                    f"CUDA library not built ({LIB_PATH}); run `python -c 'import __graft_entry__ as g; g.build()'`"
                    " or `python -m galax_gb300.build`"
                )
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status: int, what: str) -> None:
    if status != 0:
        L = load()
        msg = L.gal_last_error().decode() or L.gal_status_string(status).decode()
        raise GalaxGB300Error(f"{what} failed ({L.gal_status_string(status).decode()}): {msg}")


def solver_config(
    method: int,
    adaptive: bool,
    *,
    dt0: float = 0.0,
    rtol: float = 1e-7,
    atol: float = 1e-7,
    dtmin: float | None = None,
    dtmax: float | None = None,
    pcoeff: float = 0.0,
    icoeff: float = 1.0,
    dcoeff: float = 0.0,
    safety: float = 0.9,
    factormin: float = 0.2,
    factormax: float = 10.0,
    force_dtmin: bool = True,
    max_steps: int = 2**62,
    schedule: bool = False,
) -> SolverConfig:
    return SolverConfig(
        int(method), int(bool(adaptive)), int(max_steps), float(dt0 or 0.0), float(rtol), float(atol),
        float(dtmin or 0.0), float(dtmax or 0.0), float(pcoeff), float(icoeff), float(dcoeff), float(safety),
        float(factormin), float(factormax), int(bool(force_dtmin)), int(bool(schedule)),
    )
