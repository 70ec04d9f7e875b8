"""Shared helpers for the test suite: golden-fixture decoding and seeded
initial conditions matching the benchmark workloads."""

from __future__ import annotations

import numpy as np

from oracle import oracle as O

KIND = {"kepler": O.KEPLER, "hernquist": O.HERNQUIST, "miyamoto_nagai": O.MIYAMOTO_NAGAI, "nfw": O.NFW,
        "plummer": O.PLUMMER, "isochrone": O.ISOCHRONE, "logarithmic": O.LOGARITHMIC,
        "powerlaw_cutoff": O.POWERLAW_CUTOFF}


def golden_comps(p: dict) -> np.ndarray:
    if p["kind"] == "milky_way":
        return O.milky_way()
    if p["kind"] == "milky_way_2022":
        return O.milky_way_2022()
    if p["kind"] == "bovy_mw_2014":
        return O.bovy_mw_2014()
    if p["kind"] in ("mn3_exponential", "mn3_sech2"):
        return O.comps(O.mn3(p["m"], p["h_R"], p["h_z"], p["kind"][4:], p["positive_density"]))
    return O.comps([(KIND[p["kind"]], p["m"], p["l1"], p["l2"])])


def golden_cfg(s: dict) -> O.SolverCfg:
    kw = dict(s)
    method = kw.pop("method")
    adaptive = kw.pop("adaptive")
    return O.solver_cfg(method, adaptive, **kw)


def golden_save_ts(case: dict) -> np.ndarray:
    if "save_ts" in case:
        return np.asarray(case["save_ts"], float)
    a, b, n = case["save_ts_linspace"]
    return np.linspace(a, b, int(n))
