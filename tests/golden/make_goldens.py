"""Extract golden vectors from the reference's tests and doctests.

The reference (GalacticDynamics/galax) cannot be imported here (it needs JAX,
diffrax, unxt, ...), so its golden values are read as text from the cited lines
of its test files and docstrings and written, with the inputs each one belongs
to, into ``reference_goldens.json`` beside this script. Run:

    python tests/golden/make_goldens.py /root/reference

Only this generator reads the reference tree; the tests read the JSON.
"""

from __future__ import annotations

import json
import re
import sys
from pathlib import Path

NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")
KMS = 0.001022712165045695  # 1 km/s in kpc/Myr

# (name, file, [line numbers]): every number on those lines, in order.
POTENTIAL_SPECS = [
    ("hernquist", "tests/unit/potential/builtin/test_hernquist.py", [31], [35], [46, 47, 48]),
    ("miyamoto_nagai", "tests/unit/potential/builtin/test_miyamotonagai.py", [40], [44], [55, 56, 57]),
    ("nfw", "tests/unit/potential/builtin/test_nfw.py", [40], [44], [56, 57, 58]),
    ("plummer", "tests/unit/potential/builtin/test_plummer.py", [38], [42], [53, 54, 55]),
    ("milky_way", "tests/unit/potential/builtin/test_milkywaypotential.py", [43], [48], [61, 62, 63]),
    ("isochrone", "tests/unit/potential/builtin/test_isochrone.py", [31], [35], [46, 47, 48]),
    ("logarithmic", "tests/unit/potential/builtin/test_logarithmic.py", [38], [43], [55, 56, 57]),
    ("mn3_exponential", "tests/unit/potential/builtin/test_mn3.py", [49], [54], [67, 68, 69]),
    ("mn3_sech2", "tests/unit/potential/builtin/test_mn3.py", [124], [129], [142, 143, 144]),
    ("milky_way_2022", "tests/unit/potential/builtin/test_milkywaypotential2022.py", [43], [49], [64, 65, 66]),
    ("powerlaw_cutoff", "tests/unit/potential/builtin/test_powerlawcutoff.py", [100], [104], [115, 116, 117]),
    ("bovy_mw_2014", "tests/unit/potential/builtin/test_bovymwpotential2014.py", [32], [36], [49, 50, 51]),
]
# density and tidal-tensor goldens of the same fixtures: (density line, tidal tensor lines)
DERIVED_SPECS = {
    "hernquist": ([40], [61, 62, 63]),
    "miyamoto_nagai": ([49], [70, 71, 72]),
    "nfw": ([50], [104, 105, 106]),
    "plummer": ([47], [68, 69, 70]),
    "milky_way": ([54], [76, 77, 78]),
    "isochrone": ([40], [61, 62, 63]),
    "logarithmic": ([48], [71, 72, 73]),
    "mn3_exponential": ([61], [82, 83, 84]),
    "mn3_sech2": ([136], [157, 158, 159]),
    "milky_way_2022": ([57], [79, 80, 81]),
    "powerlaw_cutoff": ([109], [130, 131, 132]),
    "bovy_mw_2014": ([42], [64, 65, 66]),
}
# densities printed in Msun / pc^3 instead of galactic units (Msun / kpc^3)
DENSITY_SCALE = {"bovy_mw_2014": 1e9}
# parameters of each fixture: tests/unit/potential/builtin/test_common.py
# (m_tot = m = 1e12 Msun, r_s = a = b = 1 kpc); MilkyWay uses its defaults.
POTENTIAL_PARAMS = {
    "hernquist": {"kind": "hernquist", "m": 1e12, "l1": 1.0, "l2": 0.0},
    "miyamoto_nagai": {"kind": "miyamoto_nagai", "m": 1e12, "l1": 1.0, "l2": 1.0},
    "nfw": {"kind": "nfw", "m": 1e12, "l1": 1.0, "l2": 0.0},
    "plummer": {"kind": "plummer", "m": 1e12, "l1": 1.0, "l2": 0.0},
    "milky_way": {"kind": "milky_way"},
    "isochrone": {"kind": "isochrone", "m": 1e12, "l1": 1.0, "l2": 0.0},
    # v_c = 220 km/s (test_common.py:359-360), stored in m in kpc/Myr
    "logarithmic": {"kind": "logarithmic", "m": 220 * KMS, "l1": 1.0, "l2": 0.0},
    # m_tot = 1e12 Msun, h_R = h_z = 1 kpc, positive_density False (test_common.py:26-27, 305-306, 331-332)
    "mn3_exponential": {"kind": "mn3_exponential", "m": 1e12, "h_R": 1.0, "h_z": 1.0, "positive_density": False},
    "mn3_sech2": {"kind": "mn3_sech2", "m": 1e12, "h_R": 1.0, "h_z": 1.0, "positive_density": False},
    "milky_way_2022": {"kind": "milky_way_2022"},
    # m_tot = 1e12 Msun, alpha = 0.9, r_c = 1 kpc (test_powerlawcutoff.py:21-22, 47-48)
    "powerlaw_cutoff": {"kind": "powerlaw_cutoff", "m": 1e12, "l1": 1.0, "l2": 0.9},
    "bovy_mw_2014": {"kind": "bovy_mw_2014"},
}


def numbers(root: Path, rel: str, lines: list[int]) -> list[float]:
    text = (root / rel).read_text().splitlines()
    out: list[float] = []
    for ln in lines:
        line = text[ln - 1]
        # drop unit strings such as "kpc2 / Myr2" before scanning numbers
        line = re.sub(r'"[^"]*"', "", line)
        # digit-group separators (33_365_858.46)
        line = re.sub(r"(?<=\d)_(?=\d)", "", line)
        # drop identifiers (dtype=float64, CartesianPos3D, ...) so only literals remain
        line = re.sub(r"\b[A-Za-z_][A-Za-z_0-9]*", " ", line)
        out += [float(x) for x in NUM.findall(line)]
    return out


def main(root: Path) -> None:
    g: dict = {"source": "GalacticDynamics/galax tests and doctests (see 'cite' fields)", "potentials": {}, "orbits": {}}
    for name, rel, lphi, lgrad, lhess in POTENTIAL_SPECS:
        phi = numbers(root, rel, lphi)
        grad = numbers(root, rel, lgrad)
        hess = numbers(root, rel, lhess)
        assert len(phi) == 1 and len(grad) == 3 and len(hess) == 9, (name, phi, grad, hess)
        g["potentials"][name] = {
            "cite": f"{rel}:{lphi[0]},{lgrad[0]},{lhess[0]}-{lhess[-1]}",
            "params": POTENTIAL_PARAMS[name],
            "x": [1.0, 2.0, 3.0],
            "t": 0.0,
            "potential": phi[0],
            "gradient": grad,
            "hessian": hess,
            "tol": {"atol": 1e-8, "rtol": 1e-5},
        }
        ldens, ltidal = DERIVED_SPECS[name]
        dens = numbers(root, rel, ldens)
        tidal = numbers(root, rel, ltidal)
        assert len(dens) == 1 and len(tidal) == 9, (name, dens, tidal)
        g["potentials"][name]["density"] = dens[0] * DENSITY_SCALE.get(name, 1.0)
        g["potentials"][name]["tidal_tensor"] = tidal
        g["potentials"][name]["cite_derived"] = f"{rel}:{ldens[0]},{ltidal[0]}-{ltidal[-1]}"

    f = "src/galax/dynamics/_src/orbit/solver.py"
    v220 = 220 * KMS
    step = numbers(root, f, [318, 319, 320, 321])
    g["orbits"]["dopri8_single_step"] = {
        "cite": f"{f}:290-321",
        "potential": {"kind": "hernquist", "m": 1e12, "l1": 5.0, "l2": 0.0},
        "solver": {"method": 8, "adaptive": False, "dt0": 10.0},
        "y0": [[8, 0, 9, 0, v220, 0], [9, 0, 3, 0, v220, 0]],
        "t0": 0.0, "t1": 10.0, "save_ts": [10.0],
        "expect_q": [step[0:3], step[3:6]], "expect_p": [step[6:9], step[9:12]],
        "digits": 8,
    }
    run = numbers(root, f, [376, 377, 378, 379])
    g["orbits"]["dopri8_pid_lockstep_run"] = {
        "cite": f"{f}:348-379",
        "potential": {"kind": "hernquist", "m": 1e12, "l1": 5.0, "l2": 0.0},
        "solver": {"method": 8, "adaptive": True, "rtol": 1e-8, "atol": 1e-8, "lockstep": True},
        "y0": [[8, 0, 9, 0, v220, 0], [9, 0, 3, 0, v220, 0]],
        "t0": 0.0, "t1": 1000.0, "save_ts": [1000.0],
        "expect_q": [run[0:3], run[3:6]], "expect_p": [run[6:9], run[9:12]],
        "digits": 8,
    }
    s1 = numbers(root, f, [441, 442])
    g["orbits"]["dopri8_pid_solve_220kms"] = {
        "cite": f"{f}:431-442",
        "potential": {"kind": "hernquist", "m": 1e12, "l1": 5.0, "l2": 0.0},
        "solver": {"method": 8, "adaptive": True, "rtol": 1e-8, "atol": 1e-8},
        "y0": [[8, 0, 0, 0, v220, 0]], "t0": 0.0, "t1": 1000.0, "save_ts": [1000.0],
        "expect_q": [s1[0:3]], "expect_p": [s1[3:6]], "digits": 8,
    }
    s2 = numbers(root, f, [456, 457])
    g["orbits"]["dopri8_pid_solve_array"] = {
        "cite": f"{f}:451-457",
        "potential": {"kind": "hernquist", "m": 1e12, "l1": 5.0, "l2": 0.0},
        "solver": {"method": 8, "adaptive": True, "rtol": 1e-8, "atol": 1e-8},
        "y0": [[8, 0, 0, 0, 0.22499669, 0]], "t0": 0.0, "t1": 1000.0, "save_ts": [1000.0],
        "expect_q": [s2[0:3]], "expect_p": [s2[3:6]], "digits": 8,
    }

    f = "src/galax/dynamics/_src/solver.py"
    for key, lines_q, lines_p, v in (
        ("kepler_integrate_field_array", [356, 357, 359, 360], [361, 362, 364, 365], 0.22499668),
        ("kepler_integrate_field_quantity", [378, 379, 381, 382], [383, 384, 386, 387], v220),
    ):
        q = numbers(root, f, lines_q)
        p = numbers(root, f, lines_p)
        g["orbits"][key] = {
            "cite": f"{f}:{lines_q[0]}-{lines_p[-1]} (solver defaults {f}:226-232)",
            "potential": {"kind": "kepler", "m": 1e11, "l1": 0.0, "l2": 0.0},
            "solver": {"method": 8, "adaptive": True, "rtol": 1e-7, "atol": 1e-7, "dtmin": 0.05},
            "y0": [[8, 0, 0, 0, v, 0]], "t0": 0.0, "t1": 1000.0,
            "save_ts_linspace": [0.0, 1000.0, 100], "rows": [0, 1, 98, 99],
            "expect_q": [q[0:3], q[3:6], q[6:9], q[9:12]], "expect_p": [p[0:3], p[3:6], p[6:9], p[9:12]],
        }

    f = "src/galax/dynamics/_src/experimental/integrate.py"
    q = numbers(root, f, [175, 176, 178])
    p = numbers(root, f, [179, 180, 182])
    g["orbits"]["nfw_integrate_orbit"] = {
        "cite": f"{f}:157-182 (solver defaults {f}:28-35)",
        "potential": {"kind": "nfw", "m": 1e12, "l1": 15.0, "l2": 0.0},
        "solver": {"method": 8, "adaptive": True, "rtol": 1e-7, "atol": 1e-7, "dtmin": 0.3},
        "y0": [[15.0, 0, 0, 0, 0.225, 0]], "t0": 0.0, "t1": 10.0,
        "save_ts_linspace": [0.0, 10.0, 100], "rows": [0, 1, 99],
        "expect_q": [q[0:3], q[3:6], q[6:9]], "expect_p": [p[0:3], p[3:6], p[6:9]], "digits": 8,
    }

    f = "src/galax/dynamics/_src/legacy/integrator.py"
    q = numbers(root, f, [92])
    p = numbers(root, f, [94])
    g["orbits"]["legacy_integrator_1gyr"] = {
        "cite": f"{f}:76-95 (defaults {f}:161-168)",
        "potential": {"kind": "hernquist", "m": 1e12, "l1": 5.0, "l2": 0.0},
        "solver": {"method": 8, "adaptive": True, "rtol": 1e-7, "atol": 1e-7},
        "y0": [[10, 0, 0, 0, 200 * KMS, 0]], "t0": 0.0, "t1": 1000.0, "save_ts": [1000.0],
        "expect_q": [q[0:3]], "expect_p": [p[0:3]], "digits": 3,
    }

    f = "src/galax/potential/_src/params/core.py"
    rho = numbers(root, f, [72, 73])
    g["orbits"]["kepler_linear_mass"] = {
        "cite": f"{f}:52-74 (LinearParameter; compute_orbit's default OrbitSolver, orbit/solver.py:121-141)",
        "potential": {"kind": "kepler", "m": 1e12, "l1": 0.0, "l2": 0.0},
        # slope -1e3 Msun/yr = -1e9 Msun/Myr through (t = 0, 1e12 Msun)
        "slopes": [[-1e9, 0.0, 0.0]],
        "solver": {"method": 8, "adaptive": True, "rtol": 1e-8, "atol": 1e-8, "max_steps": 65536},
        "y0": [[5.0, 0.0, 0.0, 0.0, 1000 * KMS, 0.0]], "t0": 0.0, "t1": 1000.0,
        "save_ts_linspace": [0.0, 1000.0, 10], "expect_rho": rho, "rho_decimals": 3,
    }

    f = "src/galax/dynamics/_src/orbit/field_hamiltonian.py"
    fv = numbers(root, f, [118, 119])
    g["fields"] = {"hamiltonian_kepler": {
        "cite": f"{f}:103-119 (HamiltonianField(KeplerPotential(1e11)) at t = 0)",
        "potential": {"kind": "kepler", "m": 1e11, "l1": 0.0, "l2": 0.0},
        "x": [8.0, 0.0, 0.0], "v": [0.0, 0.22499668, 0.0],
        "dq_dt": fv[0:3], "dp_dt": fv[3:6], "decimals": 8,
    }}

    g["stream"] = {}
    f = "src/galax/dynamics/_src/cluster/api.py"
    rt = numbers(root, f, [198])
    g["stream"]["king_tidal_radius"] = {
        "cite": f"{f}:190-198 (King 1962, cluster/radius.py:198-214)",
        "potential": {"kind": "nfw", "m": 1e12, "l1": 20.0, "l2": 0.0},
        "x": [8.0, 0.0, 0.0], "v": [8.0, 0.0, 0.0], "mass": 1e4,
        "r_tidal": rt[0],
    }
    f = "src/galax/dynamics/_src/experimental/df.py"
    s = numbers(root, f, [117, 118, 119, 120])
    g["stream"]["fardal2015_sample"] = {
        "cite": f"{f}:106-120 (draws from jax.random.key(0), not reproducible here)",
        "potential": {"kind": "nfw", "m": 1e12, "l1": 15.0, "l2": 0.0},
        "x": [15.0, 0.0, 0.0], "v": [0.0, 220.0, 0.0], "mass": 1e5,
        "x_lead": s[0:3], "v_lead": s[3:6], "x_trail": s[6:9], "v_trail": s[9:12],
    }

    out = Path(__file__).with_name("reference_goldens.json")
    out.write_text(json.dumps(g, indent=1) + "\n")
    print(f"wrote {out}")


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
