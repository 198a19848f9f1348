"""Access to the reference golden cases stored under tests/golden/."""
import gzip
import json
import os

import numpy as np

from posidonius_gb300 import layout as L

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names(integrator="whfast"):
    """Golden cases of one integrator ("whfast", "ias15") or of all (None)."""
    out = sorted(d for d in os.listdir(GOLDEN) if os.path.isdir(os.path.join(GOLDEN, d)))
    if integrator is None:
        return out
    return [d for d in out if ("-ias15" in d) == (integrator == "ias15")]


def case_path(name, python_twin=False):
    return os.path.join(GOLDEN, name, "python_case.json.gz" if python_twin else "case.json.gz")


def case_dict(name, python_twin=False):
    with gzip.open(case_path(name, python_twin), "rb") as f:
        return json.loads(f.read())


def expected(name):
    """(n, 3) arrays of the final inertial position, velocity and acceleration."""
    with open(os.path.join(GOLDEN, name, "particles.json")) as f:
        parts = json.load(f)
    out = {}
    for key in ("inertial_position", "inertial_velocity", "inertial_acceleration"):
        out[key] = np.array([[p[key][c] for c in "xyz"] for p in parts])
    return out


def max_abs_error(body_f64, exp):
    """Largest absolute difference against the golden particle files."""
    n = exp["inertial_position"].shape[0]
    err = 0.0
    for key, sl in (("inertial_position", L.POS), ("inertial_velocity", L.VEL),
                    ("inertial_acceleration", L.ACC)):
        err = max(err, float(np.abs(body_f64[:n, sl] - exp[key]).max()))
    return err
