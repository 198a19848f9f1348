"""Copy the reference's golden WHFast and IAS15 cases into tests/golden/ (gzip-compressed).

Run once in a checkout that has the Posidonius reference mounted:

    python tests/golden/make_golden.py /root/reference

For every in-scope case of the reference's Rust integration tests
(tests/data/<case>/case.json = initial WHFast state written by
tests/common/universe.rs:36-44; tests/data/<case>/particle_<i>.json = final
inertial position/velocity/acceleration after integrating to the time limit,
tests/common/universe.rs:18-34) it writes <case>/case.json.gz and
<case>/particles.json (the particle files merged).  LeapFrog cases, and the
order cases whose case document the reference does not store, are skipped.
The Python-generated twins (posidonius/tests/data/<case>/case.json) of the three
integrator cases, which the reference steps once and compares
(tests/test_integrator.rs:58-70), are stored as <case>/python_case.json.gz.
"""
import glob
import gzip
import json
import os
import sys

IN_SCOPE = [
    "test_integrator-whfast_jacobi",
    "test_integrator-whfast_democraticheliocentric",
    "test_integrator-whfast_whds",
    "test_tides-enabled_tides",
    "test_tides-disabled_tides",
    "test_flattening-enabled_flattening",
    "test_flattening-disabled_flattening",
    "test_general_relativity-kidder1995",
    "test_general_relativity-none",
    "test_general_relativity-anderson1975",
    "test_general_relativity-newhall1983",
    "test_evolution-brown_dwarf_non_evolving",
    "test_evolution-m_dwarf_non_evolving",
    "test_evolution-brown_dwarf_leconte2011",
    "test_evolution-m_dwarf_baraffe1998",
    "test_evolution-m_dwarf_baraffe2015",
    "test_star_types-brown_dwarf",
    "test_star_types-m_dwarf",
    # wind (the solar-like star)
    "test_evolution-solar_like_non_evolving",
    "test_evolution-solar_like_baraffe1998",
    "test_evolution-solar_like_baraffe2015",
    "test_star_types-solar_like",
    "test_disk-disabled_disk",
    # dynamical tides of the solar-like host
    "test_evolution-solar_like_bolmontmathis2016",
    "test_evolution-solar_like_galletbolmont2017",
    # protoplanetary disk
    "test_disk-enabled_disk",
    # the IAS15 integrator (tests/test_integrator.rs:266-312)
    "test_integrator-ias15",
]


# Python-generated twins kept (one per coordinate system keeps the fixtures small)
PYTHON_TWINS = ["test_integrator-whfast_jacobi", "test_integrator-whfast_democraticheliocentric",
                "test_integrator-whfast_whds"]


def _write_gz(path, raw):
    with open(path, "wb") as f:
        with gzip.GzipFile(fileobj=f, mode="wb", compresslevel=9, mtime=0) as g:
            g.write(raw)


def main(ref):
    out_root = os.path.dirname(os.path.abspath(__file__))
    for case in IN_SCOPE:
        src = os.path.join(ref, "tests", "data", case)
        dst = os.path.join(out_root, case)
        os.makedirs(dst, exist_ok=True)
        with open(os.path.join(src, "case.json"), "rb") as f:
            raw = f.read()
        json.loads(raw)  # validate
        _write_gz(os.path.join(dst, "case.json.gz"), raw)
        parts = []
        for i in range(len(glob.glob(os.path.join(src, "particle_*.json")))):
            with open(os.path.join(src, f"particle_{i}.json")) as f:
                parts.append(json.load(f))
        with open(os.path.join(dst, "particles.json"), "w") as f:
            json.dump(parts, f, indent=1)
        py = os.path.join(ref, "posidonius", "tests", "data", case, "case.json")
        if case in PYTHON_TWINS and os.path.exists(py):
            with open(py, "rb") as f:
                raw = f.read()
            _write_gz(os.path.join(dst, "python_case.json.gz"), raw)
        print(case)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the Posidonius checkout>")
    main(sys.argv[1])
