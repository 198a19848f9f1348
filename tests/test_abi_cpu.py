"""C ABI checks that need no GPU: exported symbols, the C++ case reader
against the oracle's reader, error codes, and loud failure without a device."""
import ctypes
import gzip
import json
import os
import re
import subprocess

import numpy as np
import pytest

import posidonius_gb300 as pg
from oracle.case_json import load_case
from posidonius_gb300 import _lib, layout as L

from golden_cases import case_dict, case_path, names

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "posidonius_gb300.h")


@pytest.fixture(scope="module")
def built():
    from posidonius_gb300 import build
    return build.build()


def header_functions():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(posi_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (posi_\w+)", out))
    declared = header_functions()
    assert len(declared) >= 25
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    assert set(_lib.SIGNATURES) == set(declared)


def test_library_loads_and_reports_version(built):
    assert b"sm_103a" in _lib.lib().posi_version()


def _unzip(tmp_path, name, twin=False):
    p = tmp_path / (name + (".py" if twin else "") + ".json")
    with gzip.open(case_path(name, twin)) as f:
        p.write_bytes(f.read())
    return p


@pytest.mark.parametrize("name", names(None))
def test_cpp_reader_matches_oracle_reader(built, tmp_path, name):
    ref = load_case(case_dict(name))
    got = pg.read_case(_unzip(tmp_path, name))
    assert got["n"] == ref["n"]
    for k in ("sys_i64", "sys_f64", "body_i64", "body_f64", "roche", "body_ias"):
        assert np.array_equal(np.asarray(got[k]).view(np.int64) if got[k].dtype == np.float64 else got[k],
                              np.asarray(ref[k]).view(np.int64) if ref[k].dtype == np.float64 else ref[k]), k
    assert np.array_equal(got["tables"][: ref["tables"].size], ref["tables"])


def test_reader_error_codes(built, tmp_path):
    lib = _lib.lib()
    n = ctypes.c_int64()
    assert lib.posi_read_case(str(tmp_path / "missing.json").encode(), ctypes.byref(n), None, None, None, None,
                              None, None, None) == L.ERR_IO
    bad = tmp_path / "bad.json"
    bad.write_text('{"alternative_coordinates_type": ')
    assert lib.posi_read_case(str(bad).encode(), ctypes.byref(n), None, None, None, None, None, None,
                              None) == L.ERR_PARSE
    d = case_dict("test_integrator-whfast_jacobi")
    d["universe"]["consider_effects"]["disk"] = True
    p = tmp_path / "disk.json"
    p.write_text(json.dumps(d))
    assert lib.posi_read_case(str(p).encode(), ctypes.byref(n), None, None, None, None, None, None,
                              None) == L.ERR_UNSUPPORTED
    d = case_dict("test_integrator-whfast_jacobi")
    del d["alternative_coordinates_type"]
    p.write_text(json.dumps(d))
    assert lib.posi_read_case(str(p).encode(), ctypes.byref(n), None, None, None, None, None, None,
                              None) == L.ERR_UNSUPPORTED
    d = case_dict("test_integrator-whfast_jacobi")
    d["universe"]["particles"][1]["tides"]["effect"] = "Disabled"
    p.write_text(json.dumps(d))
    assert lib.posi_read_case(str(p).encode(), ctypes.byref(n), None, None, None, None, None, None,
                              None) == L.ERR_UNSUPPORTED


@pytest.mark.skipif(_lib.os.environ.get("CUDA_VISIBLE_DEVICES", None) != "" and
                    __import__("torch").cuda.is_available(), reason="a GPU is visible")
def test_product_fails_loudly_without_a_device(built, tmp_path):
    assert _lib.lib().posi_device_count() == 0
    with pytest.raises(pg.PosiError) as e:
        pg.WHFast.from_json(_unzip(tmp_path, "test_integrator-whfast_jacobi"))
    assert e.value.status == L.ERR_CUDA


def test_cli_usage_without_gpu():
    """The `posidonius` command is built beside the library and rejects a
    malformed command line before touching a device."""
    import subprocess
    from posidonius_gb300 import build as B
    B.build()
    r = subprocess.run([B.CLI], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "posidonius start" in r.stderr
    r = subprocess.run([B.CLI, "start", "only_one_arg.json"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    r = subprocess.run([B.CLI, "resume", "a.json", "b.bin", "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2


def test_unbuilt_and_unknown_mappings_are_refused(built):
    """POSI_MAP_THREAD is declared but not built: the batch refuses it (no
    silent fallback to a lane group), before any device work; an unknown
    mapping is an argument error."""
    from posidonius_gb300 import ensemble as E
    ens = E.workload_ensemble8(2, seed=1)
    with pytest.raises(pg.PosiError) as e:
        pg.Batch(ens, mapping=L.MAP_THREAD)
    assert e.value.status == L.ERR_UNSUPPORTED
    assert b"POSI_MAP_THREAD" in _lib.lib().posi_last_error()
    with pytest.raises(pg.PosiError) as e:
        pg.Batch(ens, mapping=3)
    assert e.value.status == L.ERR_ARG
