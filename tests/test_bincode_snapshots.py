"""Bincode recovery snapshots (CPU): the reference writes and restores a
snapshot as bincode whenever its path does not end in ".json"
(src/integrator/output.rs:43-51, 186-191).  Every reference golden case
(WHFast in all three coordinate systems, IAS15, the Python-generated twins)
goes JSON -> bincode -> JSON -> bincode with identical bytes on both
bincode legs, and the C++ reader reads the same flat state from the
original JSON, the bincode file and the converted JSON.  A truncated or
corrupted bincode file is refused."""
import gzip
import os

import numpy as np
import pytest

from posidonius_gb300 import _lib, layout as L

from golden_cases import case_path, names

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def built():
    from posidonius_gb300 import build
    return build.build()


def _cases():
    out = []
    for name in names():
        out.append((name, case_path(name)))
        twin = os.path.join(HERE, "golden", name, "python_case.json.gz")
        if os.path.exists(twin):
            out.append((name + "/python", twin))
    return out


def _read_flat(path):
    n = np.zeros(1, np.int64)
    nt = np.zeros(1, np.int64)
    lib = _lib.lib()
    rc = lib.posi_read_case(str(path).encode(), _lib.ptr(n, "i"), _lib.ptr(nt, "i"), None, None, None, None, None,
                            None)
    assert rc == L.OK, lib.posi_last_error()
    k = int(n[0])
    si = np.zeros(L.SI_COUNT, np.int64)
    sf = np.zeros(L.SF_COUNT, np.float64)
    bi = np.zeros((k, L.BI_COUNT), np.int64)
    bf = np.zeros((k, L.BF_COUNT), np.float64)
    tb = np.zeros(max(1, int(nt[0])), np.float64)
    ro = np.zeros(k * k, np.float64)
    rc = lib.posi_read_case(str(path).encode(), None, None, _lib.ptr(si, "i"), _lib.ptr(sf, "f"), _lib.ptr(bi, "i"),
                            _lib.ptr(bf, "f"), _lib.ptr(tb, "f"), _lib.ptr(ro, "f"))
    assert rc == L.OK, lib.posi_last_error()
    return si, sf, bi, bf, tb, ro


def _same(a, b):
    for x, y in zip(a, b):
        x, y = np.asarray(x), np.asarray(y)
        if x.dtype == np.float64:
            assert np.array_equal(x.view(np.int64), y.view(np.int64)) or np.array_equal(x, y, equal_nan=True)
        else:
            assert np.array_equal(x, y)


@pytest.mark.parametrize("name,src", _cases())
def test_json_bincode_round_trip(built, tmp_path, name, src):
    lib = _lib.lib()
    js = tmp_path / "case.json"
    with gzip.open(src) as f:
        js.write_bytes(f.read())
    b1, j2, b2 = tmp_path / "case.bin", tmp_path / "again.json", tmp_path / "again.bin"
    for a, b in ((js, b1), (b1, j2), (j2, b2)):
        rc = lib.posi_convert_snapshot(str(a).encode(), str(b).encode())
        assert rc == L.OK, (a.name, b.name, lib.posi_last_error())
    assert b1.read_bytes() == b2.read_bytes()
    flat = _read_flat(js)
    _same(flat, _read_flat(b1))
    _same(flat, _read_flat(j2))


def test_bincode_layout_sizes(built, tmp_path):
    """Fixed parts of the layout: the WHFast snapshot of a case without
    evolution tables or pair-dependent factors has the size the struct tree
    gives (every field at its declared width)."""
    lib = _lib.lib()
    js = tmp_path / "case.json"
    with gzip.open(case_path("test_integrator-whfast_jacobi")) as f:
        js.write_bytes(f.read())
    b = tmp_path / "case.bin"
    assert lib.posi_convert_snapshot(str(js).encode(), str(b).encode()) == L.OK
    axes = 24
    ctl = 4 + 4 + 24                       # TidesEffect tag, TidalModel tag, 3 doubles (or 4 for Disabled)
    del ctl
    raw = b.read_bytes()
    # time_step, half_time_step, then Universe: initial_time, time_limit
    head = np.frombuffer(raw[:32], dtype="<f8")
    import json
    doc = json.loads(js.read_text())
    assert head[0] == doc["time_step"] and head[1] == doc["half_time_step"]
    assert head[2] == doc["universe"]["initial_time"] and head[3] == doc["universe"]["time_limit"]
    # the trailing fields: timestep_warning (u64) then 2 x 10 Axes of Kahan terms
    tail = raw[-(8 + 2 * 10 * axes):]
    assert int(np.frombuffer(tail[:8], dtype="<u8")[0]) == doc["timestep_warning"]
    errs = np.frombuffer(tail[8:], dtype="<f8").reshape(2, 10, 3)
    want = np.array([[[a["x"], a["y"], a["z"]] for a in doc[k]] for k in ("inertial_velocity_errors",
                                                                           "particle_angular_momentum_errors")])
    assert np.array_equal(errs, want)


def test_bad_bincode_is_refused(built, tmp_path):
    lib = _lib.lib()
    js = tmp_path / "case.json"
    with gzip.open(case_path("test_integrator-whfast_jacobi")) as f:
        js.write_bytes(f.read())
    b = tmp_path / "case.bin"
    assert lib.posi_convert_snapshot(str(js).encode(), str(b).encode()) == L.OK
    raw = b.read_bytes()
    cut = tmp_path / "cut.bin"
    cut.write_bytes(raw[:-5])
    assert lib.posi_convert_snapshot(str(cut).encode(), str(tmp_path / "x.json").encode()) == L.ERR_PARSE
    assert b"bincode" in lib.posi_last_error()
    longer = tmp_path / "long.bin"
    longer.write_bytes(raw + b"\0")
    assert lib.posi_convert_snapshot(str(longer).encode(), str(tmp_path / "y.json").encode()) == L.ERR_PARSE
