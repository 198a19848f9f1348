"""GPU: historic records, recovery snapshots and the start/resume command.

The drop-in flow of src/main.rs + src/integrator/output.rs on the CUDA path:
historic records (156 bytes per body, output.rs:91-135) must equal the
oracle's record for record (EXACT mode, NaN matching NaN); a recovery
snapshot must read back -- with Python's json and with the C++ reader -- to
the device state it was written from; and a run resumed from a snapshot must
continue bit for bit like the uninterrupted run, history file included.
"""
import gzip
import json
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle
import posidonius_gb300 as pg
from oracle.case_json import load_case
from posidonius_gb300 import _lib, build as B, layout as L

from golden_cases import case_dict
from parity import bitwise_diffs, same_bits

pytestmark = pytest.mark.gpu

REC = struct.Struct("<ddi17d")
assert REC.size == pg.HISTORY_BYTES_PER_PARTICLE


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()


def _case(tmp_path, name, hist_period=None, rec_period=None, time_limit=None, fname=None):
    d = case_dict(name)
    if hist_period is not None:
        d["historic_snapshot_period"] = hist_period
    if rec_period is not None:
        d["recovery_snapshot_period"] = rec_period
    if time_limit is not None:
        d["universe"]["time_limit"] = time_limit
    p = tmp_path / (fname or (name + ".json"))
    p.write_text(json.dumps(d))
    return p, d


def read_history(path, n):
    data = open(path, "rb").read()
    assert len(data) % (REC.size * n) == 0
    recs = np.array([REC.unpack_from(data, k * REC.size) for k in range(len(data) // REC.size)], dtype=np.float64)
    return recs.reshape(-1, n, 20)


@pytest.mark.parametrize("name", ["test_tides-enabled_tides", "test_evolution-m_dwarf_baraffe2015",
                                  "test_integrator-whfast_democraticheliocentric",
                                  "test_disk-enabled_disk", "test_evolution-solar_like_bolmontmathis2016"])
def test_history_records_match_oracle(tmp_path, name):
    path, d = _case(tmp_path, name, hist_period=0.24)
    w = pg.restore_snapshot(path, mode=pg.EXACT)
    hist = tmp_path / "history.bin"
    w.open_history(hist)
    assert w.run(60) == 60
    w.close_history()
    n = w.get_n_particles()
    got = read_history(hist, n)
    ens, steps, _, ref = oracle.run_with_history(load_case(d), 60, init_physical=True)
    assert steps[0] == 60
    assert got.shape == ref.shape and got.shape[0] == w.get_n_historic_snapshots()
    assert same_bits(got, ref).all()
    # the dE/dt refreshed at the last trigger is part of the state too
    assert bitwise_diffs(w.get_state(), ens) == []


def test_recovery_snapshot_reads_back(tmp_path):
    name = "test_tides-enabled_tides"
    path, _ = _case(tmp_path, name, hist_period=0.4)
    w = pg.restore_snapshot(path, mode=pg.EXACT)
    w.run(37)
    snap = tmp_path / "snapshot.json"
    w.write_recovery_snapshot(snap)
    st = w.get_state()
    assert st["sys_f64"][L.SF_LAST_REC] == st["sys_f64"][L.SF_TIME]
    # Python's json reads it (NaN written as null) ...
    doc = json.loads(snap.read_text())
    assert doc["current_time"] == st["sys_f64"][L.SF_TIME]
    assert doc["current_iteration"] == 37
    back = load_case(doc)
    # the midpoint iteration count is a diagnostic of this library, not a
    # field of the case format
    back["sys_i64"][L.SI_LAST_MIDPOINT_ITERS] = st["sys_i64"][L.SI_LAST_MIDPOINT_ITERS]
    assert bitwise_diffs(st, back) == []
    assert same_bits(back["roche"], st["roche"]).all()
    # ... and so does the C++ reader of the library
    again = pg.read_case(snap)
    again["sys_i64"][L.SI_LAST_MIDPOINT_ITERS] = st["sys_i64"][L.SI_LAST_MIDPOINT_ITERS]
    assert bitwise_diffs(st, again) == []
    # a second snapshot keeps the first as a dated backup
    w.run(3)
    w.write_recovery_snapshot(snap)
    backups = [f for f in os.listdir(tmp_path) if f.startswith("snapshot.") and f.endswith(".bin")]
    assert len(backups) == 1
    assert json.loads(open(tmp_path / backups[0]).read())["current_iteration"] == 37


@pytest.mark.parametrize("mode", [pg.EXACT, pg.FAST])
def test_resume_continues_bit_for_bit(tmp_path, mode):
    name = "test_evolution-m_dwarf_baraffe2015"
    path, _ = _case(tmp_path, name, hist_period=0.8)
    straight = pg.restore_snapshot(path, mode=mode)
    straight.run(150)
    w = pg.restore_snapshot(path, mode=mode)
    w.run(70)
    snap = tmp_path / "snapshot.json"
    w.write_recovery_snapshot(snap)
    w.close()
    resumed = pg.restore_snapshot(snap, mode=mode)
    assert resumed.get_current_time() > 0.0
    resumed.run(80)
    a, b = resumed.get_state(), straight.get_state()
    # the snapshot time is the only field the two runs set differently
    b["sys_f64"][L.SF_LAST_REC] = a["sys_f64"][L.SF_LAST_REC]
    assert bitwise_diffs(a, b) == []


def test_history_open_refuses_short_file_and_truncates(tmp_path):
    path, _ = _case(tmp_path, "test_integrator-whfast_jacobi")
    w = pg.restore_snapshot(path)
    hist = tmp_path / "h.bin"
    hist.write_bytes(b"\0" * 100)
    with pytest.raises(pg.PosiError) as e:
        w.open_history(hist, expected_bytes=200)
    assert e.value.status == L.ERR_STATE
    w.open_history(hist, expected_bytes=40)
    assert os.path.getsize(hist) == 40


def _cli(*args):
    return subprocess.run([B.CLI] + [str(a) for a in args], capture_output=True, text=True, timeout=300)


def test_cli_start_resume_matches_uninterrupted_run(tmp_path):
    name = "test_tides-enabled_tides"
    # uninterrupted: 16 days
    full, _ = _case(tmp_path, name, hist_period=0.8, rec_period=4.0, time_limit=16.0, fname="full.json")
    r = _cli("start", full, tmp_path / "full_rec.json", tmp_path / "full_hist.bin", "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Simulation completed" in r.stdout
    # interrupted: 8 days, then resumed from the last recovery snapshot to 16 days
    part, _ = _case(tmp_path, name, hist_period=0.8, rec_period=4.0, time_limit=8.0, fname="part.json")
    r = _cli("start", part, tmp_path / "rec.json", tmp_path / "hist.bin", "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    # start refuses to overwrite
    r2 = _cli("start", part, tmp_path / "rec.json", tmp_path / "other.bin", "-s")
    assert r2.returncode == 101 and "already exists" in r2.stdout
    snap = json.loads((tmp_path / "rec.json").read_text())
    assert 0 < snap["current_time"] < 8.0
    r = _cli("resume", tmp_path / "rec.json", tmp_path / "hist.bin", "--time-limit", 16, "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Restored previous simulation" in r.stdout
    assert (tmp_path / "hist.bin").read_bytes() == (tmp_path / "full_hist.bin").read_bytes()
    # both runs wrote their last recovery snapshot at the same step
    a = json.loads((tmp_path / "rec.json").read_text())
    b = json.loads((tmp_path / "full_rec.json").read_text())
    assert a["current_iteration"] == b["current_iteration"]
    assert a["universe"]["particles"] == b["universe"]["particles"]


def test_generated_case_document_drives_the_cli_and_the_oracle(tmp_path):
    """A seeded system written by the case writer: `posidonius start` runs
    it to its time limit, and the library and the oracle integrate the
    document to the same bits."""
    from posidonius_gb300 import case_writer as W, ensemble as E
    ens = E.workload_single(seed=4, time_limit=4.0)
    path = tmp_path / "generated.json"
    W.write_case(path, ens)
    r = _cli("start", path, tmp_path / "rec.json", tmp_path / "hist.bin", "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Simulation completed" in r.stdout
    w = pg.restore_snapshot(path, mode=pg.EXACT)
    steps = w.run()
    assert steps == 49   # t + dt > 4.0 after 49 steps of 0.08 d
    ref, rsteps, _ = oracle.run(load_case(str(path)), max_steps=10**6, init_physical=True)
    assert rsteps[0] == steps
    assert bitwise_diffs(w.get_state(), ref) == []


def test_cli_bincode_start_resume_as_documented(tmp_path):
    """The reference's documented command lines (`posidonius start case.json
    case.bin case_history.bin`, then `posidonius resume case.bin
    case_history.bin`): bincode recovery snapshots, a resumed run that ends
    with the same history bytes and the same final snapshot bytes as an
    uninterrupted one, and a dated backup of the previous snapshot."""
    name = "test_tides-enabled_tides"
    full, _ = _case(tmp_path, name, hist_period=0.8, rec_period=4.0, time_limit=16.0, fname="full.json")
    r = _cli("start", full, tmp_path / "full.bin", tmp_path / "full_history.bin", "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    part, _ = _case(tmp_path, name, hist_period=0.8, rec_period=4.0, time_limit=8.0, fname="case.json")
    r = _cli("start", part, tmp_path / "case.bin", tmp_path / "case_history.bin", "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    backups = [f for f in os.listdir(tmp_path) if f.startswith("case.") and f.endswith(".bin") and "T" in f]
    assert len(backups) == 1, backups
    # the bincode snapshot reads back as the JSON document of the same state
    lib = _lib.lib()
    assert lib.posi_convert_snapshot(str(tmp_path / "case.bin").encode(), str(tmp_path / "case_rec.json").encode()) == L.OK
    snap = json.loads((tmp_path / "case_rec.json").read_text())
    assert 0 < snap["current_time"] < 8.0
    r = _cli("resume", tmp_path / "case.bin", tmp_path / "case_history.bin", "--time-limit", 16, "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Restored previous simulation" in r.stdout
    assert (tmp_path / "case_history.bin").read_bytes() == (tmp_path / "full_history.bin").read_bytes()
    # both runs wrote their last recovery snapshot at the same step, with the same state
    for src, dst in (("case.bin", "a.json"), ("full.bin", "b.json")):
        assert lib.posi_convert_snapshot(str(tmp_path / src).encode(), str(tmp_path / dst).encode()) == L.OK
    a = json.loads((tmp_path / "a.json").read_text())
    b = json.loads((tmp_path / "b.json").read_text())
    assert a["current_iteration"] == b["current_iteration"]
    assert a["universe"]["particles"] == b["universe"]["particles"]


@pytest.mark.parametrize("mode", [pg.EXACT, pg.FAST])
def test_bincode_resume_continues_bit_for_bit(tmp_path, mode):
    """Through the library: a bincode recovery snapshot, restored, continues
    bit for bit -- WHFast and IAS15 documents alike (the uninterrupted run
    writes a snapshot at the same step too, so that both carry the same
    last_recovery_snapshot_time, which IAS15's triggers read)."""
    for name, first in (("test_evolution-m_dwarf_baraffe2015", 5), ("test_integrator-ias15", 2)):
        path, _ = _case(tmp_path, name, hist_period=0.8, fname=name + ".json")
        straight = pg.restore_snapshot(path, mode=mode)
        assert straight.run(first) == first
        straight.write_recovery_snapshot(tmp_path / (name + "_unused.bin"))
        straight.run(7)
        w = pg.restore_snapshot(path, mode=mode)
        assert w.run(first) == first
        snap = tmp_path / (name + ".bin")
        w.write_recovery_snapshot(snap)
        w.close()
        resumed = pg.restore_snapshot(snap, mode=mode)
        assert resumed.get_current_time() > 0.0
        resumed.run(7)
        assert bitwise_diffs(resumed.get_state(), straight.get_state()) == [], name
