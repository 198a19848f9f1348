"""GPU: the IAS15 integrator (src/integrator/ias15.rs) against the oracle and
the reference's golden case.

EXACT mode must reproduce the oracle bit for bit -- positions, velocities,
accelerations, spins, the adaptive step, the accepted-step length, the count
of non-converged predictor-corrector loops and every Gauss-Radau coefficient
-- and with it the reference's test_integrator-ias15 golden (4 adaptive steps
to t = 6.8 d).  FAST mode (FMA contraction) stays within 1e-10 relative of the
oracle over the same runs.
"""
import gzip

import numpy as np
import pytest

import oracle
import posidonius_gb300 as pg
from oracle.case_json import load_case, stack
from posidonius_gb300 import ensemble as E, layout as L

from golden_cases import case_dict, case_path, expected, max_abs_error, names
from parity import bitwise_diffs, max_rel_error

pytestmark = pytest.mark.gpu

FAST_TOL = 1e-10
GOLDEN = names("ias15")


@pytest.fixture(scope="module", autouse=True)
def built():
    from posidonius_gb300 import build
    build.build()


def _json(tmp_path, name):
    p = tmp_path / (name + ".json")
    with gzip.open(case_path(name)) as f:
        p.write_bytes(f.read())
    return p


@pytest.mark.parametrize("name", GOLDEN)
def test_plain_path_exact_matches_golden_and_oracle(tmp_path, name):
    w = pg.restore_snapshot(_json(tmp_path, name), mode=pg.EXACT)
    steps = w.run()
    assert steps == 4
    st = w.get_state()
    assert st["sys_i64"][L.SI_STATUS] & L.SYS_FATAL_MASK == L.SYS_COMPLETED
    assert max_abs_error(st["body_f64"], expected(name)) == 0.0
    ref, _, _ = oracle.run(load_case(case_dict(name)), max_steps=10**6, init_physical=True)
    assert bitwise_diffs(st, ref) == []


@pytest.mark.parametrize("name", GOLDEN)
def test_plain_path_fast_within_tolerance(tmp_path, name):
    w = pg.restore_snapshot(_json(tmp_path, name), mode=pg.FAST)
    assert w.run() == 4
    st = w.get_state()
    ref, _, _ = oracle.run(load_case(case_dict(name)), max_steps=10**6, init_physical=True)
    assert max_rel_error(st, ref) <= FAST_TOL


def _golden_ensemble(k, seed=3):
    """k copies of the golden system with perturbed planets and first trial
    steps from 0.02 d to 100 d (the longest do not converge, are rejected and
    redone)."""
    rng = np.random.default_rng(seed)
    base = load_case(case_dict(GOLDEN[0]))
    trial = (0.02, 0.3, 4.0, 30.0, 100.0, 60.0)
    cases = []
    for i in range(k):
        c = {kk: (v.copy() if isinstance(v, np.ndarray) else v) for kk, v in base.items()}
        n = c["n"]
        c["body_f64"][1:n, L.POS] *= 1.0 + 1e-3 * rng.standard_normal((n - 1, 3))
        c["sys_f64"][L.SF_DT] = trial[i % len(trial)]
        c["sys_f64"][L.SF_TIME_LIMIT] = 4000.0
        cases.append(c)
    return stack(cases)


@pytest.mark.parametrize("spl", [25, 7])
def test_batched_exact_matches_oracle(spl):
    ens = _golden_ensemble(12)
    b = pg.Batch(ens, mode=pg.EXACT)
    b.initialize_physical_values()
    b.iterate(25, spl)
    st = b.get_state()
    ref, steps, _ = oracle.run(ens, max_steps=25, init_physical=True, nthreads=8)
    assert np.all(st["sys_i64"][:, L.SI_ITERATION] == steps)
    assert bitwise_diffs(st, ref) == []
    # some first tries were rejected and some predictor-corrector loops hit the limit
    assert st["sys_i64"][:, L.SI_IAS_MAX_EXCEEDED].max() >= 1


def _energy(state, s):
    """Barycentric Newtonian energy of system s."""
    G = oracle.constant(0)
    n = int(state["sys_i64"][s, L.SI_N])
    bf = state["body_f64"][s, :n]
    m, r, v = bf[:, L.BF_MASS], bf[:, L.POS], bf[:, L.VEL]
    e = 0.5 * np.sum(m * np.sum(v * v, axis=1))
    for i in range(n):
        for j in range(i + 1, n):
            e -= G * m[i] * m[j] / np.linalg.norm(r[i] - r[j])
    return e


def test_batched_synthetic_ensemble_exact_and_fast():
    """The seeded star + 7 planets systems (no evolution), IAS15 from a 0.5 d
    trial step (rejected: the predictor-corrector loop does not converge).
    EXACT: the oracle's bits.  FAST: the step sizes follow the error estimate
    of the highest-order coefficient, a rounding-level quantity, so they
    differ from the oracle's in their last digits and the two runs sample
    the orbits at slightly different times; what must agree is the physics:
    the step sizes to 1e-3 and the energy to 1e-10 relative."""
    ens = E.as_ias15(E.workload_ensemble8(64, seed=8), dt=0.5)
    ref, steps, _ = oracle.run(ens, max_steps=12, init_physical=True, nthreads=8)
    for mode in (pg.EXACT, pg.FAST):
        b = pg.Batch(ens, mode=mode)
        b.initialize_physical_values()
        b.iterate(12, 12)
        st = b.get_state()
        assert np.all(st["sys_i64"][:, L.SI_ITERATION] == 12)
        assert np.all(st["sys_i64"][:, L.SI_IAS_MAX_EXCEEDED] >= 1)
        if mode == pg.EXACT:
            assert bitwise_diffs(st, ref) == []
        else:
            assert np.abs(st["sys_f64"][:, L.SF_DT] / ref["sys_f64"][:, L.SF_DT] - 1).max() <= 1e-3
            for s in range(b.n_sys):
                e0 = _energy(ref, s)
                assert abs(_energy(st, s) - e0) <= 1e-10 * abs(e0), s


def test_recovery_snapshot_resume_is_seamless(tmp_path):
    """Stop after 2 steps, write the JSON recovery snapshot (with the
    Gauss-Radau state), restore it and finish: the same bits as one run."""
    name = GOLDEN[0]
    one = pg.restore_snapshot(_json(tmp_path, name), mode=pg.EXACT)
    assert one.run(max_steps=2) == 2
    one.write_recovery_snapshot(tmp_path / "unused.json")   # the same last_recovery_snapshot_time
    one.run()
    a = one.get_state()
    w = pg.restore_snapshot(_json(tmp_path, name), mode=pg.EXACT)
    assert w.run(max_steps=2) == 2
    snap = tmp_path / "recovery.json"
    w.write_recovery_snapshot(snap)
    r = pg.restore_snapshot(snap, mode=pg.EXACT)
    assert r.get_current_time() == w.get_current_time()
    r.run()
    b = r.get_state()
    assert bitwise_diffs(b, a) == []
    # the C++ reader and the oracle's reader agree on the written document
    got = pg.read_case(snap)
    ref = load_case(str(snap))
    for k in ("sys_i64", "sys_f64", "body_f64", "body_ias"):
        assert np.array_equal(np.asarray(got[k]).view(np.int64), np.asarray(ref[k]).view(np.int64)), k
    assert np.abs(got["body_ias"]).max() > 0


def test_history_records_match_oracle(tmp_path):
    """Historic records every 1 d of the golden run: triggers at t = 0 and,
    IAS15 moving the record time to the current time (ias15.rs:434), at
    t = 1.68 d (0 + 1 <= 1.68 after the 0.08, 0.32 and 1.28 d steps); the run
    completes at t = 6.8 d before another trigger.  Each record carries the
    adaptive step."""
    import json
    import struct
    name = GOLDEN[0]
    d = case_dict(name)
    d["historic_snapshot_period"] = 1.0
    path = tmp_path / "case.json"
    path.write_text(json.dumps(d))
    w = pg.restore_snapshot(path, mode=pg.EXACT)
    hist = tmp_path / "history.bin"
    w.open_history(hist)
    assert w.run() == 4
    w.close_history()
    n = w.get_n_particles()
    rec = struct.Struct("<ddi17d")
    data = open(hist, "rb").read()
    got = np.array([rec.unpack_from(data, k * rec.size) for k in range(len(data) // rec.size)]).reshape(-1, n, 20)
    ens, steps, _, ref = oracle.run_with_history(load_case(d), 10**6, init_physical=True)
    assert steps[0] == 4
    assert got.shape == ref.shape and got.shape[0] == w.get_n_historic_snapshots() == 2
    assert np.array_equal(got[:, 0, 0], [0.0, 0.08 + 0.32 + 1.28])
    assert np.array_equal(got[:, 0, 1], [0.08, 5.12])   # the step about to be taken
    from parity import same_bits
    assert same_bits(got, ref).all()
    assert bitwise_diffs(w.get_state(), ens) == []


def test_batched_uneven_exact_matches_oracle():
    """Systems of 2 to 10 bodies (circumbinary binaries included) by IAS15:
    lane groups of 2 to 16, every system adapting its own step."""
    ens = E.as_ias15(E.workload_uneven(96, seed=5), dt=0.1)
    ref, steps, _ = oracle.run(ens, max_steps=15, init_physical=True, nthreads=8)
    b = pg.Batch(ens, mode=pg.EXACT)
    assert b.mapping_for(10) == 16 and b.mapping_for(3) == 4 and b.mapping_for(2) == 2
    b.initialize_physical_values()
    b.iterate(15, 6)
    st = b.get_state()
    assert np.array_equal(st["sys_i64"][:, L.SI_ITERATION], steps)
    assert bitwise_diffs(st, ref) == []


def test_cli_start_resume_matches_uninterrupted_run(tmp_path):
    """`posidonius start` / `resume` on an IAS15 case: the resumed run
    continues bit for bit, history file included."""
    import json
    import subprocess
    from posidonius_gb300 import build as B

    def cli(*args):
        return subprocess.run([B.CLI] + [str(a) for a in args], capture_output=True, text=True, timeout=300)

    def case(limit, fname):
        d = case_dict(GOLDEN[0])
        d["historic_snapshot_period"] = 10.0
        d["recovery_snapshot_period"] = 20.0
        d["universe"]["time_limit"] = limit
        p = tmp_path / fname
        p.write_text(json.dumps(d))
        return p

    full = case(200.0, "full.json")
    r = cli("start", full, tmp_path / "full_rec.json", tmp_path / "full_hist.bin", "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Simulation completed" in r.stdout
    part = case(100.0, "part.json")
    r = cli("start", part, tmp_path / "rec.json", tmp_path / "hist.bin", "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    snap = json.loads((tmp_path / "rec.json").read_text())
    assert 0 < snap["current_time"] < 100.0 and snap["time_step_last_success"] > 0
    r = cli("resume", tmp_path / "rec.json", tmp_path / "hist.bin", "--time-limit", 200, "-s")
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "hist.bin").read_bytes() == (tmp_path / "full_hist.bin").read_bytes()
    a = json.loads((tmp_path / "rec.json").read_text())
    b = json.loads((tmp_path / "full_rec.json").read_text())
    assert a["current_iteration"] == b["current_iteration"]
    assert a["universe"]["particles"] == b["universe"]["particles"]
    assert a["b_6"] == b["b_6"] and a["time_step"] == b["time_step"]


def test_close_encounter_in_a_substep_freezes_like_the_oracle():
    """A planet thrown at another (0.03 AU apart, closing at 0.5 AU/d) passes
    the Roche limit at a substep of the first step: the system freezes there
    (the reference panics) with the substep's predicted state and the step's
    start time, next to a system that integrates on."""
    base = load_case(case_dict(GOLDEN[0]))
    bad = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in base.items()}
    bad["body_f64"][2, L.POS] = bad["body_f64"][1, L.POS] + np.array([0.03, 0.0, 0.0])
    bad["body_f64"][2, L.VEL] = bad["body_f64"][1, L.VEL] + np.array([-0.5, 0.0, 0.0])
    ens = stack([bad, base])
    ref, steps, _ = oracle.run(ens, max_steps=3, init_physical=True, nthreads=2)
    assert ref["sys_i64"][0, L.SI_STATUS] & L.SYS_FATAL_MASK == L.SYS_ROCHE
    assert ref["sys_f64"][0, L.SF_TIME] == 0.0
    assert np.abs(ref["body_f64"][0, :5, L.POS] - bad["body_f64"][:5, L.POS]).max() > 0   # mid-step state
    b = pg.Batch(ens, mode=pg.EXACT)
    b.initialize_physical_values()
    b.iterate(3, 3)
    assert bitwise_diffs(b.get_state(), ref) == []


@pytest.mark.parametrize("name", ["test_general_relativity-anderson1975", "test_general_relativity-newhall1983",
                                  "test_disk-enabled_disk", "test_evolution-solar_like_bolmontmathis2016",
                                  "test_evolution-solar_like_baraffe2015", "test_star_types-m_dwarf"])
def test_every_effect_under_ias15_exact(name):
    """The reference's WHFast goldens integrated by IAS15 instead: the
    N-body GR forms (their Newtonian accelerations without ignored terms),
    the disk, the wind, the dynamical tide and the evolving stars, 20
    adaptive steps, bit for bit against the oracle."""
    case = load_case(case_dict(name))
    case["sys_f64"][L.SF_TIME_LIMIT] = 400.0
    ens = E.as_ias15(stack([case]))
    ref, steps, _ = oracle.run(ens, max_steps=20, init_physical=True)
    assert steps[0] == 20
    b = pg.Batch(ens, mode=pg.EXACT)
    b.initialize_physical_values()
    b.iterate(20, 10)
    assert bitwise_diffs(b.get_state(), ref) == []


def test_mixed_batches_and_other_engines_refuse_ias15():
    """A batch holds systems of one integrator; the adjoint and the
    many-body engine take WHFast systems only."""
    from posidonius_gb300 import adjoint as A
    whf = E.workload_single(seed=1)
    ias = E.as_ias15(whf)
    both = stack([{k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in e.items()}
                  | {"n": int(e["sys_i64"][0, L.SI_N])} for e in (whf, ias)])
    both["body_ias"] = np.concatenate([np.zeros_like(ias["body_ias"]), ias["body_ias"]])
    with pytest.raises(pg.PosiError) as e:
        pg.Batch(both, mode=pg.EXACT)
    assert e.value.status == L.ERR_UNSUPPORTED
    b = pg.Batch(ias, mode=pg.FAST)
    b.initialize_physical_values()
    with pytest.raises(pg.PosiError) as e:
        A.Adjoint(b, 10, 5)
    assert e.value.status == L.ERR_UNSUPPORTED
    b.close()
    one = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ias.items()}
    with pytest.raises(pg.PosiError) as e:
        pg.ManyBody(one)
    assert e.value.status == L.ERR_UNSUPPORTED
