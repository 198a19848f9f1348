"""GPU parity: the CUDA path against the oracle and the reference goldens.

EXACT mode (reference operation order, no FMA) must agree bit for bit with
the oracle, which itself reproduces the reference's golden files exactly.
FAST mode (FMA contraction, shared reciprocals) must stay within 1e-12
relative per step of the oracle's trajectory; after the 199 steps of a golden
case the tolerance written here is 1e-10 relative.
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

FAST_TOL_199 = 1e-10
FAST_TOL_STEP = 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    from posidonius_gb300 import build
    build.build()


def _json(tmp_path, name):
    p = tmp_path / (name + ".json")
    with gzip.open(case_path(name)) as f:
        p.write_bytes(f.read())
    return p


@pytest.mark.parametrize("name", names())
def test_plain_path_exact_matches_golden_and_oracle(tmp_path, name):
    w = pg.restore_snapshot(_json(tmp_path, name), mode=pg.EXACT)
    steps = w.run()
    assert steps == 199
    st = w.get_state()
    assert max_abs_error(st["body_f64"], expected(name)) == 0.0
    ref, _, _ = oracle.run(load_case(case_dict(name)), max_steps=10**6, init_physical=True)
    assert bitwise_diffs(st, ref) == []


@pytest.mark.parametrize("name", ["test_integrator-whfast_jacobi", "test_integrator-whfast_democraticheliocentric",
                                  "test_integrator-whfast_whds", "test_evolution-brown_dwarf_non_evolving",
                                  "test_general_relativity-anderson1975", "test_general_relativity-newhall1983",
                                  "test_evolution-solar_like_non_evolving",
                                  "test_evolution-solar_like_bolmontmathis2016", "test_disk-enabled_disk"])
def test_plain_path_fast_within_tolerance(tmp_path, name):
    w = pg.restore_snapshot(_json(tmp_path, name), mode=pg.FAST)
    w.run()
    st = w.get_state()
    assert max_abs_error(st["body_f64"], expected(name)) <= 1e-12
    ref, _, _ = oracle.run(load_case(case_dict(name)), max_steps=10**6, init_physical=True)
    assert max_rel_error(st, ref) <= FAST_TOL_199


def test_fast_long_run_within_tolerance():
    """FAST build after 1e4 steps in 10 launches: <= 1e-9 relative in positions,
    velocities and angular momenta against the oracle, no frozen system."""
    ens = E.workload_ensemble8(32, seed=21)
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    b.iterate(10000, 1000)
    st = b.get_state()
    assert np.all(st["sys_i64"][:, L.SI_STATUS] & L.SYS_FATAL_MASK == 0)
    assert np.all(st["sys_i64"][:, L.SI_LAST_MIDPOINT_ITERS] < 10)
    ref, _, _ = oracle.run(ens, max_steps=10000, init_physical=True, nthreads=8)
    assert max_rel_error(st, ref) <= 1e-9


def test_fast_one_step_relative_error():
    ens = E.workload_ensemble8(64, seed=11)
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    b.iterate(1)
    ref, _, _ = oracle.run(ens, max_steps=1, init_physical=True, nthreads=4)
    assert max_rel_error(b.get_state(), ref) <= FAST_TOL_STEP


@pytest.mark.parametrize("name", ["test_integrator-whfast_jacobi", "test_integrator-whfast_whds",
                                  "test_general_relativity-anderson1975", "test_general_relativity-newhall1983"])
def test_universe_methods_exact(tmp_path, name):
    case = load_case(case_dict(name))
    w = pg.WHFast.from_json(_json(tmp_path, name), mode=pg.EXACT)
    w.initialize_physical_values()
    ref, _, _ = oracle.run(case, op=oracle.INITIALIZE)
    assert bitwise_diffs(w.get_state(), ref) == []
    for ignore in (0, 1, 2):
        w.gravity_calculate_acceleration(ignore)
        ref, _, _ = oracle.run(ref, op=oracle.GRAVITY, arg=ignore)
        assert bitwise_diffs(w.get_state(), ref) == []
    w.calculate_additional_effects(0.0, True, True, True)
    ref, _, _ = oracle.run(ref, op=oracle.ADDITIONAL_EFFECTS, arg=1 | 2 | 4, t_arg=0.0)
    assert bitwise_diffs(w.get_state(), ref) == []


def test_batched_goldens_exact():
    cases = [load_case(case_dict(n)) for n in names()]
    ens = stack(cases)
    b = pg.Batch(ens, mode=pg.EXACT)
    b.initialize_physical_values()
    b.iterate(199, 50)
    st = b.get_state()
    for s, name in enumerate(names()):
        assert max_abs_error(st["body_f64"][s], expected(name)) == 0.0, name
    ref, _, _ = oracle.run(ens, max_steps=10**6, init_physical=True, nthreads=8)
    assert bitwise_diffs(st, ref) == []


def test_batched_uneven_exact_and_mappings():
    ens = E.workload_uneven(96, seed=5)
    ref, _, _ = oracle.run(ens, max_steps=40, init_physical=True, nthreads=8)
    for mapping in (L.MAP_AUTO, L.MAP_LANES16, L.MAP_WARP):
        b = pg.Batch(ens, mode=pg.EXACT, mapping=mapping)
        b.initialize_physical_values()
        b.iterate(40, 7)
        assert bitwise_diffs(b.get_state(), ref) == [], mapping


@pytest.mark.parametrize("mode", [pg.EXACT, pg.FAST])
def test_autotune_keeps_state_and_results(mode):
    """The autotuner's trial runs leave the state untouched, its choices are
    admissible, and a tuned batch computes the same bits as an untuned one."""
    ens = E.workload_uneven(256, seed=11)
    tuned = pg.Batch(ens, mode=mode)
    tuned.initialize_physical_values()
    before = tuned.get_state()
    choice = tuned.autotune(probe_steps=5)
    assert bitwise_diffs(tuned.get_state(), before) == []
    ns = set(int(n) for n in ens["sys_i64"][:, L.SI_N])
    assert set(choice) == ns
    # the choice rule: the fastest probe, or the least SMSP time (probe time x
    # min(warps, SMSPs) / SMSPs) when several buckets fill the GPU together
    import torch
    smsps = 4 * torch.cuda.get_device_properties(0).multi_processor_count
    count = {n: int(np.sum(ens["sys_i64"][:, L.SI_N] == n)) for n in ns}
    smallest = {n: min(g for g in (2, 4, 8, 16, 32) if g >= n) for n in ns}
    shared = len(ns) > 1 and sum(-(-count[n] // (32 // smallest[n])) for n in ns) >= smsps
    for n, g in choice.items():
        assert g in (2, 4, 8, 16, 32) and g >= n and tuned.mapping_for(n) == g
        probes = tuned.autotune_report(n)
        assert g in probes and 1 not in probes

        def cost(k):
            return probes[k] * min(-(-count[n] // (32 // k)), smsps) / smsps if shared else probes[k]
        assert cost(g) == min(cost(k) for k in probes)
    plain = pg.Batch(ens, mode=mode)
    plain.initialize_physical_values()
    tuned.iterate(30, 10)
    plain.iterate(30, 10)
    assert bitwise_diffs(tuned.get_state(), plain.get_state()) == []
    if mode == pg.EXACT:
        ref, _, _ = oracle.run(ens, max_steps=30, init_physical=True, nthreads=8)
        assert bitwise_diffs(tuned.get_state(), ref) == []


def test_batched_chunking_and_plain_agree():
    ens = E.workload_ensemble8(8, seed=3)
    outs = []
    for spl in (1, 5, 20):
        b = pg.Batch(ens, mode=pg.FAST)
        b.initialize_physical_values()
        b.iterate(20, spl)
        outs.append(b.get_state())
    assert bitwise_diffs(outs[0], outs[1]) == [] and bitwise_diffs(outs[0], outs[2]) == []
    one = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    one["n"] = int(ens["sys_i64"][0, L.SI_N])
    w = pg.WHFast.from_arrays(one, mode=pg.FAST)
    w.initialize_physical_values()
    # the first step reports a recovery trigger (first snapshot), so iterate()
    # returns after it, like Ok(true) in the reference's loop
    st, done, rec = w.iterate(20)
    assert (st, done, rec) == (L.OK, 1, True)
    assert w.run(19) == 19
    plain = w.get_state()
    assert bitwise_diffs(plain, {k: (v[:1] if isinstance(v, np.ndarray) and k != "tables" else v)
                                 for k, v in outs[0].items()}) == []


def test_collision_freezes_only_that_system():
    ens = E.workload_ensemble8(4, seed=9)
    # put planet 3 of system 1 on top of planet 2, moving with it
    ens["body_f64"][1, 3, L.POS] = ens["body_f64"][1, 2, L.POS] + 1e-9
    ens["body_f64"][1, 3, L.VEL] = ens["body_f64"][1, 2, L.VEL]
    ref, _, _ = oracle.run(ens, max_steps=5, init_physical=True)
    b = pg.Batch(ens, mode=pg.EXACT)
    b.initialize_physical_values()
    b.iterate(5)
    st = b.get_state()
    assert st["sys_i64"][1, L.SI_STATUS] & L.SYS_FATAL_MASK in (L.SYS_ROCHE, L.SYS_COLLISION)
    assert st["sys_i64"][1, L.SI_STATUS] == ref["sys_i64"][1, L.SI_STATUS]
    assert st["sys_i64"][1, L.SI_FAIL_PAIR] == ref["sys_i64"][1, L.SI_FAIL_PAIR] == 2 * 1024 + 3
    assert all(st["sys_i64"][s, L.SI_ITERATION] == 5 for s in (0, 2, 3))
    assert bitwise_diffs({k: (v[[0, 2, 3]] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in st.items()},
                         {k: (v[[0, 2, 3]] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ref.items()}) == []


def test_batched_maximum_body_count_exact():
    """The largest systems of the batched kernels (POSI_MAX_BODIES = 32
    bodies, one warp per system) in all three coordinate systems and by
    IAS15, with 17- and 20-body systems in the same lane groups: bit for
    bit against the oracle."""
    cases = []
    for coords, n_small in ((L.JACOBI, 29), (L.DEMOCRATIC_HELIOCENTRIC, 29), (L.WHDS, 29), (L.JACOBI, 14),
                            (L.WHDS, 17)):
        cases.append(E.workload_large(n_small, seed=7 + n_small, coords=coords))
    ens = stack(cases, nmax=L.MAX_BODIES)
    ref, steps, _ = oracle.run(ens, max_steps=30, init_physical=True, nthreads=5)
    b = pg.Batch(ens, mode=pg.EXACT)
    assert b.mapping_for(32) == 32 and b.mapping_for(17) == 32
    b.initialize_physical_values()
    b.iterate(30, 10)
    assert np.all(b.get_state()["sys_i64"][:, L.SI_ITERATION] == 30)
    assert bitwise_diffs(b.get_state(), ref) == []
    ias = E.as_ias15(stack(cases[:2], nmax=L.MAX_BODIES), dt=0.1)
    ref, _, _ = oracle.run(ias, max_steps=5, init_physical=True, nthreads=2)
    bi = pg.Batch(ias, mode=pg.EXACT)
    bi.initialize_physical_values()
    bi.iterate(5, 5)
    assert bitwise_diffs(bi.get_state(), ref) == []


@pytest.mark.parametrize("mode", [pg.EXACT, pg.FAST])
def test_smallest_and_widest_lane_groups_agree(mode):
    """Every system on its smallest lane group (2 lanes for 2 bodies, 4 for
    3-4, 8 for 5-8, 16 for 9-10 -- the groups the autotuner picks when the
    body counts share the GPU) against every system on a whole warp: the
    same bits after 50 steps, and FAST within 1e-12 of the oracle after one
    step on the smallest groups."""
    ens = E.workload_uneven(512, seed=37)
    out = []
    for mapping in (L.MAP_LANES2, L.MAP_WARP):
        b = pg.Batch(ens, mode=mode, mapping=mapping)
        b.initialize_physical_values()
        if mapping == L.MAP_LANES2:
            assert b.mapping_for(2) == 2 and b.mapping_for(3) == 4 and b.mapping_for(9) == 16
        b.iterate(50, 25)
        out.append(b.get_state())
        b.close()
    assert bitwise_diffs(out[0], out[1]) == []
    if mode == pg.FAST:
        ref, _, _ = oracle.run(ens, max_steps=1, init_physical=True, nthreads=8)
        b = pg.Batch(ens, mode=mode, mapping=L.MAP_LANES2)
        b.initialize_physical_values()
        b.iterate(1)
        assert max_rel_error(b.get_state(), ref) <= 1e-12
        b.close()


def test_collision_first_pair_fast():
    """FAST (the pair loop over unordered pairs in rounds, the lanes keeping
    their least pair): with two overlapping pairs in one system the event
    reported is the first in (i, j) order, as in the reference, and the
    stopped system's state -- its velocities transformed at the stop --
    matches the oracle's."""
    ens = E.workload_ensemble8(4, seed=9)
    # planet 6 on top of planet 5 and planet 3 on top of planet 2: the pair
    # (2, 3) comes first in (i, j) order; the rounds meet (5, 6) as early
    ens["body_f64"][1, 6, L.POS] = ens["body_f64"][1, 5, L.POS] + 1e-9
    ens["body_f64"][1, 6, L.VEL] = ens["body_f64"][1, 5, L.VEL]
    ens["body_f64"][1, 3, L.POS] = ens["body_f64"][1, 2, L.POS] + 1e-9
    ens["body_f64"][1, 3, L.VEL] = ens["body_f64"][1, 2, L.VEL]
    ref, _, _ = oracle.run(ens, max_steps=5, init_physical=True)
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    b.iterate(5)
    st = b.get_state()
    for f in (L.SI_STATUS, L.SI_FAIL_PAIR, L.SI_FAIL_STEP, L.SI_ITERATION):
        assert st["sys_i64"][1, f] == ref["sys_i64"][1, f], f
    assert st["sys_i64"][1, L.SI_FAIL_PAIR] == 2 * 1024 + 3
    assert max_rel_error(st, ref) <= 1e-11   # 5 steps of at most 1e-12 each


def test_batched_maximum_body_count_fast():
    """The same largest systems under FAST (pairwise gravity over unordered
    pairs in rounds of shuffled terms, with odd and even body counts up to
    32 in one warp): within 1e-12 of the oracle after one step and 1e-10
    after 30."""
    cases = []
    for coords, n_small in ((L.JACOBI, 29), (L.DEMOCRATIC_HELIOCENTRIC, 29), (L.WHDS, 29), (L.JACOBI, 14),
                            (L.WHDS, 17)):
        cases.append(E.workload_large(n_small, seed=7 + n_small, coords=coords))
    ens = stack(cases, nmax=L.MAX_BODIES)
    for steps, tol in ((1, 1e-12), (30, 1e-10)):
        ref, _, _ = oracle.run(ens, max_steps=steps, init_physical=True, nthreads=5)
        b = pg.Batch(ens, mode=pg.FAST)
        b.initialize_physical_values()
        b.iterate(steps, steps)
        got = b.get_state()
        b.close()
        assert np.all(got["sys_i64"][:, L.SI_ITERATION] == steps)
        assert max_rel_error(got, ref) <= tol, (steps, max_rel_error(got, ref))


def test_empty_and_zero_step_requests():
    """An ensemble of no systems is refused; zero steps change no bit; a
    completed system stays frozen under further steps."""
    ens = E.workload_ensemble8(4, seed=2)
    empty = {k: (v[:0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    empty["n_sys"] = 0
    with pytest.raises(pg.PosiError) as e:
        pg.Batch(empty, mode=pg.EXACT)
    assert e.value.status == L.ERR_ARG
    b = pg.Batch(ens, mode=pg.EXACT)
    b.initialize_physical_values()
    before = b.get_state()
    b.iterate(0)
    assert bitwise_diffs(b.get_state(), before) == []
    short = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in ens.items()}
    short["sys_f64"][:, L.SF_TIME_LIMIT] = 0.5   # completes after 6 steps of 0.08 d
    c = pg.Batch(short, mode=pg.EXACT)
    c.initialize_physical_values()
    c.iterate(10, 10)
    done = c.get_state()
    assert np.all(done["sys_i64"][:, L.SI_STATUS] & L.SYS_FATAL_MASK == L.SYS_COMPLETED)
    assert np.all(done["sys_i64"][:, L.SI_ITERATION] == 6)
    c.iterate(5, 5)
    assert bitwise_diffs(c.get_state(), done) == []
