"""GPU: the many-body engine (posi_large_*) against the oracle and the
batched kernel.

The engine's arithmetic is the FAST formulation (contracted multiply-adds,
rsqrt gravity, order-fixed block reductions): it must stay within 1e-10
relative of the oracle's reference-order trajectory after 100 steps, agree
with the batched FAST kernel on a system both can run, repeat itself bit for
bit, and stop at the first failing pair exactly where the reference panics.
"""
import numpy as np
import pytest

import oracle
import posidonius_gb300 as pg
from oracle.case_json import stack
from posidonius_gb300 import ensemble as E, layout as L

from parity import max_rel_error

pytestmark = pytest.mark.gpu

TOL_100 = 1e-10


@pytest.fixture(scope="module", autouse=True)
def built():
    from posidonius_gb300 import build
    build.build()


def _run_large(case, steps):
    mb = pg.ManyBody(case)
    mb.initialize_physical_values()
    st = mb.iterate(steps)
    out = mb.get_state()
    mb.close()
    return st, out


@pytest.mark.parametrize("n_small", [29, 61, 125])
def test_large_matches_oracle(n_small):
    case = E.workload_large(n_small, seed=3)
    st, got = _run_large(case, 100)
    assert st == L.OK
    ref, steps, _ = oracle.run(stack([case]), max_steps=100, init_physical=True)
    assert steps[0] == 100
    assert got["sys_i64"][L.SI_ITERATION] == ref["sys_i64"][0, L.SI_ITERATION]
    assert got["sys_f64"][L.SF_TIME] == ref["sys_f64"][0, L.SF_TIME]
    assert max_rel_error(got, {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v)
                               for k, v in ref.items()}) <= TOL_100


def test_large_matches_batched_kernel():
    """A 4-body system with tides, flattening and GR in democratic-heliocentric
    coordinates, on both engines."""
    ens = E.workload_single(seed=2, coords=L.DEMOCRATIC_HELIOCENTRIC)
    case = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    case["n"] = int(case["sys_i64"][L.SI_N])
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    b.iterate(200, 200)
    ref = b.get_state()
    st, got = _run_large(case, 200)
    assert st == L.OK
    one = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ref.items()}
    assert max_rel_error(got, one) <= TOL_100


def test_large_is_deterministic():
    case = E.workload_large(253, seed=4)
    _, a = _run_large(case, 20)
    _, b = _run_large(case, 20)
    assert np.array_equal(a["body_f64"].view(np.int64), b["body_f64"].view(np.int64))


def test_large_stops_at_first_failing_pair():
    case = E.workload_large(29, seed=5)
    bf = case["body_f64"]
    # body 7 placed on body 11: a collision in the first gravity pass
    bf[7, L.POS] = bf[11, L.POS] + 1e-9
    bf[7, L.VEL] = bf[11, L.VEL]
    ref, _, res = oracle.run(stack([case]), max_steps=5, init_physical=True)
    n = case["n"]
    mb = pg.ManyBody(case)
    mb.initialize_physical_values()
    with pytest.raises(pg.PosiError) as e:
        mb.iterate(5)
    assert e.value.status == L.ERR_PHYSICS
    st = mb.get_state()
    code = int(st["sys_i64"][L.SI_STATUS]) & L.SYS_FATAL_MASK
    assert code == int(ref["sys_i64"][0, L.SI_STATUS]) & L.SYS_FATAL_MASK
    pair = int(st["sys_i64"][L.SI_FAIL_PAIR])
    rp = int(ref["sys_i64"][0, L.SI_FAIL_PAIR])
    assert (pair // n, pair % n) == (rp // 1024, rp % 1024)


@pytest.mark.parametrize("n_small", [29, 125, 509])
def test_large_jacobi_matches_oracle(n_small):
    """Jacobi coordinates: the reference's sequential recurrences (host first,
    then index order) run as grid-wide prefix scans; within 1e-10 of the
    oracle's reference-order trajectory after 100 steps (up to 512 bodies,
    several bodies per block)."""
    case = E.workload_large(n_small, seed=3, coords=L.JACOBI)
    st, got = _run_large(case, 100)
    assert st == L.OK
    ref, steps, _ = oracle.run(stack([case]), max_steps=100, init_physical=True)
    assert steps[0] == 100
    assert max_rel_error(got, {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v)
                               for k, v in ref.items()}) <= TOL_100


def test_large_jacobi_matches_batched_kernel():
    """The 4-body system with tides, flattening and GR in Jacobi coordinates,
    on both engines."""
    ens = E.workload_single(seed=2, coords=L.JACOBI)
    case = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    case["n"] = int(case["sys_i64"][L.SI_N])
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    b.iterate(200, 200)
    ref = b.get_state()
    st, got = _run_large(case, 200)
    assert st == L.OK
    one = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ref.items()}
    assert max_rel_error(got, one) <= TOL_100


def test_large_jacobi_refuses_tangents():
    mb = pg.ManyBody(E.workload_large(29, seed=3, coords=L.JACOBI))
    mb.initialize_physical_values()
    with pytest.raises(pg.PosiError) as e:
        mb.iterate_tangent(5, [(1, L.SEED_SIGMA)])
    assert e.value.status == L.ERR_UNSUPPORTED
    mb.close()


def test_large_jacobi_host_not_first():
    """The host at index 2: Jacobi order takes it first, then the others in
    index order, and the pair left out of gravity is the host and body 0."""
    case = E.workload_large(29, seed=6, coords=L.JACOBI)
    perm = np.arange(case["n"])
    perm[[0, 2]] = perm[[2, 0]]
    moved = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in case.items()}
    for k in ("body_f64", "body_i64"):
        moved[k] = np.ascontiguousarray(case[k][perm])
    moved["sys_i64"][L.SI_HOST] = 2
    st, got = _run_large(moved, 100)
    assert st == L.OK
    ref, steps, _ = oracle.run(stack([moved]), max_steps=100, init_physical=True)
    assert steps[0] == 100
    assert max_rel_error(got, {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v)
                               for k, v in ref.items()}) <= TOL_100


@pytest.mark.parametrize("n_small", [29, 125])
def test_large_whds_matches_oracle(n_small):
    """WHDS coordinates: within 1e-10 of the oracle after 100 steps."""
    case = E.workload_large(n_small, seed=3, coords=L.WHDS)
    st, got = _run_large(case, 100)
    assert st == L.OK
    ref, steps, _ = oracle.run(stack([case]), max_steps=100, init_physical=True)
    assert steps[0] == 100
    assert max_rel_error(got, {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v)
                               for k, v in ref.items()}) <= TOL_100


def test_large_whds_matches_batched_kernel():
    ens = E.workload_single(seed=2, coords=L.WHDS)
    case = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    case["n"] = int(case["sys_i64"][L.SI_N])
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    b.iterate(200, 200)
    ref = b.get_state()
    st, got = _run_large(case, 200)
    assert st == L.OK
    one = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ref.items()}
    assert max_rel_error(got, one) <= TOL_100
