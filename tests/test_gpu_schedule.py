"""GPU: balanced launch schedules (posi_batch_set_balanced).

With between one and two warps of systems per SMSP, a launch runs as
sub-launches in which warps alone on an SMSP take more steps and the systems
rotate.  Every system must still advance by exactly the requested steps, and
the states must equal those of the plain launches bit for bit (a system's
arithmetic does not depend on where or in how many pieces its steps run).
Launches of fewer than 100 steps run plain: a sub-launch costs more than a
short launch wins back.
"""
import numpy as np
import pytest

import posidonius_gb300 as pg
from posidonius_gb300 import ensemble as E, layout as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from posidonius_gb300 import build
    build.build()


def _run(ens, balanced, n_steps, spl, mode=pg.FAST):
    b = pg.Batch(ens, mode=mode, mapping=L.MAP_LANES8)
    b.set_balanced(balanced)
    b.initialize_physical_values()
    b.iterate(n_steps, spl)
    st = b.get_state()
    _, launches = b.last_timing()
    b.close()
    return st, launches


@pytest.mark.parametrize("n_steps,spl", [(200, 200), (301, 110)])
def test_balanced_schedule_matches_plain_launches(n_steps, spl):
    # 4096 systems of 8 bodies: 1024 warps, between one and two per SMSP of a
    # 152-SM part
    ens = E.workload_ensemble8(4096, seed=5)
    a, la = _run(ens, True, n_steps, spl)
    b, lb = _run(ens, False, n_steps, spl)
    assert np.all(a["sys_i64"][:, L.SI_ITERATION] == n_steps)
    for k in ("sys_i64", "sys_f64", "body_f64"):
        assert np.array_equal(np.asarray(a[k]).view(np.int64), np.asarray(b[k]).view(np.int64)), k
    assert la > lb     # the schedule ran as sub-launches (launches of >= 100 steps)


def test_balanced_schedule_exact_mode():
    ens = E.workload_ensemble8(3000, seed=6)
    a, la = _run(ens, True, 120, 120, mode=pg.EXACT)
    b, lb = _run(ens, False, 120, 120, mode=pg.EXACT)
    assert la > lb
    assert np.all(a["sys_i64"][:, L.SI_ITERATION] == 120)
    assert np.array_equal(a["body_f64"].view(np.int64), b["body_f64"].view(np.int64))


def test_side_by_side_buckets_run_plain():
    """A batch of several body counts launches its buckets side by side; a
    schedule assumes its bucket has the GPU to itself, so none is made."""
    ens = E.workload_uneven(4096, seed=7)
    assert len(np.unique(ens["sys_i64"][:, L.SI_N])) > 1
    runs = []
    for balanced in (True, False):
        b = pg.Batch(ens, mode=pg.FAST)
        b.set_balanced(balanced)
        b.initialize_physical_values()
        b.iterate(200, 200)
        runs.append((b.get_state(), b.last_timing()[1]))
        b.close()
    (a, la), (c, lc) = runs
    assert la == lc
    assert np.array_equal(a["body_f64"].view(np.int64), c["body_f64"].view(np.int64))
