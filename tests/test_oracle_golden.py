"""Pin the CPU oracle against the reference's own golden cases.

Reference test: tests/common/universe.rs:47-72 (assert_stored_positions) --
final inertial position, velocity and acceleration of every body after
integrating to time_limit = 200*dt with dt = 0.08 d, 1e-14 absolute.
The restatement meets it with zero difference.
"""
import numpy as np
import pytest

import oracle
from oracle.case_json import load_case
from posidonius_gb300 import layout as L

from golden_cases import case_dict, expected, max_abs_error, names


@pytest.mark.parametrize("name", names())
def test_oracle_matches_reference_golden(name):
    case = load_case(case_dict(name))
    ens, steps, res = oracle.run(case, max_steps=10**6, init_physical=True)
    # 200*dt time limit: the float test at src/integrator/whfast.rs:300 stops after 199 steps
    assert steps[0] == 199
    assert ens["sys_i64"][0, L.SI_STATUS] & L.SYS_FATAL_MASK == L.SYS_COMPLETED
    err = max_abs_error(ens["body_f64"][0], expected(name))
    assert err <= 1e-14
    assert err == 0.0, "restatement should be bit-exact against the Rust FP64 path"


@pytest.mark.parametrize("name", names("ias15"))
def test_oracle_ias15_matches_reference_golden(name):
    """tests/test_integrator.rs:303-312 (ias15_rust): the IAS15 restatement
    integrates the brown-dwarf case to the same bits.  The adaptive step
    starts at 0.08 d and grows by the safety factor's limit of 4 per step
    (0.32, 1.28, 5.12 d), so the run stops after 4 steps at t = 6.8 d with a
    next step of 20.48 d beyond the 16 d limit."""
    case = load_case(case_dict(name))
    assert case["sys_i64"][L.SI_INTEGRATOR] == L.INTEGRATOR_IAS15
    ens, steps, res = oracle.run(case, max_steps=10**6, init_physical=True)
    assert steps[0] == 4
    assert ens["sys_i64"][0, L.SI_STATUS] & L.SYS_FATAL_MASK == L.SYS_COMPLETED
    assert ens["sys_f64"][0, L.SF_TIME] == 0.08 + 0.32 + 1.28 + 5.12
    assert ens["sys_f64"][0, L.SF_DT] == 20.48
    assert max_abs_error(ens["body_f64"][0], expected(name)) == 0.0


def test_oracle_ias15_rejects_and_retries():
    """A first step far too long for the system (100 d against an estimate
    near 16 d) does not converge within 12 predictor-corrector iterations,
    is rejected and redone with the estimated step (ias15.rs:1187-1217)."""
    name = names("ias15")[0]
    case = load_case(case_dict(name))
    big = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in case.items()}
    big["sys_f64"][L.SF_DT] = 100.0
    big["sys_f64"][L.SF_TIME_LIMIT] = 1000.0
    ens, steps, _ = oracle.run(big, max_steps=1, init_physical=True)
    assert steps[0] == 1
    assert ens["sys_i64"][0, L.SI_IAS_MAX_EXCEEDED] == 1
    t1 = ens["sys_f64"][0, L.SF_TIME]
    assert 10.0 < t1 < 25.0 and ens["sys_f64"][0, L.SF_IAS_DT_LAST] == t1


@pytest.mark.parametrize("name", ["test_integrator-whfast_jacobi",
                                  "test_integrator-whfast_democraticheliocentric",
                                  "test_integrator-whfast_whds"])
def test_python_generated_twin_one_step(name):
    """tests/test_integrator.rs:58-70: one step of the Python-generated case
    against one step of the Rust-built case, 1e-8 (positions, velocities) and
    1e-7 (accelerations) absolute (tests/common/universe.rs:207-226)."""
    a = load_case(case_dict(name))
    b = load_case(case_dict(name, python_twin=True))
    ea, _, _ = oracle.run(a, max_steps=1, init_physical=True)
    eb, _, _ = oracle.run(b, max_steps=1, init_physical=True)
    fa, fb = ea["body_f64"][0], eb["body_f64"][0]
    assert np.abs(fa[:, L.POS] - fb[:, L.POS]).max() <= 1e-8
    assert np.abs(fa[:, L.VEL] - fb[:, L.VEL]).max() <= 1e-8
    assert np.abs(fa[:, L.ACC] - fb[:, L.ACC]).max() <= 1e-7


def test_star_order_permutation():
    """tests/test_order.rs:341-380: swapping the star and the first planet
    gives the same trajectory (assert_when_star_is_swapped, 1e-16)."""
    name = "test_integrator-whfast_jacobi"
    d = case_dict(name)
    u = d["universe"]
    u["particles"][0], u["particles"][1] = u["particles"][1], u["particles"][0]
    u["particles_evolvers"][0], u["particles_evolvers"][1] = u["particles_evolvers"][1], u["particles_evolvers"][0]
    for k in ("most_massive", "tides", "rotational_flattening", "general_relativity"):
        u["hosts"]["index"][k] = 1
    base = load_case(case_dict(name))
    swapped = load_case(d)
    e0, _, _ = oracle.run(base, max_steps=10**6, init_physical=True)
    e1, _, _ = oracle.run(swapped, max_steps=10**6, init_physical=True)
    f0 = e0["body_f64"][0]
    f1 = e1["body_f64"][0][[1, 0, 2, 3, 4]]
    for sl in (L.POS, L.VEL, L.ACC):
        assert np.abs(f0[:, sl] - f1[:, sl]).max() <= 1e-16


def test_ias15_star_order_permutation():
    """tests/test_order.rs (the IAS15 order cases): swapping the star and the
    first planet of the IAS15 case gives the same trajectory; IAS15 has no
    coordinate recurrence over the body order, so only the pair-sum order of
    the accelerations changes (1e-15 absolute after the adaptive run)."""
    name = names("ias15")[0]
    d = case_dict(name)
    u = d["universe"]
    u["particles"][0], u["particles"][1] = u["particles"][1], u["particles"][0]
    u["particles_evolvers"][0], u["particles_evolvers"][1] = u["particles_evolvers"][1], u["particles_evolvers"][0]
    for k in ("most_massive", "tides", "rotational_flattening", "general_relativity"):
        u["hosts"]["index"][k] = 1
    base = load_case(case_dict(name))
    swapped = load_case(d)
    e0, s0, _ = oracle.run(base, max_steps=10**6, init_physical=True)
    e1, s1, _ = oracle.run(swapped, max_steps=10**6, init_physical=True)
    assert s0[0] == s1[0] == 4
    f0 = e0["body_f64"][0]
    f1 = e1["body_f64"][0][[1, 0, 2, 3, 4]]
    for sl in (L.POS, L.VEL):
        assert np.abs(f0[:, sl] - f1[:, sl]).max() <= 1e-15
