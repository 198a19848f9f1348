"""CPU: the oracle's dual-number build (forward-mode derivatives of its
reference-order arithmetic), the reference the adjoint is checked against.

Its values are the plain oracle's bit for bit (the same operations on the
value parts), and its derivatives agree with central differences of the
plain oracle where differences resolve them: the orbital elements at
physical values (relative step 1e-6), the dissipation factors and Love
numbers amplified (x 5e7, x 1e6) so that a 1e-3 relative step moves the
loss well above its rounding level."""
import numpy as np
import pytest

import oracle
from posidonius_gb300 import adjoint as A, layout as L

from parity import bitwise_diffs

TOL = 1e-6
N_STEPS = 100


@pytest.fixture(scope="module", autouse=True)
def built():
    oracle.build()


def _runner(ens, n):
    out, _, _ = oracle.run(ens, max_steps=n, init_physical=True, nthreads=4)
    return out["body_f64"]


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_dual_values_are_the_plain_oracle_bit_for_bit():
    ens, el, ms, moi, ss = A.gradient_workload(3, seed=7)
    sig = ens["body_f64"][:, :, L.BF_SIGMA].copy()
    k2 = ens["body_f64"][:, :, L.BF_K2].copy()
    e0 = A.initial_ensemble(ens, el, sig, k2, ms, moi, ss)
    nd = oracle.dual_directions()
    rng = np.random.default_rng(1)
    seed = rng.normal(size=(3, e0["nmax"], L.BF_COUNT, nd))
    dual, _, _, tan = oracle.run_dual(e0, seed, N_STEPS, init_physical=True, nthreads=3)
    plain, _, _ = oracle.run(e0, max_steps=N_STEPS, init_physical=True, nthreads=3)
    assert bitwise_diffs(dual, plain) == []
    assert np.isfinite(tan).all() and np.abs(tan[:, :, L.POS]).max() > 0


@pytest.mark.parametrize("amplify", [False, True])
def test_dual_gradient_matches_central_differences(amplify):
    ens, el, ms, moi, ss = A.gradient_workload(4, seed=7)
    if amplify:
        ens["body_f64"][:, :, L.BF_SIGMA] *= 5e7
        ens["body_f64"][:, :, L.BF_K2] *= 1e6
    sig = ens["body_f64"][:, :, L.BF_SIGMA].copy()
    k2 = ens["body_f64"][:, :, L.BF_K2].copy()
    loss, gs, gk, ge = A.oracle_dual_gradient(ens, el, sig, k2, ms, moi, ss, N_STEPS, nthreads=4)
    ref = A.loss_of_parameters(ens, el, sig, k2, ms, moi, ss, N_STEPS, runner=_runner)
    assert np.array_equal(loss, ref)
    fs, fk, fe = A.finite_difference_gradient(ens, el, sig, k2, ms, moi, ss, N_STEPS, rel_step=1e-6,
                                              rel_step_tidal=1e-3, runner=_runner)
    assert _rel(ge, fe) <= TOL
    if amplify:
        # as d loss / d ln(parameter)
        assert _rel(gs * sig, fs * sig) <= TOL
        assert _rel(gk * k2, fk * k2) <= TOL
