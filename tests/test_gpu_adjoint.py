"""GPU: the adjoint of the WHFast + tides step against the exact derivatives
of the oracle.

Gradients of the differentiation workload's loss (squared final
eccentricities, relative semi-major-axis drifts, relative planetary spin-rate
changes) with respect to every body's dissipation factor and Love number and
every planet's six initial orbital elements, by the checkpointed adjoint
(torch autograd around posi_adjoint_*), against the oracle's dual-number
build: forward-mode derivatives through the reference-order arithmetic, with
no step size and no difference noise (tests/test_oracle_dual.py checks them
against central differences of the plain oracle).  Every parameter is at
its physical value; the bound is 1e-6 relative per system and parameter
group (the dissipation factors and Love numbers as d loss / d ln p, since
they span orders of magnitude), with no allowance for noise.

Over 1e4 steps a system whose planets pass close to one another is chaotic:
a 1e-13 nudge of its mean anomalies moves the oracle's own loss by 1e-7 or
more, and no two arithmetics share its trajectory.  Such systems are
identified by that sensitivity of the oracle itself and checked at 1e3
steps, inside their predictability horizon.
"""
import numpy as np
import pytest

import oracle
import posidonius_gb300 as pg
from posidonius_gb300 import adjoint as A, ensemble as E, layout as L

pytestmark = pytest.mark.gpu

ADJ_TOL = 1e-6
CHAOTIC = 1e-9   # relative loss change of the oracle under a 1e-13 nudge of the mean anomalies


@pytest.fixture(scope="module", autouse=True)
def built():
    from posidonius_gb300 import build
    build.build()
    oracle.build()


def _per_system(a, b):
    a, b = (np.asarray(x).reshape(len(x), -1) for x in (a, b))
    return np.abs(a - b).max(axis=1) / np.maximum(np.abs(b).max(axis=1), 1e-300)


def _errors(ens, el, sig, k2, ms, moi, ss, n_steps, every):
    """Per-system relative errors (elements, d/d ln sigma, d/d ln k2) of the
    adjoint against the dual oracle, the adjoint's flags and the losses."""
    loss, g_sig, g_k2, g_el, _, flags = A.adjoint_gradient(ens, el, sig, k2, ms, moi, ss, n_steps, every)
    d_loss, d_sig, d_k2, d_el = A.oracle_dual_gradient(ens, el, sig, k2, ms, moi, ss, n_steps)
    err = np.stack([_per_system(g_el, d_el), _per_system(g_sig * sig, d_sig * sig),
                    _per_system(g_k2 * k2, d_k2 * k2)], axis=1)
    return err, flags, loss, d_loss


def _oracle_sensitivity(ens, el, sig, k2, ms, moi, ss, n_steps):
    def runner(e, n):
        out, _, _ = oracle.run(e, max_steps=n, init_physical=True, nthreads=16)
        return out["body_f64"]
    l1 = A.loss_of_parameters(ens, el, sig, k2, ms, moi, ss, n_steps, runner=runner)
    el2 = el.copy()
    el2[..., 5] += 1e-13
    l2 = A.loss_of_parameters(ens, el2, sig, k2, ms, moi, ss, n_steps, runner=runner)
    return np.abs(l2 - l1) / np.abs(l1)


def _params(ens):
    return ens["body_f64"][:, :, L.BF_SIGMA].copy(), ens["body_f64"][:, :, L.BF_K2].copy()


@pytest.mark.parametrize("n_steps,every", [(120, 50), (400, 100)])
def test_adjoint_matches_oracle_derivatives(n_steps, every):
    """Every parameter at its physical value, every system."""
    ens, el, ms, moi, ss = A.gradient_workload(8, seed=7)
    sig, k2 = _params(ens)
    err, flags, loss, d_loss = _errors(ens, el, sig, k2, ms, moi, ss, n_steps, every)
    assert not flags.any()
    assert np.allclose(loss, d_loss, rtol=1e-10, atol=0)
    assert err.max() <= ADJ_TOL, err


def _workload_sample(n):
    """n systems spread over the differentiation workload (1024 systems of a
    star and three planets)."""
    ens, el, ms, moi, ss = A.gradient_workload(1024)
    idx = np.linspace(0, 1023, n).astype(int)
    ens = {k: (v[idx] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    ens["n_sys"] = n
    return ens, el[idx], ms[idx], moi[idx], ss[idx]


def test_adjoint_at_the_workloads_horizon():
    """32 systems of the workload at its 1e4 steps (checkpoints every 100):
    every system the oracle finds predictable over the run is within 1e-6,
    and most are; the chaotic rest, at 1e3 steps, are within 1e-6 too."""
    ens, el, ms, moi, ss = _workload_sample(32)
    sig, k2 = _params(ens)
    sens = _oracle_sensitivity(ens, el, sig, k2, ms, moi, ss, 10000)
    regular = sens <= CHAOTIC
    assert regular.mean() >= 0.6, regular.sum()
    err, flags, _, _ = _errors(ens, el, sig, k2, ms, moi, ss, 10000, 100)
    ok = regular & (flags == 0)
    assert (err[ok] <= ADJ_TOL).all(), (np.nonzero(ok)[0], err[ok].max(axis=1))
    rest = {k: (v[~ok] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    rest["n_sys"] = int((~ok).sum())
    if rest["n_sys"]:
        short_sens = _oracle_sensitivity(rest, el[~ok], sig[~ok], k2[~ok], ms[~ok], moi[~ok], ss[~ok], 1000)
        assert (short_sens <= CHAOTIC).all(), short_sens
        err_s, flags_s, _, _ = _errors(rest, el[~ok], sig[~ok], k2[~ok], ms[~ok], moi[~ok], ss[~ok], 1000, 100)
        assert flags_s.sum() <= A.FLAG_FROZEN      # at most one system frozen by a close encounter
        assert err_s[flags_s == 0].max() <= ADJ_TOL, err_s


def test_adjoint_flags_a_frozen_system():
    """With dissipation factors x 5e7 and Love numbers x 1e6 one system of
    this seed reaches its Roche limit: the forward run freezes it and the
    adjoint flags it; the others match the oracle's derivatives."""
    ens, el, ms, moi, ss = A.gradient_workload(4, seed=11)
    ens["body_f64"][:, :, L.BF_SIGMA] *= 5e7
    ens["body_f64"][:, :, L.BF_K2] *= 1e6
    sig, k2 = _params(ens)
    err, flags, _, _ = _errors(ens, el, sig, k2, ms, moi, ss, 300, 100)
    assert flags[2] == A.FLAG_FROZEN and flags.sum() == A.FLAG_FROZEN
    assert err[flags == 0].max() <= ADJ_TOL, err


def test_adjoint_of_identity_seed_is_consistent():
    """lam_final = e_k (one coordinate of one body): one backward run gives a
    row of the Jacobian; central differences of that coordinate agree."""
    ens, el, ms, moi, ss = A.gradient_workload(2, seed=3)
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    base = b.get_state()
    adj = A.Adjoint(b, 60, 25)
    adj.forward()
    lam = np.zeros((b.n_sys, b.nmax, 12))
    lam[:, 2, 0] = 1.0  # x of planet 2
    lam_i, grad = adj.backward(lam)
    # derivative of x_2(T) with respect to vx of planet 1 at t = 0, by differences
    h = 1e-6 * np.abs(base["body_f64"][:, 1, L.BF_VX]).max()
    outs = []
    for sgn in (1.0, -1.0):
        st = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in base.items()}
        st["body_f64"][:, 1, L.BF_VX] += sgn * h
        b.set_state(st)
        b.iterate(60, 60)
        outs.append(b.get_state()["body_f64"][:, 2, L.BF_PX])
    fd = (outs[0] - outs[1]) / (2 * h)
    assert np.abs(lam_i[:, 1, 3] - fd).max() <= 1e-5 * np.abs(fd).max(), (lam_i[:, 1, 3], fd)


def test_adjoint_rejects_unsupported_and_out_of_order():
    ens = E.workload_single(seed=1, coords=L.DEMOCRATIC_HELIOCENTRIC)
    b = pg.Batch(ens, mode=pg.FAST)
    with pytest.raises(pg.PosiError) as e:
        A.Adjoint(b, 10, 5)
    assert e.value.status == L.ERR_UNSUPPORTED
    ens = E.workload_single(seed=1)
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    adj = A.Adjoint(b, 10, 5)
    with pytest.raises(pg.PosiError) as e:
        adj.backward(np.zeros((1, b.nmax, 12)))
    assert e.value.status == L.ERR_STATE


@pytest.mark.parametrize("mode", [pg.FAST, pg.EXACT])
def test_backward_independent_of_chunking_and_repeatable(mode):
    """The backward run re-integrates each chunk from a copy of its
    checkpoint, overlapping the reverse sweep of the next chunk: the result
    must not depend on the chunk length (one chunk, uneven chunks, one tape
    buffer or two), a second backward run must repeat the first bit for bit,
    and the batch must stay at the forward run's final state."""
    ens, el, ms, moi, ss = A.gradient_workload(96, seed=4)
    rng = np.random.default_rng(9)
    n_steps = 90
    out = {}
    for every in (90, 13, 7):
        b = pg.Batch(ens, mode=mode)
        b.initialize_physical_values()
        adj = A.Adjoint(b, n_steps, every)
        adj.forward()
        final = b.get_state()
        lam = rng.standard_normal((b.n_sys, b.nmax, 12)) if every == 90 else out[90][2]
        lam_i, grad = adj.backward(lam)
        lam_i2, grad2 = adj.backward(lam)
        after = b.get_state()
        for k in ("sys_i64", "sys_f64", "body_f64"):
            assert np.array_equal(np.asarray(final[k]).view(np.int64), np.asarray(after[k]).view(np.int64)), k
        assert np.array_equal(lam_i.view(np.int64), lam_i2.view(np.int64))
        assert np.array_equal(grad.view(np.int64), grad2.view(np.int64))
        out[every] = (lam_i, grad, lam)
        adj.close()
        b.close()
    for every in (13, 7):
        for q in (0, 1):
            a, ref = out[every][q], out[90][q]
            if mode == pg.FAST:
                # the chunks are re-integrated by the forward kernel itself
                assert np.array_equal(a.view(np.int64), ref.view(np.int64)), (every, q)
            else:
                # the EXACT build records with the adjoint's own forward sweep,
                # whose last bits differ from the forward kernel's, so a chunk
                # boundary moves the recorded trajectory by rounding: per
                # field, agreement to 1e-8 of the field's largest value
                a2, r2 = a.reshape(-1, a.shape[-1]), ref.reshape(-1, ref.shape[-1])
                err = np.abs(a2 - r2).max(axis=0)
                assert np.all(err <= 1e-8 * np.abs(r2).max(axis=0)), (every, q, err)
