"""GPU: the adjoint of the WHFast + tides step against finite differences.

Gradients of the differentiation workload's loss (squared final
eccentricities, relative semi-major-axis drifts, relative planetary spin-rate
changes) with respect to every body's dissipation factor and Love number and
every planet's six initial orbital elements, by the checkpointed adjoint
(torch autograd around posi_adjoint_*), against central finite differences of
the same loss integrated by the forward kernel (relative step 1e-6 for the
orbital elements).  At physical values the dissipation factors and Love
numbers change the loss of a short run by less than its rounding level, so
their gradients are checked with both amplified (same code path) and a
1e-3 relative step, over which the loss is linear in them.
"""
import numpy as np
import pytest

import posidonius_gb300 as pg
from posidonius_gb300 import adjoint as A, ensemble as E, layout as L

pytestmark = pytest.mark.gpu

# relative agreement with central differences where they resolve the derivative
ADJ_FD_TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def built():
    from posidonius_gb300 import build
    build.build()


def _check(adj, fd, fd2):
    """Worst ratio over systems of max |adj - fd| / (ADJ_FD_TOL max |fd| +
    3 max |fd - fd2|), the maxima over the system's gradient components: the
    adjoint must agree with the difference quotient fd to ADJ_FD_TOL of the
    system's gradient, up to the quotient's own error, estimated by its
    change between two step sizes (truncation where the loss bends over the
    step, rounding noise of the loss where the step is small).  Norms per
    system, not per component: a component whose two quotients agree by
    chance would otherwise get a bound below the quotient's real error."""
    adj, fd, fd2 = (x.reshape(x.shape[0], -1) for x in (adj, fd, fd2))
    err = np.abs(adj - fd).max(axis=1)
    bound = ADJ_FD_TOL * np.abs(fd).max(axis=1) + 3.0 * np.abs(fd - fd2).max(axis=1) + 1e-300
    return float((err / bound).max())


@pytest.mark.parametrize("n_steps,every", [(120, 50), (400, 100)])
def test_adjoint_elements_match_finite_differences(n_steps, every):
    """Physical parameters: the orbital-element gradients (relative steps 1e-6
    and 1e-5)."""
    ens, el, ms, moi, ss = A.gradient_workload(4, seed=7)
    sig = ens["body_f64"][:, :, L.BF_SIGMA].copy()
    k2 = ens["body_f64"][:, :, L.BF_K2].copy()
    loss, g_sig, g_k2, g_el, _, flags = A.adjoint_gradient(ens, el, sig, k2, ms, moi, ss, n_steps, every)
    assert not flags.any()
    _, _, f_el = A.finite_difference_gradient(ens, el, sig, k2, ms, moi, ss, n_steps, rel_step=1e-6)
    _, _, f_el2 = A.finite_difference_gradient(ens, el, sig, k2, ms, moi, ss, n_steps, rel_step=1e-5)
    ref = A.loss_of_parameters(ens, el, sig, k2, ms, moi, ss, n_steps)
    assert np.allclose(loss, ref, rtol=1e-10, atol=0)
    err = _check(g_el, f_el, f_el2)
    assert err <= 1.0, (err, g_el, f_el, f_el2)


def test_adjoint_tidal_parameters_match_finite_differences():
    """Dissipation factors x 5e7 and Love numbers x 1e6: their effect on the
    loss becomes large enough for central differences (relative steps 1e-2
    and 1e-3; the loss is linear in them over that range) to resolve it; the
    code path is the one the physical parameters take.  A system the forward
    run froze (Roche limit) is flagged and left out."""
    ens, el, ms, moi, ss = A.gradient_workload(4, seed=11)
    sig = ens["body_f64"][:, :, L.BF_SIGMA].copy() * 5e7
    k2 = ens["body_f64"][:, :, L.BF_K2].copy() * 1e6
    ens["body_f64"][:, :, L.BF_SIGMA] = sig
    ens["body_f64"][:, :, L.BF_K2] = k2
    n_steps, every = 300, 100
    loss, g_sig, g_k2, g_el, _, flags = A.adjoint_gradient(ens, el, sig, k2, ms, moi, ss, n_steps, every)
    assert flags[2] == A.FLAG_FROZEN and flags.sum() == A.FLAG_FROZEN
    keep = flags == 0
    f_sig, f_k2, _ = A.finite_difference_gradient(ens, el, sig, k2, ms, moi, ss, n_steps, rel_step_tidal=1e-2)
    f_sig2, f_k22, _ = A.finite_difference_gradient(ens, el, sig, k2, ms, moi, ss, n_steps, rel_step_tidal=1e-3)
    # compared as d loss / d ln(parameter): the bodies' dissipation factors
    # span five orders of magnitude, and a raw-unit norm would let the
    # smallest one's (noise-dominated) component set every system's bound
    s, k = sig[keep], k2[keep]
    errs = {"sigma": _check(g_sig[keep] * s, f_sig[keep] * s, f_sig2[keep] * s),
            "k2": _check(g_k2[keep] * k, f_k2[keep] * k, f_k22[keep] * k)}
    assert max(errs.values()) <= 1.0, (errs, g_sig * sig, f_sig * sig, f_sig2 * sig, g_k2 * k2, f_k2 * k2,
                                       f_k22 * k2)


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
