"""GPU: forward-mode derivatives of the many-body engine
(posi_large_iterate_tangent).

* The primal state of a tangent run is the plain run's state.
* Tangents along a dissipation factor, a Love number and an initial velocity
  agree with central finite differences of the engine's own trajectories.
  The tidal parameters are amplified (dissipation factors x 5e7, Love
  numbers x 1e3) so that a finite-difference step moves the state well above
  FP64 rounding; the code path is the one physical values take.
* The check allows FD_TOL relative plus three times the change of the
  difference quotient between two step sizes (its own truncation and
  rounding noise), both as maxima over all bodies of a field.  At these
  amplifications the state is far from linear in a dissipation factor: the
  quotient's truncation error falls as h^2 (1.1e-5 of the derivative at a
  relative step of 1e-2 over 100 steps, 4.7e-3 at 2e-1), while below 1e-3
  its rounding noise dominates.
"""
import numpy as np
import pytest

import posidonius_gb300 as pg
from posidonius_gb300 import ensemble as E, layout as L

pytestmark = pytest.mark.gpu

FD_TOL = 1e-6
STEPS = 100
FIELDS = {"r": L.POS, "v": L.VEL, "L": L.ANG}


@pytest.fixture(scope="module", autouse=True)
def built():
    from posidonius_gb300 import build
    build.build()


def _case(n_small=29, seed=3):
    case = E.workload_large(n_small, seed=seed)
    case["body_f64"][1:3, L.BF_SIGMA] *= 5e7
    case["body_f64"][1:3, L.BF_K2] *= 1e3
    return case


def _final(case, steps=STEPS):
    mb = pg.ManyBody(case)
    mb.initialize_physical_values()
    assert mb.iterate(steps) == L.OK
    out = mb.get_state()["body_f64"]
    mb.close()
    return out


def _tangent(case, seeds, tangents=None, steps=STEPS):
    mb = pg.ManyBody(case)
    mb.initialize_physical_values()
    rc, tan = mb.iterate_tangent(steps, seeds, tangents)
    assert rc == L.OK
    out = mb.get_state()["body_f64"]
    mb.close()
    return out, tan


def _fd(case, perturb, h):
    """Central difference of the final state for perturb(case copy, +-h)."""
    def run(s):
        c = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in case.items()}
        perturb(c, s)
        return _final(c)
    return (run(h) - run(-h)) / (2 * h)


def _check(tan, fd, fd2, label):
    """tan [n, 12] against the difference quotients fd, fd2 [n, BF_COUNT]."""
    for name, sl in FIELDS.items():
        k = {"r": 0, "v": 3, "L": 6}[name]
        t = tan[:, k:k + 3]
        f, f2 = fd[:, sl], fd2[:, sl]
        scale = np.abs(f).max()
        if scale == 0.0:
            assert np.abs(t).max() == 0.0, (label, name)
            continue
        bound = FD_TOL * scale + 3.0 * np.abs(f - f2).max()
        worst = np.abs(t - f).max() / bound
        assert worst <= 1.0, (label, name, worst, scale)


def test_tangent_primal_matches_plain_run():
    """The integrated state of a tangent run (positions, velocities, spin
    angular momenta, spins and their compensation terms) is the plain run's
    bit for bit: every primal sum is formed in the same order.  The stored
    gravity acceleration of the last evaluation -- a diagnostic that enters
    the state only through dt a, far below a velocity's last bit -- may
    differ by a few ulps: the pair loop's instantiation with tangents is
    compiled with other multiply-add contractions."""
    case = _case()
    plain = _final(case)
    prim, _ = _tangent(case, [(1, L.SEED_SIGMA), (2, L.SEED_SIGMA)])
    acc = [L.BF_AX, L.BF_AY, L.BF_AZ]
    state = [f for f in range(L.BF_COUNT) if f not in acc]
    np.testing.assert_array_equal(prim[:, state].view(np.int64), plain[:, state].view(np.int64))
    assert np.abs(prim[:, acc] - plain[:, acc]).max() <= 1e-14 * np.abs(plain[:, acc]).max()


@pytest.mark.parametrize("body", [1, 2])
def test_dissipation_factor_tangent_matches_finite_differences(body):
    case = _case()
    sig = case["body_f64"][body, L.BF_SIGMA]
    _, tan = _tangent(case, [(body, L.SEED_SIGMA)])

    def perturb(c, s):
        c["body_f64"][body, L.BF_SIGMA] = sig + s

    h = 1e-2 * sig
    fd, fd2 = _fd(case, perturb, h), _fd(case, perturb, h / 2)
    _check(tan[0], fd, fd2, f"sigma of body {body}")


def test_love_number_tangent_matches_finite_differences():
    case = _case()
    k2 = case["body_f64"][1, L.BF_K2]
    _, tan = _tangent(case, [(1, L.SEED_K2)])

    def perturb(c, s):
        c["body_f64"][1, L.BF_K2] = k2 + s

    h = 1e-2 * k2
    fd, fd2 = _fd(case, perturb, h), _fd(case, perturb, h / 2)
    _check(tan[0], fd, fd2, "k2 of body 1")


def test_initial_velocity_tangent_matches_finite_differences():
    """No parameter seed: the tangent of an initial velocity component of a
    small body and of a planet (gravity, Kepler drift and the transforms)."""
    case = _case()
    n = case["n"]
    seeds = [(-1, L.SEED_SIGMA), (-1, L.SEED_SIGMA)]
    t0 = np.zeros((2, n, 12))
    t0[0, 5, 3] = 1.0      # v_x of body 5
    t0[1, 1, 4] = 1.0      # v_y of planet 1
    _, tan = _tangent(case, seeds, t0)
    for d, (b, q) in enumerate([(5, 0), (1, 1)]):
        v = case["body_f64"][b, L.BF_VX + q]

        def perturb(c, s, b=b, q=q, v=v):
            c["body_f64"][b, L.BF_VX + q] = v + s

        h = 1e-6 * np.abs(case["body_f64"][b, L.VEL]).max()
        fd, fd2 = _fd(case, perturb, h), _fd(case, perturb, h / 2)
        _check(tan[d], fd, fd2, f"v[{q}] of body {b}")


def test_tangent_directions_are_independent():
    """Three directions (one launch of four, the last a zero padding
    direction) give the tangents of three one-direction launches."""
    case = _case()
    seeds = [(1, L.SEED_SIGMA), (2, L.SEED_SIGMA), (1, L.SEED_K2)]
    _, tan3 = _tangent(case, seeds, steps=20)
    for d, s in enumerate(seeds):
        _, one = _tangent(case, [s], steps=20)
        for k in range(0, 12, 3):
            scale = np.abs(one[0][:, k:k + 3]).max()
            assert np.abs(tan3[d][:, k:k + 3] - one[0][:, k:k + 3]).max() <= 1e-12 * scale, (d, k)


def test_tangent_rejects_bad_seeds():
    case = _case()
    mb = pg.ManyBody(case)
    with pytest.raises(pg.PosiError) as e:
        mb.iterate_tangent(1, [(case["n"], L.SEED_SIGMA)])
    assert e.value.status == L.ERR_ARG
    with pytest.raises(pg.PosiError):
        mb.iterate_tangent(1, [(1, 7)])
    with pytest.raises(pg.PosiError):
        mb.iterate_tangent(1, [(1, 0)] * 5)
    mb.close()
