"""CPU checks of the adjoint building blocks (no GPU).

``posidonius_gb300/csrc/adjoint_blocks.cuh`` and the generated
``adjoint_effects.cuh`` are host-and-device code; here they are compiled for
the CPU (tests/adjoint_host/adjoint_host.cpp) and checked:

* Stumpff functions c0..c5 against their power series;
* the Kepler drift against the classical two-body solution (eccentric
  anomaly), and its VJP against central finite differences;
* the forward effect blocks, assembled per system, against the oracle's
  ``calculate_additional_effects`` (the reference's evaluation);
* every effect-block VJP against central finite differences.
"""
import ctypes
import math
import os
import subprocess

import numpy as np
import pytest

import oracle
from posidonius_gb300 import ensemble as E, layout as L

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "adjoint_host", "adjoint_host.cpp")
BUILD = os.path.join(HERE, "adjoint_host", "_build")
SO = os.path.join(BUILD, "libadjoint_host.so")

f64p = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def lib():
    os.makedirs(BUILD, exist_ok=True)
    deps = [SRC] + [os.path.join(HERE, "..", "posidonius_gb300", "csrc", f)
                    for f in ("adjoint_blocks.cuh", "adjoint_effects.cuh")]
    if not os.path.exists(SO) or any(os.path.getmtime(d) > os.path.getmtime(SO) for d in deps):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", SRC, "-o", SO])
    h = ctypes.CDLL(SO)
    h.h_stumpff6.argtypes = [ctypes.c_double, f64p]
    h.h_kepler_fwd.argtypes = [ctypes.c_double, ctypes.c_double, f64p, f64p, f64p, f64p]
    h.h_kepler_fwd.restype = ctypes.c_double
    h.h_kepler_vjp.argtypes = [ctypes.c_double, ctypes.c_double, f64p, f64p, ctypes.c_double, f64p, f64p, f64p, f64p]
    h.h_effects_fwd.argtypes = [ctypes.c_int, f64p, f64p, f64p]
    h.h_effects_vjp.argtypes = [ctypes.c_int, f64p, f64p, f64p, f64p]
    h.h_kepler_jvp.argtypes = [ctypes.c_double, ctypes.c_double, f64p, f64p, ctypes.c_double, f64p, f64p, f64p,
                               f64p]
    h.h_effects_jvp.argtypes = [ctypes.c_int, f64p, f64p, f64p, f64p]
    return h


def P(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(f64p)


def stumpff_series(z, n):
    s, term, k = 0.0, None, 0
    while True:
        term = (-z) ** k / math.factorial(2 * k + n)
        s += term
        if abs(term) < 1e-18 * abs(s) and k > 3:
            return s
        k += 1


@pytest.mark.parametrize("z", [0.0, 1e-3, -0.05, 0.09, 0.3, -0.7, 2.5, 9.0, -4.0])
def test_stumpff(lib, z):
    c = np.zeros(6)
    lib.h_stumpff6(z, P(c)) if False else lib.h_stumpff6(z, c.ctypes.data_as(f64p))
    for n in range(6):
        ref = stumpff_series(z, n)
        assert abs(c[n] - ref) <= 2e-13 * max(1.0, abs(ref)) / (1.0 if n < 4 else min(1.0, abs(z) + 1e-3)), (n, c[n], ref)


def two_body(mu, r, v, dt):
    """Classical elliptic propagation through the eccentric anomaly."""
    r, v = np.asarray(r, float), np.asarray(v, float)
    rn = np.linalg.norm(r)
    a = 1.0 / (2.0 / rn - v @ v / mu)
    n = math.sqrt(mu / a**3)
    ecosE0 = 1.0 - rn / a
    esinE0 = (r @ v) / math.sqrt(mu * a)
    E0 = math.atan2(esinE0, ecosE0)
    e = math.hypot(ecosE0, esinE0)
    M0 = E0 - esinE0
    M = M0 + n * dt
    Ex = M
    for _ in range(100):
        Ex -= (Ex - e * math.sin(Ex) - M) / (1.0 - e * math.cos(Ex))
    dE = Ex - E0
    f = a / rn * (math.cos(dE) - 1.0) + 1.0
    g = dt + (math.sin(dE) - dE) / n
    r1 = f * r + g * v
    r1n = np.linalg.norm(r1)
    fd = -a * a * n * math.sin(dE) / (r1n * rn)
    gd = a / r1n * (math.cos(dE) - 1.0) + 1.0
    return r1, fd * r + gd * v


def _orbit(rng, mu):
    a = rng.uniform(0.01, 0.07)
    e = rng.uniform(0.0, 0.3)
    pos, vel = E.kepler_to_cartesian(mu, a, e, rng.uniform(0, 0.05), *rng.uniform(0, 2 * np.pi, 3))
    return pos, vel


@pytest.mark.parametrize("seed", range(6))
def test_kepler_forward_matches_two_body(lib, seed):
    rng = np.random.default_rng(seed)
    mu = E.G * 0.08
    r, v = _orbit(rng, mu)
    for dt in (0.04, 0.5, -0.04):
        r1, v1 = np.zeros(3), np.zeros(3)
        X = lib.h_kepler_fwd(mu, dt, P(r), P(v), r1.ctypes.data_as(f64p), v1.ctypes.data_as(f64p))
        assert np.isfinite(X)
        rr, vv = two_body(mu, r, v, dt)
        assert np.abs(r1 - rr).max() <= 1e-12 * np.linalg.norm(rr)
        assert np.abs(v1 - vv).max() <= 1e-11 * np.linalg.norm(vv)


@pytest.mark.parametrize("seed", range(6))
def test_kepler_vjp_matches_finite_differences(lib, seed):
    rng = np.random.default_rng(100 + seed)
    mu = E.G * rng.uniform(0.08, 1.0)
    r, v = _orbit(rng, mu)
    dt = 0.04
    lr1, lv1 = rng.normal(size=3), rng.normal(size=3) * 10.0

    def fwd(x):
        r1, v1 = np.zeros(3), np.zeros(3)
        lib.h_kepler_fwd(mu, dt, P(x[:3]), P(x[3:]), r1.ctypes.data_as(f64p), v1.ctypes.data_as(f64p))
        return lr1 @ r1 + lv1 @ v1

    r1, v1 = np.zeros(3), np.zeros(3)
    X = lib.h_kepler_fwd(mu, dt, P(r), P(v), r1.ctypes.data_as(f64p), v1.ctypes.data_as(f64p))
    lr0, lv0 = np.zeros(3), np.zeros(3)
    lib.h_kepler_vjp(mu, dt, P(r), P(v), X, P(lr1), P(lv1), lr0.ctypes.data_as(f64p), lv0.ctypes.data_as(f64p))
    x0 = np.concatenate([r, v])
    got = np.concatenate([lr0, lv0])
    fd = np.zeros(6)
    for k in range(6):
        h = 1e-6 * (np.linalg.norm(r) if k < 3 else np.linalg.norm(v))
        xp, xm = x0.copy(), x0.copy()
        xp[k] += h
        xm[k] -= h
        fd[k] = (fwd(xp) - fwd(xm)) / (2 * h)
    scale = np.abs(fd).max()
    assert np.abs(got - fd).max() <= 1e-7 * scale, (got, fd)


def _system(seed=0):
    ens = E.workload_single(seed=seed)
    state, _, _ = oracle.run(ens, max_steps=7, init_physical=True)
    return state


def _planet_inputs(st, p):
    bf = st["body_f64"][0]
    h = int(st["sys_i64"][0, L.SI_HOST])
    r = bf[p, L.POS] - bf[h, L.POS]
    hv = bf[p, L.VEL] - bf[h, L.VEL]
    S = bf[p, L.ANG] / bf[p, L.BF_MOI]
    H = bf[h, L.ANG] / bf[h, L.BF_MOI]
    Pp = bf[p, L.SPIN]
    Q = bf[h, L.SPIN]
    inp = np.concatenate([r, hv, S, H, Pp, Q, [bf[p, L.BF_SIGMA], bf[h, L.BF_SIGMA], bf[p, L.BF_K2], bf[h, L.BF_K2]]])
    c = np.array([bf[p, L.BF_MASS], bf[h, L.BF_MASS], bf[p, L.BF_RADIUS], bf[h, L.BF_RADIUS], bf[p, L.BF_K2F],
                  bf[h, L.BF_K2F], bf[p, L.BF_MASS_G], bf[h, L.BF_MASS_G], bf[p, L.BF_MOI], bf[h, L.BF_MOI]])
    return inp, c


def test_effect_blocks_match_oracle_evaluation(lib):
    """Per-planet blocks, assembled (host: -sum (m_p/m_h) a_p and sum of the
    torques), reproduce the oracle's calculate_additional_effects."""
    st = _system()
    t = float(st["sys_f64"][0, L.SF_TIME])
    ref, _, _ = oracle.run(st, op=oracle.ADDITIONAL_EFFECTS, arg=2 | 4, t_arg=t)
    bf = st["body_f64"][0]
    n = int(st["sys_i64"][0, L.SI_N])
    h = int(st["sys_i64"][0, L.SI_HOST])
    acc = np.zeros((n, 3))
    dl = np.zeros((n, 3))
    for p in range(n):
        if p == h:
            continue
        inp, c = _planet_inputs(st, p)
        for which in range(3):
            out = np.zeros(9)
            lib.h_effects_fwd(which, P(inp), P(c), out.ctypes.data_as(f64p))
            acc[p] += out[0:3]
            dl[p] += out[3:6]
            acc[h] -= bf[p, L.BF_MASS] / bf[h, L.BF_MASS] * out[0:3]
            dl[h] += out[6:9]
    ra = ref["body_f64"][0][:n, L.BF_ADDAX:L.BF_ADDAZ + 1]
    rd = ref["body_f64"][0][:n, L.BF_DLX:L.BF_DLZ + 1]
    for b in range(n):
        assert np.abs(acc[b] - ra[b]).max() <= 1e-11 * np.abs(ra[b]).max(), (b, acc[b], ra[b])
        assert np.abs(dl[b] - rd[b]).max() <= 1e-11 * np.abs(rd[b]).max(), (b, dl[b], rd[b])


@pytest.mark.parametrize("which", [0, 1, 2])
def test_effect_block_vjp_matches_finite_differences(lib, which):
    st = _system(3)
    rng = np.random.default_rng(which)
    nin = 22 if which == 0 else 18
    for p in (1, 2, 3):
        inp, c = _planet_inputs(st, p)
        out0 = np.zeros(9)
        lib.h_effects_fwd(which, P(inp), P(c), out0.ctypes.data_as(f64p))
        # adjoints scaled so that every output group contributes comparably
        bout = rng.normal(size=9)
        for g in range(3):
            sc = np.abs(out0[3 * g:3 * g + 3]).max()
            bout[3 * g:3 * g + 3] /= sc if sc > 0 else 1.0
        bin_ = np.zeros(22)
        lib.h_effects_vjp(which, P(inp), P(c), P(bout), bin_.ctypes.data_as(f64p))

        def f(x):
            o = np.zeros(9)
            lib.h_effects_fwd(which, P(x), P(c), o.ctypes.data_as(f64p))
            return bout @ o

        groups = [slice(0, 3), slice(3, 6), slice(6, 9), slice(9, 12), slice(12, 15), slice(15, 18)]
        for k in range(nin):
            g = next((gg for gg in groups if gg.start <= k < gg.stop), None)
            scale = np.linalg.norm(inp[g]) if g is not None else abs(inp[k])
            hstep = 1e-6 * (scale if scale > 0 else 1.0)
            xp, xm = inp.copy(), inp.copy()
            xp[k] += hstep
            xm[k] -= hstep
            fd = (f(xp) - f(xm)) / (2 * hstep)
            # compare in units of the input scale (|d f / d ln x|)
            err = abs(bin_[k] - fd) * (scale if scale > 0 else 1.0)
            ref = max(abs(fd) * (scale if scale > 0 else 1.0), 1e-9)
            assert err <= 1e-5 * ref + 1e-12, (which, p, k, bin_[k], fd)


@pytest.mark.parametrize("seed", range(4))
def test_kepler_jvp_matches_finite_differences(lib, seed):
    rng = np.random.default_rng(200 + seed)
    mu = E.G * rng.uniform(0.08, 1.0)
    r, v = _orbit(rng, mu)
    dt = 0.05
    dr, dv = rng.normal(size=3) * np.linalg.norm(r), rng.normal(size=3) * np.linalg.norm(v)
    r1, v1 = np.zeros(3), np.zeros(3)
    X = lib.h_kepler_fwd(mu, dt, P(r), P(v), r1.ctypes.data_as(f64p), v1.ctypes.data_as(f64p))
    dr1, dv1 = np.zeros(3), np.zeros(3)
    lib.h_kepler_jvp(mu, dt, P(r), P(v), X, P(dr), P(dv), dr1.ctypes.data_as(f64p), dv1.ctypes.data_as(f64p))
    h = 1e-6
    outs = []
    for sg in (1.0, -1.0):
        a, b = np.zeros(3), np.zeros(3)
        lib.h_kepler_fwd(mu, dt, P(r + sg * h * dr), P(v + sg * h * dv), a.ctypes.data_as(f64p),
                         b.ctypes.data_as(f64p))
        outs.append(np.concatenate([a, b]))
    fd = (outs[0] - outs[1]) / (2 * h)
    got = np.concatenate([dr1, dv1])
    assert np.abs(got - fd).max() <= 1e-7 * np.abs(fd).max(), (got, fd)


@pytest.mark.parametrize("which", [0, 1, 2])
def test_effect_block_jvp_matches_vjp(lib, which):
    """<v, J u> from the tangent sweep equals <J^T v, u> from the reverse sweep."""
    st = _system(3)
    rng = np.random.default_rng(10 + which)
    for p in (1, 2, 3):
        inp, c = _planet_inputs(st, p)
        u = rng.normal(size=22) * np.abs(inp)
        vv = rng.normal(size=9)
        dout = np.zeros(9)
        lib.h_effects_jvp(which, P(inp), P(c), P(u), dout.ctypes.data_as(f64p))
        bin_ = np.zeros(22)
        lib.h_effects_vjp(which, P(inp), P(c), P(vv), bin_.ctypes.data_as(f64p))
        lhs, rhs = vv @ dout, bin_ @ u
        assert abs(lhs - rhs) <= 1e-10 * (np.abs(vv * dout).sum() + 1e-300), (which, p, lhs, rhs)
