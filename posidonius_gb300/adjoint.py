"""Gradients of WHFast trajectories: the adjoint behind ``torch.autograd``.

:class:`Adjoint` drives the C ABI's checkpointed reverse mode
(``posi_adjoint_*``): a forward run of a :class:`~posidonius_gb300.Batch` that
keeps its state every ``checkpoint_every`` steps, then a backward run that
re-integrates each chunk on the GPU, records its steps and sweeps them in
reverse with the hand-derived vector-Jacobian products of the step.

:class:`WHFastTrajectory` wraps it as a ``torch.autograd.Function``: initial
positions, velocities and spin angular momenta, plus every body's tidal
dissipation factor and Love number, in; the state after ``n_steps`` out.
PyTorch is the gradient binding only: the trajectory and its adjoint run in
the CUDA library; torch differentiates what the caller builds around it
(orbital elements -> Cartesian state, final state -> loss).

:func:`elements_to_state` and :func:`orbital_elements` are those torch-side
maps for star + planets systems (the reference's
``calculate_cartesian_coordinates`` / ``calculate_keplerian_orbital_elements``
in src/tools.rs, and the pseudo-synchronous spin of src/tools.rs:909-927),
and :func:`tidal_loss` is the objective of the differentiation workload: the
sum of squared final eccentricities, squared relative semi-major-axis drifts
and squared relative planetary spin-rate changes.

For one system of many bodies (:class:`~posidonius_gb300.ManyBody`) with a
few tidal parameters of interest, :func:`many_body_dissipation_gradient`
takes the same loss's derivatives in forward mode: the engine carries the
tangents of every body's state along each parameter direction
(``posi_large_iterate_tangent``), and the derivative of the loss is the
final-state gradient (torch) dotted with each tangent -- the same numbers a
reverse sweep yields, at the cost of one run with a few directions.
"""
import ctypes
import math

import numpy as np

from . import layout as L
from ._lib import check, lib

LAM_FIELDS = 12   # adjoint of (r, v, L, S) per body
GRAD_FIELDS = 2   # d/d dissipation factor, d/d Love number
FLAG_KEPLER = L.ADJ_KEPLER
FLAG_ZERO_INERTIA = L.ADJ_ZERO_INERTIA
FLAG_FROZEN = L.ADJ_FROZEN


class Adjoint:
    """Checkpointed reverse mode over a Batch (posi_adjoint_*)."""

    def __init__(self, batch, n_steps, checkpoint_every=100):
        st = ctypes.c_int(0)
        h = lib().posi_adjoint_create(batch._h, int(n_steps), int(checkpoint_every), ctypes.byref(st))
        if not h:
            check(st.value)
        self._h = ctypes.c_void_p(h)
        self.batch = batch
        self.n_steps = int(n_steps)

    def close(self):
        if getattr(self, "_h", None):
            lib().posi_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self):
        check(lib().posi_adjoint_forward(self._h))

    def backward(self, lam_final, lam_initial=None, grad=None):
        """lam_final: [n_sys, nmax, 12] (numpy, or a contiguous CUDA float64
        tensor); returns (lam_initial, grad) of the same kind.  Per-system
        flags (FLAG_* bits; gradients of a flagged system are not meaningful)
        are kept in ``self.flags``."""
        ns, nm = self.batch.n_sys, self.batch.nmax
        if isinstance(lam_final, np.ndarray):
            lam_final = np.ascontiguousarray(lam_final, dtype=np.float64).reshape(ns, nm, LAM_FIELDS)
            if lam_initial is None:
                lam_initial = np.zeros((ns, nm, LAM_FIELDS))
            if grad is None:
                grad = np.zeros((ns, nm, GRAD_FIELDS))
            ptrs = [a.ctypes.data for a in (lam_final, lam_initial, grad)]
        else:  # torch tensors on the batch's device
            import torch
            lam_final = lam_final.contiguous().to(torch.float64)
            if lam_initial is None:
                lam_initial = torch.zeros((ns, nm, LAM_FIELDS), dtype=torch.float64, device=lam_final.device)
            if grad is None:
                grad = torch.zeros((ns, nm, GRAD_FIELDS), dtype=torch.float64, device=lam_final.device)
            torch.cuda.synchronize(lam_final.device)
            ptrs = [t.data_ptr() for t in (lam_final, lam_initial, grad)]
        self.flags = np.zeros(ns, dtype=np.int32)
        check(lib().posi_adjoint_backward(self._h, ctypes.c_void_p(ptrs[0]), ctypes.c_void_p(ptrs[1]),
                                          ctypes.c_void_p(ptrs[2]), ctypes.c_void_p(self.flags.ctypes.data)))
        return lam_initial, grad

    def last_timing(self):
        """(forward_ms, backward_ms, record_ms, reverse_ms) of the last runs."""
        v = [ctypes.c_double() for _ in range(4)]
        check(lib().posi_adjoint_last_timing(self._h, *[ctypes.byref(x) for x in v]))
        return tuple(x.value for x in v)


def _torch():
    import torch
    return torch


class WHFastTrajectory:
    """``apply(r0, v0, L0, sigma, k2)`` -> ``(r, v, L)`` after n_steps.

    Shapes [n_sys, nmax, 3] and [n_sys, nmax]; float64.  The batch supplies
    everything else (masses, radii, effect flags, time step); spins start at
    L / I (the reference's initialize_physical_values)."""

    def __init__(self, batch, n_steps, checkpoint_every=100):
        self.batch = batch
        self.adjoint = Adjoint(batch, n_steps, checkpoint_every)
        self.base = batch.get_state()
        torch = _torch()

        engine = self

        class Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, r0, v0, L0, sigma, k2):
                final = engine.run(r0, v0, L0, sigma, k2)
                out = [torch.as_tensor(final["body_f64"][..., sl], dtype=torch.float64, device=r0.device)
                       for sl in (L.POS, L.VEL, L.ANG)]
                return tuple(out)

            @staticmethod
            def backward(ctx, gr, gv, gL):
                ns, nm = engine.batch.n_sys, engine.batch.nmax
                lam = torch.zeros((ns, nm, 12), dtype=torch.float64, device=gr.device)
                if gr is not None:
                    lam[..., 0:3] = gr
                if gv is not None:
                    lam[..., 3:6] = gv
                if gL is not None:
                    lam[..., 6:9] = gL
                lam_init, grad = engine.adjoint.backward(lam.contiguous())
                moi = torch.as_tensor(engine.base["body_f64"][..., L.BF_MOI], dtype=torch.float64, device=gr.device)
                inv = torch.where(moi != 0, 1.0 / torch.where(moi != 0, moi, torch.ones_like(moi)), torch.zeros_like(moi))
                # initial spins are L0 / I
                gL0 = lam_init[..., 6:9] + lam_init[..., 9:12] * inv[..., None]
                return lam_init[..., 0:3], lam_init[..., 3:6], gL0, grad[..., 0], grad[..., 1]

        self.Fn = Fn

    def run(self, r0, v0, L0, sigma, k2):
        st = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in self.base.items()}
        bf = st["body_f64"]
        bf[..., L.POS] = r0.detach().cpu().numpy()
        bf[..., L.VEL] = v0.detach().cpu().numpy()
        Lh = L0.detach().cpu().numpy()
        bf[..., L.ANG] = Lh
        moi = bf[..., L.BF_MOI]
        safe = np.where(moi != 0, moi, 1.0)
        bf[..., L.SPIN] = np.where((moi != 0)[..., None], Lh / safe[..., None], 0.0)
        bf[..., L.BF_NSV2] = np.sum(bf[..., L.SPIN] ** 2, axis=-1)
        bf[..., L.BF_SIGMA] = sigma.detach().cpu().numpy()
        bf[..., L.BF_K2] = k2.detach().cpu().numpy()
        self.batch.set_state(st)
        self.adjoint.forward()
        return self.batch.get_state()

    def __call__(self, r0, v0, L0, sigma, k2):
        return self.Fn.apply(r0, v0, L0, sigma, k2)


# ---------------------------------------------------------------------------
# torch-side maps of the differentiation workload (star + planets systems)
# ---------------------------------------------------------------------------
def kepler_to_cartesian(gm, a, e, inc, omega, node, mean_anomaly, iters=40):
    """Elliptic orbital elements -> position, velocity relative to the central
    body (Kepler's equation by Newton's method); torch, broadcasting."""
    torch = _torch()
    E = mean_anomaly + e * torch.sin(mean_anomaly)
    for _ in range(iters):
        E = E - (E - e * torch.sin(E) - mean_anomaly) / (1.0 - e * torch.cos(E))
    cE, sE = torch.cos(E), torch.sin(E)
    b = a * torch.sqrt(1.0 - e * e)
    xo, yo = a * (cE - e), b * sE
    n = torch.sqrt(gm / a ** 3)
    edot = n / (1.0 - e * cE)
    vxo, vyo = -a * sE * edot, b * cE * edot
    co, so = torch.cos(omega), torch.sin(omega)
    cn, sn = torch.cos(node), torch.sin(node)
    ci, si = torch.cos(inc), torch.sin(inc)
    r11, r12 = cn * co - sn * so * ci, -cn * so - sn * co * ci
    r21, r22 = sn * co + cn * so * ci, -sn * so + cn * co * ci
    r31, r32 = so * si, co * si
    pos = torch.stack([r11 * xo + r12 * yo, r21 * xo + r22 * yo, r31 * xo + r32 * yo], dim=-1)
    vel = torch.stack([r11 * vxo + r12 * vyo, r21 * vxo + r22 * vyo, r31 * vxo + r32 * vyo], dim=-1)
    return pos, vel


def pseudo_synchronous_spin(a, e, inc, node, star_mass, planet_mass):
    """src/tools.rs:909-927: pseudo-synchronous rotation, zero obliquity."""
    from .ensemble import G_SI, M_SUN, AU, HOUR
    torch = _torch()
    alpha = ((1.0 + 7.5 * e ** 2 + 45.0 / 8.0 * e ** 4 + 5.0 / 16.0 * e ** 6) / (1.0 + 3.0 * e ** 2 + 3.0 / 8.0 * e ** 4)
             / (1.0 - e ** 2) ** 1.5)
    w = alpha * torch.sqrt(G_SI * M_SUN * (star_mass + planet_mass)) * (a * AU) ** (-1.5) * HOUR * 24.0
    return torch.stack([w * torch.sin(inc) * torch.sin(node), -w * torch.sin(inc) * torch.cos(node),
                        w * torch.cos(inc)], dim=-1)


def elements_to_state(elements, masses, moi, star_spin):
    """elements [S, P, 6] (a, e, i, argument of pericentre, node, mean
    anomaly) of P planets around body 0 -> barycentric r, v [S, P+1, 3] and
    spin angular momenta L [S, P+1, 3]; masses [S, P+1], moi [S, P+1],
    star_spin [S, 3] (fixed)."""
    from .ensemble import G
    torch = _torch()
    a, e, inc, om, no, M = elements.unbind(-1)
    ms, mp = masses[:, :1], masses[:, 1:]
    pos, vel = kepler_to_cartesian(G * (ms + mp), a, e, inc, om, no, M)
    zeros = torch.zeros_like(pos[:, :1])
    hpos = torch.cat([zeros, pos], dim=1)
    hvel = torch.cat([zeros, vel], dim=1)
    mt = masses.sum(dim=1, keepdim=True)
    cmp = (masses[..., None] * hpos).sum(dim=1, keepdim=True) / mt[..., None]
    cmv = (masses[..., None] * hvel).sum(dim=1, keepdim=True) / mt[..., None]
    spin_p = pseudo_synchronous_spin(a, e, inc, no, ms, mp)
    spin = torch.cat([star_spin[:, None, :], spin_p], dim=1)
    return hpos - cmp, hvel - cmv, moi[..., None] * spin


def orbital_elements(r, v, masses):
    """Semi-major axis and eccentricity of every planet relative to body 0."""
    from .ensemble import G
    torch = _torch()
    rr = r[:, 1:] - r[:, :1]
    vv = v[:, 1:] - v[:, :1]
    mu = G * (masses[:, :1] + masses[:, 1:])
    d = torch.linalg.norm(rr, dim=-1)
    v2 = (vv * vv).sum(-1)
    a = 1.0 / (2.0 / d - v2 / mu)
    h = torch.linalg.cross(rr, vv)
    evec = torch.linalg.cross(vv, h) / mu[..., None] - rr / d[..., None]
    e = torch.linalg.norm(evec, dim=-1)
    return a, e


def tidal_loss(r, v, Lspin, masses, moi, a0, spin0):
    """Per-system loss: sum_p e_p^2 + ((a_p - a0_p) / a0_p)^2 +
    ((|Omega_p| - |Omega0_p|) / |Omega0_p|)^2."""
    torch = _torch()
    a, e = orbital_elements(r, v, masses)
    w = torch.linalg.norm(Lspin[:, 1:], dim=-1) / moi[:, 1:]
    return (e ** 2 + ((a - a0) / a0) ** 2 + ((w - spin0) / spin0) ** 2).sum(dim=1)


def gradient_workload(n_systems=1024, seed=None, dt=0.08):
    """Systems of the differentiation workload: the 0.08 Msun star + 3 planets
    of the single-system workload (elements drawn the same way), returned as
    (case ensemble, elements [S, 3, 6], masses [S, 4], moi [S, 4],
    star_spin [S, 3])."""
    from . import ensemble as E
    rng = np.random.default_rng(E.SEED_BASE + E.WORKLOAD_IDS["gradient"] if seed is None else seed)
    cases, els, ms, mois, sspin = [], [], [], [], []
    for _ in range(n_systems):
        star = E._star()
        masses = np.exp(rng.uniform(np.log(0.3), np.log(3.0), size=3)) * E.M_EARTH
        a = np.sort(rng.uniform(0.01, 0.05, size=3))
        bodies, el = [star], []
        for k in range(3):
            b = E._planet(rng, star.mass, a[k], mass=masses[k])
            bodies.append(b)
        # recover the drawn elements from the generator's relative state
        for b in bodies[1:]:
            el.append(_elements_of(E.G * (star.mass + b.mass), b.pos, b.vel))
        case = E.make_system(bodies, dt=dt)
        cases.append(case)
        els.append(el)
        ms.append([b.mass for b in bodies])
        mois.append(case["body_f64"][:, L.BF_MOI])
        sspin.append(star.spin)
    return (E.stack_systems(cases), np.array(els), np.array(ms), np.array(mois), np.array(sspin))


def _elements_of(mu, r, v):
    """(a, e, i, argument of pericentre, node, mean anomaly) of a bound orbit."""
    r, v = np.asarray(r, float), np.asarray(v, float)
    d = np.linalg.norm(r)
    h = np.cross(r, v)
    inc = math.acos(h[2] / np.linalg.norm(h))
    node = math.atan2(h[0], -h[1])
    evec = np.cross(v, h) / mu - r / d
    e = np.linalg.norm(evec)
    a = 1.0 / (2.0 / d - v @ v / mu)
    nvec = np.array([math.cos(node), math.sin(node), 0.0])
    # argument of pericentre and true anomaly in the orbital plane
    hz = h / np.linalg.norm(h)
    def ang(x, y):
        return math.atan2(np.cross(x, y) @ hz, x @ y)
    om = ang(nvec, evec)
    f = ang(evec, r)
    E_ = 2.0 * math.atan2(math.sqrt(1 - e) * math.sin(f / 2), math.sqrt(1 + e) * math.cos(f / 2))
    M = E_ - e * math.sin(E_)
    return [a, e, inc, om, node, M]


def _state_arrays(elements, sigma, k2, masses, moi, star_spin):
    """numpy initial state (r, v, L, S) of the workload's systems."""
    torch = _torch()
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64)
    with torch.no_grad():
        r0, v0, L0 = elements_to_state(t(elements), t(masses), t(moi), t(star_spin))
    r0, v0, L0 = r0.numpy(), v0.numpy(), L0.numpy()
    moi = np.asarray(moi)
    S0 = L0 / np.where(moi != 0, moi, 1.0)[..., None]
    return r0, v0, L0, S0


def initial_ensemble(ens, elements, sigma, k2, masses, moi, star_spin):
    """Copy of the workload ensemble with the initial state built from the
    given parameters (one parameter set per system)."""
    r0, v0, L0, S0 = _state_arrays(elements, sigma, k2, masses, moi, star_spin)
    out = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in ens.items()}
    n = r0.shape[1]
    bf = out["body_f64"]
    bf[:, :n, L.POS] = r0
    bf[:, :n, L.VEL] = v0
    bf[:, :n, L.ANG] = L0
    bf[:, :n, L.SPIN] = S0
    bf[:, :n, L.BF_NSV2] = np.sum(S0 ** 2, axis=-1)
    bf[:, :n, L.BF_SIGMA] = sigma
    bf[:, :n, L.BF_K2] = k2
    return out


def loss_from_final(final_body_f64, elements, masses, moi):
    """Per-system loss of final states [S, n, BF_COUNT] (numpy)."""
    torch = _torch()
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64)
    n = np.asarray(masses).shape[1]
    fin = final_body_f64[:, :n]
    with torch.no_grad():
        el = t(elements)
        a0 = el[..., 0]
        spin0 = torch.linalg.norm(pseudo_synchronous_spin(el[..., 0], el[..., 1], el[..., 2], el[..., 4],
                                                          t(masses)[:, :1], t(masses)[:, 1:]), dim=-1)
        out = tidal_loss(t(fin[..., L.POS]), t(fin[..., L.VEL]), t(fin[..., L.ANG]), t(masses), t(moi), a0, spin0)
    return out.numpy()


def gpu_runner(mode=None):
    """Runner for loss_of_parameters: integrates an ensemble on the GPU and
    returns the final body_f64."""
    def run(ens, n_steps):
        import posidonius_gb300 as pg
        batch = pg.Batch(ens, mode=pg.FAST if mode is None else mode)
        batch.initialize_physical_values()
        batch.iterate(n_steps, min(n_steps, 1000))
        fin = batch.get_state()["body_f64"]
        batch.close()
        return fin
    return run


def loss_of_parameters(ens, elements, sigma, k2, masses, moi, star_spin, n_steps, mode=None, runner=None):
    """Per-system loss after n_steps for parameter sets given per system (no
    gradient): one batched run of all of them (GPU unless a runner is given)."""
    run = runner or gpu_runner(mode)
    e0 = initial_ensemble(ens, elements, sigma, k2, masses, moi, star_spin)
    return loss_from_final(run(e0, n_steps), elements, masses, moi)


def finite_difference_gradient(ens, elements, sigma, k2, masses, moi, star_spin, n_steps, rel_step=1e-6,
                               rel_step_tidal=None, mode=None, runner=None):
    """Central finite differences of the per-system loss with respect to
    (sigma [nb], k2 [nb], elements [np, 6]) of every system, all perturbed
    copies integrated in one batch.  Returns (d/dsigma, d/dk2, d/delements).
    The step is rel_step x |parameter| (angles: x max(|angle|, 1), e:
    x max(e, 0.05)); sigma and k2 use rel_step_tidal when given (the loss is
    nearly linear in them and their effect over a short run is close to the
    loss's rounding level, so a larger relative step resolves it)."""
    rel_tidal = rel_step if rel_step_tidal is None else rel_step_tidal
    elements = np.asarray(elements, float)
    sigma, k2 = np.asarray(sigma, float), np.asarray(k2, float)
    S, nb = sigma.shape
    npl = elements.shape[1]
    params = [("sigma", b, None) for b in range(nb)] + [("k2", b, None) for b in range(nb)] + \
             [("el", p, c) for p in range(npl) for c in range(6)]
    P = len(params)
    reps = 2 * P
    idx = np.repeat(np.arange(S), reps)
    E2 = {k: (v[idx] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    E2["n_sys"] = S * reps
    el2 = np.repeat(elements, reps, axis=0)
    sg2 = np.repeat(sigma, reps, axis=0)
    k22 = np.repeat(k2, reps, axis=0)
    steps = np.zeros((S, P))
    for s in range(S):
        for j, (kind, b, c) in enumerate(params):
            for sgn, off in ((1.0, 0), (-1.0, 1)):
                row = s * reps + 2 * j + off
                if kind == "sigma":
                    h = rel_tidal * abs(sigma[s, b])
                    sg2[row, b] += sgn * h
                elif kind == "k2":
                    h = rel_tidal * abs(k2[s, b])
                    k22[row, b] += sgn * h
                else:
                    x = elements[s, b, c]
                    h = rel_step * (abs(x) if c == 0 else max(abs(x), 1.0 if c >= 2 else 0.05))
                    el2[row, b, c] += sgn * h
                steps[s, j] = h
    loss = loss_of_parameters(E2, el2, sg2, k22, np.repeat(masses, reps, axis=0), np.repeat(moi, reps, axis=0),
                              np.repeat(star_spin, reps, axis=0), n_steps, mode=mode,
                              runner=runner).reshape(S, P, 2)
    g = (loss[..., 0] - loss[..., 1]) / (2.0 * steps)
    g = np.where(steps > 0, g, 0.0)
    return g[:, :nb], g[:, nb:2 * nb], g[:, 2 * nb:].reshape(S, npl, 6)


def oracle_dual_gradient(ens, elements, sigma, k2, masses, moi, star_spin, n_steps, nthreads=None):
    """The same per-system loss gradient with respect to (sigma, k2,
    elements) from the oracle's dual-number build: the initial state's
    derivatives with respect to the elements (torch Jacobian of
    elements_to_state) and unit rates of every body's sigma and k2 seed
    forward-mode derivatives through n_steps of the oracle's reference-order
    arithmetic; the loss gradient at the final state (torch) then contracts
    them.  Exact derivatives of the computed map, no step size: the
    reference the adjoint is checked against.  Returns (loss [S], d/dsigma
    [S, nb], d/dk2 [S, nb], d/delements [S, np, 6])."""
    import os

    import oracle
    torch = _torch()
    elements = np.asarray(elements, float)
    masses, moi = np.asarray(masses, float), np.asarray(moi, float)
    S, npl = elements.shape[0], elements.shape[1]
    nb = npl + 1
    nd = oracle.dual_directions()
    if 2 * nb + 6 * npl > nd:
        raise ValueError(f"{2 * nb + 6 * npl} directions needed, the dual build carries {nd}")
    e0 = initial_ensemble(ens, elements, sigma, k2, masses, moi, star_spin)
    nmax = int(e0["nmax"])
    seed = np.zeros((S, nmax, L.BF_COUNT, nd))
    for b in range(nb):
        seed[:, b, L.BF_SIGMA, b] = 1.0
        seed[:, b, L.BF_K2, nb + b] = 1.0
    t = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float64)
    for s in range(S):
        ms, mi, ss = t(masses[s:s + 1]), t(moi[s:s + 1]), t(star_spin[s:s + 1])

        def state_of(el):
            r0, v0, L0 = elements_to_state(el[None], ms, mi, ss)
            return torch.cat([r0[0], v0[0], L0[0]], dim=-1)   # [nb, 9]

        J = torch.autograd.functional.jacobian(state_of, t(elements[s])).numpy()  # [nb, 9, npl, 6]
        J = J.reshape(nb, 9, npl * 6)
        cols = slice(2 * nb, 2 * nb + 6 * npl)
        seed[s, :nb, L.POS, cols] = J[:, 0:3]
        seed[s, :nb, L.VEL, cols] = J[:, 3:6]
        seed[s, :nb, L.ANG, cols] = J[:, 6:9]
        inv = np.where(moi[s] != 0, 1.0 / np.where(moi[s] != 0, moi[s], 1.0), 0.0)
        seed[s, :nb, L.SPIN, cols] = J[:, 6:9] * inv[:, None, None]
    res = oracle.run_dual(e0, seed, n_steps, init_physical=True, nthreads=nthreads or os.cpu_count() or 1)
    fin, T = res[0]["body_f64"][:, :nb], res[3][:, :nb]
    r, v, Ls = (t(fin[..., sl]).requires_grad_(True) for sl in (L.POS, L.VEL, L.ANG))
    el = t(elements).requires_grad_(True)
    a0 = el[..., 0]
    spin0 = torch.linalg.norm(pseudo_synchronous_spin(el[..., 0], el[..., 1], el[..., 2], el[..., 4],
                                                      t(masses)[:, :1], t(masses)[:, 1:]), dim=-1)
    loss = tidal_loss(r, v, Ls, t(masses), t(moi), a0, spin0)
    loss.sum().backward()
    g = np.einsum("sbq,sbqk->sk", r.grad.numpy(), T[:, :, L.POS, :]) + \
        np.einsum("sbq,sbqk->sk", v.grad.numpy(), T[:, :, L.VEL, :]) + \
        np.einsum("sbq,sbqk->sk", Ls.grad.numpy(), T[:, :, L.ANG, :])
    g_el = g[:, 2 * nb:2 * nb + 6 * npl].reshape(S, npl, 6) + el.grad.numpy()
    return loss.detach().numpy(), g[:, :nb], g[:, nb:2 * nb], g_el


def adjoint_gradient(ens, elements, sigma, k2, masses, moi, star_spin, n_steps, checkpoint_every=100,
                     device="cuda", mode=None):
    """Per-system loss and its gradient with respect to (sigma, k2, elements)
    by the adjoint (torch autograd around WHFastTrajectory).  Returns
    (loss [S], d/dsigma, d/dk2, d/delements, (forward_ms, backward_ms),
    flags [S]) -- gradients of systems with flags != 0 are not meaningful."""
    import posidonius_gb300 as pg
    torch = _torch()
    batch = pg.Batch(ens, mode=pg.FAST if mode is None else mode)
    batch.initialize_physical_values()
    traj = WHFastTrajectory(batch, n_steps, checkpoint_every)
    t = lambda x, g=False: torch.tensor(np.asarray(x), dtype=torch.float64, device=device, requires_grad=g)
    el = t(elements, True)
    sg = t(sigma, True)
    kk = t(k2, True)
    ms, mi, ss = t(masses), t(moi), t(star_spin)
    r0, v0, L0 = elements_to_state(el, ms, mi, ss)
    n = r0.shape[1]
    nm = batch.nmax
    if nm > n:  # pad to the batch's body slots
        pad = lambda x: torch.cat([x, torch.zeros(x.shape[0], nm - n, *x.shape[2:], dtype=x.dtype, device=x.device)],
                                  dim=1)
        r0, v0, L0, sgp, kkp = pad(r0), pad(v0), pad(L0), pad(sg), pad(kk)
    else:
        sgp, kkp = sg, kk
    r, v, Ls = traj(r0, v0, L0, sgp, kkp)
    r, v, Ls = r[:, :n], v[:, :n], Ls[:, :n]
    a0 = el[..., 0]
    spin0 = torch.linalg.norm(pseudo_synchronous_spin(el[..., 0], el[..., 1], el[..., 2], el[..., 4], ms[:, :1],
                                                      ms[:, 1:]), dim=-1)
    loss = tidal_loss(r, v, Ls, ms, mi, a0, spin0)
    loss.sum().backward()
    timing = traj.adjoint.last_timing()
    out = (loss.detach().cpu().numpy(), sg.grad.cpu().numpy(), kk.grad.cpu().numpy(), el.grad.cpu().numpy(), timing,
           traj.adjoint.flags.copy())
    traj.adjoint.close()
    batch.close()
    return out


def tangent_loss_gradient(final_body_f64, tangents, host, planets, a0, spin0):
    """Loss of :func:`tidal_loss` over ``planets`` (relative to ``host``) of a
    final many-body state [n, BF_COUNT], and its derivative along each
    tangent direction (tangents [D, n, 12]: r, v, L, S per body):
    d loss = sum over bodies of (d loss / d r, v, L) . tangent."""
    torch = _torch()
    idx = [int(host)] + [int(p) for p in planets]
    fin = np.asarray(final_body_f64)[idx]
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64)
    r = t(fin[:, L.POS])[None].requires_grad_(True)
    v = t(fin[:, L.VEL])[None].requires_grad_(True)
    Ls = t(fin[:, L.ANG])[None].requires_grad_(True)
    loss = tidal_loss(r, v, Ls, t(fin[:, L.BF_MASS])[None], t(fin[:, L.BF_MOI])[None], t(a0)[None],
                      t(spin0)[None]).sum()
    gr, gv, gL = torch.autograd.grad(loss, (r, v, Ls))
    tan = t(np.asarray(tangents)[:, idx])
    grad = (gr[0] * tan[..., 0:3]).sum((1, 2)) + (gv[0] * tan[..., 3:6]).sum((1, 2)) + \
        (gL[0] * tan[..., 6:9]).sum((1, 2))
    return float(loss.detach()), grad.numpy()


def many_body_dissipation_gradient(case, n_steps, planets=(1, 2)):
    """d loss / d (dissipation factor) of each of ``planets`` after ``n_steps``
    of the many-body engine, the loss :func:`tidal_loss` of those planets
    (initial semi-major axes and spin rates as the targets).  Returns
    (loss, gradient [len(planets)], engine milliseconds of the tangent run,
    final state)."""
    from . import ManyBody
    torch = _torch()
    mb = ManyBody(case)
    try:
        mb.initialize_physical_values()
        init = mb.get_state()
        host = int(init["sys_i64"][L.SI_HOST])
        idx = [host] + list(planets)
        b0 = init["body_f64"][idx]
        t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64)
        with torch.no_grad():
            a0, _ = orbital_elements(t(b0[:, L.POS])[None], t(b0[:, L.VEL])[None], t(b0[:, L.BF_MASS])[None])
        spin0 = np.linalg.norm(b0[1:, L.ANG], axis=-1) / b0[1:, L.BF_MOI]
        _, tan = mb.iterate_tangent(n_steps, [(int(p), L.SEED_SIGMA) for p in planets])
        ms = mb.last_timing()
        final = mb.get_state()
    finally:
        mb.close()
    loss, grad = tangent_loss_gradient(final["body_f64"], tan, host, planets, a0[0].numpy(), spin0)
    return loss, grad, ms, final


def main(argv=None):
    """``python -m posidonius_gb300.adjoint --systems S --steps K --every C``:
    one gradient of the differentiation workload's loss; prints the forward
    and backward times (CUDA events) as JSON."""
    import argparse
    import json
    p = argparse.ArgumentParser(description=main.__doc__)
    p.add_argument("--systems", type=int, default=1024)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--every", type=int, default=100)
    p.add_argument("--seed", type=int, default=1)
    a = p.parse_args(argv)
    ens, el, ms, moi, ss = gradient_workload(a.systems, seed=a.seed)
    sig = ens["body_f64"][:, :, L.BF_SIGMA].copy()
    k2 = ens["body_f64"][:, :, L.BF_K2].copy()
    loss, g_sig, g_k2, g_el, tm, flags = adjoint_gradient(ens, el, sig, k2, ms, moi, ss, a.steps, a.every)
    print(json.dumps({"systems": a.systems, "steps": a.steps, "every": a.every, "forward_ms": tm[0],
                      "backward_ms": tm[1], "record_ms": tm[2], "reverse_ms": tm[3],
                      "systems_flagged": int((flags != 0).sum())}))


if __name__ == "__main__":
    main()
