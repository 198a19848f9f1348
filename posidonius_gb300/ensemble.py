"""Synthetic planetary-system ensembles in the flat layout.

Builds seeded systems the way a Posidonius case script does
(``cases/trappist1.py`` of the reference is the template): a constant-time-lag
tidal host with oblate rotational flattening and Kidder (1995) general
relativity, planets on Keplerian orbits given by orbital elements,
pseudo-synchronous planetary spins (``src/tools.rs:909-927``), masses turned
into ``mass_g = mass * K2`` and barycentric coordinates obtained with the
reference's pairwise centre-of-mass accumulation
(``src/particles/universe.rs:663-697``).

Workloads (seed = 20261203 + workload id):

* ``single``  -- 0.08 Msun star + 3 planets, a in [0.01, 0.05] AU;
* ``ensemble8`` -- star + 7 planets, a in [0.01, 0.07] AU with at least 8
  mutual Hill radii between neighbours;
* ``uneven`` -- 2..10 bodies per system, 20 % circumbinary binaries, each of
  tides / flattening / GR on with probability 0.7;
* ``large`` -- one system: a 1 Msun star, 2 tidally active planets (1-10
  M_earth, 0.02-0.05 AU) and n_small massive bodies (1e-3 - 1e-1 M_earth,
  a in 0.1-1 AU, e <= 0.1, i <= 2 deg), democratic heliocentric, dt = 0.1 d.

Dissipation factors follow the reference's own cgs conversion (x 3.845764e64,
``tests/common/stars.rs:183``): star 2.006e-60 -> 2.006*3.845764e4, planet
2.006e-55*Qscale -> 2.006*3.845764e9*Qscale.
"""
import numpy as np

from . import layout as L

# src/constants.rs
M_SUN = 1.9818e30
G_SI = 6.67428e-11
AU = 1.49597870700e11
DAY = 24.0 * 3600.0
HOUR = 3600.0
G = G_SI / (AU * AU * AU) * M_SUN * (DAY * DAY)
K2 = G
M_EARTH = 1.0 / 332946.050895
R_SUN = 6.957e8 / AU
R_EARTH = 6.3781e6 / AU
TWO_PI = 2.0 * np.pi
DEG2RAD = np.pi / 180.0

SEED_BASE = 20261203
WORKLOAD_IDS = {"single": 0, "ensemble8": 1, "uneven": 2, "gradient": 3, "large": 4}


def kepler_to_cartesian(gm, a, e, inc, omega, node, mean_anomaly):
    """Position and velocity relative to the central body for an elliptic orbit
    (Kepler's equation solved by Newton's method)."""
    E = mean_anomaly + e * np.sin(mean_anomaly)
    for _ in range(50):
        dE = (E - e * np.sin(E) - mean_anomaly) / (1.0 - e * np.cos(E))
        E = E - dE
        if abs(dE) < 1e-15:
            break
    cE, sE = np.cos(E), np.sin(E)
    b = a * np.sqrt(1.0 - e * e)
    xo, yo = a * (cE - e), b * sE
    n = np.sqrt(gm / a**3)
    edot = n / (1.0 - e * cE)
    vxo, vyo = -a * sE * edot, b * cE * edot
    co, so = np.cos(omega), np.sin(omega)
    cn, sn = np.cos(node), np.sin(node)
    ci, si = np.cos(inc), np.sin(inc)
    r11, r12 = cn * co - sn * so * ci, -cn * so - sn * co * ci
    r21, r22 = sn * co + cn * so * ci, -sn * so + cn * co * ci
    r31, r32 = so * si, co * si
    pos = np.array([r11 * xo + r12 * yo, r21 * xo + r22 * yo, r31 * xo + r32 * yo])
    vel = np.array([r11 * vxo + r12 * vyo, r21 * vxo + r22 * vyo, r31 * vxo + r32 * vyo])
    return pos, vel


def pseudo_synchronization_period(a, e, star_mass, planet_mass):
    """src/tools.rs:909-917 (days)."""
    alpha = ((1.0 + 15.0 / 2.0 * e**2 + 45.0 / 8.0 * e**4 + 5.0 / 16.0 * e**6) / (1.0 + 3.0 * e**2 + 3.0 / 8.0 * e**4)
             / (1.0 - e**2) ** 1.5)
    pseudo_rot = alpha * np.sqrt(G_SI * M_SUN * (star_mass + planet_mass))
    angular_frequency = pseudo_rot * (a * AU) ** (-1.5) * HOUR * 24.0
    return TWO_PI / angular_frequency


def spin_vector(angular_frequency, inclination, obliquity, node):
    """src/tools.rs:919-927."""
    return np.array([angular_frequency * np.sin(obliquity + inclination) * np.sin(node),
                     -angular_frequency * np.sin(obliquity + inclination) * np.cos(node),
                     angular_frequency * np.cos(obliquity + inclination)])


class Body:
    def __init__(self, mass, radius, rg2, pos, vel, spin, tides=None, flat=None, gr=L.EFFECT_DISABLED):
        self.mass, self.radius, self.rg2 = float(mass), float(radius), float(rg2)
        self.pos, self.vel, self.spin = np.asarray(pos, float), np.asarray(vel, float), np.asarray(spin, float)
        self.tides = tides    # (kind, sigma, k2) or None
        self.flat = flat      # (kind, k2f) or None
        self.gr = gr


def make_system(bodies, dt=0.08, coords=L.JACOBI, tides=True, flat=True, gr=True, time_limit=1e30,
                hist_period=1e30, rec_period=1e30):
    """Flat single-system dict (Universe::new + WHFast::new semantics) from
    heliocentric bodies; body 0 must be the most massive."""
    n = len(bodies)
    si = np.zeros(L.SI_COUNT, np.int64)
    sf = np.zeros(L.SF_COUNT, np.float64)
    bi = np.zeros((n, L.BI_COUNT), np.int64)
    bf = np.zeros((n, L.BF_COUNT), np.float64)
    masses = np.array([b.mass for b in bodies])
    host = int(np.argmax(masses))
    si[L.SI_N] = n
    si[L.SI_HOST] = host
    si[L.SI_COORDS] = coords
    has_central = {k: any((getattr(b, k) or (0,))[0] == L.EFFECT_CENTRAL if k != "gr" else b.gr == L.EFFECT_CENTRAL
                          for b in bodies) for k in ("tides", "flat", "gr")}
    si[L.SI_TIDES] = int(tides and has_central["tides"])
    si[L.SI_FLAT] = int(flat and has_central["flat"])
    si[L.SI_GR] = int(gr and has_central["gr"])
    si[L.SI_EVOLUTION] = 0
    sf[L.SF_DT] = dt
    sf[L.SF_HALF_DT] = 0.5 * dt
    sf[L.SF_TIME_LIMIT] = time_limit
    sf[L.SF_LAST_HIST] = -1.0
    sf[L.SF_HIST_PERIOD] = hist_period
    sf[L.SF_LAST_REC] = -1.0
    sf[L.SF_REC_PERIOD] = rec_period
    # centre of mass by the reference's pairwise accumulation (universe.rs:663-697)
    cmp, cmv, cmm = np.zeros(3), np.zeros(3), 0.0
    for b in bodies:
        cmp = cmp * cmm + b.pos * b.mass
        cmv = cmv * cmm + b.vel * b.mass
        new = cmm + b.mass
        if new > 0.0:
            cmp = cmp / new
            cmv = cmv / new
        cmm = new
    for k, b in enumerate(bodies):
        F = bf[k]
        F[L.BF_MASS] = b.mass
        F[L.BF_MASS_G] = b.mass * K2
        F[L.BF_RADIUS] = b.radius
        F[L.BF_RG2] = b.rg2
        moi = b.mass * b.rg2 * b.radius**2
        F[L.BF_MOI] = moi
        F[L.POS] = b.pos - cmp
        F[L.VEL] = b.vel - cmv
        F[L.SPIN] = b.spin
        F[L.BF_NSV2] = float(b.spin @ b.spin)
        F[L.ANG] = moi * b.spin
        if b.tides is not None:
            bi[k, L.BI_TIDES_KIND] = b.tides[0]
            F[L.BF_SIGMA] = b.tides[1]
            F[L.BF_K2] = b.tides[2]
        if b.flat is not None:
            bi[k, L.BI_FLAT_KIND] = b.flat[0]
            F[L.BF_K2F] = b.flat[1]
        bi[k, L.BI_GR_KIND] = b.gr
    return {"sys_i64": si, "sys_f64": sf, "body_i64": bi, "body_f64": bf, "tables": np.zeros(1),
            "roche": np.zeros((n, n)), "n": n}


def stack_systems(cases, nmax=None):
    """Stack single-system dicts into one padded ensemble of nmax bodies."""
    nmax = int(nmax or max(c["n"] for c in cases))
    ns = len(cases)
    ens = {
        "sys_i64": np.zeros((ns, L.SI_COUNT), np.int64),
        "sys_f64": np.zeros((ns, L.SF_COUNT), np.float64),
        "body_i64": np.zeros((ns, nmax, L.BI_COUNT), np.int64),
        "body_f64": np.zeros((ns, nmax, L.BF_COUNT), np.float64),
        "roche": np.zeros((ns, nmax, nmax), np.float64),
        "nmax": nmax, "n_sys": ns,
    }
    tabs, off = [], 0
    for k, c in enumerate(cases):
        n = c["n"]
        ens["sys_i64"][k] = c["sys_i64"]
        ens["sys_f64"][k] = c["sys_f64"]
        ens["body_i64"][k, :n] = c["body_i64"]
        ens["body_f64"][k, :n] = c["body_f64"]
        ens["roche"][k, :n, :n] = c["roche"]
        ev = ens["body_i64"][k, :n, L.BI_EVO_LEN] > 0
        ens["body_i64"][k, :n, L.BI_EVO_OFFSET] = np.where(ev, ens["body_i64"][k, :n, L.BI_EVO_OFFSET] + off, 0)
        tabs.append(np.asarray(c["tables"], np.float64))
        off += len(c["tables"])
    ens["tables"] = np.concatenate(tabs)
    return ens


def _star(mass=0.08, radius_factor=0.117, rg2=0.2, period_days=3.3, k2=0.307):
    sigma = 2.006 * 3.845764e4
    spin = np.array([0.0, 0.0, TWO_PI / period_days])
    return Body(mass, radius_factor * R_SUN, rg2, np.zeros(3), np.zeros(3), spin,
                tides=(L.EFFECT_CENTRAL, sigma, k2), flat=(L.EFFECT_CENTRAL, k2), gr=L.EFFECT_CENTRAL)


def _planet(rng, star_mass, a, host_pos=None, host_vel=None, e_max=0.05, i_max_deg=1.0, mass=None):
    if mass is None:
        mass = np.exp(rng.uniform(np.log(0.3), np.log(3.0))) * M_EARTH
    m_earth = mass / M_EARTH
    radius = m_earth**0.27 * R_EARTH
    qscale = np.exp(rng.uniform(np.log(0.1), np.log(10.0)))
    sigma = 2.006 * 3.845764e9 * qscale
    e = rng.uniform(0.0, e_max)
    inc = rng.uniform(0.0, i_max_deg) * DEG2RAD
    omega, node, mean_anom = rng.uniform(0.0, TWO_PI, size=3)
    gm = G * (star_mass + mass)
    pos, vel = kepler_to_cartesian(gm, a, e, inc, omega, node, mean_anom)
    if host_pos is not None:
        pos, vel = pos + host_pos, vel + host_vel
    period = pseudo_synchronization_period(a, e, star_mass, mass)
    spin = spin_vector(TWO_PI / period, inc, 0.0, node)
    return Body(mass, radius, 0.575**2, pos, vel, spin, tides=(L.EFFECT_ORBITING, sigma, 0.305),
                flat=(L.EFFECT_ORBITING, 0.9532), gr=L.EFFECT_ORBITING)


def _hill_ok(a, masses, star_mass, spacing):
    """Rows of `a` (candidates x n) whose neighbours are at least `spacing`
    mutual Hill radii apart."""
    a = np.atleast_2d(a)
    rh = ((masses[:-1] + masses[1:]) / (3.0 * star_mass)) ** (1.0 / 3.0) * 0.5 * (a[:, :-1] + a[:, 1:])
    return np.all(a[:, 1:] - a[:, :-1] >= spacing * rh, axis=1)


def _semi_major_axes(rng, n, lo, hi, masses=None, star_mass=None, spacing=0.0):
    """Sorted uniform draws in [lo, hi]; with spacing > 0, drawn from that
    distribution conditioned on every neighbouring pair being `spacing`
    mutual Hill radii apart (what rejection and redraw converges to).

    The condition reads a[k+1] >= c_k a[k] with c_k = (1+f_k)/(1-f_k),
    f_k = spacing/2 ((m_k+m_k+1)/(3 M))^(1/3).  The map y_0 = a_0 - lo,
    y_k = a_k - c_(k-1) a_(k-1) has unit Jacobian and sends the feasible set
    onto the simplex {y >= 0, sum_k w_k y_k <= hi - lo prod c}, w_k =
    prod_(j>=k) c_j, so a uniform point of that simplex is an exact draw."""
    if spacing <= 0.0 or n < 2:
        return np.sort(rng.uniform(lo, hi, size=n))
    f = 0.5 * spacing * ((masses[:-1] + masses[1:]) / (3.0 * star_mass)) ** (1.0 / 3.0)
    c = (1.0 + f) / (1.0 - f)
    # many-planet systems of the uneven workload do not fit the range: widen it
    hi = max(hi, 1.25 * lo * np.prod(c))
    budget = hi - lo * np.prod(c)
    w = np.array([np.prod(c[k:]) for k in range(n)])  # weight of y_k in a[n-1]
    u = rng.dirichlet(np.ones(n + 1))[:n]
    y = budget * u / w
    a = np.empty(n)
    a[0] = lo + y[0]
    for k in range(1, n):
        a[k] = c[k - 1] * a[k - 1] + y[k]
    return a


def system_single(rng, n_planets=3, a_range=(0.01, 0.05), spacing=0.0, coords=L.JACOBI, **kw):
    star = _star()
    masses = np.exp(rng.uniform(np.log(0.3), np.log(3.0), size=n_planets)) * M_EARTH
    a = _semi_major_axes(rng, n_planets, a_range[0], a_range[1], masses, star.mass, spacing)
    planets = []
    for k in range(n_planets):
        planets.append(_planet(rng, star.mass, a[k], mass=masses[k]))
    return make_system([star] + planets, coords=coords, **kw)


def workload_single(seed=None, **kw):
    rng = np.random.default_rng(SEED_BASE + WORKLOAD_IDS["single"] if seed is None else seed)
    return stack_systems([system_single(rng, 3, (0.01, 0.05), **kw)])


def workload_ensemble8(n_systems=4096, seed=None, **kw):
    rng = np.random.default_rng(SEED_BASE + WORKLOAD_IDS["ensemble8"] if seed is None else seed)
    return stack_systems([system_single(rng, 7, (0.01, 0.07), spacing=8.0, **kw) for _ in range(n_systems)])


def workload_uneven(n_systems=16384, seed=None, **kw):
    rng = np.random.default_rng(SEED_BASE + WORKLOAD_IDS["uneven"] if seed is None else seed)
    cases = []
    for _ in range(n_systems):
        n_bodies = int(rng.integers(2, 11))
        flags = rng.uniform(size=3) < 0.7
        if n_bodies >= 3 and rng.uniform() < 0.2:
            cases.append(_binary_system(rng, n_bodies, flags, **kw))
        else:
            cases.append(system_single(rng, n_bodies - 1, (0.01, 0.07), spacing=8.0, tides=bool(flags[0]),
                                       flat=bool(flags[1]), gr=bool(flags[2]), **kw))
    return stack_systems(cases, nmax=10)


def _binary_system(rng, n_bodies, flags, **kw):
    """Two stars (0.1-1 Msun, separation 0.05-0.2 AU) and circumbinary
    planets beyond three separations; the heavier star hosts the effects."""
    m1, m2 = sorted(rng.uniform(0.1, 1.0, size=2), reverse=True)
    sep = rng.uniform(0.05, 0.2)
    star = _star(mass=m1, radius_factor=m1**0.8, rg2=0.1, period_days=10.0, k2=0.03)
    gm = G * (m1 + m2)
    pos, vel = kepler_to_cartesian(gm, sep, rng.uniform(0.0, 0.05), 0.0, *rng.uniform(0.0, TWO_PI, size=3))
    companion = Body(m2, m2**0.8 * R_SUN, 0.1, pos, vel, np.array([0.0, 0.0, TWO_PI / 10.0]),
                     tides=(L.EFFECT_ORBITING, 2.006 * 3.845764e4, 0.03), flat=(L.EFFECT_ORBITING, 0.03),
                     gr=L.EFFECT_ORBITING)
    n_pl = n_bodies - 2
    a = np.sort(rng.uniform(3.0 * sep, 3.0 * sep + 0.3, size=n_pl)) if n_pl > 0 else []
    bary_pos = companion.pos * m2 / (m1 + m2)
    bary_vel = companion.vel * m2 / (m1 + m2)
    planets = [_planet(rng, m1 + m2, a[k], bary_pos, bary_vel) for k in range(n_pl)]
    return make_system([star, companion] + planets, tides=bool(flags[0]), flat=bool(flags[1]), gr=bool(flags[2]),
                       **kw)


def workload_large(n_small=1021, seed=None, dt=0.1, coords=L.DEMOCRATIC_HELIOCENTRIC, **kw):
    """One system of 3 + n_small bodies (the many-body workload).  Every body
    is a tidal orbiting body of the star -- the reference sums the star's
    torque over all bodies -- with zero dissipation factor and Love number for
    the small bodies."""
    rng = np.random.default_rng(SEED_BASE + WORKLOAD_IDS["large"] if seed is None else seed)
    star = _star(mass=1.0, radius_factor=1.0, rg2=0.07, period_days=25.0, k2=0.03)
    bodies = [star]
    a_pl = np.sort(rng.uniform(0.02, 0.05, size=2))
    for a in a_pl:
        m = rng.uniform(1.0, 10.0) * M_EARTH
        bodies.append(_planet(rng, star.mass, a, mass=m))
    for _ in range(n_small):
        m = np.exp(rng.uniform(np.log(1e-3), np.log(1e-1))) * M_EARTH
        a = rng.uniform(0.1, 1.0)
        b = _planet(rng, star.mass, a, e_max=0.1, i_max_deg=2.0, mass=m)
        b.tides = (L.EFFECT_ORBITING, 0.0, 0.0)
        b.flat = None
        b.gr = L.EFFECT_DISABLED
        bodies.append(b)
    for b in bodies[1:3]:
        b.flat = None
        b.gr = L.EFFECT_DISABLED
    star.flat = None
    star.gr = L.EFFECT_DISABLED
    return make_system(bodies, dt=dt, coords=coords, tides=True, flat=False, gr=False, **kw)


def as_ias15(ens, dt=None):
    """The same systems integrated by IAS15 (src/integrator/ias15.rs): a copy
    of the ensemble with the integrator set, a fresh Gauss-Radau state
    (``body_ias`` zeros, no accepted step yet) and, if given, the first trial
    step ``dt`` in days (IAS15 adapts it from there)."""
    out = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in ens.items()}
    out["sys_i64"][:, L.SI_INTEGRATOR] = L.INTEGRATOR_IAS15
    out["sys_i64"][:, L.SI_IAS_MAX_EXCEEDED] = 0
    out["sys_f64"][:, L.SF_IAS_DT_LAST] = 0.0
    if dt is not None:
        out["sys_f64"][:, L.SF_DT] = dt
        out["sys_f64"][:, L.SF_HALF_DT] = 0.5 * dt
    out["body_ias"] = np.zeros(out["body_f64"].shape[:2] + (L.IAS_COUNT,), np.float64)
    return out
