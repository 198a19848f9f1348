"""Flat system -> Posidonius JSON case document (WHFast or Ias15).

The counterpart of the reference's own case generator
(``posidonius/particles/universe.py:313-366`` with the integrator writers):
the serde form of ``WHFast`` (src/integrator/whfast.rs:99-120) or ``Ias15``
(src/integrator/ias15.rs:28-224) around a ``Universe``
(src/particles/universe.rs:50-63), padded to the reference's MAX_PARTICLES
(src/constants.rs:3) with disabled dummy particles, so that ``posidonius
start`` -- the reference's or this repository's -- can run a system built
with ``posidonius_gb300.ensemble``.  Fields the integrator recomputes before
it uses them (heliocentric copies, effect scratch values, alternative
coordinates) are written as zeros, as the reference's generator leaves them.

    from posidonius_gb300 import case_writer, ensemble
    case_writer.write_case("case.json", ensemble.workload_single())
"""
import json

import numpy as np

from . import layout as L

MAX_PARTICLES = 10      # src/constants.rs:3
NO_HOST = MAX_PARTICLES + 1

EVOLUTION_NAMES = {L.EVO_LECONTE2011: "Leconte2011", L.EVO_BARAFFE1998: "Baraffe1998",
                   L.EVO_BARAFFE2015: "Baraffe2015", L.EVO_BOLMONT_MATHIS2016: "BolmontMathis2016",
                   L.EVO_GALLET_BOLMONT2017: "GalletBolmont2017"}
GR_NAMES = {L.GR_KIDDER1995: "Kidder1995", L.GR_ANDERSON1975: "Anderson1975", L.GR_NEWHALL1983: "Newhall1983"}
COORD_NAMES = {L.JACOBI: "Jacobi", L.DEMOCRATIC_HELIOCENTRIC: "DemocraticHeliocentric", L.WHDS: "WHDS"}


def _axes(v=(0.0, 0.0, 0.0)):
    return {"x": float(v[0]), "y": float(v[1]), "z": float(v[2])}


def _coords():
    return {"position": _axes(), "velocity": _axes()}


def _kind_tag(kind):
    return {L.EFFECT_CENTRAL: "CentralBody", L.EFFECT_ORBITING: "OrbitingBody"}[kind]


def _particle(F=None, I=None, idx=0, gr_impl="Kidder1995", host_mg=0.0, gr_on=False):
    """One particle entry; F / I are the body's flat fields (None: a dummy)."""
    z = np.zeros(L.BF_COUNT) if F is None else F
    zi = np.zeros(L.BI_COUNT, dtype=np.int64) if I is None else I
    tk, fk, gk = int(zi[L.BI_TIDES_KIND]), int(zi[L.BI_FLAT_KIND]), int(zi[L.BI_GR_KIND])
    dk, wk, evo = int(zi[L.BI_DISK_KIND]), int(zi[L.BI_WIND_KIND]), int(zi[L.BI_EVO_TYPE])
    if tk == L.EFFECT_DISABLED:
        tides_effect = "Disabled"
    else:
        tides_effect = {_kind_tag(tk): {"ConstantTimeLag": {
            "dissipation_factor": float(z[L.BF_DISS_FACTOR]),
            "dissipation_factor_scale": float(z[L.BF_DISS_SCALE]),
            "love_number": float(z[L.BF_K2])}}}
    if fk == L.EFFECT_DISABLED:
        flat_effect = "Disabled"
    else:
        flat_effect = {_kind_tag(fk): {"OblateSpheroid": {"love_number": float(z[L.BF_K2F])}}}
    if gk == L.EFFECT_DISABLED:
        gr_effect = "Disabled"
    elif gk == L.EFFECT_CENTRAL:
        gr_effect = {"CentralBody": gr_impl}
    else:
        gr_effect = "OrbitingBody"
    if dk == L.EFFECT_CENTRAL:
        disk_effect = {"CentralBody": {
            "alpha": float(z[L.BF_DISK_ALPHA]), "inner_edge_distance": float(z[L.BF_DISK_INNER]),
            "lifetime": float(z[L.BF_DISK_LIFETIME]), "mean_molecular_weight": float(z[L.BF_DISK_MU]),
            "outer_edge_distance": float(z[L.BF_DISK_OUTER]),
            "surface_density_normalization": float(z[L.BF_DISK_SIGMA0])}}
    elif dk == L.EFFECT_ORBITING:
        disk_effect = "OrbitingBody"
    else:
        disk_effect = "Disabled"
    mass, mass_g = float(z[L.BF_MASS]), float(z[L.BF_MASS_G])
    # src/effects/general_relativity.rs:86-109 (the generator's GR factor)
    gr_factor = host_mg * mass_g / np.power(host_mg + mass_g, 2) if (gr_on and gk == L.EFFECT_ORBITING and mass != 0) \
        else 0.0
    return {
        "angular_momentum": _axes(z[L.BF_LX:L.BF_LZ + 1]),
        "dangular_momentum_dt": _axes(z[L.BF_DLX:L.BF_DLZ + 1]),
        "disk": {"coordinates": _coords(), "effect": disk_effect,
                 "parameters": {"internal": {"distance": 0.0, "migration_timescale": float(z[L.BF_DISK_MTS]),
                                             "norm_velocity_vector": 0.0, "norm_velocity_vector_2": 0.0},
                                "output": {"acceleration": _axes()}}},
        "evolution": _evolution_tag(evo, mass),
        "general_relativity": {"coordinates": _coords(), "effect": gr_effect,
                               "parameters": {"internal": {"distance": 0.0, "factor": float(gr_factor),
                                                           "norm_velocity_vector": 0.0,
                                                           "norm_velocity_vector_2": 0.0, "radial_velocity": 0.0},
                                              "output": {"acceleration": _axes(), "dangular_momentum_dt": _axes()}}},
        "heliocentric_distance": 0.0, "heliocentric_norm_velocity_vector": 0.0,
        "heliocentric_norm_velocity_vector_2": 0.0, "heliocentric_position": _axes(),
        "heliocentric_radial_velocity": 0.0, "heliocentric_velocity": _axes(),
        "id": int(idx),
        "inertial_acceleration": _axes(z[L.BF_AX:L.BF_AZ + 1]),
        "inertial_additional_acceleration": _axes(z[L.BF_ADDAX:L.BF_ADDAZ + 1]),
        "inertial_position": _axes(z[L.BF_PX:L.BF_PZ + 1]),
        "inertial_velocity": _axes(z[L.BF_VX:L.BF_VZ + 1]),
        "mass": mass, "mass_g": mass_g,
        "moment_of_inertia": float(z[L.BF_MOI]),
        "norm_spin_vector_2": float(z[L.BF_NSV2]),
        "radius": float(z[L.BF_RADIUS]),
        "radius_of_gyration_2": float(z[L.BF_RG2]),
        "reference": "MostMassiveParticle",
        "rotational_flattening": {
            "coordinates": _coords(), "effect": flat_effect,
            "parameters": {"internal": {
                "distance": 0.0, "factor_for_the_force_induced_by_planet_rotation": 0.0,
                "factor_for_the_force_induced_by_star_rotation": 0.0,
                "orthogonal_component_of_the_force_induced_by_planet_rotation": 0.0,
                "orthogonal_component_of_the_force_induced_by_star_rotation": 0.0,
                "radial_component_of_the_force_induced_by_rotation": 0.0,
                "scalar_product_of_vector_position_with_planetary_spin": 0.0,
                "scalar_product_of_vector_position_with_stellar_spin": 0.0, "shape": _axes()},
                "output": {"acceleration": _axes(), "dangular_momentum_dt": _axes()}}},
        "spin": _axes(z[L.BF_SX:L.BF_SZ + 1]),
        "tides": {
            "coordinates": {"position": _axes(z[L.BF_TD_PX:L.BF_TD_PZ + 1]),
                            "velocity": _axes(z[L.BF_TD_VX:L.BF_TD_VZ + 1])},
            "effect": tides_effect,
            "parameters": {"internal": {
                "denergy_dt": float(z[L.BF_DENERGY_DT]), "distance": float(z[L.BF_TD_DIST]),
                "lag_angle": float(z[L.BF_LAG_ANGLE]),
                "orthogonal_component_of_the_tidal_force_due_to_planetary_tide": float(z[L.BF_TD_ORTHO]),
                "orthogonal_component_of_the_tidal_force_due_to_stellar_tide": 0.0,
                "radial_component_of_the_tidal_force": 0.0,
                "radial_component_of_the_tidal_force_dissipative_part_when_star_as_point_mass":
                    float(z[L.BF_TD_DPM]),
                "radial_velocity": float(z[L.BF_TD_VR]),
                "scalar_product_of_vector_position_with_planetary_spin": 0.0,
                "scalar_product_of_vector_position_with_stellar_spin": 0.0,
                "scaled_dissipation_factor": float(z[L.BF_SIGMA]), "shape": _axes()},
                "output": {"acceleration": _axes(),
                           "dangular_momentum_dt": _axes(z[L.BF_TD_LX:L.BF_TD_LZ + 1])}}},
        "wind": {"effect": "Interaction" if wk == 1 else "Disabled",
                 "parameters": {"input": {"k_factor": float(z[L.BF_WIND_K]),
                                          "rotation_saturation": float(z[L.BF_WIND_RSAT])},
                                "internal": {"rotation_saturation_2": float(z[L.BF_WIND_RSAT2])},
                                "output": {"dangular_momentum_dt": _axes()}}},
    }


def _evolution_tag(evo, mass):
    if evo == L.EVO_NON_EVOLVING:
        return "NonEvolving"
    if evo == L.EVO_LECONTE_CHABRIER2013:
        return {"LeconteChabrier2013": False}
    return {EVOLUTION_NAMES[evo]: float(mass)}


def _evolver(I, F, tables):
    """One Evolver (src/effects/evolution.rs:20-28): the columns each
    evolution type interpolates, from the flat tables block."""
    evo = L.EVO_NON_EVOLVING if I is None else int(I[L.BI_EVO_TYPE])
    out = {"evolution": _evolution_tag(evo, 0.0 if F is None else float(F[L.BF_MASS])),
           "inverse_tidal_q_factor": [], "left_index": 0 if I is None else int(I[L.BI_EVO_LEFT]),
           "love_number": [], "radius": [], "radius_of_gyration_2": [], "time": []}
    n = 0 if I is None else int(I[L.BI_EVO_LEN])
    if evo == L.EVO_NON_EVOLVING or n == 0:
        return out
    off = int(I[L.BI_EVO_OFFSET])
    col = [np.asarray(tables[off + k * n: off + (k + 1) * n], dtype=np.float64).tolist() for k in range(4)]
    out["time"], out["radius"] = col[0], col[1]
    if evo in (L.EVO_BARAFFE2015, L.EVO_LECONTE2011, L.EVO_LECONTE_CHABRIER2013):
        out["radius_of_gyration_2"] = col[2]
    if evo == L.EVO_LECONTE_CHABRIER2013:
        out["love_number"] = col[3]
    if evo in (L.EVO_BOLMONT_MATHIS2016, L.EVO_GALLET_BOLMONT2017):
        out["inverse_tidal_q_factor"] = col[3]
    return out


def case_document(case):
    """The JSON document (a dict) of one system: ``case`` is a single-system
    flat dict (``oracle``-style ``load_case`` output, ``WHFast.get_state()``
    or one system of an ensemble) with sys_i64, sys_f64, body_i64, body_f64,
    tables and, for IAS15, body_ias."""
    si, sf = np.asarray(case["sys_i64"]).reshape(-1), np.asarray(case["sys_f64"]).reshape(-1)
    n = int(si[L.SI_N])
    if n > MAX_PARTICLES:
        raise ValueError(f"the reference's case documents hold at most {MAX_PARTICLES} particles")
    bf = np.asarray(case["body_f64"]).reshape(-1, L.BF_COUNT)
    bi = np.asarray(case["body_i64"]).reshape(-1, L.BI_COUNT)
    tables = np.asarray(case.get("tables", np.zeros(1))).reshape(-1)
    host = int(si[L.SI_HOST])
    flags = {k: bool(si[f]) for k, f in (("tides", L.SI_TIDES), ("rotational_flattening", L.SI_FLAT),
                                         ("general_relativity", L.SI_GR), ("disk", L.SI_DISK),
                                         ("wind", L.SI_WIND), ("evolution", L.SI_EVOLUTION))}
    gr_impl = GR_NAMES[int(si[L.SI_GR_IMPL])]
    host_mg = float(bf[host, L.BF_MASS_G])
    particles = [_particle(bf[b], bi[b], b, gr_impl, host_mg, flags["general_relativity"]) for b in range(n)]
    particles += [_particle() for _ in range(MAX_PARTICLES - n)]
    evolvers = [_evolver(bi[b], bf[b], tables) for b in range(n)] + [_evolver(None, None, None)
                                                                      for _ in range(MAX_PARTICLES - n)]
    # universe.py:324-337: the hosts of disabled effects point past the vector
    index = {"most_massive": host,
             "tides": host if flags["tides"] else (host if flags["rotational_flattening"] else NO_HOST),
             "rotational_flattening": host if flags["rotational_flattening"] else NO_HOST,
             "general_relativity": host if flags["general_relativity"] else NO_HOST,
             "disk": host if flags["disk"] else NO_HOST}
    roche = np.zeros(MAX_PARTICLES * MAX_PARTICLES)
    if case.get("roche") is not None:
        r = np.asarray(case["roche"]).reshape(-1)
        rr = r[: n * n] if r.size >= n * n else np.zeros(n * n)
        roche[: n * n] = rr    # calculate_roche_radiuses fills the first n*n in rows of n
    universe = {
        "consider_effects": flags,
        "general_relativity_implementation": gr_impl,
        "hosts": {"index": index,
                  "most_massive": {"all": True, "disk": flags["disk"],
                                   "general_relativity": flags["general_relativity"],
                                   "rotational_flattening": flags["rotational_flattening"],
                                   "tides": flags["tides"]}},
        "initial_time": float(sf[L.SF_INITIAL_TIME]),
        "n_particles": n,
        "pair_dependent_scaled_dissipation_factor": {},
        "particles": particles,
        "particles_evolvers": evolvers,
        "roche_radiuses": roche.tolist(),
        "time_limit": float(sf[L.SF_TIME_LIMIT]),
    }
    doc = {
        "current_iteration": int(si[L.SI_ITERATION]),
        "current_time": float(sf[L.SF_TIME]),
        "hash": 0,
        "historic_snapshot_period": float(sf[L.SF_HIST_PERIOD]),
        "last_historic_snapshot_time": float(sf[L.SF_LAST_HIST]),
        "last_recovery_snapshot_time": float(sf[L.SF_LAST_REC]),
        "n_historic_snapshots": int(si[L.SI_N_HIST]),
        "recovery_snapshot_period": float(sf[L.SF_REC_PERIOD]),
        "time_step": float(sf[L.SF_DT]),
        "universe": universe,
    }
    if int(si[L.SI_INTEGRATOR]) == L.INTEGRATOR_IAS15:
        ias = np.asarray(case.get("body_ias", np.zeros((n, L.IAS_COUNT)))).reshape(-1, L.IAS_COUNT)
        zeros3 = [0.0] * (3 * MAX_PARTICLES)

        def block(base):
            out = list(zeros3)
            for b in range(n):
                out[3 * b: 3 * b + 3] = [float(x) for x in ias[b, base: base + 3]]
            return out

        for name, base in (("b", L.IAS_B), ("e", L.IAS_E), ("br", L.IAS_BR), ("er", L.IAS_ER),
                           ("sb", L.IAS_SB), ("se", L.IAS_SE), ("sbr", L.IAS_SBR), ("ser", L.IAS_SER)):
            for j in range(7):
                doc[f"{name}_{j}"] = block(base + 3 * j)
        for name in ("g", "sg"):
            for j in range(7):
                doc[f"{name}_{j}"] = list(zeros3)
        doc["csx"], doc["csv"], doc["css"] = block(L.IAS_CSX), block(L.IAS_CSV), block(L.IAS_CSS)
        for name in ("a0", "angular_momentum0", "at", "dangular_momentum_dt0", "dangular_momentum_dtt", "v0", "x0"):
            doc[name] = list(zeros3)
        doc["s"] = [0.0] * 9
        doc["n_particles"] = n
        doc["integrator_iterations_max_exceeded"] = int(si[L.SI_IAS_MAX_EXCEEDED])
        doc["time_step_last_success"] = float(sf[L.SF_IAS_DT_LAST])
    else:
        doc["alternative_coordinates_type"] = COORD_NAMES[int(si[L.SI_COORDS])]
        doc["half_time_step"] = float(sf[L.SF_HALF_DT])
        doc["timestep_warning"] = int(si[L.SI_TIMESTEP_WARNING])
        doc["inertial_velocity_errors"] = [_axes(bf[b, L.BF_EVX:L.BF_EVZ + 1]) for b in range(n)] + \
            [_axes() for _ in range(MAX_PARTICLES - n)]
        doc["particle_angular_momentum_errors"] = [_axes(bf[b, L.BF_ELX:L.BF_ELZ + 1]) for b in range(n)] + \
            [_axes() for _ in range(MAX_PARTICLES - n)]
        doc["particles_alternative_coordinates"] = [
            {"acceleration": _axes(), "mass": 0.0, "mass_g": 0.0, "position": _axes(), "velocity": _axes()}
            for _ in range(MAX_PARTICLES)]
    return doc


def _single(case):
    """One system of an ensemble dict (n_sys == 1) or a single-system dict."""
    if "n_sys" not in case:
        return case
    if case["n_sys"] != 1:
        raise ValueError("write one system per case document")
    out = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in case.items()}
    return out


def _json_safe(x):
    """serde_json writes non-finite floats as null."""
    if isinstance(x, dict):
        return {k: _json_safe(v) for k, v in x.items()}
    if isinstance(x, list):
        return [_json_safe(v) for v in x]
    if isinstance(x, float) and not np.isfinite(x):
        return None
    return x


def write_case(path, case):
    """Write one system as a Posidonius JSON case document (keys sorted, as
    the reference's test documents are stored)."""
    with open(path, "w") as f:
        json.dump(_json_safe(case_document(_single(case))), f, indent=2, sort_keys=True, allow_nan=False)
