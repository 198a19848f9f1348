"""Reference JSON case -> flat system layout (test infrastructure).

Reads a Posidonius WHFast case / recovery snapshot written by serde
(``src/integrator/output.rs:28-54`` write, ``:205-241`` read; the layout is
the serde form of ``WHFast`` in ``src/integrator/whfast.rs:99-120``) with
Python's ``json`` module (correctly rounded float parsing) and packs it into
the flat layout declared in ``include/posidonius_gb300.h``.

This is the checker's own reader: the product parses JSON in C++
(``posi_universe_from_json``); tests compare the two.
"""
import json

import numpy as np

from posidonius_gb300 import layout as L

EVOLUTION_CODES = {
    "NonEvolving": L.EVO_NON_EVOLVING,
    "Leconte2011": L.EVO_LECONTE2011,
    "Baraffe1998": L.EVO_BARAFFE1998,
    "Baraffe2015": L.EVO_BARAFFE2015,
    "BolmontMathis2016": L.EVO_BOLMONT_MATHIS2016,
    "GalletBolmont2017": L.EVO_GALLET_BOLMONT2017,
}
DYNAMICAL = (L.EVO_BOLMONT_MATHIS2016, L.EVO_GALLET_BOLMONT2017)


class Unsupported(ValueError):
    """The case uses a part of Posidonius outside the WHFast/CTL/oblate/Kidder path."""


def _evolution_code(evo):
    if isinstance(evo, str):
        if evo in EVOLUTION_CODES:
            return EVOLUTION_CODES[evo]
        raise Unsupported(f"evolution {evo}")
    (name, arg), = evo.items()
    if name == "LeconteChabrier2013":
        if arg:
            raise Unsupported("LeconteChabrier2013(true) dynamical tides")
        return L.EVO_LECONTE_CHABRIER2013
    if name in EVOLUTION_CODES:
        return EVOLUTION_CODES[name]
    raise Unsupported(f"evolution {name}")


def _effect(effect, model_key):
    """(kind, params) of a serde externally-tagged effect enum."""
    if effect == "Disabled":
        return L.EFFECT_DISABLED, None
    if effect == "OrbitingBody" or effect == {"OrbitingBody": None}:
        return L.EFFECT_ORBITING, None
    (tag, inner), = effect.items()
    kind = {"CentralBody": L.EFFECT_CENTRAL, "OrbitingBody": L.EFFECT_ORBITING}[tag]
    if model_key is None:
        return kind, inner
    if not isinstance(inner, dict) or model_key not in inner:
        raise Unsupported(f"model {inner}")
    return kind, inner[model_key]


def load_case(path_or_dict):
    """Return a dict of flat arrays for one system (nmax = n)."""
    d = path_or_dict
    if not isinstance(d, dict):
        with open(d) as f:
            d = json.load(f)
    ias15 = "alternative_coordinates_type" not in d and "b_0" in d and "time_step_last_success" in d
    if "alternative_coordinates_type" not in d and not ias15:
        raise Unsupported("neither a WHFast nor an IAS15 case")
    u = d["universe"]
    n = int(u["n_particles"])
    ce = u["consider_effects"]

    gr_impl = u["general_relativity_implementation"]
    gr_codes = {"Kidder1995": L.GR_KIDDER1995, "Anderson1975": L.GR_ANDERSON1975, "Newhall1983": L.GR_NEWHALL1983}
    if ce["general_relativity"] and gr_impl not in gr_codes:
        raise Unsupported(f"general relativity {gr_impl}")
    hosts = u["hosts"]
    host = int(hosts["index"]["most_massive"])
    for eff in ("tides", "rotational_flattening", "general_relativity", "disk"):
        if ce[eff] and int(hosts["index"][eff]) != host:
            raise Unsupported(f"{eff} host is not the most massive body")

    si = np.zeros(L.SI_COUNT, dtype=np.int64)
    sf = np.zeros(L.SF_COUNT, dtype=np.float64)
    bi = np.zeros((n, L.BI_COUNT), dtype=np.int64)
    bf = np.zeros((n, L.BF_COUNT), dtype=np.float64)
    si[L.SI_N] = n
    si[L.SI_HOST] = host
    if ias15:
        si[L.SI_INTEGRATOR] = L.INTEGRATOR_IAS15
        si[L.SI_IAS_MAX_EXCEEDED] = int(d["integrator_iterations_max_exceeded"])
        sf[L.SF_IAS_DT_LAST] = d["time_step_last_success"]
    else:
        si[L.SI_COORDS] = {"Jacobi": L.JACOBI, "DemocraticHeliocentric": L.DEMOCRATIC_HELIOCENTRIC,
                           "WHDS": L.WHDS}[d["alternative_coordinates_type"]]
    si[L.SI_TIDES] = int(ce["tides"])
    si[L.SI_FLAT] = int(ce["rotational_flattening"])
    si[L.SI_GR] = int(ce["general_relativity"])
    si[L.SI_GR_IMPL] = gr_codes.get(gr_impl, L.GR_KIDDER1995)
    si[L.SI_WIND] = int(ce["wind"])
    si[L.SI_DISK] = int(ce["disk"])
    si[L.SI_EVOLUTION] = int(ce["evolution"])
    si[L.SI_ITERATION] = int(d["current_iteration"])
    si[L.SI_N_HIST] = int(d["n_historic_snapshots"])
    si[L.SI_TIMESTEP_WARNING] = int(d.get("timestep_warning", 0))
    sf[L.SF_DT] = d["time_step"]
    sf[L.SF_HALF_DT] = d.get("half_time_step", 0.0)
    sf[L.SF_TIME] = d["current_time"]
    sf[L.SF_TIME_LIMIT] = u["time_limit"]
    sf[L.SF_LAST_HIST] = d["last_historic_snapshot_time"]
    sf[L.SF_HIST_PERIOD] = d["historic_snapshot_period"]
    sf[L.SF_LAST_REC] = d["last_recovery_snapshot_time"]
    sf[L.SF_REC_PERIOD] = d["recovery_snapshot_period"]
    sf[L.SF_INITIAL_TIME] = u["initial_time"]

    tables = []
    off = 0
    for b in range(n):
        p = u["particles"][b]
        ev = u["particles_evolvers"][b]
        tk, tparams = _effect(p["tides"]["effect"], "ConstantTimeLag")
        fk, fparams = _effect(p["rotational_flattening"]["effect"], "OblateSpheroid")
        gk, gimpl = _effect(p["general_relativity"]["effect"], None)
        wk = 1 if p["wind"]["effect"] == "Interaction" else 0
        if p["wind"]["effect"] not in ("Interaction", "Disabled"):
            raise Unsupported(f"wind {p['wind']['effect']}")
        # the wind torque output is summed into dL/dt whatever the flags
        # (src/particles/universe.rs:589-591); only interacting bodies under
        # the wind effect recompute it, the others must hold zero
        if not (ce["wind"] and wk):
            o = p["wind"]["parameters"]["output"]["dangular_momentum_dt"]
            if o["x"] != 0.0 or o["y"] != 0.0 or o["z"] != 0.0:
                raise Unsupported("stale wind torque output")
        if gk == L.EFFECT_CENTRAL and gimpl != gr_impl and ce["general_relativity"]:
            raise Unsupported(f"general relativity host {gimpl} differs from the universe's {gr_impl}")
        if ce["tides"] and b != host and tk != L.EFFECT_ORBITING:
            # The reference's host torque loop visits every body and divides
            # by the stale distance 0 of a non-orbiting one (NaN spin).
            raise Unsupported("tides on with a non-orbiting body")
        # Outputs of disabled effects are summed into dL/dt by the reference
        # (src/particles/universe.rs:589-591); they must be zero here.
        for eff, on in (("tides", ce["tides"]), ("rotational_flattening", ce["rotational_flattening"]),
                        ("general_relativity", ce["general_relativity"])):
            if not on:
                o = p[eff]["parameters"]["output"]["dangular_momentum_dt"]
                if o["x"] != 0.0 or o["y"] != 0.0 or o["z"] != 0.0:
                    raise Unsupported(f"stale {eff} torque output")
        if b == host:
            hv = p["heliocentric_velocity"]
            if hv["x"] != 0.0 or hv["y"] != 0.0 or hv["z"] != 0.0:
                raise Unsupported("host with non-zero heliocentric velocity")
        bi[b, L.BI_TIDES_KIND] = tk
        bi[b, L.BI_FLAT_KIND] = fk
        bi[b, L.BI_GR_KIND] = gk
        bi[b, L.BI_WIND_KIND] = wk
        dk, dprops = _effect(p["disk"]["effect"], None)
        if ce["disk"] and b == host and dk != L.EFFECT_CENTRAL:
            raise Unsupported("disk host is not a central body")
        bi[b, L.BI_DISK_KIND] = dk
        bf[b, L.BF_DISK_MTS] = p["disk"]["parameters"]["internal"]["migration_timescale"]
        evo_code = _evolution_code(p["evolution"])
        evo_ev = _evolution_code(ev["evolution"])
        if evo_code != evo_ev:
            raise Unsupported("particle and evolver evolution types differ")
        if evo_code in DYNAMICAL and (b != host or not ce["tides"] or tk != L.EFFECT_CENTRAL):
            # the planet-dependent branch keeps stale entries in the reference
            # (src/effects/tides/constant_time_lag.rs:131-135 removes the host's key)
            raise Unsupported("dynamical-tide evolution on a body other than the tidal host")
        bi[b, L.BI_EVO_TYPE] = evo_code
        bi[b, L.BI_EVO_LEFT] = int(ev["left_index"])
        nrow = len(ev["time"])
        if evo_code != L.EVO_NON_EVOLVING and nrow > 0:
            block = np.zeros(4 * nrow)
            block[0:nrow] = ev["time"]
            block[nrow:2 * nrow] = ev["radius"]
            if len(ev["radius_of_gyration_2"]) == nrow:
                block[2 * nrow:3 * nrow] = ev["radius_of_gyration_2"]
            if len(ev["love_number"]) == nrow:
                block[3 * nrow:4 * nrow] = ev["love_number"]
            if evo_code in DYNAMICAL:
                # the dynamical-tide evolutions interpolate no Love number:
                # their 4th column holds the inverse tidal Q factor
                if len(ev.get("inverse_tidal_q_factor", [])) != nrow:
                    raise Unsupported("dynamical-tide evolution without its inverse tidal Q factor")
                block[3 * nrow:4 * nrow] = ev["inverse_tidal_q_factor"]
            bi[b, L.BI_EVO_OFFSET] = off
            bi[b, L.BI_EVO_LEN] = nrow
            tables.append(block)
            off += 4 * nrow
        F = bf[b]
        F[L.BF_MASS] = p["mass"]
        F[L.BF_MASS_G] = p["mass_g"]
        F[L.BF_RADIUS] = p["radius"]
        F[L.BF_RG2] = p["radius_of_gyration_2"]
        F[L.BF_MOI] = p["moment_of_inertia"]
        if tparams is not None:
            F[L.BF_DISS_FACTOR] = tparams["dissipation_factor"]
            F[L.BF_DISS_SCALE] = tparams["dissipation_factor_scale"]
        if dk == L.EFFECT_CENTRAL:
            for f, key in ((L.BF_DISK_INNER, "inner_edge_distance"), (L.BF_DISK_OUTER, "outer_edge_distance"),
                           (L.BF_DISK_LIFETIME, "lifetime"), (L.BF_DISK_ALPHA, "alpha"),
                           (L.BF_DISK_SIGMA0, "surface_density_normalization"),
                           (L.BF_DISK_MU, "mean_molecular_weight")):
                F[f] = dprops[key]
        F[L.BF_WIND_K] = p["wind"]["parameters"]["input"]["k_factor"]
        F[L.BF_WIND_RSAT] = p["wind"]["parameters"]["input"]["rotation_saturation"]
        F[L.BF_WIND_RSAT2] = p["wind"]["parameters"]["internal"]["rotation_saturation_2"]
        for k, key in enumerate(("x", "y", "z")):
            F[L.BF_PX + k] = p["inertial_position"][key]
            F[L.BF_VX + k] = p["inertial_velocity"][key]
            F[L.BF_AX + k] = p["inertial_acceleration"][key]
            F[L.BF_LX + k] = p["angular_momentum"][key]
            F[L.BF_SX + k] = p["spin"][key]
            if not ias15:
                F[L.BF_EVX + k] = d["inertial_velocity_errors"][b][key]
                F[L.BF_ELX + k] = d["particle_angular_momentum_errors"][b][key]
            F[L.BF_ADDAX + k] = p["inertial_additional_acceleration"][key]
            F[L.BF_DLX + k] = p["dangular_momentum_dt"][key]
        F[L.BF_NSV2] = p["norm_spin_vector_2"]
        F[L.BF_SIGMA] = p["tides"]["parameters"]["internal"]["scaled_dissipation_factor"]
        F[L.BF_K2] = tparams["love_number"] if tparams else 0.0
        F[L.BF_K2F] = fparams["love_number"] if fparams else 0.0
        tint = p["tides"]["parameters"]["internal"]
        F[L.BF_DENERGY_DT] = tint["denergy_dt"]
        F[L.BF_LAG_ANGLE] = tint["lag_angle"]
        F[L.BF_TD_DIST] = tint["distance"]
        F[L.BF_TD_VR] = tint["radial_velocity"]
        F[L.BF_TD_ORTHO] = tint["orthogonal_component_of_the_tidal_force_due_to_planetary_tide"]
        F[L.BF_TD_DPM] = tint["radial_component_of_the_tidal_force_dissipative_part_when_star_as_point_mass"]
        for k, key in enumerate(("x", "y", "z")):
            F[L.BF_TD_PX + k] = p["tides"]["coordinates"]["position"][key]
            F[L.BF_TD_VX + k] = p["tides"]["coordinates"]["velocity"][key]
            F[L.BF_TD_LX + k] = p["tides"]["parameters"]["output"]["dangular_momentum_dt"][key]
    # calculate_roche_radiuses fills the first n*n entries in rows of n
    # (src/particles/universe.rs:177-196)
    rr = u["roche_radiuses"]
    roche = np.zeros((n, n), dtype=np.float64)
    if len(rr) >= n * n:
        roche = np.array(rr[: n * n], dtype=np.float64).reshape(n, n)
    tab = np.concatenate(tables) if tables else np.zeros(1)
    ias = np.zeros((n, L.IAS_COUNT), dtype=np.float64)
    if ias15:
        # the serde arrays b_0..b_6, e_*, br_*, er_*, sb_*, se_*, sbr_*, ser_*
        # hold 3*MAX_PARTICLES values (body i component c at 3*i + c)
        for base, name in ((L.IAS_B, "b"), (L.IAS_E, "e"), (L.IAS_BR, "br"), (L.IAS_ER, "er"),
                           (L.IAS_SB, "sb"), (L.IAS_SE, "se"), (L.IAS_SBR, "sbr"), (L.IAS_SER, "ser")):
            for j in range(7):
                arr = np.asarray(d[f"{name}_{j}"], dtype=np.float64)[: 3 * n].reshape(n, 3)
                ias[:, base + 3 * j: base + 3 * j + 3] = arr
        for base, name in ((L.IAS_CSX, "csx"), (L.IAS_CSV, "csv"), (L.IAS_CSS, "css")):
            ias[:, base: base + 3] = np.asarray(d[name], dtype=np.float64)[: 3 * n].reshape(n, 3)
    return {"sys_i64": si, "sys_f64": sf, "body_i64": bi, "body_f64": bf, "tables": tab,
            "roche": roche, "n": n, "body_ias": ias}


def stack(cases, nmax=None):
    """Stack single-system dicts into one padded ensemble (nmax bodies)."""
    nmax = nmax or max(c["n"] for c in cases)
    ns = len(cases)
    si = np.zeros((ns, L.SI_COUNT), dtype=np.int64)
    sf = np.zeros((ns, L.SF_COUNT), dtype=np.float64)
    bi = np.zeros((ns, nmax, L.BI_COUNT), dtype=np.int64)
    bf = np.zeros((ns, nmax, L.BF_COUNT), dtype=np.float64)
    roche = np.zeros((ns, nmax, nmax), dtype=np.float64)
    ias = np.zeros((ns, nmax, L.IAS_COUNT), dtype=np.float64)
    tabs = []
    off = 0
    for k, c in enumerate(cases):
        n = c["n"]
        si[k] = c["sys_i64"]
        sf[k] = c["sys_f64"]
        bi[k, :n] = c["body_i64"]
        bf[k, :n] = c["body_f64"]
        roche[k, :n, :n] = c["roche"]
        if "body_ias" in c:
            ias[k, :n] = c["body_ias"]
        evolving = bi[k, :n, L.BI_EVO_LEN] > 0
        bi[k, :n, L.BI_EVO_OFFSET] = np.where(evolving, bi[k, :n, L.BI_EVO_OFFSET] + off, 0)
        tabs.append(c["tables"])
        off += len(c["tables"])
    return {"sys_i64": si, "sys_f64": sf, "body_i64": bi, "body_f64": bf,
            "tables": np.concatenate(tabs), "roche": roche, "nmax": nmax, "n_sys": ns, "body_ias": ias}
