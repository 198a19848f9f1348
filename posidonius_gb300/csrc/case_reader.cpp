// case_reader.cpp -- see case_reader.hpp.
#include "case_reader.hpp"

#include <cmath>
#include <cstring>

namespace posi {
namespace {

struct Ctx {
    std::string err;
    int code = POSI_OK;
    bool fail(int c, const std::string& m) {
        if (code == POSI_OK) { code = c; err = m; }
        return false;
    }
};

const json::Value* req(Ctx& c, const json::Value* v, const char* key) {
    if (!v) return nullptr;
    const json::Value* r = v->find(key);
    if (!r) c.fail(POSI_ERR_PARSE, std::string("missing field '") + key + "'");
    return r;
}

double num(Ctx& c, const json::Value* v, const char* key) {
    const json::Value* r = req(c, v, key);
    if (!r) return 0.;
    if (r->kind == json::Value::Null) return std::nan("");  // serde_json writes non-finite floats as null
    if (!r->is_number()) { c.fail(POSI_ERR_PARSE, std::string("field '") + key + "' is not a number"); return 0.; }
    return r->num();
}

bool boolean(Ctx& c, const json::Value* v, const char* key) {
    const json::Value* r = req(c, v, key);
    if (!r) return false;
    if (r->kind != json::Value::Bool) { c.fail(POSI_ERR_PARSE, std::string("field '") + key + "' is not a boolean"); return false; }
    return r->b;
}

void axes(Ctx& c, const json::Value* v, const char* key, double out[3]) {
    const json::Value* r = req(c, v, key);
    out[0] = num(c, r, "x");
    out[1] = num(c, r, "y");
    out[2] = num(c, r, "z");
}

// Externally tagged effect enum -> (kind, model parameters or nullptr).
int effect_kind(Ctx& c, const json::Value* eff, const char* model, const json::Value** params,
                std::string* tag_inner = nullptr) {
    *params = nullptr;
    if (!eff) return POSI_EFFECT_DISABLED;
    if (eff->is_string()) {
        if (eff->text == "Disabled") return POSI_EFFECT_DISABLED;
        if (eff->text == "OrbitingBody") return POSI_EFFECT_ORBITING;
        c.fail(POSI_ERR_PARSE, "unknown effect " + eff->text);
        return POSI_EFFECT_DISABLED;
    }
    if (!eff->is_object() || eff->members.size() != 1) { c.fail(POSI_ERR_PARSE, "malformed effect"); return 0; }
    const std::string& tag = eff->members[0].first;
    const json::Value& inner = eff->members[0].second;
    int kind;
    if (tag == "CentralBody") kind = POSI_EFFECT_CENTRAL;
    else if (tag == "OrbitingBody") kind = POSI_EFFECT_ORBITING;
    else { c.fail(POSI_ERR_PARSE, "unknown effect tag " + tag); return 0; }
    if (!model) {
        if (tag_inner && inner.is_string()) *tag_inner = inner.text;
        return kind;
    }
    const json::Value* m = inner.find(model);
    if (!m) { c.fail(POSI_ERR_UNSUPPORTED, std::string("effect model other than ") + model); return kind; }
    *params = m;
    return kind;
}

int evolution_code(Ctx& c, const json::Value* e) {
    if (!e) return POSI_EVO_NON_EVOLVING;
    if (e->is_string()) {
        if (e->text == "NonEvolving") return POSI_EVO_NON_EVOLVING;
        c.fail(POSI_ERR_UNSUPPORTED, "evolution " + e->text);
        return 0;
    }
    if (!e->is_object() || e->members.size() != 1) { c.fail(POSI_ERR_PARSE, "malformed evolution"); return 0; }
    const std::string& name = e->members[0].first;
    const json::Value& arg = e->members[0].second;
    if (name == "Leconte2011") return POSI_EVO_LECONTE2011;
    if (name == "Baraffe1998") return POSI_EVO_BARAFFE1998;
    if (name == "Baraffe2015") return POSI_EVO_BARAFFE2015;
    if (name == "BolmontMathis2016") return POSI_EVO_BOLMONT_MATHIS2016;
    if (name == "GalletBolmont2017") return POSI_EVO_GALLET_BOLMONT2017;
    if (name == "LeconteChabrier2013") {
        if (arg.kind == json::Value::Bool && arg.b) {
            c.fail(POSI_ERR_UNSUPPORTED, "LeconteChabrier2013(true) dynamical tides");
            return 0;
        }
        return POSI_EVO_LECONTE_CHABRIER2013;
    }
    c.fail(POSI_ERR_UNSUPPORTED, "evolution " + name + " (dynamical tides)");
    return 0;
}

bool zero_axes(Ctx& c, const json::Value* v) {
    double a[3];
    axes(c, v, "dangular_momentum_dt", a);
    return a[0] == 0. && a[1] == 0. && a[2] == 0.;
}

}  // namespace

int read_case(const json::Value& doc, FlatSystem& out, std::string& err) {
    Ctx c;
    if (!doc.is_object()) { err = "case is not a JSON object"; return POSI_ERR_PARSE; }
    // WHFast documents carry the alternative coordinates, Ias15 ones the
    // Gauss-Radau coefficients (src/integrator/ias15.rs:28-224)
    const bool ias15 = !doc.find("alternative_coordinates_type") && doc.find("b_0") &&
                       doc.find("time_step_last_success");
    if (!doc.find("alternative_coordinates_type") && !ias15) {
        err = "neither a WHFast nor an IAS15 case (LeapFrog is outside this path)";
        return POSI_ERR_UNSUPPORTED;
    }
    const json::Value* u = req(c, &doc, "universe");
    const json::Value* ce = req(c, u, "consider_effects");
    const int64_t n = (int64_t)num(c, u, "n_particles");
    if (c.code != POSI_OK) { err = c.err; return c.code; }
    if (n < 1 || n > POSI_MAX_BODIES) { err = "n_particles out of range"; return POSI_ERR_UNSUPPORTED; }
    const bool tides = boolean(c, ce, "tides");
    const bool flat = boolean(c, ce, "rotational_flattening");
    const bool gr = boolean(c, ce, "general_relativity");
    const bool disk = boolean(c, ce, "disk");
    const bool wind = boolean(c, ce, "wind");
    const bool evo = boolean(c, ce, "evolution");

    const json::Value* gri = req(c, u, "general_relativity_implementation");
    int gr_code = POSI_GR_KIDDER1995;
    std::string gr_name = gri && gri->is_string() ? gri->text : std::string();
    if (gr_name == "Anderson1975") gr_code = POSI_GR_ANDERSON1975;
    else if (gr_name == "Newhall1983") gr_code = POSI_GR_NEWHALL1983;
    else if (gr && gr_name != "Kidder1995") c.fail(POSI_ERR_UNSUPPORTED, "general relativity implementation " + gr_name);
    const json::Value* hosts = req(c, u, "hosts");
    const json::Value* hidx = req(c, hosts, "index");
    const int64_t host = (int64_t)num(c, hidx, "most_massive");
    if (tides && (int64_t)num(c, hidx, "tides") != host) c.fail(POSI_ERR_UNSUPPORTED, "tidal host is not the most massive body");
    if (flat && (int64_t)num(c, hidx, "rotational_flattening") != host)
        c.fail(POSI_ERR_UNSUPPORTED, "flattening host is not the most massive body");
    if (gr && (int64_t)num(c, hidx, "general_relativity") != host)
        c.fail(POSI_ERR_UNSUPPORTED, "general-relativity host is not the most massive body");
    if (disk && (int64_t)num(c, hidx, "disk") != host)
        c.fail(POSI_ERR_UNSUPPORTED, "disk host is not the most massive body");
    if (c.code != POSI_OK) { err = c.err; return c.code; }
    if (host < 0 || host >= n) { err = "host index out of range"; return POSI_ERR_PARSE; }

    out.n = n;
    out.si.assign(POSI_SI_COUNT, 0);
    out.sf.assign(POSI_SF_COUNT, 0.);
    out.bi.assign((size_t)n * POSI_BI_COUNT, 0);
    out.bf.assign((size_t)n * POSI_BF_COUNT, 0.);
    out.tables.clear();
    out.roche.assign((size_t)n * n, 0.);

    int coords = POSI_JACOBI;
    out.ias.assign((size_t)n * POSI_IAS_COUNT, 0.);
    if (!ias15) {
        const json::Value* act = req(c, &doc, "alternative_coordinates_type");
        coords = -1;
        if (act && act->is_string()) {
            if (act->text == "Jacobi") coords = POSI_JACOBI;
            else if (act->text == "DemocraticHeliocentric") coords = POSI_DEMOCRATIC_HELIOCENTRIC;
            else if (act->text == "WHDS") coords = POSI_WHDS;
        }
        if (coords < 0) { err = "unknown alternative_coordinates_type"; return POSI_ERR_PARSE; }
    } else {
        // the serde arrays hold 3 * MAX_PARTICLES values, body i component c at 3i + c
        struct Blk { int base; const char* name; };
        static const Blk blocks[] = {{POSI_IAS_B, "b"}, {POSI_IAS_E, "e"}, {POSI_IAS_BR, "br"},
                                     {POSI_IAS_ER, "er"}, {POSI_IAS_SB, "sb"}, {POSI_IAS_SE, "se"},
                                     {POSI_IAS_SBR, "sbr"}, {POSI_IAS_SER, "ser"}};
        auto arr3 = [&](const std::string& key, int base) {
            const json::Value* a = req(c, &doc, key.c_str());
            if (!a) return;
            if (!a->is_array() || (int64_t)a->items.size() < 3 * n) {
                c.fail(POSI_ERR_PARSE, "field '" + key + "' is shorter than 3 * n_particles");
                return;
            }
            for (int64_t b = 0; b < n; ++b)
                for (int k = 0; k < 3; ++k) {
                    const json::Value& x = a->items[(size_t)(3 * b + k)];
                    if (!x.is_number()) { c.fail(POSI_ERR_PARSE, "field '" + key + "' holds a non-number"); return; }
                    out.ias[(size_t)b * POSI_IAS_COUNT + base + k] = x.num();
                }
        };
        for (const Blk& bk : blocks)
            for (int j = 0; j < 7; ++j) arr3(std::string(bk.name) + "_" + std::to_string(j), bk.base + 3 * j);
        arr3("csx", POSI_IAS_CSX);
        arr3("csv", POSI_IAS_CSV);
        arr3("css", POSI_IAS_CSS);
        out.si[POSI_SI_INTEGRATOR] = POSI_INTEGRATOR_IAS15;
        out.si[POSI_SI_IAS_MAX_EXCEEDED] = (int64_t)num(c, &doc, "integrator_iterations_max_exceeded");
        out.sf[POSI_SF_IAS_DT_LAST] = num(c, &doc, "time_step_last_success");
        if (c.code != POSI_OK) { err = c.err; return c.code; }
    }
    out.si[POSI_SI_N] = n;
    out.si[POSI_SI_HOST] = host;
    out.si[POSI_SI_COORDS] = coords;
    out.si[POSI_SI_TIDES] = tides;
    out.si[POSI_SI_FLAT] = flat;
    out.si[POSI_SI_GR] = gr;
    out.si[POSI_SI_GR_IMPL] = gr_code;
    out.si[POSI_SI_WIND] = wind;
    out.si[POSI_SI_DISK] = disk;
    out.si[POSI_SI_EVOLUTION] = evo;
    out.si[POSI_SI_ITERATION] = (int64_t)num(c, &doc, "current_iteration");
    out.si[POSI_SI_N_HIST] = (int64_t)num(c, &doc, "n_historic_snapshots");
    if (!ias15) out.si[POSI_SI_TIMESTEP_WARNING] = (int64_t)num(c, &doc, "timestep_warning");
    out.sf[POSI_SF_DT] = num(c, &doc, "time_step");
    if (!ias15) out.sf[POSI_SF_HALF_DT] = num(c, &doc, "half_time_step");
    out.sf[POSI_SF_TIME] = num(c, &doc, "current_time");
    out.sf[POSI_SF_TIME_LIMIT] = num(c, u, "time_limit");
    out.sf[POSI_SF_LAST_HIST] = num(c, &doc, "last_historic_snapshot_time");
    out.sf[POSI_SF_HIST_PERIOD] = num(c, &doc, "historic_snapshot_period");
    out.sf[POSI_SF_LAST_REC] = num(c, &doc, "last_recovery_snapshot_time");
    out.sf[POSI_SF_REC_PERIOD] = num(c, &doc, "recovery_snapshot_period");
    out.sf[POSI_SF_INITIAL_TIME] = num(c, u, "initial_time");

    const json::Value* parts = req(c, u, "particles");
    const json::Value* evols = req(c, u, "particles_evolvers");
    const json::Value* verr = ias15 ? nullptr : req(c, &doc, "inertial_velocity_errors");
    const json::Value* lerr = ias15 ? nullptr : req(c, &doc, "particle_angular_momentum_errors");
    if (c.code != POSI_OK) { err = c.err; return c.code; }
    if (!parts->is_array() || (int64_t)parts->items.size() < n || !evols->is_array() ||
        (int64_t)evols->items.size() < n ||
        (!ias15 && (!verr->is_array() || (int64_t)verr->items.size() < n || !lerr->is_array() ||
                    (int64_t)lerr->items.size() < n))) {
        err = "particle arrays shorter than n_particles";
        return POSI_ERR_PARSE;
    }
    for (int64_t b = 0; b < n; ++b) {
        const json::Value& p = parts->items[b];
        const json::Value& ev = evols->items[b];
        int64_t* I = &out.bi[(size_t)b * POSI_BI_COUNT];
        double* F = &out.bf[(size_t)b * POSI_BF_COUNT];
        const json::Value* tides_v = req(c, &p, "tides");
        const json::Value* flat_v = req(c, &p, "rotational_flattening");
        const json::Value* gr_v = req(c, &p, "general_relativity");
        const json::Value *tparams = nullptr, *fparams = nullptr, *gparams = nullptr;
        std::string gr_impl;
        const int tk = effect_kind(c, req(c, tides_v, "effect"), "ConstantTimeLag", &tparams);
        const int fk = effect_kind(c, req(c, flat_v, "effect"), "OblateSpheroid", &fparams);
        const int gk = effect_kind(c, req(c, gr_v, "effect"), nullptr, &gparams, &gr_impl);
        if (c.code != POSI_OK) { err = c.err; return c.code; }
        if (gr && gk == POSI_EFFECT_CENTRAL && gr_impl != gr_name)
            c.fail(POSI_ERR_UNSUPPORTED, "general-relativity host " + gr_impl + " differs from the universe's " + gr_name);
        if (tides && b != host && tk != POSI_EFFECT_ORBITING)
            c.fail(POSI_ERR_UNSUPPORTED, "tides on with a non-orbiting body (the reference's host torque is NaN)");
        if (tides && b == host && tk != POSI_EFFECT_CENTRAL) c.fail(POSI_ERR_UNSUPPORTED, "tidal host is not a central body");
        if (flat && b == host && fk != POSI_EFFECT_CENTRAL) c.fail(POSI_ERR_UNSUPPORTED, "flattening host is not a central body");
        if (gr && b == host && gk != POSI_EFFECT_CENTRAL) c.fail(POSI_ERR_UNSUPPORTED, "GR host is not a central body");
        // Outputs of effects that are off (or of bodies outside an effect) are
        // summed by the reference as they stand; they must be zero here.
        const json::Value* tout = req(c, req(c, tides_v, "parameters"), "output");
        const json::Value* fout = req(c, req(c, flat_v, "parameters"), "output");
        const json::Value* gout = req(c, req(c, gr_v, "parameters"), "output");
        if ((!tides || (b != host && tk != POSI_EFFECT_ORBITING)) && !zero_axes(c, tout))
            c.fail(POSI_ERR_UNSUPPORTED, "stale tidal torque output");
        if ((!flat || (b != host && fk != POSI_EFFECT_ORBITING)) && !zero_axes(c, fout))
            c.fail(POSI_ERR_UNSUPPORTED, "stale flattening torque output");
        if ((!gr || (b != host && gk != POSI_EFFECT_ORBITING)) && !zero_axes(c, gout))
            c.fail(POSI_ERR_UNSUPPORTED, "stale general-relativity torque output");
        // wind (src/effects/wind.rs): "Interaction" or "Disabled"; its torque
        // output is summed whatever the flags (src/particles/universe.rs:589-591)
        const json::Value* wind_v = req(c, &p, "wind");
        const json::Value* weff = req(c, wind_v, "effect");
        if (c.code != POSI_OK) { err = c.err; return c.code; }
        int wk = 0;
        if (weff->is_string() && weff->text == "Interaction") wk = 1;
        else if (!(weff->is_string() && weff->text == "Disabled")) c.fail(POSI_ERR_UNSUPPORTED, "unknown wind effect");
        const json::Value* wpar = req(c, wind_v, "parameters");
        if (!(wind && wk) && !zero_axes(c, req(c, wpar, "output")))
            c.fail(POSI_ERR_UNSUPPORTED, "stale wind torque output");
        I[POSI_BI_WIND_KIND] = wk;
        // disk (src/effects/disk.rs:43-47): "Disabled", "OrbitingBody" or
        // {"CentralBody": DiskProperties}
        {
            const json::Value* deff = req(c, req(c, &p, "disk"), "effect");
            if (c.code != POSI_OK) { err = c.err; return c.code; }
            int dk = POSI_EFFECT_DISABLED;
            if (deff->is_string()) {
                if (deff->text == "OrbitingBody") dk = POSI_EFFECT_ORBITING;
                else if (deff->text != "Disabled") c.fail(POSI_ERR_PARSE, "unknown disk effect " + deff->text);
            } else if (deff->is_object() && deff->members.size() == 1 && deff->members[0].first == "CentralBody") {
                dk = POSI_EFFECT_CENTRAL;
                const json::Value* dp = &deff->members[0].second;
                F[POSI_BF_DISK_INNER] = num(c, dp, "inner_edge_distance");
                F[POSI_BF_DISK_OUTER] = num(c, dp, "outer_edge_distance");
                F[POSI_BF_DISK_LIFETIME] = num(c, dp, "lifetime");
                F[POSI_BF_DISK_ALPHA] = num(c, dp, "alpha");
                F[POSI_BF_DISK_SIGMA0] = num(c, dp, "surface_density_normalization");
                F[POSI_BF_DISK_MU] = num(c, dp, "mean_molecular_weight");
            } else {
                c.fail(POSI_ERR_PARSE, "malformed disk effect");
            }
            if (disk && b == host && dk != POSI_EFFECT_CENTRAL) c.fail(POSI_ERR_UNSUPPORTED, "disk host is not a central body");
            I[POSI_BI_DISK_KIND] = dk;
            F[POSI_BF_DISK_MTS] = num(c, req(c, req(c, req(c, &p, "disk"), "parameters"), "internal"), "migration_timescale");
        }
        F[POSI_BF_WIND_K] = num(c, req(c, wpar, "input"), "k_factor");
        F[POSI_BF_WIND_RSAT] = num(c, req(c, wpar, "input"), "rotation_saturation");
        F[POSI_BF_WIND_RSAT2] = num(c, req(c, wpar, "internal"), "rotation_saturation_2");
        if (b == host) {
            double hv[3];
            axes(c, &p, "heliocentric_velocity", hv);
            if (hv[0] != 0. || hv[1] != 0. || hv[2] != 0.)
                c.fail(POSI_ERR_UNSUPPORTED, "host with a non-zero heliocentric velocity");
        }
        const int evo_p = evolution_code(c, req(c, &p, "evolution"));
        const int evo_e = evolution_code(c, req(c, &ev, "evolution"));
        if (c.code != POSI_OK) { err = c.err; return c.code; }
        if (evo_p != evo_e) { err = "particle and evolver evolution types differ"; return POSI_ERR_UNSUPPORTED; }
        I[POSI_BI_TIDES_KIND] = tk;
        I[POSI_BI_FLAT_KIND] = fk;
        I[POSI_BI_GR_KIND] = gk;
        const bool dynamical = evo_p == POSI_EVO_BOLMONT_MATHIS2016 || evo_p == POSI_EVO_GALLET_BOLMONT2017;
        if (dynamical && (b != host || !tides || tk != POSI_EFFECT_CENTRAL)) {
            // the planet-dependent branch keeps stale entries in the reference
            // (src/effects/tides/constant_time_lag.rs:131-135 removes the host's key)
            err = "dynamical-tide evolution on a body other than the tidal host";
            return POSI_ERR_UNSUPPORTED;
        }
        I[POSI_BI_EVO_TYPE] = evo_p;
        I[POSI_BI_EVO_LEFT] = (int64_t)num(c, &ev, "left_index");
        const json::Value* tt = req(c, &ev, "time");
        if (c.code != POSI_OK) { err = c.err; return c.code; }
        const int64_t rows = tt->is_array() ? (int64_t)tt->items.size() : 0;
        if (evo_p != POSI_EVO_NON_EVOLVING && rows > 0) {
            const size_t off = out.tables.size();
            out.tables.resize(off + 4 * (size_t)rows, 0.);
            // the dynamical-tide evolutions interpolate no Love number: their
            // 4th column holds the inverse tidal Q factor
            const char* names[4] = {"time", "radius", "radius_of_gyration_2",
                                    dynamical ? "inverse_tidal_q_factor" : "love_number"};
            for (int k = 0; k < 4; ++k) {
                const json::Value* col = req(c, &ev, names[k]);
                if (!col || !col->is_array()) continue;
                if ((int64_t)col->items.size() == rows) {
                    for (int64_t r = 0; r < rows; ++r) out.tables[off + (size_t)k * rows + r] = col->items[r].num();
                } else if (k < 2 && !col->items.empty()) {
                    err = "evolution table columns of different lengths";
                    return POSI_ERR_PARSE;
                }
            }
            I[POSI_BI_EVO_OFFSET] = (int64_t)off;
            I[POSI_BI_EVO_LEN] = rows;
        }
        F[POSI_BF_MASS] = num(c, &p, "mass");
        F[POSI_BF_MASS_G] = num(c, &p, "mass_g");
        F[POSI_BF_RADIUS] = num(c, &p, "radius");
        F[POSI_BF_RG2] = num(c, &p, "radius_of_gyration_2");
        F[POSI_BF_MOI] = num(c, &p, "moment_of_inertia");
        axes(c, &p, "inertial_position", &F[POSI_BF_PX]);
        axes(c, &p, "inertial_velocity", &F[POSI_BF_VX]);
        axes(c, &p, "inertial_acceleration", &F[POSI_BF_AX]);
        axes(c, &p, "angular_momentum", &F[POSI_BF_LX]);
        axes(c, &p, "spin", &F[POSI_BF_SX]);
        F[POSI_BF_NSV2] = num(c, &p, "norm_spin_vector_2");
        if (!ias15) {
            const json::Value& ve = verr->items[b];
            const json::Value& le = lerr->items[b];
            F[POSI_BF_EVX] = num(c, &ve, "x"); F[POSI_BF_EVY] = num(c, &ve, "y"); F[POSI_BF_EVZ] = num(c, &ve, "z");
            F[POSI_BF_ELX] = num(c, &le, "x"); F[POSI_BF_ELY] = num(c, &le, "y"); F[POSI_BF_ELZ] = num(c, &le, "z");
        }
        axes(c, &p, "inertial_additional_acceleration", &F[POSI_BF_ADDAX]);
        axes(c, &p, "dangular_momentum_dt", &F[POSI_BF_DLX]);
        const json::Value* tint = req(c, req(c, tides_v, "parameters"), "internal");
        F[POSI_BF_SIGMA] = num(c, tint, "scaled_dissipation_factor");
        F[POSI_BF_DENERGY_DT] = num(c, tint, "denergy_dt");
        F[POSI_BF_LAG_ANGLE] = num(c, tint, "lag_angle");
        F[POSI_BF_TD_DIST] = num(c, tint, "distance");
        F[POSI_BF_TD_VR] = num(c, tint, "radial_velocity");
        F[POSI_BF_TD_ORTHO] = num(c, tint, "orthogonal_component_of_the_tidal_force_due_to_planetary_tide");
        F[POSI_BF_TD_DPM] = num(c, tint, "radial_component_of_the_tidal_force_dissipative_part_when_star_as_point_mass");
        {
            const json::Value* tco = req(c, tides_v, "coordinates");
            axes(c, tco, "position", &F[POSI_BF_TD_PX]);
            axes(c, tco, "velocity", &F[POSI_BF_TD_VX]);
            axes(c, tout, "dangular_momentum_dt", &F[POSI_BF_TD_LX]);
        }
        F[POSI_BF_K2] = tparams ? num(c, tparams, "love_number") : 0.;
        F[POSI_BF_DISS_FACTOR] = tparams ? num(c, tparams, "dissipation_factor") : 0.;
        F[POSI_BF_DISS_SCALE] = tparams ? num(c, tparams, "dissipation_factor_scale") : 0.;
        F[POSI_BF_K2F] = fparams ? num(c, fparams, "love_number") : 0.;
        if (c.code != POSI_OK) { err = c.err; return c.code; }
    }
    // calculate_roche_radiuses fills the first n*n entries in rows of n
    // (src/particles/universe.rs:177-196)
    const json::Value* rr = u->find("roche_radiuses");
    if (rr && rr->is_array() && (int64_t)rr->items.size() >= n * n) {
        for (int64_t k = 0; k < n * n; ++k) out.roche[(size_t)k] = rr->items[(size_t)k].num();
    }
    if (c.code != POSI_OK) { err = c.err; return c.code; }
    return POSI_OK;
}

}  // namespace posi
