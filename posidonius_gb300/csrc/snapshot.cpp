// snapshot.cpp -- see snapshot.hpp.
#include "snapshot.hpp"

#include <cmath>
#include <cstdlib>
#include <cstring>

namespace posi {

std::string format_double(double v) {
    if (!std::isfinite(v)) return "null";  // serde_json writes non-finite floats as null
    char buf[40];
    for (int prec = 1; prec <= 17; ++prec) {
        std::snprintf(buf, sizeof buf, "%.*g", prec, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    std::string s(buf);
    if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
    return s;
}

namespace {

void indent_to(std::string& out, int n) { out.append((size_t)n, ' '); }

void write_string(const std::string& s, std::string& out) {
    out += '"';
    for (unsigned char c : s) {
        switch (c) {
            case '"': out += "\\\""; break;
            case '\\': out += "\\\\"; break;
            case '\n': out += "\\n"; break;
            case '\r': out += "\\r"; break;
            case '\t': out += "\\t"; break;
            default:
                if (c < 0x20) {
                    char b[8];
                    std::snprintf(b, sizeof b, "\\u%04x", c);
                    out += b;
                } else {
                    out += (char)c;
                }
        }
    }
    out += '"';
}

void set_number(json::Value& v, double x) {
    if (!std::isfinite(x)) { v.kind = json::Value::Null; v.text.clear(); return; }
    v.kind = json::Value::Number;
    v.text = format_double(x);
}

void set_integer(json::Value& v, int64_t x) {
    v.kind = json::Value::Number;
    v.text = std::to_string(x);
}

json::Value* member(json::Value* v, const char* key) {
    if (!v || v->kind != json::Value::Object) return nullptr;
    for (auto& m : v->members)
        if (m.first == key) return &m.second;
    return nullptr;
}

bool set_axes(json::Value* v, const double* a) {
    json::Value *x = member(v, "x"), *y = member(v, "y"), *z = member(v, "z");
    if (!x || !y || !z) return false;
    set_number(*x, a[0]);
    set_number(*y, a[1]);
    set_number(*z, a[2]);
    return true;
}

}  // namespace

void write_json(const json::Value& v, std::string& out, int indent) {
    switch (v.kind) {
        case json::Value::Null: out += "null"; break;
        case json::Value::Bool: out += v.b ? "true" : "false"; break;
        case json::Value::Number: out += v.text; break;
        case json::Value::String: write_string(v.text, out); break;
        case json::Value::Array:
            if (v.items.empty()) { out += "[]"; break; }
            out += "[\n";
            for (size_t k = 0; k < v.items.size(); ++k) {
                indent_to(out, indent + 2);
                write_json(v.items[k], out, indent + 2);
                out += k + 1 < v.items.size() ? ",\n" : "\n";
            }
            indent_to(out, indent);
            out += "]";
            break;
        case json::Value::Object:
            if (v.members.empty()) { out += "{}"; break; }
            out += "{\n";
            for (size_t k = 0; k < v.members.size(); ++k) {
                indent_to(out, indent + 2);
                write_string(v.members[k].first, out);
                out += ": ";
                write_json(v.members[k].second, out, indent + 2);
                out += k + 1 < v.members.size() ? ",\n" : "\n";
            }
            indent_to(out, indent);
            out += "}";
            break;
    }
}

bool update_case_document(json::Value& doc, int64_t n, const int64_t* si, const double* sf, const int64_t* bi,
                          const double* bf, const double* roche, const double* ias, std::string& err) {
    auto need = [&](json::Value* v, const char* what) {
        if (!v) err = std::string("case document lacks ") + what;
        return v != nullptr;
    };
    json::Value* u = member(&doc, "universe");
    if (!need(u, "universe")) return false;
    struct F { const char* key; double v; };
    const F f64s[] = {{"current_time", sf[POSI_SF_TIME]},
                      {"last_recovery_snapshot_time", sf[POSI_SF_LAST_REC]},
                      {"last_historic_snapshot_time", sf[POSI_SF_LAST_HIST]},
                      {"historic_snapshot_period", sf[POSI_SF_HIST_PERIOD]},
                      {"recovery_snapshot_period", sf[POSI_SF_REC_PERIOD]}};
    for (const F& f : f64s) {
        json::Value* v = member(&doc, f.key);
        if (!need(v, f.key)) return false;
        set_number(*v, f.v);
    }
    const bool ias15 = si[POSI_SI_INTEGRATOR] == POSI_INTEGRATOR_IAS15;
    struct I { const char* key; int64_t v; };
    const I i64s[] = {{"current_iteration", si[POSI_SI_ITERATION]},
                      {"n_historic_snapshots", si[POSI_SI_N_HIST]},
                      {ias15 ? "integrator_iterations_max_exceeded" : "timestep_warning",
                       ias15 ? si[POSI_SI_IAS_MAX_EXCEEDED] : si[POSI_SI_TIMESTEP_WARNING]},
                      {"hash", 0}};
    for (const I& f : i64s) {
        json::Value* v = member(&doc, f.key);
        if (!need(v, f.key)) return false;
        set_integer(*v, f.v);
    }
    if (ias15) {
        // src/integrator/ias15.rs:28-224: the adaptive step and the per-body
        // Gauss-Radau state that carries over to the next step (the arrays
        // hold 3 * MAX_PARTICLES values, body i component c at 3i + c; the
        // scratch arrays g, at, x0, v0, a0, ... are rewritten by every step
        // and keep the values the document had)
        const F fs[] = {{"time_step", sf[POSI_SF_DT]}, {"time_step_last_success", sf[POSI_SF_IAS_DT_LAST]}};
        for (const F& f : fs) {
            json::Value* v = member(&doc, f.key);
            if (!need(v, f.key)) return false;
            set_number(*v, f.v);
        }
        if (!ias) { err = "IAS15 state missing"; return false; }
        struct Blk { int base; const char* name; };
        static const Blk blocks[] = {{POSI_IAS_B, "b"}, {POSI_IAS_E, "e"}, {POSI_IAS_BR, "br"},
                                     {POSI_IAS_ER, "er"}, {POSI_IAS_SB, "sb"}, {POSI_IAS_SE, "se"},
                                     {POSI_IAS_SBR, "sbr"}, {POSI_IAS_SER, "ser"}};
        auto put = [&](const std::string& key, int base) {
            json::Value* a = member(&doc, key.c_str());
            if (!a || a->kind != json::Value::Array || (int64_t)a->items.size() < 3 * n) {
                err = "case document lacks " + key;
                return false;
            }
            for (int64_t b = 0; b < n; ++b)
                for (int k = 0; k < 3; ++k)
                    set_number(a->items[(size_t)(3 * b + k)], ias[(size_t)b * POSI_IAS_COUNT + base + k]);
            return true;
        };
        for (const Blk& bk : blocks)
            for (int j = 0; j < 7; ++j)
                if (!put(std::string(bk.name) + "_" + std::to_string(j), bk.base + 3 * j)) return false;
        if (!put("csx", POSI_IAS_CSX) || !put("csv", POSI_IAS_CSV) || !put("css", POSI_IAS_CSS)) return false;
    }
    json::Value* tl = member(u, "time_limit");
    if (!need(tl, "time_limit")) return false;
    set_number(*tl, sf[POSI_SF_TIME_LIMIT]);
    json::Value* parts = member(u, "particles");
    json::Value* evols = member(u, "particles_evolvers");
    json::Value* verr = ias15 ? nullptr : member(&doc, "inertial_velocity_errors");
    json::Value* lerr = ias15 ? nullptr : member(&doc, "particle_angular_momentum_errors");
    if (!need(parts, "particles") || !need(evols, "particles_evolvers") ||
        (!ias15 && (!need(verr, "inertial_velocity_errors") || !need(lerr, "particle_angular_momentum_errors"))))
        return false;
    for (int64_t b = 0; b < n; ++b) {
        const double* F = bf + (size_t)b * POSI_BF_COUNT;
        json::Value* p = &parts->items[(size_t)b];
        const struct { const char* key; int field; } vecs[] = {
            {"inertial_position", POSI_BF_PX}, {"inertial_velocity", POSI_BF_VX},
            {"inertial_acceleration", POSI_BF_AX}, {"inertial_additional_acceleration", POSI_BF_ADDAX},
            {"angular_momentum", POSI_BF_LX}, {"spin", POSI_BF_SX}, {"dangular_momentum_dt", POSI_BF_DLX}};
        for (const auto& v : vecs)
            if (!set_axes(member(p, v.key), F + v.field)) { err = std::string("particle lacks ") + v.key; return false; }
        const struct { const char* key; int field; } scal[] = {
            {"norm_spin_vector_2", POSI_BF_NSV2}, {"radius", POSI_BF_RADIUS},
            {"radius_of_gyration_2", POSI_BF_RG2}, {"moment_of_inertia", POSI_BF_MOI}};
        for (const auto& v : scal) {
            json::Value* x = member(p, v.key);
            if (!need(x, v.key)) return false;
            set_number(*x, F[v.field]);
        }
        json::Value* tides = member(p, "tides");
        json::Value* tint = member(member(tides, "parameters"), "internal");
        json::Value* tout = member(member(tides, "parameters"), "output");
        json::Value* tco = member(tides, "coordinates");
        if (!need(tint, "tides internals") || !need(tout, "tides outputs") || !need(tco, "tides coordinates"))
            return false;
        const struct { const char* key; int field; } tsc[] = {
            {"denergy_dt", POSI_BF_DENERGY_DT}, {"lag_angle", POSI_BF_LAG_ANGLE}, {"distance", POSI_BF_TD_DIST},
            {"radial_velocity", POSI_BF_TD_VR},
            {"orthogonal_component_of_the_tidal_force_due_to_planetary_tide", POSI_BF_TD_ORTHO},
            {"radial_component_of_the_tidal_force_dissipative_part_when_star_as_point_mass", POSI_BF_TD_DPM}};
        for (const auto& v : tsc) {
            json::Value* x = member(tint, v.key);
            if (!need(x, v.key)) return false;
            set_number(*x, F[v.field]);
        }
        if (!set_axes(member(tco, "position"), F + POSI_BF_TD_PX) || !set_axes(member(tco, "velocity"), F + POSI_BF_TD_VX) ||
            !set_axes(member(tout, "dangular_momentum_dt"), F + POSI_BF_TD_LX)) {
            err = "tides coordinates";
            return false;
        }
        // the disk's migration timescale of the last evaluation (read by the
        // historic records)
        {
            json::Value* dint = member(member(member(p, "disk"), "parameters"), "internal");
            json::Value* mts = dint ? member(dint, "migration_timescale") : nullptr;
            if (mts) set_number(*mts, F[POSI_BF_DISK_MTS]);
        }
        if (!ias15 &&
            (!set_axes(&verr->items[(size_t)b], F + POSI_BF_EVX) || !set_axes(&lerr->items[(size_t)b], F + POSI_BF_ELX))) {
            err = "Kahan error arrays";
            return false;
        }
        json::Value* li = member(&evols->items[(size_t)b], "left_index");
        if (!need(li, "left_index")) return false;
        set_integer(*li, bi[(size_t)b * POSI_BI_COUNT + POSI_BI_EVO_LEFT]);
    }
    json::Value* rr = member(u, "roche_radiuses");
    if (roche && rr && rr->kind == json::Value::Array && (int64_t)rr->items.size() >= n * n) {
        for (int64_t k = 0; k < n * n; ++k) set_number(rr->items[(size_t)k], roche[k]);
    }
    return true;
}

void encode_history_record(const double* rec, int64_t n, std::vector<unsigned char>& out) {
    auto put_f64 = [&](double x) {
        unsigned char b[8];
        std::memcpy(b, &x, 8);  // little-endian on every supported host
        out.insert(out.end(), b, b + 8);
    };
    for (int64_t b = 0; b < n; ++b) {
        const double* R = rec + (size_t)b * kHistoryFields;
        put_f64(R[0]);
        put_f64(R[1]);
        const int32_t id = (int32_t)R[2];
        unsigned char ib[4];
        std::memcpy(ib, &id, 4);
        out.insert(out.end(), ib, ib + 4);
        for (int k = 3; k < kHistoryFields; ++k) put_f64(R[k]);
    }
}

}  // namespace posi
