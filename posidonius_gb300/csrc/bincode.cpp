// bincode.cpp -- bincode <-> JSON document codec of the recovery snapshots.
//
// The types of the reference's WHFast and Ias15 snapshots are written down
// once, below, in a small schema notation (their field order, widths and
// enum variant order are the format: src/integrator/whfast.rs:91-130,
// src/integrator/ias15.rs:30-125, src/particles/{universe,particle,axes}.rs,
// src/effects/{tides/common,tides/constant_time_lag,rotational_flattening/
// common,rotational_flattening/oblate_spheroid,general_relativity,wind,disk,
// evolution}.rs).  One walker encodes a JSON document by the schema, one
// decodes bytes into a JSON document.
#include "bincode.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "snapshot.hpp"

namespace posi {
namespace {

// ---- schema ----------------------------------------------------------------
//   Name = { field: Type; ... }          struct
//   Name = < Unit | Newtype(Type) >      enum, variants in declaration order
//   Types: f64 usize u64 u32 i32 bool, [Type; N], Vec<Type>, Map<Key, Value>,
//   a Name, or ! (a payload this library does not support).
std::string schema_text() {
    std::string s = R"(
Axes = { x: f64; y: f64; z: f64; }
Reference = < MostMassiveParticle | Particle(usize) >

ConstantTimeLagParameters = { dissipation_factor: f64; dissipation_factor_scale: f64; love_number: f64; }
TidalModel = < ConstantTimeLag(ConstantTimeLagParameters) | CreepCoplanar(!) | Kaula(!) >
TidesEffect = < CentralBody(TidalModel) | OrbitingBody(TidalModel) | Disabled >
TidesInternal = { distance: f64; radial_velocity: f64; scaled_dissipation_factor: f64;
    scalar_product_of_vector_position_with_stellar_spin: f64;
    scalar_product_of_vector_position_with_planetary_spin: f64;
    orthogonal_component_of_the_tidal_force_due_to_stellar_tide: f64;
    orthogonal_component_of_the_tidal_force_due_to_planetary_tide: f64;
    radial_component_of_the_tidal_force: f64;
    radial_component_of_the_tidal_force_dissipative_part_when_star_as_point_mass: f64;
    shape: Axes; denergy_dt: f64; lag_angle: f64; }
AccelerationAndTorque = { acceleration: Axes; dangular_momentum_dt: Axes; }
TidesParameters = { internal: TidesInternal; output: AccelerationAndTorque; }
PositionVelocity = { position: Axes; velocity: Axes; }
Tides = { effect: TidesEffect; parameters: TidesParameters; coordinates: PositionVelocity; }

OblateSpheroidParameters = { love_number: f64; }
FlatteningModel = < OblateSpheroid(OblateSpheroidParameters) | CreepCoplanar(!) >
FlatteningEffect = < CentralBody(FlatteningModel) | OrbitingBody(FlatteningModel) | Disabled >
FlatteningInternal = { distance: f64; scalar_product_of_vector_position_with_stellar_spin: f64;
    scalar_product_of_vector_position_with_planetary_spin: f64;
    radial_component_of_the_force_induced_by_rotation: f64;
    factor_for_the_force_induced_by_star_rotation: f64;
    factor_for_the_force_induced_by_planet_rotation: f64;
    orthogonal_component_of_the_force_induced_by_star_rotation: f64;
    orthogonal_component_of_the_force_induced_by_planet_rotation: f64;
    shape: Axes; }
FlatteningParameters = { internal: FlatteningInternal; output: AccelerationAndTorque; }
RotationalFlattening = { effect: FlatteningEffect; parameters: FlatteningParameters; coordinates: PositionVelocity; }

GrImplementation = < Kidder1995 | Anderson1975 | Newhall1983 | Disabled >
GrEffect = < CentralBody(GrImplementation) | OrbitingBody | Disabled >
GrInternal = { distance: f64; radial_velocity: f64; norm_velocity_vector: f64; norm_velocity_vector_2: f64;
    factor: f64; }
GrParameters = { internal: GrInternal; output: AccelerationAndTorque; }
GeneralRelativity = { effect: GrEffect; parameters: GrParameters; coordinates: PositionVelocity; }

WindEffect = < Interaction | Disabled >
WindInput = { k_factor: f64; rotation_saturation: f64; }
WindInternal = { rotation_saturation_2: f64; }
WindOutput = { dangular_momentum_dt: Axes; }
WindParameters = { input: WindInput; internal: WindInternal; output: WindOutput; }
Wind = { effect: WindEffect; parameters: WindParameters; }

DiskProperties = { inner_edge_distance: f64; outer_edge_distance: f64; lifetime: f64; alpha: f64;
    surface_density_normalization: f64; mean_molecular_weight: f64; }
DiskEffect = < CentralBody(DiskProperties) | OrbitingBody | Disabled >
DiskInternal = { distance: f64; norm_velocity_vector: f64; norm_velocity_vector_2: f64; migration_timescale: f64; }
DiskOutput = { acceleration: Axes; }
DiskParameters = { internal: DiskInternal; output: DiskOutput; }
Disk = { effect: DiskEffect; parameters: DiskParameters; coordinates: PositionVelocity; }

EvolutionType = < GalletBolmont2017(f64) | BolmontMathis2016(f64) | Baraffe2015(f64) | Leconte2011(f64)
    | Baraffe1998(f64) | LeconteChabrier2013(bool) | NonEvolving >
Evolver = { evolution: EvolutionType; time: Vec<f64>; radius: Vec<f64>; radius_of_gyration_2: Vec<f64>;
    love_number: Vec<f64>; inverse_tidal_q_factor: Vec<f64>; left_index: usize; }

Particle = { id: usize; mass: f64; mass_g: f64; radius: f64;
    inertial_position: Axes; inertial_velocity: Axes; inertial_acceleration: Axes;
    inertial_additional_acceleration: Axes; heliocentric_position: Axes; heliocentric_velocity: Axes;
    heliocentric_distance: f64; heliocentric_radial_velocity: f64; heliocentric_norm_velocity_vector: f64;
    heliocentric_norm_velocity_vector_2: f64; spin: Axes; norm_spin_vector_2: f64; angular_momentum: Axes;
    dangular_momentum_dt: Axes; radius_of_gyration_2: f64; moment_of_inertia: f64; reference: Reference;
    tides: Tides; rotational_flattening: RotationalFlattening; general_relativity: GeneralRelativity;
    wind: Wind; disk: Disk; evolution: EvolutionType; }

HostIndices = { most_massive: usize; tides: usize; rotational_flattening: usize; general_relativity: usize;
    disk: usize; }
HostMostMassive = { all: bool; general_relativity: bool; tides: bool; rotational_flattening: bool; disk: bool; }
Hosts = { index: HostIndices; most_massive: HostMostMassive; }
ConsiderEffects = { tides: bool; rotational_flattening: bool; general_relativity: bool; disk: bool; wind: bool;
    evolution: bool; }
Universe = { initial_time: f64; time_limit: f64; particles: [Particle; 10]; particles_evolvers: Vec<Evolver>;
    n_particles: usize; consider_effects: ConsiderEffects; general_relativity_implementation: GrImplementation;
    hosts: Hosts; pair_dependent_scaled_dissipation_factor: Map<usize, f64>; roche_radiuses: [f64; 100]; }

CoordinatesType = < Jacobi | DemocraticHeliocentric | WHDS >
AlternativeCoordinates = { mass: f64; mass_g: f64; position: Axes; velocity: Axes; acceleration: Axes; }
WHFast = { time_step: f64; half_time_step: f64; universe: Universe; current_time: f64; current_iteration: usize;
    recovery_snapshot_period: f64; historic_snapshot_period: f64; last_recovery_snapshot_time: f64;
    last_historic_snapshot_time: f64; n_historic_snapshots: usize; hash: u64;
    particles_alternative_coordinates: [AlternativeCoordinates; 10]; alternative_coordinates_type: CoordinatesType;
    timestep_warning: usize; inertial_velocity_errors: [Axes; 10]; particle_angular_momentum_errors: [Axes; 10]; }
)";
    // Ias15: scalars, then its per-coordinate arrays of 3 x 10 doubles (the
    // seven coefficients of b, br, g, e, er, four buffers, the seven of the
    // spin forms sb, sbr, sg, se, ser, three torque / spin buffers, the
    // compensated-sum terms) and the nine summation coefficients
    s += "Ias15 = { time_step: f64; universe: Universe; current_time: f64; current_iteration: u32;\n"
         "    recovery_snapshot_period: f64; historic_snapshot_period: f64; last_recovery_snapshot_time: f64;\n"
         "    last_historic_snapshot_time: f64; n_historic_snapshots: usize; hash: u64; n_particles: usize;\n"
         "    integrator_iterations_max_exceeded: i32; time_step_last_success: f64;\n";
    auto seven = [&](const char* p) {
        for (int k = 0; k < 7; ++k) s += std::string("    ") + p + "_" + std::to_string(k) + ": [f64; 30];\n";
    };
    for (const char* p : {"b", "br", "g", "e", "er"}) seven(p);
    for (const char* p : {"at", "x0", "v0", "a0"}) s += std::string("    ") + p + ": [f64; 30];\n";
    for (const char* p : {"sb", "sbr", "sg", "se", "ser"}) seven(p);
    for (const char* p : {"dangular_momentum_dtt", "dangular_momentum_dt0", "angular_momentum0", "csx", "csv", "css"})
        s += std::string("    ") + p + ": [f64; 30];\n";
    s += "    s: [f64; 9]; }\n";
    return s;
}

struct Type;
using TypeP = std::shared_ptr<Type>;
struct Type {
    enum Kind { F64, U64, U32, I32, Bool, Array, Vec, Map, Named, Unsupported } kind = F64;
    int64_t n = 0;         // Array length
    TypeP a, b;            // element / key, value
    std::string name;      // Named
};
struct Field {
    std::string name;
    TypeP type;            // null: unit variant
};
struct Def {
    bool is_enum = false;
    std::vector<Field> fields;  // struct fields or enum variants
};

class Schema {
public:
    std::map<std::string, Def> defs;
    std::string error;

    bool parse(const std::string& text) {
        s_ = text.c_str();
        for (;;) {
            ws();
            if (!*s_) return true;
            std::string name = ident();
            if (name.empty() || !expect('=')) return fail("definition");
            ws();
            Def d;
            if (*s_ == '{') {
                ++s_;
                for (;;) {
                    ws();
                    if (*s_ == '}') { ++s_; break; }
                    Field f;
                    f.name = ident();
                    if (f.name.empty() || !expect(':')) return fail("field of " + name);
                    f.type = type();
                    if (!f.type || !expect(';')) return fail("field type of " + name);
                    d.fields.push_back(f);
                }
            } else if (*s_ == '<') {
                ++s_;
                d.is_enum = true;
                for (;;) {
                    Field v;
                    v.name = ident();
                    if (v.name.empty()) return fail("variant of " + name);
                    ws();
                    if (*s_ == '(') {
                        ++s_;
                        v.type = type();
                        if (!v.type || !expect(')')) return fail("variant payload of " + name);
                    }
                    d.fields.push_back(v);
                    ws();
                    if (*s_ == '|') { ++s_; continue; }
                    if (*s_ == '>') { ++s_; break; }
                    return fail("variant list of " + name);
                }
            } else {
                return fail("body of " + name);
            }
            defs[name] = d;
        }
    }

private:
    const char* s_ = nullptr;
    bool fail(const std::string& what) { error = "schema: " + what; return false; }
    void ws() { while (*s_ == ' ' || *s_ == '\n' || *s_ == '\t' || *s_ == '\r') ++s_; }
    bool expect(char c) { ws(); if (*s_ != c) return false; ++s_; return true; }
    std::string ident() {
        ws();
        const char* b = s_;
        while ((*s_ >= 'a' && *s_ <= 'z') || (*s_ >= 'A' && *s_ <= 'Z') || (*s_ >= '0' && *s_ <= '9') || *s_ == '_') ++s_;
        return std::string(b, s_);
    }
    TypeP type() {
        ws();
        auto t = std::make_shared<Type>();
        if (*s_ == '!') { ++s_; t->kind = Type::Unsupported; return t; }
        if (*s_ == '[') {
            ++s_;
            t->kind = Type::Array;
            t->a = type();
            if (!t->a || !expect(';')) return nullptr;
            ws();
            t->n = std::strtoll(s_, const_cast<char**>(&s_), 10);
            if (t->n <= 0 || !expect(']')) return nullptr;
            return t;
        }
        const std::string id = ident();
        if (id == "f64") t->kind = Type::F64;
        else if (id == "usize" || id == "u64") t->kind = Type::U64;
        else if (id == "u32") t->kind = Type::U32;
        else if (id == "i32") t->kind = Type::I32;
        else if (id == "bool") t->kind = Type::Bool;
        else if (id == "Vec") {
            t->kind = Type::Vec;
            if (!expect('<') || !(t->a = type()) || !expect('>')) return nullptr;
        } else if (id == "Map") {
            t->kind = Type::Map;
            if (!expect('<') || !(t->a = type()) || !expect(',') || !(t->b = type()) || !expect('>')) return nullptr;
        } else if (!id.empty()) {
            t->kind = Type::Named;
            t->name = id;
        } else {
            return nullptr;
        }
        return t;
    }
};

const Schema& schema() {
    static Schema sc;
    static std::once_flag once;
    std::call_once(once, [] {
        if (!sc.parse(schema_text())) std::fprintf(stderr, "posidonius_gb300: %s\n", sc.error.c_str());
    });
    return sc;
}

// ---- encoder ---------------------------------------------------------------
class Encoder {
public:
    Encoder(const Schema& sc, std::string& out) : sc_(sc), out_(out) {}
    std::string error;

    bool named(const std::string& name, const json::Value& v, const std::string& where) {
        auto it = sc_.defs.find(name);
        if (it == sc_.defs.end()) return fail(where, "unknown type " + name);
        const Def& d = it->second;
        if (!d.is_enum) {
            if (!v.is_object()) return fail(where, "object expected");
            for (const Field& f : d.fields) {
                const json::Value* m = v.find(f.name.c_str());
                if (!m) return fail(where, "missing field " + f.name);
                if (!value(*f.type, *m, where + "." + f.name)) return false;
            }
            return true;
        }
        // enum: "Unit" or {"Variant": payload}
        std::string tag;
        const json::Value* payload = nullptr;
        if (v.is_string()) {
            tag = v.text;
        } else if (v.is_object() && v.members.size() == 1) {
            tag = v.members[0].first;
            payload = &v.members[0].second;
        } else {
            return fail(where, "enum value expected");
        }
        for (size_t k = 0; k < d.fields.size(); ++k) {
            const Field& f = d.fields[k];
            if (f.name != tag) continue;
            u32((uint32_t)k);
            if (!f.type) return payload ? fail(where, tag + " takes no payload") : true;
            if (!payload) return fail(where, tag + " needs a payload");
            return value(*f.type, *payload, where + "." + tag);
        }
        return fail(where, "unknown variant " + tag);
    }

private:
    const Schema& sc_;
    std::string& out_;
    bool fail(const std::string& where, const std::string& what) { error = where + ": " + what; return false; }
    void raw(const void* p, size_t n) {
        // little-endian host layout (x86-64 and AArch64 alike)
        out_.append((const char*)p, n);
    }
    void u32(uint32_t x) { raw(&x, 4); }
    void u64(uint64_t x) { raw(&x, 8); }

    bool value(const Type& t, const json::Value& v, const std::string& where) {
        switch (t.kind) {
            case Type::F64: {
                double x;
                if (v.kind == json::Value::Null) {
                    const uint64_t qnan = 0x7ff8000000000000ull;
                    std::memcpy(&x, &qnan, 8);
                } else if (v.is_number()) {
                    x = std::strtod(v.text.c_str(), nullptr);
                } else {
                    return fail(where, "number expected");
                }
                raw(&x, 8);
                return true;
            }
            case Type::U64: {
                if (!v.is_number() || v.text.find_first_of(".eE-") != std::string::npos)
                    return fail(where, "unsigned integer expected");
                u64(std::strtoull(v.text.c_str(), nullptr, 10));
                return true;
            }
            case Type::U32: {
                if (!v.is_number() || v.text.find_first_of(".eE-") != std::string::npos)
                    return fail(where, "unsigned integer expected");
                u32((uint32_t)std::strtoull(v.text.c_str(), nullptr, 10));
                return true;
            }
            case Type::I32: {
                if (!v.is_number() || v.text.find_first_of(".eE") != std::string::npos)
                    return fail(where, "integer expected");
                const int32_t x = (int32_t)std::strtoll(v.text.c_str(), nullptr, 10);
                raw(&x, 4);
                return true;
            }
            case Type::Bool: {
                if (v.kind != json::Value::Bool) return fail(where, "bool expected");
                const unsigned char c = v.b ? 1 : 0;
                raw(&c, 1);
                return true;
            }
            case Type::Array: {
                if (!v.is_array() || (int64_t)v.items.size() != t.n)
                    return fail(where, "array of " + std::to_string(t.n) + " expected");
                for (size_t k = 0; k < v.items.size(); ++k)
                    if (!value(*t.a, v.items[k], where + "[" + std::to_string(k) + "]")) return false;
                return true;
            }
            case Type::Vec: {
                if (!v.is_array()) return fail(where, "array expected");
                u64(v.items.size());
                for (size_t k = 0; k < v.items.size(); ++k)
                    if (!value(*t.a, v.items[k], where + "[" + std::to_string(k) + "]")) return false;
                return true;
            }
            case Type::Map: {
                if (!v.is_object()) return fail(where, "object expected");
                u64(v.members.size());
                for (const auto& m : v.members) {
                    json::Value key;
                    key.kind = json::Value::Number;
                    key.text = m.first;
                    if (!value(*t.a, key, where + " key") || !value(*t.b, m.second, where + "[" + m.first + "]"))
                        return false;
                }
                return true;
            }
            case Type::Named: return named(t.name, v, where);
            case Type::Unsupported: return fail(where, "not supported by this library");
        }
        return false;
    }
};

// ---- decoder ---------------------------------------------------------------
class Decoder {
public:
    Decoder(const Schema& sc, const std::string& in) : sc_(sc), p_((const unsigned char*)in.data()), e_(p_ + in.size()) {}
    std::string error;
    bool done() const { return p_ == e_; }
    size_t left() const { return (size_t)(e_ - p_); }

    bool named(const std::string& name, json::Value& v, const std::string& where) {
        auto it = sc_.defs.find(name);
        if (it == sc_.defs.end()) return fail(where, "unknown type " + name);
        const Def& d = it->second;
        if (!d.is_enum) {
            v.kind = json::Value::Object;
            v.members.reserve(d.fields.size());
            for (const Field& f : d.fields) {
                v.members.emplace_back(f.name, json::Value());
                if (!value(*f.type, v.members.back().second, where + "." + f.name)) return false;
            }
            return true;
        }
        uint32_t k;
        if (!take(&k, 4)) return fail(where, "truncated");
        if (k >= d.fields.size()) return fail(where, "variant index " + std::to_string(k) + " out of range");
        const Field& f = d.fields[k];
        if (!f.type) {
            v.kind = json::Value::String;
            v.text = f.name;
            return true;
        }
        v.kind = json::Value::Object;
        v.members.emplace_back(f.name, json::Value());
        return value(*f.type, v.members.back().second, where + "." + f.name);
    }

private:
    const Schema& sc_;
    const unsigned char* p_;
    const unsigned char* e_;
    bool fail(const std::string& where, const std::string& what) { error = where + ": " + what; return false; }
    bool take(void* dst, size_t n) {
        if ((size_t)(e_ - p_) < n) return false;
        std::memcpy(dst, p_, n);
        p_ += n;
        return true;
    }

    bool value(const Type& t, json::Value& v, const std::string& where) {
        switch (t.kind) {
            case Type::F64: {
                double x;
                if (!take(&x, 8)) return fail(where, "truncated");
                if (std::isnan(x)) {
                    v.kind = json::Value::Null;
                } else {
                    v.kind = json::Value::Number;
                    v.text = format_double(x);
                }
                return true;
            }
            case Type::U64: {
                uint64_t x;
                if (!take(&x, 8)) return fail(where, "truncated");
                v.kind = json::Value::Number;
                v.text = std::to_string(x);
                return true;
            }
            case Type::U32: {
                uint32_t x;
                if (!take(&x, 4)) return fail(where, "truncated");
                v.kind = json::Value::Number;
                v.text = std::to_string(x);
                return true;
            }
            case Type::I32: {
                int32_t x;
                if (!take(&x, 4)) return fail(where, "truncated");
                v.kind = json::Value::Number;
                v.text = std::to_string(x);
                return true;
            }
            case Type::Bool: {
                unsigned char c;
                if (!take(&c, 1)) return fail(where, "truncated");
                if (c > 1) return fail(where, "bool byte " + std::to_string(c));
                v.kind = json::Value::Bool;
                v.b = c == 1;
                return true;
            }
            case Type::Array:
            case Type::Vec: {
                uint64_t n = (uint64_t)t.n;
                if (t.kind == Type::Vec) {
                    if (!take(&n, 8)) return fail(where, "truncated");
                    if (n > left()) return fail(where, "length " + std::to_string(n) + " beyond the data");
                }
                v.kind = json::Value::Array;
                v.items.resize((size_t)n);
                for (uint64_t k = 0; k < n; ++k)
                    if (!value(*t.a, v.items[(size_t)k], where + "[" + std::to_string(k) + "]")) return false;
                return true;
            }
            case Type::Map: {
                uint64_t n;
                if (!take(&n, 8)) return fail(where, "truncated");
                if (n > left()) return fail(where, "length beyond the data");
                v.kind = json::Value::Object;
                for (uint64_t k = 0; k < n; ++k) {
                    json::Value key, val;
                    if (!value(*t.a, key, where + " key") || !value(*t.b, val, where + "[]")) return false;
                    v.members.emplace_back(key.text, std::move(val));
                }
                return true;
            }
            case Type::Named: return named(t.name, v, where);
            case Type::Unsupported: return fail(where, "not supported by this library");
        }
        return false;
    }
};

}  // namespace

bool is_bincode_path(const std::string& path) {
    const size_t dot = path.find_last_of('.');
    const size_t slash = path.find_last_of('/');
    const bool has_ext = dot != std::string::npos && (slash == std::string::npos || dot > slash);
    return !(has_ext && path.substr(dot + 1) == "json");
}

bool json_to_bincode(const json::Value& doc, std::string& out, std::string& err) {
    const Schema& sc = schema();
    if (!sc.error.empty()) { err = sc.error; return false; }
    const char* root = doc.find("half_time_step") ? "WHFast" : doc.find("b_0") ? "Ias15" : nullptr;
    if (!root) { err = "bincode: neither a WHFast nor an Ias15 document"; return false; }
    out.clear();
    Encoder enc(sc, out);
    if (!enc.named(root, doc, root)) { err = "bincode: " + enc.error; return false; }
    return true;
}

bool bincode_to_json(const std::string& bytes, json::Value& doc, std::string& err) {
    const Schema& sc = schema();
    if (!sc.error.empty()) { err = sc.error; return false; }
    std::string first;
    for (const char* root : {"WHFast", "Ias15"}) {
        json::Value v;
        Decoder dec(sc, bytes);
        if (dec.named(root, v, root) && dec.done()) {
            doc = std::move(v);
            return true;
        }
        if (first.empty()) first = dec.error.empty() ? std::string(root) + ": trailing bytes" : dec.error;
    }
    err = "bincode: neither a WHFast nor an Ias15 snapshot (" + first + ")";
    return false;
}

}  // namespace posi
