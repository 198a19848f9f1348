// whfast_oracle.cpp -- CPU restatement of Posidonius's WHFast + additional
// effects path in FP64.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke test
// and the CPU-baseline / reference legs of bench.py load it to produce the
// expected results and the CPU timing.  The product library never links,
// loads or calls it.
//
// It restates, function by function and in the same floating-point operation
// order, the reference functions cited beside each routine below (paths are
// inside the posidonius project).  It must be compiled without FMA
// contraction (-ffp-contract=off), which is Rust's default, so that every
// +, -, *, / and sqrt rounds exactly as in the Rust binary.  `powi` follows
// LLVM's expansion of llvm.powi (binary exponentiation, the same product
// order as compiler-rt's __powidf2).
//
// Parity pin: tests/test_oracle_golden.py runs this restatement on the
// reference's own golden cases (tests/data/<case>/case.json of the reference)
// and checks the final inertial positions, velocities and accelerations
// against tests/data/<case>/particle_*.json at the reference's 1e-14 absolute
// tolerance (tests/common/universe.rs:47-72 of the reference).
//
// Built with -DORACLE_COUNT_FLOPS the same code counts every FP64 operation
// (+ - * / sqrt each count 1), which gives the algorithmic flops per step.
// Built with -DORACLE_DUAL every value carries ORACLE_ND directional
// derivatives (forward-mode dual numbers): the exact derivatives of the
// computed map -- the same operation order, branches taken on the values --
// with respect to the seeded inputs (oracle_dual_io), with no step size and
// no difference noise.  Terms the reference evaluates through powf / exp
// (Roche radii, the dynamical tide, the disk) carry no derivative there.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/posidonius_gb300.h"

namespace orc {

// ---------------------------------------------------------------------------
// Arithmetic type: plain double, or a counting wrapper.
// ---------------------------------------------------------------------------
#ifdef ORACLE_COUNT_FLOPS
static thread_local int64_t g_flops = 0, g_divs = 0, g_sqrts = 0;
struct real {
    double v;
    real() : v(0.) {}
    real(double x) : v(x) {}
    explicit operator double() const { return v; }
};
static inline real operator+(real a, real b) { ++g_flops; return real(a.v + b.v); }
static inline real operator-(real a, real b) { ++g_flops; return real(a.v - b.v); }
static inline real operator*(real a, real b) { ++g_flops; return real(a.v * b.v); }
static inline real operator/(real a, real b) { ++g_flops; ++g_divs; return real(a.v / b.v); }
static inline real operator-(real a) { return real(-a.v); }
static inline real& operator+=(real& a, real b) { a = a + b; return a; }
static inline real& operator-=(real& a, real b) { a = a - b; return a; }
static inline real& operator*=(real& a, real b) { a = a * b; return a; }
static inline real& operator/=(real& a, real b) { a = a / b; return a; }
static inline bool operator<(real a, real b) { return a.v < b.v; }
static inline bool operator>(real a, real b) { return a.v > b.v; }
static inline bool operator<=(real a, real b) { return a.v <= b.v; }
static inline bool operator>=(real a, real b) { return a.v >= b.v; }
static inline bool operator==(real a, real b) { return a.v == b.v; }
static inline bool operator!=(real a, real b) { return a.v != b.v; }
static inline real rsqrt_(real a) { ++g_flops; ++g_sqrts; return real(std::sqrt(a.v)); }
static inline real rabs(real a) { return real(std::fabs(a.v)); }
static inline real rfloor(real a) { return real(std::floor(a.v)); }
static inline bool risnan(real a) { return std::isnan(a.v); }
static inline double dv(real a) { return a.v; }
#elif defined(ORACLE_DUAL)
#ifndef ORACLE_ND
#define ORACLE_ND 26
#endif
constexpr int ND = ORACLE_ND;
struct real {
    double v;
    double d[ND];
    real() : v(0.) { for (int k = 0; k < ND; ++k) d[k] = 0.; }
    real(double x) : v(x) { for (int k = 0; k < ND; ++k) d[k] = 0.; }
    explicit operator double() const { return v; }
};
static inline real operator+(const real& a, const real& b) {
    real r(a.v + b.v);
    for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
static inline real operator-(const real& a, const real& b) {
    real r(a.v - b.v);
    for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
static inline real operator*(const real& a, const real& b) {
    real r(a.v * b.v);
    for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
static inline real operator/(const real& a, const real& b) {
    real r(a.v / b.v);
    const double ib = 1. / b.v;
    for (int k = 0; k < ND; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
static inline real operator-(const real& a) {
    real r(-a.v);
    for (int k = 0; k < ND; ++k) r.d[k] = -a.d[k];
    return r;
}
static inline real& operator+=(real& a, const real& b) { a = a + b; return a; }
static inline real& operator-=(real& a, const real& b) { a = a - b; return a; }
static inline real& operator*=(real& a, const real& b) { a = a * b; return a; }
static inline real& operator/=(real& a, const real& b) { a = a / b; return a; }
static inline bool operator<(const real& a, const real& b) { return a.v < b.v; }
static inline bool operator>(const real& a, const real& b) { return a.v > b.v; }
static inline bool operator<=(const real& a, const real& b) { return a.v <= b.v; }
static inline bool operator>=(const real& a, const real& b) { return a.v >= b.v; }
static inline bool operator==(const real& a, const real& b) { return a.v == b.v; }
static inline bool operator!=(const real& a, const real& b) { return a.v != b.v; }
static inline real rsqrt_(const real& a) {
    real r(std::sqrt(a.v));
    const double h = r.v > 0. ? 0.5 / r.v : 0.;
    for (int k = 0; k < ND; ++k) r.d[k] = a.d[k] * h;
    return r;
}
static inline real rabs(const real& a) { return a.v < 0. ? -a : a; }
static inline real rfloor(const real& a) { return real(std::floor(a.v)); }
static inline bool risnan(const real& a) { return std::isnan(a.v); }
static inline double dv(const real& a) { return a.v; }
#else
typedef double real;
static inline real rsqrt_(real a) { return std::sqrt(a); }
static inline real rabs(real a) { return std::fabs(a); }
static inline real rfloor(real a) { return std::floor(a); }
static inline bool risnan(real a) { return std::isnan(a); }
static inline double dv(real a) { return a; }
#endif

// LLVM's llvm.powi expansion for a constant exponent (SelectionDAG ExpandPowI,
// identical product order to compiler-rt __powidf2): square-and-multiply from
// the low bit, the first factor taken without multiplying by 1.
static inline real powi(real x, int n) {
    real res = 0.;
    bool have = false;
    real cur = x;
    unsigned v = (unsigned)n;
    while (v) {
        if (v & 1u) {
            if (have) res = res * cur; else { res = cur; have = true; }
        }
        v >>= 1;
        if (v) cur = cur * cur;
    }
    return res;
}

// src/constants.rs:20-61
static const int WHFAST_NMAX_QUART = 64;
static const int WHFAST_NMAX_NEWT = 32;
static const double DBL_EPSILON_ = 2.2204460492503131e-16;
static const double DBL_EPSILON_2 = DBL_EPSILON_ * DBL_EPSILON_;
static const int IMPLICIT_MIDPOINT_MIN_ITER = 3;
static const int IMPLICIT_MIDPOINT_MAX_ITER = 10;
static const double PI = 3.141592653589793;
static const double DAY = 24. * 3600.;
static const double M_SUN = 1.9818e30;
static const double G_SI = 6.67428e-11;
static const double AU = 1.49597870700e11;
static const double SPEED_OF_LIGHT = (2.99792458e8 / AU) * DAY;
static const double SPEED_OF_LIGHT_2 = SPEED_OF_LIGHT * SPEED_OF_LIGHT;
static const double G = G_SI / (AU * AU * AU) * M_SUN * (DAY * DAY);
static const double K2 = G;
static const double R_SUN = 6.957e8 / AU;
static const double SUN_DYN_FREQ_2 = K2 / (R_SUN * R_SUN * R_SUN);
static const double SMOOTHING_FACTOR_DYN_TIDE_COROTATION = 1.0e-5 * 86400.;
static const double BOLTZMANN_CONSTANT = 1.380649e-23 / (M_SUN * AU * AU) * DAY * DAY;
static const double MASS_HYDROGEN_ATOM = 1.672162841e-27 / M_SUN;
static const double MAX_DISTANCE = 100.;
static const double MAX_DISTANCE_2 = MAX_DISTANCE * MAX_DISTANCE;

struct V3 { real x, y, z; };

// src/effects/tides/common.rs:35-79 (ConstantTimeLag subset)
struct Tides {
    int kind = POSI_EFFECT_DISABLED;
    real love_number = 0.;           // ConstantTimeLagParameters.love_number
    real distance = 0., radial_velocity = 0., scaled_dissipation_factor = 0.;
    real rscal_star = 0., rscal_planet = 0.;
    real ortho_star = 0., ortho_planet = 0., radial = 0., radial_diss_pm = 0.;
    real denergy_dt = 0., lag_angle = 0.;
    real diss_factor = 0., diss_scale = 0.;   // ConstantTimeLag inputs (:13-19)
    // the host's pair-dependent dissipation factor for this body (:20-93);
    // unset (false) when the dynamical tide is not excited
    bool pair_set = false;
    real pair_sigma = 0.;
    V3 out_acc{0., 0., 0.}, out_dldt{0., 0., 0.};
    V3 pos{0., 0., 0.}, vel{0., 0., 0.};
};
// src/effects/rotational_flattening/common.rs:8-62 (OblateSpheroid subset)
struct Flat {
    int kind = POSI_EFFECT_DISABLED;
    real love_number = 0.;
    real distance = 0., rscal_star = 0., rscal_planet = 0., radial = 0.;
    real factor_star = 0., factor_planet = 0., ortho_star = 0., ortho_planet = 0.;
    V3 out_acc{0., 0., 0.}, out_dldt{0., 0., 0.};
    V3 pos{0., 0., 0.}, vel{0., 0., 0.};
};
// src/effects/general_relativity.rs:10-59 (Kidder1995 subset)
struct GR {
    int kind = POSI_EFFECT_DISABLED;
    real distance = 0., radial_velocity = 0., norm_v = 0., norm_v2 = 0., factor = 0.;
    V3 out_acc{0., 0., 0.}, out_dldt{0., 0., 0.};
    V3 pos{0., 0., 0.}, vel{0., 0., 0.};
};
// src/effects/disk.rs:6-56
struct Disk {
    int kind = POSI_EFFECT_DISABLED;
    real inner = 0., outer = 0., lifetime = 0., alpha = 0., sigma0 = 0., mu = 0.;   // DiskProperties
    real distance = 0., nv = 0., nv2 = 0., migration_timescale = 0.;
    V3 out_acc{0., 0., 0.};
    V3 pos{0., 0., 0.}, vel{0., 0., 0.};
};
// src/particles/particle.rs:16-52
struct Particle {
    int id = 0;
    real mass = 0., mass_g = 0., radius = 0.;
    V3 r{0., 0., 0.}, v{0., 0., 0.}, a{0., 0., 0.}, a_add{0., 0., 0.};
    V3 hr{0., 0., 0.}, hv{0., 0., 0.};
    real hd = 0., hvr = 0., hnv = 0., hnv2 = 0.;
    V3 spin{0., 0., 0.};
    real nsv2 = 0.;
    V3 L{0., 0., 0.}, dLdt{0., 0., 0.};
    real rg2 = 0., moi = 0.;
    Tides tides;
    Flat flat;
    GR gr;
    Disk disk;
    // src/effects/wind.rs:6-40
    int wind_kind = 0;          // 1: Interaction
    real wind_k = 0., wind_rsat = 0., wind_rsat2 = 0.;
    V3 wind_dldt{0., 0., 0.};
    int evolution = POSI_EVO_NON_EVOLVING;
};
// src/effects/evolution.rs:20-28
struct Evolver {
    int type = POSI_EVO_NON_EVOLVING;
    const double *time = nullptr, *radius = nullptr, *rg2 = nullptr, *love = nullptr;
    int64_t len = 0;
    int64_t left_index = 0;
};
// src/integrator/whfast.rs:123-130
struct AltCoords {
    real mass = 0., mass_g = 0.;
    V3 pos{0., 0., 0.}, vel{0., 0., 0.}, acc{0., 0., 0.};
};

// src/integrator/whfast.rs:99-120 + src/particles/universe.rs:50-63
struct Sim {
    int n = 0, host = 0, coords = POSI_JACOBI;
    bool tides = false, flat = false, gr = false, evolution = false, wind = false, disk = false;
    int gr_impl = POSI_GR_KIDDER1995;   // Universe.general_relativity_implementation
    real dt = 0., half_dt = 0., t = 0., time_limit = 0.;
    real last_hist = -1., hist_period = 0., last_rec = -1., rec_period = 0.;
    int64_t iteration = 0, n_hist = 0, timestep_warning = 0, status = 0, fail_step = 0, fail_pair = 0;
    int64_t last_midpoint_iters = 0;
    std::vector<Particle> p;
    std::vector<Evolver> ev;
    std::vector<AltCoords> alt;
    std::vector<V3> errv, errL;
    std::vector<real> roche;
    // src/integrator/ias15.rs:28-224 (IAS15 systems): per body POSI_IAS_COUNT
    // values (posi_ias15_field), the last accepted step and the count of
    // predictor-corrector loops that hit the iteration limit
    int integrator = POSI_INTEGRATOR_WHFAST;
    std::vector<real> ias;
    real ias_dt_last = 0.;
    int64_t ias_max_exceeded = 0;
    bool fatal() const { return (status & POSI_SYS_FATAL_MASK) != 0; }
};

// ---------------------------------------------------------------------------
// src/particles/common.rs:3-14 calculate_spin
// ---------------------------------------------------------------------------
static void calculate_spin(Sim& s) {
    for (int i = 0; i < s.n; ++i) {
        Particle& q = s.p[i];
        if (q.moi == 0.) {
            s.status = (s.status & ~int64_t(POSI_SYS_FATAL_MASK)) | POSI_SYS_ZERO_INERTIA;
            return;
        }
        q.spin.x = q.L.x / q.moi;
        q.spin.y = q.L.y / q.moi;
        q.spin.z = q.L.z / q.moi;
        q.nsv2 = powi(q.spin.x, 2) + powi(q.spin.y, 2) + powi(q.spin.z, 2);
    }
}

// ---------------------------------------------------------------------------
// src/tools.rs:884-907 find_indices_around_target_value and
// src/tools.rs:840-860 linear_interpolation
// ---------------------------------------------------------------------------
static void find_indices_around_target_value(const double* data, int64_t ndata, double target,
                                             int64_t* left, int64_t* right) {
    int64_t last = ndata - 1;
    int64_t pos = -1;
    for (int64_t k = 0; k < ndata; ++k) {
        if (data[k] > target) { pos = k; break; }
    }
    if (pos < 0) {
        if (data[last] > target) { *left = 0; *right = 0; } else { *left = last; *right = last; }
    } else if (pos == 0) {
        *left = 0; *right = 0;
    } else {
        *left = pos - 1; *right = pos;
    }
}

static real linear_interpolation(real target_x, const double* x, const double* y, int64_t n, int64_t* left_out) {
    int64_t left, right;
    find_indices_around_target_value(x, n, dv(target_x), &left, &right);
    real target_y;
    if (left == right) {
        target_y = y[left];
    } else {
        real x_left = x[left];
        real target_percent = (target_x - x_left) / (real(x[right]) - x_left);
        target_y = real(y[left]) * (real(1.) - target_percent) + real(y[right]) * target_percent;
    }
    *left_out = left;
    return target_y;
}

// src/effects/evolution.rs:446-513 Evolver::idx / radius / radius_of_gyration_2 / love_number
static int64_t evolver_idx(const Evolver& e) {
    const int64_t security_shift = 10;
    return e.left_index > security_shift ? e.left_index - security_shift : 0;
}
static real evolver_radius(Evolver& e, real t, real current) {
    if (e.type == POSI_EVO_NON_EVOLVING) return current;
    int64_t i0 = evolver_idx(e), left = 0;
    real r = linear_interpolation(t, e.time + i0, e.radius + i0, e.len - i0, &left);
    e.left_index += left;
    return r;
}
static real evolver_rg2(Evolver& e, real t, real current) {
    if (e.type == POSI_EVO_BARAFFE2015 || e.type == POSI_EVO_LECONTE2011 || e.type == POSI_EVO_LECONTE_CHABRIER2013) {
        int64_t i0 = evolver_idx(e), left = 0;
        real r = linear_interpolation(t, e.time + i0, e.rg2 + i0, e.len - i0, &left);
        e.left_index += left;
        return r;
    }
    return current;
}
static real evolver_love(Evolver& e, real t, real current) {
    if (e.type == POSI_EVO_LECONTE_CHABRIER2013) {
        int64_t i0 = evolver_idx(e), left = 0;
        real r = linear_interpolation(t, e.time + i0, e.love + i0, e.len - i0, &left);
        e.left_index += left;
        return r;
    }
    return current;
}

// src/effects/evolution.rs:516-546 (the love number update writes to a copy
// of the parameters in the reference, so only the index bookkeeping remains)
static void non_spin_dependent_evolving_quantities(Sim& s, real t) {
    for (int i = 0; i < s.n; ++i) {
        Particle& q = s.p[i];
        Evolver& e = s.ev[i];
        real new_radius = evolver_radius(e, t, q.radius);
        real new_rg2 = evolver_rg2(e, t, q.rg2);
        if (new_radius != q.radius || new_rg2 != q.rg2) {
            q.radius = new_radius;
            q.rg2 = new_rg2;
            q.moi = q.mass * q.rg2 * powi(q.radius, 2);
        }
        if (q.tides.kind != POSI_EFFECT_DISABLED) {
            (void)evolver_love(e, t, q.tides.love_number);
        }
    }
}

static bool dynamical(int type) {
    return type == POSI_EVO_BOLMONT_MATHIS2016 || type == POSI_EVO_GALLET_BOLMONT2017;
}

// src/effects/evolution.rs:487-512 (the 4th table column of a dynamical-tide
// evolution holds the inverse tidal Q factor)
static real evolver_inverse_tidal_q_factor(Evolver& e, real t, real current) {
    if (dynamical(e.type)) {
        int64_t i0 = evolver_idx(e), left = 0;
        real r = linear_interpolation(t, e.time + i0, e.love + i0, e.len - i0, &left);
        e.left_index += left;
        return r;
    }
    return current;
}

// src/effects/evolution.rs:548-567
static void spin_dependent_evolving_quantities(Sim& s, real t) {
    for (int i = 0; i < s.n; ++i) {
        Particle& q = s.p[i];
        Evolver& e = s.ev[i];
        if (dynamical(e.type)) {
            real inverse_tidal_q_factor = evolver_inverse_tidal_q_factor(e, t, 0.);
            real epsilon_squared = q.nsv2 / SUN_DYN_FREQ_2;
            q.tides.lag_angle = real(3.0) * epsilon_squared * inverse_tidal_q_factor / real(4.0);
        } else {
            q.tides.lag_angle = 0.;
        }
    }
}

// src/particles/universe.rs:305-316
static void calculate_spin_and_evolving_quantities(Sim& s, real t, bool evolution) {
    if (evolution && s.evolution) non_spin_dependent_evolving_quantities(s, t);
    calculate_spin(s);
    if (evolution && s.evolution) spin_dependent_evolving_quantities(s, t);
}

// src/particles/universe.rs:177-196
static void calculate_roche_radiuses(Sim& s) {
    const int n = s.n;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            const Particle& a = s.p[i];
            const Particle& b = s.p[j];
            if (a.mass > b.mass) {
                s.roche[i * n + j] = (b.radius / 0.462) * real(std::pow(dv(a.mass / b.mass), 1. / 3.));
            } else {
                s.roche[i * n + j] = (a.radius / 0.462) * real(std::pow(dv(b.mass / a.mass), 1. / 3.));
            }
        }
    }
}

static void set_fatal(Sim& s, int code, int i, int j) {
    if (s.fatal()) return;
    s.status = (s.status & ~int64_t(POSI_SYS_FATAL_MASK)) | code;
    s.fail_step = s.iteration;
    s.fail_pair = int64_t(i) * 1024 + j;
}

// src/particles/universe.rs:198-303 (ignore_terms: 0 None, 1 WHFastOne, 2 WHFastTwo)
static void gravity_calculate_acceleration(Sim& s, int ignore_terms) {
    const int n = s.n, mm = s.host;
    std::vector<V3> acc(n, V3{0., 0., 0.});
    for (int i = 0; i < n; ++i) {
        const Particle& a = s.p[i];
        for (int j = 0; j < n; ++j) {
            if (i == j) continue;
            const Particle& b = s.p[j];
            real dx = a.r.x - b.r.x;
            real dy = a.r.y - b.r.y;
            real dz = a.r.z - b.r.z;
            real distance_2 = dx * dx + dy * dy + dz * dz;
            if (i < j) {
                if (distance_2 <= powi(s.roche[i * n + j], 2)) { set_fatal(s, POSI_SYS_ROCHE, i, j); return; }
                if (distance_2 <= powi(a.radius + b.radius, 2)) { set_fatal(s, POSI_SYS_COLLISION, i, j); return; }
                if (MAX_DISTANCE_2 > 0. && i == mm && distance_2 > MAX_DISTANCE_2) { set_fatal(s, POSI_SYS_EJECTED, i, j); return; }
            }
            if (ignore_terms == 1 &&
                ((i == mm && mm == 0 && j == 1) || (i == mm && mm > 0 && j == 0) ||
                 (j == mm && mm == 0 && i == 1) || (j == mm && mm > 0 && i == 0))) {
                continue;
            }
            if (ignore_terms == 2 && (i == mm || j == mm)) continue;
            real distance = rsqrt_(distance_2);
            real prefact = -G / (distance * distance * distance) * b.mass;
            acc[i].x += prefact * dx;
            acc[i].y += prefact * dy;
            acc[i].z += prefact * dz;
        }
    }
    for (int i = 0; i < n; ++i) s.p[i].a = acc[i];
}

// src/particles/universe.rs:318-351
static void inertial_to_heliocentric(Sim& s) {
    Particle& h = s.p[s.host];
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        q.hr.x = q.r.x - h.r.x;
        q.hr.y = q.r.y - h.r.y;
        q.hr.z = q.r.z - h.r.z;
        q.hv.x = q.v.x - h.v.x;
        q.hv.y = q.v.y - h.v.y;
        q.hv.z = q.v.z - h.v.z;
        q.hd = rsqrt_(powi(q.hr.x, 2) + powi(q.hr.y, 2) + powi(q.hr.z, 2));
        q.hvr = (q.hr.x * q.hv.x + q.hr.y * q.hv.y + q.hr.z * q.hv.z) / q.hd;
        q.hnv2 = powi(q.hv.x - h.hv.x, 2) + powi(q.hv.y - h.hv.y, 2) + powi(q.hv.z - h.hv.z, 2);
        q.hnv = rsqrt_(q.hnv2);
    }
    h.hr = V3{0., 0., 0.};
    h.hv = V3{0., 0., 0.};
    h.hd = 0.; h.hvr = 0.; h.hnv2 = 0.; h.hnv = 0.;
}

// src/particles/universe.rs:353-426 with
// src/effects/tides/common.rs:143-170,202-217,
// src/effects/rotational_flattening/common.rs:93-120,148-161,
// src/effects/general_relativity.rs:86-109,153-174
static void initialize(Sim& s, bool dl, bool acc) {
    // src/effects/wind.rs:62-70
    if (dl && s.wind) {
        for (int i = 0; i < s.n; ++i)
            if (s.p[i].wind_kind == 1) s.p[i].wind_dldt = V3{0., 0., 0.};
    }
    const bool it = (dl && s.tides) || (acc && s.tides);
    const bool ifl = (dl && s.flat) || (acc && s.flat);
    const bool igr = (dl && s.gr && s.gr_impl == POSI_GR_KIDDER1995) || (acc && s.gr);
    if (it || ifl || igr) {
        Particle& h = s.p[s.host];
        if (it && h.tides.kind == POSI_EFFECT_CENTRAL) {
            // tides::copy_heliocentric_coordinates
            h.tides.pos = h.hr; h.tides.vel = h.hv; h.tides.distance = h.hd; h.tides.radial_velocity = h.hvr;
            for (int i = 0; i < s.n; ++i) {
                if (i == s.host) continue;
                Particle& q = s.p[i];
                if (q.tides.kind == POSI_EFFECT_ORBITING) {
                    q.tides.pos = q.hr; q.tides.vel = q.hv; q.tides.distance = q.hd; q.tides.radial_velocity = q.hvr;
                }
            }
            // tides::initialize
            h.tides.rscal_star = 0.; h.tides.rscal_planet = 0.;
            h.tides.out_acc = V3{0., 0., 0.}; h.tides.out_dldt = V3{0., 0., 0.};
            for (int i = 0; i < s.n; ++i) {
                if (i == s.host) continue;
                Particle& q = s.p[i];
                if (q.tides.kind == POSI_EFFECT_ORBITING) {
                    q.tides.rscal_star = q.tides.pos.x * h.spin.x + q.tides.pos.y * h.spin.y + q.tides.pos.z * h.spin.z;
                    q.tides.rscal_planet = q.tides.pos.x * q.spin.x + q.tides.pos.y * q.spin.y + q.tides.pos.z * q.spin.z;
                    q.tides.out_acc = V3{0., 0., 0.}; q.tides.out_dldt = V3{0., 0., 0.};
                }
            }
        }
        if (ifl && h.flat.kind == POSI_EFFECT_CENTRAL) {
            h.flat.pos = h.hr; h.flat.vel = h.hv; h.flat.distance = h.hd;
            for (int i = 0; i < s.n; ++i) {
                if (i == s.host) continue;
                Particle& q = s.p[i];
                if (q.flat.kind == POSI_EFFECT_ORBITING) { q.flat.pos = q.hr; q.flat.vel = q.hv; q.flat.distance = q.hd; }
            }
            h.flat.rscal_star = 0.; h.flat.rscal_planet = 0.;
            h.flat.out_acc = V3{0., 0., 0.}; h.flat.out_dldt = V3{0., 0., 0.};
            for (int i = 0; i < s.n; ++i) {
                if (i == s.host) continue;
                Particle& q = s.p[i];
                if (q.flat.kind == POSI_EFFECT_ORBITING) {
                    q.flat.rscal_star = q.flat.pos.x * h.spin.x + q.flat.pos.y * h.spin.y + q.flat.pos.z * h.spin.z;
                    q.flat.rscal_planet = q.flat.pos.x * q.spin.x + q.flat.pos.y * q.spin.y + q.flat.pos.z * q.spin.z;
                    q.flat.out_acc = V3{0., 0., 0.}; q.flat.out_dldt = V3{0., 0., 0.};
                }
            }
        }
        if (igr && h.gr.kind == POSI_EFFECT_CENTRAL) {
            h.gr.pos = h.hr; h.gr.vel = h.hv; h.gr.distance = h.hd; h.gr.radial_velocity = h.hvr;
            h.gr.norm_v = h.hnv; h.gr.norm_v2 = h.hnv2;
            for (int i = 0; i < s.n; ++i) {
                if (i == s.host) continue;
                Particle& q = s.p[i];
                if (q.gr.kind == POSI_EFFECT_ORBITING) {
                    q.gr.pos = q.hr; q.gr.vel = q.hv; q.gr.distance = q.hd; q.gr.radial_velocity = q.hvr;
                    q.gr.norm_v = q.hnv; q.gr.norm_v2 = q.hnv2;
                }
            }
            // general_relativity::initialize: not for Newhall1983
            if (s.gr_impl != POSI_GR_NEWHALL1983) {
                h.gr.factor = 0.;
                h.gr.out_acc = V3{0., 0., 0.}; h.gr.out_dldt = V3{0., 0., 0.};
                for (int i = 0; i < s.n; ++i) {
                    if (i == s.host) continue;
                    Particle& q = s.p[i];
                    if (q.gr.kind == POSI_EFFECT_ORBITING) {
                        q.gr.factor = h.mass_g * q.mass_g / powi(h.mass_g + q.mass_g, 2);
                        q.gr.out_acc = V3{0., 0., 0.}; q.gr.out_dldt = V3{0., 0., 0.};
                    }
                }
            }
        }
    }
    // src/effects/disk.rs:83-97, :134-150
    if (acc && s.disk) {
        Particle& h = s.p[s.host];
        if (h.disk.kind == POSI_EFFECT_CENTRAL) {
            h.disk.pos = h.hr; h.disk.vel = h.hv; h.disk.distance = h.hd; h.disk.nv = h.hnv; h.disk.nv2 = h.hnv2;
            for (int i = 0; i < s.n; ++i) {
                if (i == s.host) continue;
                Particle& q = s.p[i];
                if (q.disk.kind == POSI_EFFECT_ORBITING) {
                    q.disk.pos = q.hr; q.disk.vel = q.hv; q.disk.distance = q.hd; q.disk.nv = q.hnv; q.disk.nv2 = q.hnv2;
                }
            }
            h.disk.out_acc = V3{0., 0., 0.};
            for (int i = 0; i < s.n; ++i) {
                if (i == s.host) continue;
                if (s.p[i].disk.kind == POSI_EFFECT_ORBITING) s.p[i].disk.out_acc = V3{0., 0., 0.};
            }
        }
    }
    if (acc) {
        for (int i = 0; i < s.n; ++i) s.p[i].a_add = V3{0., 0., 0.};
    }
}

// ---------------------------------------------------------------------------
// Constant-time-lag tides: src/effects/tides/constant_time_lag.rs
// ---------------------------------------------------------------------------
// :206-264 (the pair-dependent dissipation factor is the particle's own for
// every non-dynamical evolution, :144-165)
// src/tools.rs:251-285
static void perihelion_distance_and_eccentricity(real gm, V3 p, V3 v, real* q, real* e) {
    real hx = p.y * v.z - p.z * v.y;
    real hy = p.z * v.x - p.x * v.z;
    real hz = p.x * v.y - p.y * v.x;
    real h2 = real(std::pow(dv(hx), 2.)) + real(std::pow(dv(hy), 2.)) + real(std::pow(dv(hz), 2.));
    real v2 = v.x * v.x + v.y * v.y + v.z * v.z;
    real r = rsqrt_(p.x * p.x + p.y * p.y + p.z * p.z);
    real sv = h2 / gm;
    real temp = real(1.) + sv * (v2 / gm - real(2.) / r);
    *e = temp <= real(0.) ? real(0.) : rsqrt_(temp);
    *q = sv / (real(1.) + *e);
}

// src/effects/tides/constant_time_lag.rs:20-93: the host's dissipation factor
// for each orbiting body when the host's evolution has a dynamical tide (the
// planet-dependent branch, :95-140, is refused by the loader)
static void pair_dependent_scaled_dissipation_factors(Sim& s) {
    Particle& h = s.p[s.host];
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        q.tides.pair_set = false;
        if (!dynamical(s.ev[s.host].type) || q.tides.kind != POSI_EFFECT_ORBITING) continue;
        real host_norm_spin_vector = rsqrt_(h.nsv2);
        real scale = h.tides.kind == POSI_EFFECT_CENTRAL ? h.tides.diss_scale : real(0.);
        real factor = h.tides.kind == POSI_EFFECT_CENTRAL ? h.tides.diss_factor : real(0.);
        real gm = h.mass_g + q.mass_g;
        real peri, ecc;
        perihelion_distance_and_eccentricity(gm, q.tides.pos, q.tides.vel, &peri, &ecc);
        real mean_motion = rsqrt_(gm) * real(std::pow(dv(peri / (real(1.0) - ecc)), -1.5));
        real half = rabs(host_norm_spin_vector - mean_motion);
        if (half < host_norm_spin_vector) {
            if (half < SMOOTHING_FACTOR_DYN_TIDE_COROTATION) half = SMOOTHING_FACTOR_DYN_TIDE_COROTATION;
            real inv = real(1.) / half;
            q.tides.pair_sigma = scale * (real(2.0) * K2 / (real(3.0) * powi(h.radius, 5)) * h.tides.lag_angle * inv + factor);
            q.tides.pair_set = true;
        }
    }
}

// :144-165 get_pair_dependent_scaled_dissipation_factor_or_else for the host
static real host_sigma_for(const Sim& s, const Particle& q) {
    const Particle& h = s.p[s.host];
    if (dynamical(s.ev[s.host].type) && q.tides.pair_set) return q.tides.pair_sigma;
    return h.tides.scaled_dissipation_factor;
}

static void tides_orthogonal(Sim& s) {
    Particle& h = s.p[s.host];
    for (int pass = 0; pass < 2; ++pass) {
        const bool central_body = (pass == 0);
        for (int i = 0; i < s.n; ++i) {
            if (i == s.host) continue;
            Particle& q = s.p[i];
            if (q.tides.kind != POSI_EFFECT_ORBITING) continue;
            real distance_7 = powi(q.tides.distance, 7);
            if (central_body) {
                q.tides.ortho_star = real(4.5) * powi(q.mass, 2) * powi(h.radius, 10) * host_sigma_for(s, q) / distance_7;
            } else {
                q.tides.ortho_planet = real(4.5) * powi(h.mass, 2) * powi(q.radius, 10) * q.tides.scaled_dissipation_factor / distance_7;
            }
        }
    }
}

// :266-307
static void tides_radial(Sim& s) {
    Particle& h = s.p[s.host];
    real host_mass_2 = h.mass * h.mass;
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.tides.kind != POSI_EFFECT_ORBITING) continue;
        real host_love = (h.tides.kind == POSI_EFFECT_CENTRAL) ? h.tides.love_number : real(0.);
        real particle_mass_2 = q.mass * q.mass;
        real conservative = real(-3.0) * K2 / powi(q.tides.distance, 7)
            * (particle_mass_2 * powi(h.radius, 5) * host_love + host_mass_2 * powi(q.radius, 5) * q.tides.love_number);
        real factor1 = real(-13.5) * q.tides.radial_velocity / powi(q.tides.distance, 8);
        real term1 = particle_mass_2 * powi(h.radius, 10) * host_sigma_for(s, q);
        real term2 = host_mass_2 * powi(q.radius, 10) * q.tides.scaled_dissipation_factor;
        q.tides.radial_diss_pm = factor1 * term2;
        real dissipative = q.tides.radial_diss_pm + factor1 * term1;
        q.tides.radial = conservative + dissipative;
    }
}

// :309-332
static V3 tidal_force(const Particle& h, const Particle& q) {
    const Tides& t = q.tides;
    real factor3 = t.radial + (t.ortho_star + t.ortho_planet) * t.radial_velocity / t.distance;
    V3 f;
    f.x = factor3 * t.pos.x / t.distance
        + t.ortho_star / t.distance * (h.spin.y * t.pos.z - h.spin.z * t.pos.y - t.vel.x)
        + t.ortho_planet / t.distance * (q.spin.y * t.pos.z - q.spin.z * t.pos.y - t.vel.x);
    f.y = factor3 * t.pos.y / t.distance
        + t.ortho_star / t.distance * (h.spin.z * t.pos.x - h.spin.x * t.pos.z - t.vel.y)
        + t.ortho_planet / t.distance * (q.spin.z * t.pos.x - q.spin.x * t.pos.z - t.vel.y);
    f.z = factor3 * t.pos.z / t.distance
        + t.ortho_star / t.distance * (h.spin.x * t.pos.y - h.spin.y * t.pos.x - t.vel.z)
        + t.ortho_planet / t.distance * (q.spin.x * t.pos.y - q.spin.y * t.pos.x - t.vel.z);
    return f;
}

// :171-204
static V3 tides_torque(const Particle& h, const Particle& q, bool central_body) {
    V3 rs;
    real orth, rscal;
    if (!central_body) { rs = q.spin; rscal = q.tides.rscal_planet; orth = q.tides.ortho_planet; }
    else { rs = h.spin; rscal = q.tides.rscal_star; orth = q.tides.ortho_star; }
    const Tides& t = q.tides;
    real d = t.distance;
    V3 r;
    r.x = orth * (d * rs.x - rscal * t.pos.x / d - real(1.0) / d * (t.pos.y * t.vel.z - t.pos.z * t.vel.y));
    r.y = orth * (d * rs.y - rscal * t.pos.y / d - real(1.0) / d * (t.pos.z * t.vel.x - t.pos.x * t.vel.z));
    r.z = orth * (d * rs.z - rscal * t.pos.z / d - real(1.0) / d * (t.pos.x * t.vel.y - t.pos.y * t.vel.x));
    return r;
}

// src/effects/tides/common.rs:312-370 (ConstantTimeLag branch)
static void tidal_acceleration(Sim& s) {
    Particle& h = s.p[s.host];
    real factor2 = real(1.) / h.mass;
    V3 sum{0., 0., 0.};
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.tides.kind != POSI_EFFECT_ORBITING) continue;
        V3 f = tidal_force(h, q);
        real factor1 = real(1.) / q.mass;
        sum.x += f.x; sum.y += f.y; sum.z += f.z;
        q.tides.out_acc.x = factor1 * f.x;
        q.tides.out_acc.y = factor1 * f.y;
        q.tides.out_acc.z = factor1 * f.z;
    }
    h.tides.out_acc.x = real(-1.0) * factor2 * sum.x;
    h.tides.out_acc.y = real(-1.0) * factor2 * sum.y;
    h.tides.out_acc.z = real(-1.0) * factor2 * sum.z;
}

// src/effects/tides/common.rs:223-261 (every non-host body is an orbiting
// body here; the loader rejects cases where it is not)
static void tides_dangular_momentum_dt(Sim& s) {
    Particle& h = s.p[s.host];
    const real factor = -1.0;
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.tides.kind != POSI_EFFECT_ORBITING) continue;
        V3 t = tides_torque(h, q, false);
        q.tides.out_dldt.x = factor * t.x;
        q.tides.out_dldt.y = factor * t.y;
        q.tides.out_dldt.z = factor * t.z;
    }
    V3 sum{0., 0., 0.};
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        if (h.tides.kind != POSI_EFFECT_CENTRAL) continue;
        V3 t = tides_torque(h, s.p[i], true);
        sum.x += factor * t.x; sum.y += factor * t.y; sum.z += factor * t.z;
    }
    h.tides.out_dldt = sum;
}

// src/effects/tides/common.rs:263-279
static void tides_denergy_dt(Sim& s) {
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.tides.kind != POSI_EFFECT_ORBITING) continue;
        Tides& t = q.tides;
        real factor2 = t.ortho_planet / t.distance;
        t.denergy_dt = -((real(1.0) / t.distance * (t.radial_diss_pm + factor2 * t.radial_velocity))
                    * (t.pos.x * t.vel.x + t.pos.y * t.vel.y + t.pos.z * t.vel.z)
                    + factor2
                    * ((q.spin.y * t.pos.z - q.spin.z * t.pos.y - t.vel.x) * t.vel.x
                    + (q.spin.z * t.pos.x - q.spin.x * t.pos.z - t.vel.y) * t.vel.y
                    + (q.spin.x * t.pos.y - q.spin.y * t.pos.x - t.vel.z) * t.vel.z))
                    - (t.out_dldt.x * q.spin.x + t.out_dldt.y * q.spin.y + t.out_dldt.z * q.spin.z);
    }
}

// ---------------------------------------------------------------------------
// Rotational flattening (oblate spheroid):
// src/effects/rotational_flattening/oblate_spheroid.rs, common.rs
// ---------------------------------------------------------------------------
// oblate_spheroid.rs:12-49
static void flat_orthogonal(Sim& s) {
    Particle& h = s.p[s.host];
    real host_love = (h.flat.kind == POSI_EFFECT_CENTRAL) ? h.flat.love_number : real(0.);
    for (int pass = 0; pass < 2; ++pass) {
        const bool central_body = (pass == 0);
        for (int i = 0; i < s.n; ++i) {
            if (i == s.host) continue;
            Particle& q = s.p[i];
            if (q.flat.kind != POSI_EFFECT_ORBITING) continue;
            Flat& f = q.flat;
            if (central_body) {
                f.factor_star = q.mass * host_love * h.nsv2 * powi(h.radius, 5) / real(6.);
                f.ortho_star = real(-6.) * f.factor_star * f.rscal_star / (h.nsv2 * powi(f.distance, 5));
            } else {
                f.factor_planet = h.mass * f.love_number * q.nsv2 * powi(q.radius, 5) / real(6.);
                f.ortho_planet = real(-6.) * f.factor_planet * f.rscal_planet / (q.nsv2 * powi(f.distance, 5));
            }
        }
    }
}

// oblate_spheroid.rs:51-60
static void flat_radial(Sim& s) {
    Particle& h = s.p[s.host];
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.flat.kind != POSI_EFFECT_ORBITING) continue;
        Flat& f = q.flat;
        f.radial = real(-3.) / powi(f.distance, 5) * (f.factor_planet + f.factor_star)
            + real(15.) / powi(f.distance, 7) * (f.factor_star * f.rscal_star * f.rscal_star / h.nsv2
                + f.factor_planet * f.rscal_planet * f.rscal_planet / q.nsv2);
    }
}

// oblate_spheroid.rs:83-97 via common.rs:203-237
static void flat_acceleration(Sim& s) {
    Particle& h = s.p[s.host];
    real factor2 = real(1.) / h.mass;
    V3 sum{0., 0., 0.};
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.flat.kind != POSI_EFFECT_ORBITING) continue;
        Flat& f = q.flat;
        V3 F;
        F.x = f.radial * f.pos.x + f.ortho_planet * q.spin.x + f.ortho_star * h.spin.x;
        F.y = f.radial * f.pos.y + f.ortho_planet * q.spin.y + f.ortho_star * h.spin.y;
        F.z = f.radial * f.pos.z + f.ortho_planet * q.spin.z + f.ortho_star * h.spin.z;
        sum.x += F.x; sum.y += F.y; sum.z += F.z;
        real factor1 = real(1.) / q.mass;
        f.out_acc.x = factor1 * F.x;
        f.out_acc.y = factor1 * F.y;
        f.out_acc.z = factor1 * F.z;
    }
    h.flat.out_acc.x = real(-1.0) * factor2 * sum.x;
    h.flat.out_acc.y = real(-1.0) * factor2 * sum.y;
    h.flat.out_acc.z = real(-1.0) * factor2 * sum.z;
}

// oblate_spheroid.rs:62-81
static V3 flat_torque(const Particle& h, const Particle& q, bool central_body) {
    V3 rs = h.spin;
    real orth;
    if (!central_body) { rs = q.spin; orth = q.flat.ortho_planet; }
    else { orth = q.flat.ortho_star; }
    const V3& p = q.flat.pos;
    V3 t;
    t.x = orth * (p.y * rs.z - p.z * rs.y);
    t.y = orth * (p.z * rs.x - p.x * rs.z);
    t.z = orth * (p.x * rs.y - p.y * rs.x);
    return t;
}

// common.rs:165-201
static void flat_dangular_momentum_dt(Sim& s) {
    Particle& h = s.p[s.host];
    const real factor = -1.0;
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.flat.kind != POSI_EFFECT_ORBITING) continue;
        V3 t = flat_torque(h, q, false);
        q.flat.out_dldt.x = factor * t.x;
        q.flat.out_dldt.y = factor * t.y;
        q.flat.out_dldt.z = factor * t.z;
    }
    V3 sum{0., 0., 0.};
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        if (h.flat.kind != POSI_EFFECT_CENTRAL) continue;
        V3 t = flat_torque(h, s.p[i], true);
        sum.x += factor * t.x; sum.y += factor * t.y; sum.z += factor * t.z;
    }
    h.flat.out_dldt = sum;
}

// ---------------------------------------------------------------------------
// General relativity, Kidder (1995): src/effects/general_relativity.rs
// ---------------------------------------------------------------------------
// :187-239
static void gr_first_order(Sim& s) {
    Particle& h = s.p[s.host];
    V3 sum{0., 0., 0.};
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.gr.kind != POSI_EFFECT_ORBITING) continue;
        GR& g = q.gr;
        real mg = h.mass_g + q.mass_g;
        real distance_2 = powi(g.distance, 2);
        real radial_velocity_2 = powi(g.radial_velocity, 2);
        real radial = -mg / (distance_2 * SPEED_OF_LIGHT_2)
            * ((real(1.0) + real(3.0) * g.factor) * g.norm_v2
               - real(2.0) * (real(2.0) + g.factor) * mg / g.distance
               - real(1.5) * g.factor * radial_velocity_2);
        real ortho = mg / (distance_2 * SPEED_OF_LIGHT_2)
            * real(2.0) * (real(2.0) - g.factor) * g.radial_velocity * g.norm_v;
        V3 a;
        a.x = radial * g.pos.x / g.distance + ortho * g.vel.x / g.norm_v;
        a.y = radial * g.pos.y / g.distance + ortho * g.vel.y / g.norm_v;
        a.z = radial * g.pos.z / g.distance + ortho * g.vel.z / g.norm_v;
        sum.x += q.mass / h.mass * a.x;
        sum.y += q.mass / h.mass * a.y;
        sum.z += q.mass / h.mass * a.z;
        g.out_acc = a;
    }
    h.gr.out_acc.x = real(-1.0) * sum.x;
    h.gr.out_acc.y = real(-1.0) * sum.y;
    h.gr.out_acc.z = real(-1.0) * sum.z;
}

// :241-298
static void gr_second_order(Sim& s) {
    Particle& h = s.p[s.host];
    V3 sum{0., 0., 0.};
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.gr.kind != POSI_EFFECT_ORBITING) continue;
        GR& g = q.gr;
        const real f = g.factor;
        real mg = h.mass_g + q.mass_g;
        real distance_2 = powi(g.distance, 2);
        real nv2 = g.norm_v2;
        real nv4 = powi(nv2, 2);
        real vr2 = powi(g.radial_velocity, 2);
        real vr4 = powi(vr2, 2);
        real f2 = powi(f, 2);
        real radial = -mg / (distance_2 * SPEED_OF_LIGHT_2)
            * (real(3.0 / 4.0) * (real(12.0) + real(29.0) * f) * (powi(mg, 2) / distance_2)
               + f * (real(3.0) - real(4.0) * f) * nv4
               + real(15.0 / 8.0) * f * (real(1.0) - real(3.0) * f) * vr4
               - real(3.0 / 2.0) * f * (real(3.0) - real(4.0) * f) * vr2 * nv2
               - real(0.5) * f * (real(13.0) - real(4.0) * f) * (mg / g.distance) * nv2
               - (real(2.0) + real(25.0) * f + real(2.0) * f2) * (mg / g.distance) * vr2);
        real ortho = -mg / (distance_2 * SPEED_OF_LIGHT_2)
            * real(-0.5) * g.radial_velocity
            * (f * (real(15.0) + real(4.0) * f) * nv2
               - (real(4.0) + real(41.0) * f + real(8.0) * f2) * (mg / g.distance)
               - real(3.0) * f * (real(3.0) + real(2.0) * f) * vr2);
        V3 a;
        a.x = radial * g.pos.x / g.distance + ortho * g.vel.x;
        a.y = radial * g.pos.y / g.distance + ortho * g.vel.y;
        a.z = radial * g.pos.z / g.distance + ortho * g.vel.z;
        sum.x += q.mass / h.mass * a.x;
        sum.y += q.mass / h.mass * a.y;
        sum.z += q.mass / h.mass * a.z;
        g.out_acc.x += a.x; g.out_acc.y += a.y; g.out_acc.z += a.z;
    }
    h.gr.out_acc.x += real(-1.0) * sum.x;
    h.gr.out_acc.y += real(-1.0) * sum.y;
    h.gr.out_acc.z += real(-1.0) * sum.z;
}

// :300-456
static void gr_spin_orbit(Sim& s) {
    Particle& h = s.p[s.host];
    V3 sL{h.moi * h.spin.x, h.moi * h.spin.y, h.moi * h.spin.z};
    V3 sum{0., 0., 0.};
    h.gr.out_dldt = V3{0., 0., 0.};
    const real fa = G / SPEED_OF_LIGHT_2;
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.gr.kind != POSI_EFFECT_ORBITING) continue;
        GR& g = q.gr;
        real M = h.mass + q.mass;
        real dM = h.mass - q.mass;
        real mass_factor = dM / M;
        V3 pL{q.moi * q.spin.x, q.moi * q.spin.y, q.moi * q.spin.z};
        V3 nn{g.pos.x / g.distance, g.pos.y / g.distance, g.pos.z / g.distance};
        real msx = mass_factor * M * (pL.x / q.mass - sL.x / h.mass);
        real msy = mass_factor * M * (pL.y / q.mass - sL.y / h.mass);
        real msz = mass_factor * M * (pL.z / q.mass - sL.z / h.mass);
        real e1x = real(6.) * nn.x * ((nn.y * g.vel.z - nn.z * g.vel.y) * (real(2.) * (sL.x + pL.x) + msx));
        real e1y = real(6.) * nn.y * ((nn.z * g.vel.x - nn.x * g.vel.z) * (real(2.) * (sL.y + pL.y) + msy));
        real e1z = real(6.) * nn.z * ((nn.x * g.vel.y - nn.y * g.vel.x) * (real(2.) * (sL.z + pL.z) + msz));
        V3 e7{real(7.) * (sL.x + pL.x) + real(3.) * msx,
              real(7.) * (sL.y + pL.y) + real(3.) * msy,
              real(7.) * (sL.z + pL.z) + real(3.) * msz};
        real e2x = g.vel.y * e7.z - g.vel.z * e7.y;
        real e2y = g.vel.z * e7.x - g.vel.x * e7.z;
        real e2z = g.vel.x * e7.y - g.vel.y * e7.x;
        V3 e3s{real(3.) * (sL.x + pL.x) + msx, real(3.) * (sL.y + pL.y) + msy, real(3.) * (sL.z + pL.z) + msz};
        real e3x = real(3.) * g.radial_velocity * (nn.y * e3s.z - nn.z * e3s.y);
        real e3y = real(3.) * g.radial_velocity * (nn.z * e3s.x - nn.x * e3s.z);
        real e3z = real(3.) * g.radial_velocity * (nn.x * e3s.y - nn.y * e3s.x);
        real ax = fa * (e1x - e2x + e3x);
        real ay = fa * (e1y - e2y + e3y);
        real az = fa * (e1z - e2z + e3z);
        sum.x += q.mass / h.mass * ax;
        sum.y += q.mass / h.mass * ay;
        sum.z += q.mass / h.mass * az;
        g.out_acc.x += ax; g.out_acc.y += ay; g.out_acc.z += az;
        // Kidder 1995 eq. 2.4a
        real mu = (h.mass * q.mass) / M;
        V3 lo{mu * (g.pos.y * g.vel.z - g.pos.z * g.vel.y),
              mu * (g.pos.z * g.vel.x - g.pos.x * g.vel.z),
              mu * (g.pos.x * g.vel.y - g.pos.y * g.vel.x)};
        real fm = real(2.) + real(3. / 2.) * q.mass / h.mass;
        real h1x = fm * (lo.y * sL.z - lo.z * sL.y);
        real h1y = fm * (lo.z * sL.x - lo.x * sL.z);
        real h1z = fm * (lo.x * sL.y - lo.y * sL.x);
        real h2x = pL.y * sL.z - pL.z * sL.y;
        real h2y = pL.z * sL.x - pL.x * sL.z;
        real h2z = pL.x * sL.y - pL.y * sL.x;
        real sp = nn.x * pL.x + nn.y * pL.y + nn.z * pL.z;
        real h3x = real(3.) * sp * (nn.y * sL.z - nn.z * sL.y);
        real h3y = real(3.) * sp * (nn.z * sL.x - nn.x * sL.z);
        real h3z = real(3.) * sp * (nn.x * sL.y - nn.y * sL.x);
        h.gr.out_dldt.x += fa * (h1x - h2x + h3x);
        h.gr.out_dldt.y += fa * (h1y - h2y + h3y);
        h.gr.out_dldt.z += fa * (h1z - h2z + h3z);
        // Kidder 1995 eq. 2.4b
        real fm2 = real(2.) + real(3. / 2.) * h.mass / q.mass;
        real q1x = fm2 * (lo.y * pL.z - lo.z * pL.y);
        real q1y = fm2 * (lo.z * pL.x - lo.x * pL.z);
        real q1z = fm2 * (lo.x * pL.y - lo.y * pL.x);
        real q2x = sL.y * pL.z - sL.z * pL.y;
        real q2y = sL.z * pL.x - sL.x * pL.z;
        real q2z = sL.x * pL.y - sL.y * pL.x;
        real ss = nn.x * sL.x + nn.y * sL.y + nn.z * sL.z;
        real q3x = real(3.) * ss * (nn.y * pL.z - nn.z * pL.y);
        real q3y = real(3.) * ss * (nn.z * pL.x - nn.x * pL.z);
        real q3z = real(3.) * ss * (nn.x * pL.y - nn.y * pL.x);
        g.out_dldt.x = fa * (q1x - q2x + q3x);
        g.out_dldt.y = fa * (q1y - q2y + q3y);
        g.out_dldt.z = fa * (q1z - q2z + q3z);
    }
    h.gr.out_acc.x += real(-1.0) * sum.x;
    h.gr.out_acc.y += real(-1.0) * sum.y;
    h.gr.out_acc.z += real(-1.0) * sum.z;
}

// ---------------------------------------------------------------------------
// General relativity after REBOUNDx gr.c: src/effects/general_relativity.rs
// ---------------------------------------------------------------------------
// Bodies other than the host, in index order (the reference's
// particles.iter().chain(more_particles.iter())).
static std::vector<int> others(const Sim& s) {
    std::vector<int> o;
    for (int i = 0; i < s.n; ++i)
        if (i != s.host) o.push_back(i);
    return o;
}

// :661-697 -- the integrator's gravity accelerations plus the host terms it
// ignored (WHFastOne: the first other body only; WHFastTwo: all).  The
// separation is the host's inertial position minus the body's heliocentric
// (GR) position, as in the reference.
static void gr_newtonian_accelerations(Sim& s, int ignore, V3& ha, std::vector<V3>& na) {
    const std::vector<int> o = others(s);
    Particle& h = s.p[s.host];
    ha = h.a;
    na.assign(o.size(), V3{0., 0., 0.});
    for (size_t k = 0; k < o.size(); ++k) na[k] = s.p[o[k]].a;
    if (ignore == 1 || ignore == 2) {
        const size_t np = ignore == 1 ? 1 : o.size();
        for (size_t k = 0; k < np && k < o.size(); ++k) {
            const Particle& q = s.p[o[k]];
            real dx = h.r.x - q.gr.pos.x, dy = h.r.y - q.gr.pos.y, dz = h.r.z - q.gr.pos.z;
            real r2 = powi(dx, 2) + powi(dy, 2) + powi(dz, 2);
            real r = rsqrt_(r2);
            real prefac = G / (r2 * r);
            real pms = prefac * h.mass;
            real pmp = prefac * q.mass;
            ha.x -= pmp * dx; ha.y -= pmp * dy; ha.z -= pmp * dz;
            na[k].x += pms * dx; na[k].y += pms * dy; na[k].z += pms * dz;
        }
    }
}

// :461-535 with the Jacobi transforms :537-634
static void gr_anderson1975(Sim& s, int ignore) {
    const std::vector<int> o = others(s);
    const size_t no = o.size();
    Particle& h = s.p[s.host];
    V3 ha;
    std::vector<V3> na;
    gr_newtonian_accelerations(s, ignore, ha, na);
    std::vector<V3> jp(no, V3{0., 0., 0.}), jv(no, V3{0., 0., 0.}), ja(no, V3{0., 0., 0.});
    real eta = h.mass;
    real sx = eta * h.r.x, sy = eta * h.r.y, sz = eta * h.r.z;
    real svx = eta * h.v.x, svy = eta * h.v.y, svz = eta * h.v.z;
    real sax = eta * ha.x, say = eta * ha.y, saz = eta * ha.z;
    for (size_t k = 0; k < no; ++k) {
        const Particle& q = s.p[o[k]];
        if (q.gr.kind != POSI_EFFECT_ORBITING) continue;
        real ei = real(1.) / eta;
        eta += q.mass;
        real pme = eta * ei;
        jp[k].x = q.r.x - sx * ei; jp[k].y = q.r.y - sy * ei; jp[k].z = q.r.z - sz * ei;
        jv[k].x = q.v.x - svx * ei; jv[k].y = q.v.y - svy * ei; jv[k].z = q.v.z - svz * ei;
        ja[k].x = na[k].x - sax * ei; ja[k].y = na[k].y - say * ei; ja[k].z = na[k].z - saz * ei;
        sx = sx * pme + q.mass * jp[k].x; sy = sy * pme + q.mass * jp[k].y; sz = sz * pme + q.mass * jp[k].z;
        svx = svx * pme + q.mass * jv[k].x; svy = svy * pme + q.mass * jv[k].y; svz = svz * pme + q.mass * jv[k].z;
        sax = sax * pme + q.mass * ja[k].x; say = say * pme + q.mass * ja[k].y; saz = saz * pme + q.mass * ja[k].z;
    }
    const real mtot = eta;
    const real mu = h.mass_g;
    for (size_t k = 0; k < no; ++k) {
        const Particle& q = s.p[o[k]];
        if (q.gr.kind != POSI_EFFECT_ORBITING) continue;
        V3 vi = jv[k];
        real vi2 = powi(jv[k].x, 2) + powi(jv[k].y, 2) + powi(jv[k].z, 2);
        real ri = rsqrt_(powi(jp[k].x, 2) + powi(jp[k].y, 2) + powi(jp[k].z, 2));
        real fa = (real(0.5) * vi2 + real(3.) * mu / ri) / SPEED_OF_LIGHT_2;
        for (int it = 0; it < 10; ++it) {
            V3 old = vi;
            vi.x = jv[k].x / (real(1.) - fa);
            vi.y = jv[k].y / (real(1.) - fa);
            vi.z = jv[k].z / (real(1.) - fa);
            vi2 = vi.x * vi.x + vi.y * vi.y + vi.z * vi.z;
            fa = (real(0.5) * vi2 + real(3.) * mu / ri) / SPEED_OF_LIGHT_2;
            real dvx = vi.x - old.x, dvy = vi.y - old.y, dvz = vi.z - old.z;
            if ((dvx * dvx + dvy * dvy + dvz * dvz) / vi2 < DBL_EPSILON_2) break;
        }
        real fb = (mu / ri - real(1.5) * vi2) * mu / (ri * ri * ri) / SPEED_OF_LIGHT_2;
        real rdotrdot = jp[k].x * jv[k].x + jp[k].y * jv[k].y + jp[k].z * jv[k].z;
        V3 vidot{ja[k].x + fb * jp[k].x, ja[k].y + fb * jp[k].y, ja[k].z + fb * jp[k].z};
        real vdotvdot = vi.x * vidot.x + vi.y * vidot.y + vi.z * vidot.z;
        real fd = (vdotvdot - real(3.) * mu / (ri * ri * ri) * rdotrdot) / SPEED_OF_LIGHT_2;
        ja[k].x = fb * (real(1.) - fa) * jp[k].x - fa * ja[k].x - fd * vi.x;
        ja[k].y = fb * (real(1.) - fa) * jp[k].y - fa * ja[k].y - fd * vi.y;
        ja[k].z = fb * (real(1.) - fa) * jp[k].z - fa * ja[k].z - fd * vi.z;
    }
    // Jacobi -> inertial with a zero Jacobi star acceleration
    eta = mtot;
    sax = eta * real(0.); say = eta * real(0.); saz = eta * real(0.);
    std::vector<V3> pa(no, V3{0., 0., 0.});
    for (size_t kk = no; kk-- > 0;) {
        const Particle& q = s.p[o[kk]];
        if (q.gr.kind != POSI_EFFECT_ORBITING) continue;
        real ei = real(1.) / eta;
        sax = (sax - q.mass * ja[kk].x) * ei;
        say = (say - q.mass * ja[kk].y) * ei;
        saz = (saz - q.mass * ja[kk].z) * ei;
        pa[kk].x = ja[kk].x + sax; pa[kk].y = ja[kk].y + say; pa[kk].z = ja[kk].z + saz;
        eta -= q.mass;
        sax *= eta; say *= eta; saz *= eta;
    }
    real mi = real(1.) / eta;
    for (size_t k = 0; k < no; ++k) {
        Particle& q = s.p[o[k]];
        if (q.gr.kind == POSI_EFFECT_ORBITING) q.gr.out_acc = pa[k];
    }
    h.gr.out_acc = V3{sax * mi, say * mi, saz * mi};
}

// :702-898 -- every pair of bodies, the host first then the others in index
// order; the constant part once, the acceleration-dependent part iterated.
// The convergence test keeps the reference's form: a component's relative
// change is taken only where |a| < 1e-30, otherwise the previous value stays.
static void gr_newhall1983(Sim& s, int ignore) {
    std::vector<int> ord{s.host};
    for (int i : others(s)) ord.push_back(i);
    const size_t N = ord.size();
    V3 ha;
    std::vector<V3> na;
    gr_newtonian_accelerations(s, ignore, ha, na);
    std::vector<V3> an(N);
    an[0] = ha;
    for (size_t k = 1; k < N; ++k) an[k] = na[k - 1];
    auto P = [&](size_t t) -> const Particle& { return s.p[ord[t]]; };
    auto on = [&](size_t t) { return P(t).gr.kind != POSI_EFFECT_DISABLED; };
    std::vector<std::vector<real>> rs(N, std::vector<real>(N, real(0.)));
    std::vector<std::vector<V3>> drs(N, std::vector<V3>(N, V3{0., 0., 0.}));
    for (size_t i = 0; i < N; ++i)
        for (size_t j = 0; j < N; ++j) {
            if (j == i || !(on(i) || on(j))) continue;
            drs[i][j] = V3{P(i).r.x - P(j).r.x, P(i).r.y - P(j).r.y, P(i).r.z - P(j).r.z};
            rs[i][j] = rsqrt_(powi(drs[i][j].x, 2) + powi(drs[i][j].y, 2) + powi(drs[i][j].z, 2));
        }
    std::vector<V3> ac(N, V3{0., 0., 0.});
    for (size_t i = 0; i < N; ++i) {
        const Particle& pi = P(i);
        real cx = 0., cy = 0., cz = 0.;
        for (size_t j = 0; j < N; ++j) {
            if (j == i || !(on(i) || on(j))) continue;
            const Particle& pj = P(j);
            real dxij = drs[i][j].x, dyij = drs[i][j].y, dzij = drs[i][j].z;
            real rij2 = powi(rs[i][j], 2);
            real rij3 = rij2 * rs[i][j];
            real a1 = 0.;
            for (size_t k = 0; k < N; ++k)
                if (k != i) a1 += (real(4.) / SPEED_OF_LIGHT_2) * G * P(k).mass / rs[i][k];
            real a2 = 0.;
            for (size_t l = 0; l < N; ++l)
                if (l != j) a2 += (real(1.) / SPEED_OF_LIGHT_2) * G * P(l).mass / rs[l][j];
            real vi2 = powi(pi.v.x, 2) + powi(pi.v.y, 2) + powi(pi.v.z, 2);
            real a3 = -vi2 / SPEED_OF_LIGHT_2;
            real vj2 = powi(pj.v.x, 2) + powi(pj.v.y, 2) + powi(pj.v.z, 2);
            real a4 = real(-2.) * vj2 / SPEED_OF_LIGHT_2;
            real a5 = (real(4.) / SPEED_OF_LIGHT_2) * (pi.v.x * pj.v.x + pi.v.y * pj.v.y + pi.v.z * pj.v.z);
            real a6_0 = dxij * pj.v.x + dyij * pj.v.y + dzij * pj.v.z;
            real a6 = (real(3.) / (real(2.) * SPEED_OF_LIGHT_2)) * powi(a6_0, 2) / rij2;
            real f1 = a1 + a2 + a3 + a4 + a5 + a6;
            cx += G * pj.mass * dxij * f1 / rij3;
            cy += G * pj.mass * dyij * f1 / rij3;
            cz += G * pj.mass * dzij * f1 / rij3;
            real dvx = pi.v.x - pj.v.x, dvy = pi.v.y - pj.v.y, dvz = pi.v.z - pj.v.z;
            real f2 = dxij * (real(4.) * pi.v.x - real(3.) * pj.v.x) + dyij * (real(4.) * pi.v.y - real(3.) * pj.v.y) +
                      dzij * (real(4.) * pi.v.z - real(3.) * pj.v.z);
            cx += G * pj.mass * f2 * dvx / rij3 / SPEED_OF_LIGHT_2;
            cy += G * pj.mass * f2 * dvy / rij3 / SPEED_OF_LIGHT_2;
            cz += G * pj.mass * f2 * dvz / rij3 / SPEED_OF_LIGHT_2;
        }
        ac[i] = V3{cx, cy, cz};
    }
    std::vector<V3> anew(N, V3{0., 0., 0.}), aold(N);
    const real dev_limit = 1.0e-30;
    for (int it = 0; it < 10; ++it) {
        aold = anew;
        for (size_t i = 0; i < N; ++i) {
            real nx = 0., ny = 0., nz = 0.;
            for (size_t j = 0; j < N; ++j) {
                if (j == i || !(on(i) || on(j))) continue;
                const Particle& pj = P(j);
                real dxij = drs[i][j].x, dyij = drs[i][j].y, dzij = drs[i][j].z;
                real rij = rs[i][j];
                real rij2 = powi(rij, 2);
                real rij3 = rij2 * rij;
                real sx_ = an[j].x + aold[j].x, sy_ = an[j].y + aold[j].y, sz_ = an[j].z + aold[j].z;
                real dot = dxij * sx_ + dyij * sy_ + dzij * sz_;
                nx += (G * pj.mass * dxij / rij3) * dot / (real(2.) * SPEED_OF_LIGHT_2) +
                      (real(7.) / (real(2.) * SPEED_OF_LIGHT_2)) * G * pj.mass * sx_ / rij;
                ny += (G * pj.mass * dyij / rij3) * dot / (real(2.) * SPEED_OF_LIGHT_2) +
                      (real(7.) / (real(2.) * SPEED_OF_LIGHT_2)) * G * pj.mass * sy_ / rij;
                nz += (G * pj.mass * dzij / rij3) * dot / (real(2.) * SPEED_OF_LIGHT_2) +
                      (real(7.) / (real(2.) * SPEED_OF_LIGHT_2)) * G * pj.mass * sz_ / rij;
            }
            anew[i] = V3{ac[i].x + nx, ac[i].y + ny, ac[i].z + nz};
        }
        real maxdev = 0., dx = 0., dy = 0., dz = 0.;
        for (size_t i = 0; i < N; ++i) {
            if (!on(i)) continue;
            if (rabs(anew[i].x) < dev_limit) dx = rabs(anew[i].x - aold[i].x) / anew[i].x;
            if (rabs(anew[i].y) < dev_limit) dy = rabs(anew[i].y - aold[i].y) / anew[i].y;
            if (rabs(anew[i].z) < dev_limit) dz = rabs(anew[i].z - aold[i].z) / anew[i].z;
            if (dx > maxdev) maxdev = dx;
            if (dy > maxdev) maxdev = dy;
            if (dz > maxdev) maxdev = dz;
        }
        if (maxdev < dev_limit) break;
    }
    for (size_t k = 1; k < N; ++k) {
        Particle& q = s.p[ord[k]];
        if (q.gr.kind == POSI_EFFECT_ORBITING) q.gr.out_acc = anew[k];
    }
    s.p[s.host].gr.out_acc = anew[0];
}

// src/effects/wind.rs:72-91 (Bolmont & Mathis 2016 eq. 14)
static void calculate_wind_factor(Sim& s) {
    for (int i = 0; i < s.n; ++i) {
        Particle& q = s.p[i];
        if (q.wind_kind != 1) continue;
        real threshold = rsqrt_(q.nsv2);
        real w = threshold >= q.wind_rsat ? q.wind_rsat2 : q.nsv2;
        q.wind_dldt.x = real(-1.) * q.wind_k * q.spin.x * w * rsqrt_(q.radius / R_SUN * real(1.) / q.mass);
        q.wind_dldt.y = real(-1.) * q.wind_k * q.spin.y * w * rsqrt_(q.radius / R_SUN * real(1.) / q.mass);
        q.wind_dldt.z = real(-1.) * q.wind_k * q.spin.z * w * rsqrt_(q.radius / R_SUN * real(1.) / q.mass);
    }
}

// src/effects/disk.rs:154-203 (DiskProperties::calculate_migration_timescale)
static real disk_migration_timescale(const Disk& dp, real time, real host_mass, real host_mass_g,
                                     real particle_mass, real distance, real semi_major_axis) {
    real keplerian_frequency = rsqrt_(host_mass_g / powi(distance, 3));
    real disk_temperature = real(280.0) * real(std::pow(dv(distance), -0.5)) * host_mass;
    real speed_of_sound_squared = BOLTZMANN_CONSTANT * disk_temperature / (dp.mu * MASS_HYDROGEN_ATOM);
    real viscosity = dp.alpha * speed_of_sound_squared / keplerian_frequency;
    real gas_radial_velocity = real(-3.0) * viscosity / (real(2.0) * semi_major_axis);
    real initial_density = dp.sigma0 * (real(1.) / distance) * real(std::exp(dv(real(-1.0) * distance / dp.outer))) *
                           (real(1.0) - rsqrt_(dp.inner / distance));
    real density = 0.;
    if (distance > dp.inner) density = initial_density * real(std::exp(dv(-time / dp.lifetime)));
    real y = real(2.0) * density * powi(semi_major_axis, 2) / particle_mass;
    real m = y < real(1.0) ? y : real(1.0);   // f64::min(1.0, y)
    real a_dot = gas_radial_velocity * m;
    return -semi_major_axis / a_dot;
}

// src/effects/disk.rs:205-268
static void disk_interaction_acceleration(Sim& s, real t) {
    Particle& h = s.p[s.host];
    if (h.disk.kind != POSI_EFFECT_CENTRAL) return;
    real factor2 = real(1.) / h.mass;
    V3 sum{0., 0., 0.};
    for (int i = 0; i < s.n; ++i) {
        if (i == s.host) continue;
        Particle& q = s.p[i];
        if (q.disk.kind == POSI_EFFECT_ORBITING) {
            Disk& d = q.disk;
            real sma = (q.mass_g + h.mass_g) * d.distance / (real(2.0) * (q.mass_g + h.mass_g) - d.distance * d.nv2);
            d.migration_timescale = disk_migration_timescale(h.disk, t, h.mass, h.mass_g, q.mass, d.distance, sma);
            real factor1 = real(1.) / q.mass;
            real factor_migration = -q.mass / d.migration_timescale;
            real ecc_ts = real(0.1) * d.migration_timescale;
            real factor_ecc = -q.mass * real(2.0) / ecc_ts;
            real inc_ts = ecc_ts;
            real factor_inc = -q.mass * real(2.0) / inc_ts;
            V3 fm{factor_migration * d.vel.x, factor_migration * d.vel.y, factor_migration * d.vel.z};
            real sp = real(1.0) / (d.distance * d.distance) * (d.pos.x * d.vel.x + d.pos.y * d.vel.y + d.pos.z * d.vel.z);
            V3 fe{factor_ecc * sp * d.pos.x, factor_ecc * sp * d.pos.y, factor_ecc * sp * d.pos.z};
            V3 fi{0.0, 0.0, factor_inc * d.vel.z};
            V3 ft{fm.x + fe.x + fi.x, fm.y + fe.y + fi.y, fm.z + fe.z + fi.z};
            sum.x += ft.x; sum.y += ft.y; sum.z += ft.z;
            d.out_acc = V3{factor1 * ft.x, factor1 * ft.y, factor1 * ft.z};
        }
        h.disk.out_acc = V3{real(-1.0) * factor2 * sum.x, real(-1.0) * factor2 * sum.y, real(-1.0) * factor2 * sum.z};
    }
}

// src/particles/universe.rs:580-614
static void calculate_dangular_momentum_dt(Sim& s) {
    for (int i = 0; i < s.n; ++i) {
        Particle& q = s.p[i];
        q.dLdt.x = q.tides.out_dldt.x + q.flat.out_dldt.x + q.gr.out_dldt.x + q.wind_dldt.x;
        q.dLdt.y = q.tides.out_dldt.y + q.flat.out_dldt.y + q.gr.out_dldt.y + q.wind_dldt.y;
        q.dLdt.z = q.tides.out_dldt.z + q.flat.out_dldt.z + q.gr.out_dldt.z + q.wind_dldt.z;
    }
}

// src/particles/universe.rs:540-567
static void add_additional_acceleration_corrections(Sim& s) {
    for (int i = 0; i < s.n; ++i) {
        Particle& q = s.p[i];
        if (s.tides) { q.a_add.x += q.tides.out_acc.x; q.a_add.y += q.tides.out_acc.y; q.a_add.z += q.tides.out_acc.z; }
        if (s.disk) { q.a_add.x += q.disk.out_acc.x; q.a_add.y += q.disk.out_acc.y; q.a_add.z += q.disk.out_acc.z; }
        if (s.flat) { q.a_add.x += q.flat.out_acc.x; q.a_add.y += q.flat.out_acc.y; q.a_add.z += q.flat.out_acc.z; }
        if (s.gr) { q.a_add.x += q.gr.out_acc.x; q.a_add.y += q.gr.out_acc.y; q.a_add.z += q.gr.out_acc.z; }
    }
}

// src/particles/universe.rs:428-538
static void calculate_additional_effects(Sim& s, real t, bool evolution, bool dl, bool acc, int ignore) {
    initialize(s, dl, acc);
    calculate_spin_and_evolving_quantities(s, t, evolution);
    if (s.fatal()) return;
    if (dl && s.wind) calculate_wind_factor(s);
    if (s.tides || s.flat) {
        if ((dl && (s.tides || s.flat)) || (acc && (s.tides || s.disk || s.flat || s.gr))) {
            pair_dependent_scaled_dissipation_factors(s);
            if (s.tides) tides_orthogonal(s);
            if (s.flat) flat_orthogonal(s);
            if (acc && (s.tides || s.flat)) {
                if (s.tides) { tides_radial(s); tidal_acceleration(s); }
                if (s.flat) { flat_radial(s); flat_acceleration(s); }
            }
            if (dl && (s.tides || s.flat)) {
                if (s.tides) tides_dangular_momentum_dt(s);
                if (s.flat) flat_dangular_momentum_dt(s);
            }
        }
    }
    if (acc && s.gr) {
        if (s.p[s.host].gr.kind == POSI_EFFECT_CENTRAL) {
            if (s.gr_impl == POSI_GR_ANDERSON1975) {
                gr_anderson1975(s, ignore);
            } else if (s.gr_impl == POSI_GR_NEWHALL1983) {
                gr_newhall1983(s, ignore);
            } else {
                gr_first_order(s);
                gr_second_order(s);
                gr_spin_orbit(s);
            }
        }
    }
    if (acc && s.disk) disk_interaction_acceleration(s, t);
    if (dl) {
        if (s.tides || s.flat || (s.gr && s.gr_impl == POSI_GR_KIDDER1995) || s.wind) calculate_dangular_momentum_dt(s);
    }
    if (acc) add_additional_acceleration_corrections(s);
}

// ---------------------------------------------------------------------------
// WHFast: src/integrator/whfast.rs
// ---------------------------------------------------------------------------
// :424-451
static bool converged_velocity_dependent_forces_integration(const Sim& s, const std::vector<V3>& fv,
                                                            const std::vector<V3>& fL,
                                                            const std::vector<V3>& pv,
                                                            const std::vector<V3>& pL, bool spin) {
    real fv2 = 0., dv2 = 0., fL2 = 0., dL2 = 0.;
    for (int i = 0; i < s.n; ++i) {
        real dvx = fv[i].x - pv[i].x, dvy = fv[i].y - pv[i].y, dvz = fv[i].z - pv[i].z;
        dv2 += powi(dvx, 2) + powi(dvy, 2) + powi(dvz, 2);
        fv2 += powi(fv[i].x, 2) + powi(fv[i].y, 2) + powi(fv[i].z, 2);
        if (spin) {
            real dsx = fL[i].x - pL[i].x, dsy = fL[i].y - pL[i].y, dsz = fL[i].z - pL[i].z;
            dL2 += powi(dsx, 2) + powi(dsy, 2) + powi(dsz, 2);
            fL2 += powi(fL[i].x, 2) + powi(fL[i].y, 2) + powi(fL[i].z, 2);
        }
    }
    return (spin && dv2 / fv2 < real(DBL_EPSILON_2) && dL2 / fL2 < real(DBL_EPSILON_2)) ||
           (!spin && dv2 / fv2 < real(DBL_EPSILON_2));
}

// :322-422
static void integrate_velocity_dependent_forces(Sim& s, real dt, bool spin, bool evolution) {
    const int n = s.n;
    std::vector<V3> ov(n), oL(n), fv(n), fL(n), pv(n), pL(n), dvc(n, V3{0., 0., 0.}), dLc(n, V3{0., 0., 0.});
    for (int i = 0; i < n; ++i) { ov[i] = s.p[i].v; oL[i] = s.p[i].L; fv[i] = ov[i]; fL[i] = oL[i]; }
    bool converged = false;
    int iters = 0;
    for (int it = 0; it < IMPLICIT_MIDPOINT_MAX_ITER; ++it) {
        iters = it + 1;
        pv = fv; pL = fL;
        inertial_to_heliocentric(s);
        calculate_additional_effects(s, s.t, evolution && it == 0, spin, true, s.coords == POSI_JACOBI ? 1 : 2);
        if (s.fatal()) return;
        for (int i = 0; i < n; ++i) {
            const Particle& q = s.p[i];
            dvc[i].x = dt * q.a_add.x - s.errv[i].x;
            dvc[i].y = dt * q.a_add.y - s.errv[i].y;
            dvc[i].z = dt * q.a_add.z - s.errv[i].z;
            fv[i].x = ov[i].x + dvc[i].x;
            fv[i].y = ov[i].y + dvc[i].y;
            fv[i].z = ov[i].z + dvc[i].z;
            if (spin) {
                dLc[i].x = dt * q.dLdt.x - s.errL[i].x;
                dLc[i].y = dt * q.dLdt.y - s.errL[i].y;
                dLc[i].z = dt * q.dLdt.z - s.errL[i].z;
                fL[i].x = oL[i].x + dLc[i].x;
                fL[i].y = oL[i].y + dLc[i].y;
                fL[i].z = oL[i].z + dLc[i].z;
            }
        }
        if (it >= IMPLICIT_MIDPOINT_MIN_ITER - 1 && converged_velocity_dependent_forces_integration(s, fv, fL, pv, pL, spin)) {
            converged = true;
            break;
        }
        for (int i = 0; i < n; ++i) {
            Particle& q = s.p[i];
            q.v.x = real(0.5) * (ov[i].x + fv[i].x);
            q.v.y = real(0.5) * (ov[i].y + fv[i].y);
            q.v.z = real(0.5) * (ov[i].z + fv[i].z);
            if (spin) {
                q.L.x = real(0.5) * (oL[i].x + fL[i].x);
                q.L.y = real(0.5) * (oL[i].y + fL[i].y);
                q.L.z = real(0.5) * (oL[i].z + fL[i].z);
            }
        }
    }
    s.last_midpoint_iters = iters;
    if (!converged) s.status |= POSI_SYS_WARN_NONCONVERGED;
    for (int i = 0; i < n; ++i) {
        Particle& q = s.p[i];
        q.v = fv[i];
        s.errv[i].x = (q.v.x - ov[i].x) - dvc[i].x;
        s.errv[i].y = (q.v.y - ov[i].y) - dvc[i].y;
        s.errv[i].z = (q.v.z - ov[i].z) - dvc[i].z;
        if (spin) {
            q.L = fL[i];
            s.errL[i].x = (q.L.x - oL[i].x) - dLc[i].x;
            s.errL[i].y = (q.L.y - oL[i].y) - dLc[i].y;
            s.errL[i].z = (q.L.z - oL[i].z) - dLc[i].z;
        }
    }
}

// :844-876
static void stumpff_cs3(real z_in, real cs[4]) {
    static const double invfactorial[14] = {1., 1., 1. / 2., 1. / 6., 1. / 24., 1. / 120., 1. / 720., 1. / 5040.,
                                            1. / 40320., 1. / 362880., 1. / 3628800., 1. / 39916800.,
                                            1. / 479001600., 1. / 6227020800.};
    real z = z_in;
    int n = 0;
    while (rabs(z) > real(0.1)) { z = z / real(4.); n += 1; }
    const int nmax = 13;
    real c_odd = invfactorial[nmax];
    real c_even = invfactorial[nmax - 1];
    int np = nmax - 2;
    while (np >= 3) {
        c_odd = real(invfactorial[np]) - z * c_odd;
        c_even = real(invfactorial[np - 1]) - z * c_even;
        np -= 2;
    }
    cs[3] = c_odd;
    cs[2] = c_even;
    cs[1] = real(invfactorial[1]) - z * c_odd;
    cs[0] = real(invfactorial[0]) - z * c_even;
    while (n > 0) {
        cs[3] = (cs[2] + cs[0] * cs[3]) * real(0.25);
        cs[2] = cs[1] * cs[1] * real(0.5);
        cs[1] = cs[0] * cs[1];
        cs[0] = real(2.) * cs[0] * cs[0] - real(1.);
        n -= 1;
    }
}

// :835-842
static void stiefel_gs3(real beta, real x, real gs[4]) {
    real x2 = powi(x, 2);
    stumpff_cs3(beta * x2, gs);
    gs[1] = gs[1] * x;
    gs[2] = gs[2] * x2;
    gs[3] = gs[3] * (x2 * x);
}

// :676-833
static void kepler_individual_step(Sim& s, int i, real mass_g, real dt) {
    V3 p1p = s.alt[i].pos, p1v = s.alt[i].vel;
    real r0 = rsqrt_(powi(p1p.x, 2) + powi(p1p.y, 2) + powi(p1p.z, 2));
    real r0i = real(1.) / r0;
    real v2 = powi(p1v.x, 2) + powi(p1v.y, 2) + powi(p1v.z, 2);
    real beta = real(2.) * mass_g * r0i - v2;
    real eta0 = p1p.x * p1v.x + p1p.y * p1v.y + p1p.z * p1v.z;
    real zeta0 = mass_g - beta * r0;
    real x;
    real gs[4];
    real invperiod = 0.;
    real x_per_period;
    bool x_per_period_nan;
    if (beta > real(0.)) {
        real sqrt_beta = rsqrt_(beta);
        invperiod = sqrt_beta * beta / (real(2.) * real(PI) * mass_g);
        x_per_period = real(2.) * real(PI) / sqrt_beta;
        x_per_period_nan = risnan(x_per_period);
        if (rabs(dt) * invperiod > real(1.) && s.timestep_warning == 0) {
            s.status |= POSI_SYS_WARN_TIMESTEP;
            s.timestep_warning += 1;
        }
        real dtr0i = dt * r0i;
        x = dtr0i * (real(1.) - dtr0i * eta0 * real(0.5) * r0i);
    } else {
        x = 0.;
        x_per_period = 0.;
        x_per_period_nan = true;
    }
    int converged = 0;
    real old_x = x;
    stiefel_gs3(beta, x, gs);
    real eta0_gs1_zeta0_gs2 = eta0 * gs[1] + zeta0 * gs[2];
    real ri = real(1.) / (r0 + eta0_gs1_zeta0_gs2);
    x = ri * (x * eta0_gs1_zeta0_gs2 - eta0 * gs[2] - zeta0 * gs[3] + dt);
    if (!x_per_period_nan && rabs(x - old_x) > real(0.01) * x_per_period) {
        x = beta * dt / mass_g;
        real prev_x[WHFAST_NMAX_QUART + 1];
        for (int k = 0; k <= WHFAST_NMAX_QUART; ++k) prev_x[k] = 0.;
        bool done = false;
        for (int n_lag = 1; n_lag < WHFAST_NMAX_QUART && !done; ++n_lag) {
            stiefel_gs3(beta, x, gs);
            real f = r0 * x + eta0 * gs[2] + zeta0 * gs[3] - dt;
            real fp = r0 + eta0 * gs[1] + zeta0 * gs[2];
            real fpp = eta0 * gs[0] + zeta0 * gs[1];
            real denom = fp + rsqrt_(rabs(real(16.) * fp * fp - real(20.) * f * fpp));
            x = (x * denom - real(5.) * f) / denom;
            for (int k = 1; k < n_lag; ++k) {
                if (x == prev_x[k]) { converged = 1; done = true; break; }
            }
            if (!done) prev_x[n_lag] = x;
        }
        real e = eta0 * gs[1] + zeta0 * gs[2];
        ri = real(1.) / (r0 + e);
    } else {
        real old_x2;
        for (int k = 1; k < WHFAST_NMAX_NEWT; ++k) {
            old_x2 = old_x;
            old_x = x;
            stiefel_gs3(beta, x, gs);
            real e = eta0 * gs[1] + zeta0 * gs[2];
            ri = real(1.) / (r0 + e);
            x = ri * (x * e - eta0 * gs[2] - zeta0 * gs[3] + dt);
            if (x == old_x || x == old_x2) { converged = 1; break; }
        }
    }
    if (converged == 0) {
        real x_min, x_max;
        if (beta > real(0.)) {
            x_min = x_per_period * rfloor(dt * invperiod);
            x_max = x_min + x_per_period;
        } else {
            real h2 = r0 * r0 * v2 - eta0 * eta0;
            real q = h2 / mass_g / (real(1.) + rsqrt_(real(1.) - h2 * beta / (mass_g * mass_g)));
            real vq = rsqrt_(h2) / q;
            x_min = real(1.) / (vq + r0 / dt);
            x_max = dt / q;
        }
        x = (x_max + x_min) / real(2.);
        int guard = 0;
        for (;;) {
            stiefel_gs3(beta, x, gs);
            real sres = r0 * x + eta0 * gs[2] + zeta0 * gs[3] - dt;
            if (sres >= real(0.)) x_max = x; else x_min = x;
            x = (x_max + x_min) / real(2.);
            if (rabs(x_max - x_min) / x_max <= real(1e-15)) break;
            if (++guard > 4096) { set_fatal(s, POSI_SYS_BISECTION_LIMIT, i, i); break; }
        }
        real e = eta0 * gs[1] + zeta0 * gs[2];
        ri = real(1.) / (r0 + e);
    }
    if (risnan(ri)) {
        ri = 0.; gs[1] = 0.; gs[2] = 0.; gs[3] = 0.;
    }
    real f = -mass_g * gs[2] * r0i;
    real g = dt - mass_g * gs[3];
    real fd = -mass_g * gs[1] * r0i * ri;
    real gd = -mass_g * gs[2] * ri;
    AltCoords& pj = s.alt[i];
    pj.pos.x += f * p1p.x + g * p1v.x;
    pj.pos.y += f * p1p.y + g * p1v.y;
    pj.pos.z += f * p1p.z + g * p1v.z;
    pj.vel.x += fd * p1p.x + gd * p1v.x;
    pj.vel.y += fd * p1p.y + gd * p1v.y;
    pj.vel.z += fd * p1p.z + gd * p1v.z;
}

// :628-672
static void kepler_steps(Sim& s, real dt) {
    const int mm = s.host;
    if (s.coords == POSI_JACOBI) {
        real gm = s.p[mm].mass_g;
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            gm += s.alt[i].mass_g;
            kepler_individual_step(s, i, gm, dt);
        }
    } else if (s.coords == POSI_DEMOCRATIC_HELIOCENTRIC) {
        real gm = s.p[mm].mass_g;
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            kepler_individual_step(s, i, gm, dt);
        }
    } else {
        real gm0 = s.p[mm].mass_g;
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            kepler_individual_step(s, i, gm0 + s.alt[i].mass_g, dt);
        }
    }
    AltCoords& st = s.alt[mm];
    st.pos.x += dt * st.vel.x;
    st.pos.y += dt * st.vel.y;
    st.pos.z += dt * st.vel.z;
}

// :889-933
static void inertial_to_jacobi_posvel(Sim& s) {
    const int mm = s.host;
    const Particle& star = s.p[mm];
    real m0 = star.mass;
    real eta = m0;
    real sx = eta * star.r.x, sy = eta * star.r.y, sz = eta * star.r.z;
    real svx = eta * star.v.x, svy = eta * star.v.y, svz = eta * star.v.z;
    for (int i = 0; i < s.n; ++i) {
        if (i == mm) continue;
        const Particle& q = s.p[i];
        AltCoords& a = s.alt[i];
        real ei = real(1.) / eta;
        eta += q.mass;
        real pme = eta * ei;
        a.mass = q.mass;
        a.mass_g = q.mass_g;
        a.pos.x = q.r.x - sx * ei;
        a.pos.y = q.r.y - sy * ei;
        a.pos.z = q.r.z - sz * ei;
        a.vel.x = q.v.x - svx * ei;
        a.vel.y = q.v.y - svy * ei;
        a.vel.z = q.v.z - svz * ei;
        sx = sx * pme + q.mass * a.pos.x;
        sy = sy * pme + q.mass * a.pos.y;
        sz = sz * pme + q.mass * a.pos.z;
        svx = svx * pme + q.mass * a.vel.x;
        svy = svy * pme + q.mass * a.vel.y;
        svz = svz * pme + q.mass * a.vel.z;
    }
    real mtot = eta;
    real mtot_i = real(1.) / mtot;
    AltCoords& st = s.alt[mm];
    st.mass = mtot;
    st.pos.x = sx * mtot_i; st.pos.y = sy * mtot_i; st.pos.z = sz * mtot_i;
    st.vel.x = svx * mtot_i; st.vel.y = svy * mtot_i; st.vel.z = svz * mtot_i;
}

// :935-963
static void inertial_to_jacobi_acc(Sim& s) {
    const int mm = s.host;
    const Particle& star = s.p[mm];
    real eta = star.mass;
    real sax = eta * star.a.x, say = eta * star.a.y, saz = eta * star.a.z;
    for (int i = 0; i < s.n; ++i) {
        if (i == mm) continue;
        const Particle& q = s.p[i];
        AltCoords& a = s.alt[i];
        real ei = real(1.) / eta;
        eta += q.mass;
        real pme = eta * ei;
        a.acc.x = q.a.x - sax * ei;
        a.acc.y = q.a.y - say * ei;
        a.acc.z = q.a.z - saz * ei;
        sax = sax * pme + q.mass * a.acc.x;
        say = say * pme + q.mass * a.acc.y;
        saz = saz * pme + q.mass * a.acc.z;
    }
    real mtot_i = real(1.) / eta;
    AltCoords& st = s.alt[mm];
    st.acc.x = sax * mtot_i; st.acc.y = say * mtot_i; st.acc.z = saz * mtot_i;
}

// :973-1023
static void inertial_to_whds_and_dh_posvel(Sim& s) {
    const int mm = s.host;
    const Particle& star = s.p[mm];
    AltCoords& st = s.alt[mm];
    st.pos = V3{0., 0., 0.}; st.vel = V3{0., 0., 0.}; st.mass = 0.; st.mass_g = 0.;
    for (int k = -1; k < s.n; ++k) {
        if (k == mm) continue;
        const Particle& q = (k < 0) ? star : s.p[k];
        st.pos.x += q.r.x * q.mass; st.pos.y += q.r.y * q.mass; st.pos.z += q.r.z * q.mass;
        st.vel.x += q.v.x * q.mass; st.vel.y += q.v.y * q.mass; st.vel.z += q.v.z * q.mass;
        st.mass += q.mass;
        st.mass_g += q.mass_g;
    }
    real mtot = st.mass;
    st.pos.x /= mtot; st.pos.y /= mtot; st.pos.z /= mtot;
    st.vel.x /= mtot; st.vel.y /= mtot; st.vel.z /= mtot;
    for (int i = 0; i < s.n; ++i) {
        if (i == mm) continue;
        const Particle& q = s.p[i];
        AltCoords& a = s.alt[i];
        a.pos.x = q.r.x - star.r.x; a.pos.y = q.r.y - star.r.y; a.pos.z = q.r.z - star.r.z;
        a.vel.x = q.v.x - st.vel.x; a.vel.y = q.v.y - st.vel.y; a.vel.z = q.v.z - st.vel.z;
        a.mass = q.mass;
        a.mass_g = q.mass_g;
        if (s.coords == POSI_WHDS) {
            real factor = (star.mass + q.mass) / star.mass;
            a.vel.x *= factor; a.vel.y *= factor; a.vel.z *= factor;
        }
    }
}

// :1034-1080
static void jacobi_to_inertial_posvel(Sim& s) {
    const int mm = s.host;
    AltCoords& st = s.alt[mm];
    real m0 = st.mass;
    real eta = m0;
    real sx = eta * st.pos.x, sy = eta * st.pos.y, sz = eta * st.pos.z;
    real svx = eta * st.vel.x, svy = eta * st.vel.y, svz = eta * st.vel.z;
    for (int i = s.n - 1; i >= 0; --i) {
        if (i == mm) continue;
        Particle& q = s.p[i];
        const AltCoords& a = s.alt[i];
        real ei = real(1.) / eta;
        sx = (sx - q.mass * a.pos.x) * ei;
        sy = (sy - q.mass * a.pos.y) * ei;
        sz = (sz - q.mass * a.pos.z) * ei;
        svx = (svx - q.mass * a.vel.x) * ei;
        svy = (svy - q.mass * a.vel.y) * ei;
        svz = (svz - q.mass * a.vel.z) * ei;
        q.r.x = a.pos.x + sx; q.r.y = a.pos.y + sy; q.r.z = a.pos.z + sz;
        q.v.x = a.vel.x + svx; q.v.y = a.vel.y + svy; q.v.z = a.vel.z + svz;
        eta -= q.mass;
        sx *= eta; sy *= eta; sz *= eta;
        svx *= eta; svy *= eta; svz *= eta;
    }
    real mtot_i = real(1.) / eta;
    Particle& star = s.p[mm];
    star.r.x = sx * mtot_i; star.r.y = sy * mtot_i; star.r.z = sz * mtot_i;
    star.v.x = svx * mtot_i; star.v.y = svy * mtot_i; star.v.z = svz * mtot_i;
}

// :1090-1155
static void whds_and_dh_to_inertial_posvel(Sim& s) {
    const int mm = s.host;
    AltCoords& st = s.alt[mm];
    Particle& star = s.p[mm];
    {
        real mtot = st.mass;
        V3 nsp = st.pos;
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            const AltCoords& a = s.alt[i];
            const Particle& q = s.p[i];
            nsp.x -= a.pos.x * q.mass / mtot;
            nsp.y -= a.pos.y * q.mass / mtot;
            nsp.z -= a.pos.z * q.mass / mtot;
        }
        star.r = nsp;
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            const AltCoords& a = s.alt[i];
            Particle& q = s.p[i];
            q.r.x = a.pos.x + star.r.x; q.r.y = a.pos.y + star.r.y; q.r.z = a.pos.z + star.r.z;
        }
    }
    real m0 = star.mass;
    V3 nsv = st.vel;
    for (int i = 0; i < s.n; ++i) {
        if (i == mm) continue;
        const AltCoords& a = s.alt[i];
        Particle& q = s.p[i];
        if (s.coords == POSI_WHDS) {
            real factor = (m0 + q.mass) / m0;
            q.v.x = a.vel.x / factor + st.vel.x;
            q.v.y = a.vel.y / factor + st.vel.y;
            q.v.z = a.vel.z / factor + st.vel.z;
        } else {
            q.v.x = a.vel.x + st.vel.x;
            q.v.y = a.vel.y + st.vel.y;
            q.v.z = a.vel.z + st.vel.z;
        }
        real factor = (s.coords == POSI_WHDS) ? q.mass / (m0 + q.mass) : q.mass / m0;
        nsv.x -= a.vel.x * factor;
        nsv.y -= a.vel.y * factor;
        nsv.z -= a.vel.z * factor;
    }
    star.v = nsv;
}

static void inertial_to_alternative_posvel(Sim& s) {
    if (s.coords == POSI_JACOBI) inertial_to_jacobi_posvel(s); else inertial_to_whds_and_dh_posvel(s);
}
static void alternative_to_inertial_posvel(Sim& s) {
    if (s.coords == POSI_JACOBI) jacobi_to_inertial_posvel(s); else whds_and_dh_to_inertial_posvel(s);
}

// :495-556
static void jump_step(Sim& s, real dt) {
    const int mm = s.host;
    if (s.coords == POSI_JACOBI) return;
    real m0 = s.p[mm].mass;
    real px = 0., py = 0., pz = 0.;
    if (s.coords == POSI_DEMOCRATIC_HELIOCENTRIC) {
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            const AltCoords& a = s.alt[i];
            const Particle& q = s.p[i];
            px += q.mass * a.vel.x; py += q.mass * a.vel.y; pz += q.mass * a.vel.z;
        }
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            AltCoords& a = s.alt[i];
            a.pos.x += dt * px / m0;
            a.pos.y += dt * py / m0;
            a.pos.z += dt * pz / m0;
        }
    } else {
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            const AltCoords& a = s.alt[i];
            const Particle& q = s.p[i];
            real factor = m0 + q.mass;
            px += q.mass * a.vel.x / factor; py += q.mass * a.vel.y / factor; pz += q.mass * a.vel.z / factor;
        }
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            AltCoords& a = s.alt[i];
            const Particle& q = s.p[i];
            real factor = m0 + q.mass;
            a.pos.x += dt * (px - (q.mass * a.vel.x / factor));
            a.pos.y += dt * (py - (q.mass * a.vel.y / factor));
            a.pos.z += dt * (pz - (q.mass * a.vel.z / factor));
        }
    }
}

// :558-625
static void interaction_step(Sim& s, real dt) {
    const int mm = s.host;
    if (s.coords == POSI_JACOBI) {
        inertial_to_jacobi_acc(s);
        const real softening = 1e-12;
        real eta = s.p[mm].mass;
        int k = 0;
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            AltCoords& a = s.alt[i];
            eta += a.mass;
            a.vel.x += dt * a.acc.x;
            a.vel.y += dt * a.acc.y;
            a.vel.z += dt * a.acc.z;
            if (k > 0) {
                real rj2i = real(1.) / (powi(a.pos.x, 2) + powi(a.pos.y, 2) + powi(a.pos.z, 2) + softening);
                real rji = rsqrt_(rj2i);
                real rj3im = rji * rj2i * G * eta;
                real prefac = dt * rj3im;
                a.vel.x += prefac * a.pos.x;
                a.vel.y += prefac * a.pos.y;
                a.vel.z += prefac * a.pos.z;
            }
            ++k;
        }
    } else if (s.coords == POSI_DEMOCRATIC_HELIOCENTRIC) {
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            AltCoords& a = s.alt[i];
            const Particle& q = s.p[i];
            a.vel.x += dt * q.a.x; a.vel.y += dt * q.a.y; a.vel.z += dt * q.a.z;
        }
    } else {
        real m0 = s.p[mm].mass;
        for (int i = 0; i < s.n; ++i) {
            if (i == mm) continue;
            AltCoords& a = s.alt[i];
            const Particle& q = s.p[i];
            real factor = m0 + q.mass;
            a.vel.x += dt * factor * q.a.x / m0;
            a.vel.y += dt * factor * q.a.y / m0;
            a.vel.z += dt * factor * q.a.z / m0;
        }
    }
}

// :226-233
static int initialize_physical_values(Sim& s) {
    if (s.t != real(0.)) return POSI_ERR_STATE;
    calculate_spin_and_evolving_quantities(s, s.t, true);
    calculate_roche_radiuses(s);
    return POSI_OK;
}

// Historic records (src/integrator/output.rs:91-135), as 20 doubles per body:
// t, dt, id, position, spin, velocity, mass, radius, rg2, love number,
// scaled dissipation factor, lag angle, denergy_dt, migration timescale (the
// disk is not on this path: 0).  Collected only when a buffer is attached.
thread_local double* g_hist = nullptr;
thread_local int64_t g_hist_cap = 0, g_hist_len = 0;

static void write_historic_snapshot(const Sim& s) {
    if (!g_hist) return;
    for (int i = 0; i < s.n; ++i) {
        if (g_hist_len >= g_hist_cap) return;
        const Particle& q = s.p[i];
        double* R = g_hist + g_hist_len * 20;
        const real rec[20] = {s.t, s.dt, real((double)q.id), q.r.x, q.r.y, q.r.z, q.spin.x, q.spin.y, q.spin.z,
                              q.v.x, q.v.y, q.v.z, q.mass, q.radius, q.rg2,
                              q.tides.kind != POSI_EFFECT_DISABLED ? q.tides.love_number : real(0.),
                              q.tides.scaled_dissipation_factor, q.tides.lag_angle, q.tides.denergy_dt,
                              q.disk.migration_timescale};
        for (int k = 0; k < 20; ++k) R[k] = static_cast<double>(rec[k]);
        ++g_hist_len;
    }
}

// :235-305 (the historic snapshot goes to the attached record buffer; its
// side effects on the state -- the evolution update and the spin refresh --
// are reproduced)
static int iterate(Sim& s, bool* recovery_trigger) {
    bool first = s.last_hist < real(0.);
    bool hist_trig = s.last_hist + s.hist_period <= s.t;
    bool rec_trig = s.last_rec + s.rec_period <= s.t;
    if (first || hist_trig) {
        inertial_to_heliocentric(s);
        calculate_spin_and_evolving_quantities(s, s.t, true);
        if (s.fatal()) return POSI_ERR_PHYSICS;
        if (s.tides) tides_denergy_dt(s);
        write_historic_snapshot(s);
        if (!first) s.last_hist += s.hist_period; else s.last_hist = 0.;
        s.n_hist += 1;
    }
    const int ignore = (s.coords == POSI_JACOBI) ? 1 : 2;
    // whfast.rs:270-274: GR adds a spin torque only in Kidder1995
    const bool spin = s.tides || s.flat || s.evolution || (s.gr && s.gr_impl == POSI_GR_KIDDER1995);
    integrate_velocity_dependent_forces(s, s.half_dt, spin, true);
    if (s.fatal()) return POSI_ERR_PHYSICS;
    // part 1: :469-479
    inertial_to_alternative_posvel(s);
    kepler_steps(s, s.half_dt);
    jump_step(s, s.half_dt);
    alternative_to_inertial_posvel(s);
    if (s.fatal()) return POSI_ERR_PHYSICS;
    gravity_calculate_acceleration(s, ignore);
    if (s.fatal()) return POSI_ERR_PHYSICS;
    // part 2: :482-491
    interaction_step(s, s.dt);
    jump_step(s, s.half_dt);
    kepler_steps(s, s.half_dt);
    alternative_to_inertial_posvel(s);
    if (s.fatal()) return POSI_ERR_PHYSICS;
    integrate_velocity_dependent_forces(s, s.half_dt, spin, false);
    if (s.fatal()) return POSI_ERR_PHYSICS;
    s.t += s.dt;
    s.iteration += 1;
    if (s.t + s.dt > s.time_limit) return POSI_COMPLETED;
    *recovery_trigger = first || rec_trig;
    return POSI_OK;
}

#include "ias15_oracle.inc"

// ---------------------------------------------------------------------------
// Flat layout <-> Sim
// ---------------------------------------------------------------------------
static void load(Sim& s, int64_t nmax, const int64_t* si, const double* sf, const int64_t* bi, const double* bf,
                 const double* tables, const double* roche, const double* ias) {
    s.n = (int)si[POSI_SI_N];
    s.integrator = (int)si[POSI_SI_INTEGRATOR];
    s.ias_max_exceeded = si[POSI_SI_IAS_MAX_EXCEEDED];
    s.ias_dt_last = sf[POSI_SF_IAS_DT_LAST];
    s.ias.assign((size_t)si[POSI_SI_N] * POSI_IAS_COUNT, real(0.));
    if (ias)
        for (size_t k = 0; k < s.ias.size(); ++k) s.ias[k] = ias[k];
    s.host = (int)si[POSI_SI_HOST];
    s.coords = (int)si[POSI_SI_COORDS];
    s.tides = si[POSI_SI_TIDES] != 0;
    s.flat = si[POSI_SI_FLAT] != 0;
    s.gr = si[POSI_SI_GR] != 0;
    s.gr_impl = (int)si[POSI_SI_GR_IMPL];
    s.wind = si[POSI_SI_WIND] != 0;
    s.disk = si[POSI_SI_DISK] != 0;
    s.evolution = si[POSI_SI_EVOLUTION] != 0;
    s.iteration = si[POSI_SI_ITERATION];
    s.n_hist = si[POSI_SI_N_HIST];
    s.timestep_warning = si[POSI_SI_TIMESTEP_WARNING];
    s.status = si[POSI_SI_STATUS];
    s.fail_step = si[POSI_SI_FAIL_STEP];
    s.fail_pair = si[POSI_SI_FAIL_PAIR];
    s.last_midpoint_iters = si[POSI_SI_LAST_MIDPOINT_ITERS];
    s.dt = sf[POSI_SF_DT];
    s.half_dt = sf[POSI_SF_HALF_DT];
    s.t = sf[POSI_SF_TIME];
    s.time_limit = sf[POSI_SF_TIME_LIMIT];
    s.last_hist = sf[POSI_SF_LAST_HIST];
    s.hist_period = sf[POSI_SF_HIST_PERIOD];
    s.last_rec = sf[POSI_SF_LAST_REC];
    s.rec_period = sf[POSI_SF_REC_PERIOD];
    const int n = s.n;
    s.p.assign(n, Particle());
    s.ev.assign(n, Evolver());
    s.alt.assign(n, AltCoords());
    s.errv.assign(n, V3{0., 0., 0.});
    s.errL.assign(n, V3{0., 0., 0.});
    s.roche.assign((size_t)n * n, real(0.));
    for (int b = 0; b < n; ++b) {
        const int64_t* I = bi + (size_t)b * POSI_BI_COUNT;
        const double* F = bf + (size_t)b * POSI_BF_COUNT;
        Particle& q = s.p[b];
        q.id = b;
        q.mass = F[POSI_BF_MASS]; q.mass_g = F[POSI_BF_MASS_G]; q.radius = F[POSI_BF_RADIUS];
        q.rg2 = F[POSI_BF_RG2]; q.moi = F[POSI_BF_MOI];
        q.r = V3{F[POSI_BF_PX], F[POSI_BF_PY], F[POSI_BF_PZ]};
        q.v = V3{F[POSI_BF_VX], F[POSI_BF_VY], F[POSI_BF_VZ]};
        q.a = V3{F[POSI_BF_AX], F[POSI_BF_AY], F[POSI_BF_AZ]};
        q.L = V3{F[POSI_BF_LX], F[POSI_BF_LY], F[POSI_BF_LZ]};
        q.spin = V3{F[POSI_BF_SX], F[POSI_BF_SY], F[POSI_BF_SZ]};
        q.nsv2 = F[POSI_BF_NSV2];
        q.a_add = V3{F[POSI_BF_ADDAX], F[POSI_BF_ADDAY], F[POSI_BF_ADDAZ]};
        q.dLdt = V3{F[POSI_BF_DLX], F[POSI_BF_DLY], F[POSI_BF_DLZ]};
        s.errv[b] = V3{F[POSI_BF_EVX], F[POSI_BF_EVY], F[POSI_BF_EVZ]};
        s.errL[b] = V3{F[POSI_BF_ELX], F[POSI_BF_ELY], F[POSI_BF_ELZ]};
        q.tides.kind = (int)I[POSI_BI_TIDES_KIND];
        q.tides.scaled_dissipation_factor = F[POSI_BF_SIGMA];
        q.tides.love_number = F[POSI_BF_K2];
        q.tides.denergy_dt = F[POSI_BF_DENERGY_DT];
        q.tides.lag_angle = F[POSI_BF_LAG_ANGLE];
        q.tides.distance = F[POSI_BF_TD_DIST];
        q.tides.radial_velocity = F[POSI_BF_TD_VR];
        q.tides.ortho_planet = F[POSI_BF_TD_ORTHO];
        q.tides.radial_diss_pm = F[POSI_BF_TD_DPM];
        q.tides.pos = V3{F[POSI_BF_TD_PX], F[POSI_BF_TD_PY], F[POSI_BF_TD_PZ]};
        q.tides.vel = V3{F[POSI_BF_TD_VX], F[POSI_BF_TD_VY], F[POSI_BF_TD_VZ]};
        q.tides.out_dldt = V3{F[POSI_BF_TD_LX], F[POSI_BF_TD_LY], F[POSI_BF_TD_LZ]};
        q.flat.kind = (int)I[POSI_BI_FLAT_KIND];
        q.flat.love_number = F[POSI_BF_K2F];
        q.gr.kind = (int)I[POSI_BI_GR_KIND];
        q.wind_kind = (int)I[POSI_BI_WIND_KIND];
        q.disk.kind = (int)I[POSI_BI_DISK_KIND];
        q.disk.inner = F[POSI_BF_DISK_INNER];
        q.disk.outer = F[POSI_BF_DISK_OUTER];
        q.disk.lifetime = F[POSI_BF_DISK_LIFETIME];
        q.disk.alpha = F[POSI_BF_DISK_ALPHA];
        q.disk.sigma0 = F[POSI_BF_DISK_SIGMA0];
        q.disk.mu = F[POSI_BF_DISK_MU];
        q.disk.migration_timescale = F[POSI_BF_DISK_MTS];
        q.tides.diss_factor = F[POSI_BF_DISS_FACTOR];
        q.tides.diss_scale = F[POSI_BF_DISS_SCALE];
        q.wind_k = F[POSI_BF_WIND_K];
        q.wind_rsat = F[POSI_BF_WIND_RSAT];
        q.wind_rsat2 = F[POSI_BF_WIND_RSAT2];
        q.evolution = (int)I[POSI_BI_EVO_TYPE];
        Evolver& e = s.ev[b];
        e.type = q.evolution;
        e.len = I[POSI_BI_EVO_LEN];
        e.left_index = I[POSI_BI_EVO_LEFT];
        if (e.type != POSI_EVO_NON_EVOLVING && e.len > 0) {
            const double* base = tables + I[POSI_BI_EVO_OFFSET];
            e.time = base; e.radius = base + e.len; e.rg2 = base + 2 * e.len; e.love = base + 3 * e.len;
        } else {
            e.type = POSI_EVO_NON_EVOLVING;
        }
    }
    if (roche) {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) s.roche[(size_t)i * n + j] = roche[(size_t)i * nmax + j];
    }
}

static void store(const Sim& s, int64_t nmax, int64_t* si, double* sf, int64_t* bi, double* bf, double* roche,
                  double* ias) {
    si[POSI_SI_IAS_MAX_EXCEEDED] = s.ias_max_exceeded;
    sf[POSI_SF_IAS_DT_LAST] = dv(s.ias_dt_last);
    sf[POSI_SF_DT] = dv(s.dt);
    if (ias)
        for (size_t k = 0; k < s.ias.size(); ++k) ias[k] = dv(s.ias[k]);
    si[POSI_SI_ITERATION] = s.iteration;
    si[POSI_SI_N_HIST] = s.n_hist;
    si[POSI_SI_TIMESTEP_WARNING] = s.timestep_warning;
    si[POSI_SI_STATUS] = s.status;
    si[POSI_SI_FAIL_STEP] = s.fail_step;
    si[POSI_SI_FAIL_PAIR] = s.fail_pair;
    si[POSI_SI_LAST_MIDPOINT_ITERS] = s.last_midpoint_iters;
    sf[POSI_SF_TIME] = dv(s.t);
    sf[POSI_SF_LAST_HIST] = dv(s.last_hist);
    sf[POSI_SF_LAST_REC] = dv(s.last_rec);
    for (int b = 0; b < s.n; ++b) {
        int64_t* I = bi + (size_t)b * POSI_BI_COUNT;
        double* F = bf + (size_t)b * POSI_BF_COUNT;
        const Particle& q = s.p[b];
        F[POSI_BF_RADIUS] = dv(q.radius); F[POSI_BF_RG2] = dv(q.rg2); F[POSI_BF_MOI] = dv(q.moi);
        F[POSI_BF_PX] = dv(q.r.x); F[POSI_BF_PY] = dv(q.r.y); F[POSI_BF_PZ] = dv(q.r.z);
        F[POSI_BF_VX] = dv(q.v.x); F[POSI_BF_VY] = dv(q.v.y); F[POSI_BF_VZ] = dv(q.v.z);
        F[POSI_BF_AX] = dv(q.a.x); F[POSI_BF_AY] = dv(q.a.y); F[POSI_BF_AZ] = dv(q.a.z);
        F[POSI_BF_LX] = dv(q.L.x); F[POSI_BF_LY] = dv(q.L.y); F[POSI_BF_LZ] = dv(q.L.z);
        F[POSI_BF_SX] = dv(q.spin.x); F[POSI_BF_SY] = dv(q.spin.y); F[POSI_BF_SZ] = dv(q.spin.z);
        F[POSI_BF_NSV2] = dv(q.nsv2);
        F[POSI_BF_EVX] = dv(s.errv[b].x); F[POSI_BF_EVY] = dv(s.errv[b].y); F[POSI_BF_EVZ] = dv(s.errv[b].z);
        F[POSI_BF_ELX] = dv(s.errL[b].x); F[POSI_BF_ELY] = dv(s.errL[b].y); F[POSI_BF_ELZ] = dv(s.errL[b].z);
        F[POSI_BF_ADDAX] = dv(q.a_add.x); F[POSI_BF_ADDAY] = dv(q.a_add.y); F[POSI_BF_ADDAZ] = dv(q.a_add.z);
        F[POSI_BF_DLX] = dv(q.dLdt.x); F[POSI_BF_DLY] = dv(q.dLdt.y); F[POSI_BF_DLZ] = dv(q.dLdt.z);
        F[POSI_BF_DENERGY_DT] = dv(q.tides.denergy_dt);
        F[POSI_BF_LAG_ANGLE] = dv(q.tides.lag_angle);
        F[POSI_BF_DISK_MTS] = dv(q.disk.migration_timescale);
        F[POSI_BF_TD_DIST] = dv(q.tides.distance);
        F[POSI_BF_TD_VR] = dv(q.tides.radial_velocity);
        F[POSI_BF_TD_ORTHO] = dv(q.tides.ortho_planet);
        F[POSI_BF_TD_DPM] = dv(q.tides.radial_diss_pm);
        F[POSI_BF_TD_PX] = dv(q.tides.pos.x); F[POSI_BF_TD_PY] = dv(q.tides.pos.y); F[POSI_BF_TD_PZ] = dv(q.tides.pos.z);
        F[POSI_BF_TD_VX] = dv(q.tides.vel.x); F[POSI_BF_TD_VY] = dv(q.tides.vel.y); F[POSI_BF_TD_VZ] = dv(q.tides.vel.z);
        F[POSI_BF_TD_LX] = dv(q.tides.out_dldt.x); F[POSI_BF_TD_LY] = dv(q.tides.out_dldt.y); F[POSI_BF_TD_LZ] = dv(q.tides.out_dldt.z);
        I[POSI_BI_EVO_LEFT] = s.ev[b].left_index;
    }
    if (roche) {
        for (int i = 0; i < s.n; ++i)
            for (int j = 0; j < s.n; ++j) roche[(size_t)i * nmax + j] = dv(s.roche[(size_t)i * s.n + j]);
    }
}

#ifdef ORACLE_DUAL
// Seeds and tangents of the dual build, [n_sys][nmax][POSI_BF_COUNT][ND]:
// the derivatives of a body's inputs along each direction (position,
// velocity, spin angular momentum and spin, dissipation factor, Love
// number), and on return those of its final position, velocity, spin
// angular momentum and spin.
static const double* g_dual_seed = nullptr;
static double* g_dual_out = nullptr;

static void seed3(V3& x, const double* S, int f) {
    for (int k = 0; k < ND; ++k) {
        x.x.d[k] = S[(f + 0) * ND + k];
        x.y.d[k] = S[(f + 1) * ND + k];
        x.z.d[k] = S[(f + 2) * ND + k];
    }
}
static void out3(const V3& x, double* T, int f) {
    for (int k = 0; k < ND; ++k) {
        T[(f + 0) * ND + k] = x.x.d[k];
        T[(f + 1) * ND + k] = x.y.d[k];
        T[(f + 2) * ND + k] = x.z.d[k];
    }
}
static void dual_seed(Sim& s, const double* S) {
    for (int b = 0; b < s.n; ++b) {
        const double* B = S + (size_t)b * POSI_BF_COUNT * ND;
        Particle& q = s.p[b];
        seed3(q.r, B, POSI_BF_PX);
        seed3(q.v, B, POSI_BF_VX);
        seed3(q.L, B, POSI_BF_LX);
        seed3(q.spin, B, POSI_BF_SX);
        for (int k = 0; k < ND; ++k) {
            q.tides.scaled_dissipation_factor.d[k] = B[POSI_BF_SIGMA * ND + k];
            q.tides.love_number.d[k] = B[POSI_BF_K2 * ND + k];
        }
    }
}
static void dual_tangents(const Sim& s, double* T) {
    for (int b = 0; b < s.n; ++b) {
        double* B = T + (size_t)b * POSI_BF_COUNT * ND;
        const Particle& q = s.p[b];
        out3(q.r, B, POSI_BF_PX);
        out3(q.v, B, POSI_BF_VX);
        out3(q.L, B, POSI_BF_LX);
        out3(q.spin, B, POSI_BF_SX);
    }
}
#endif

}  // namespace orc

// ---------------------------------------------------------------------------
// C entry points (ctypes)
// ---------------------------------------------------------------------------
enum oracle_op {
    ORACLE_ITERATE = 0,            // initialise if asked, then up to max_steps WHFast steps
    ORACLE_GRAVITY = 1,            // gravity_calculate_acceleration(arg)
    ORACLE_ADDITIONAL_EFFECTS = 2, // inertial_to_heliocentric + calculate_additional_effects
    ORACLE_INITIALIZE = 3          // initialize_physical_values
};

extern "C" {

// Runs `op` on every system of the flat-layout ensemble, in place.
// roche: n_sys*nmax*nmax doubles (in/out) or NULL.
// For ORACLE_ITERATE: steps_done[s] receives the steps performed and
// result[s] the last iterate() code.  nthreads <= 0 uses the hardware count.
int oracle_run(int op, int64_t n_sys, int64_t nmax, int64_t* sys_i64, double* sys_f64, int64_t* body_i64,
               double* body_f64, const double* tables, double* roche, double* body_ias, int64_t max_steps,
               int init_physical, int arg, double t_arg, int nthreads, int64_t* steps_done, int64_t* result) {
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    if (nthreads > n_sys) nthreads = (int)std::max<int64_t>(1, n_sys);
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        orc::Sim s;
        for (;;) {
            int64_t k = next.fetch_add(1);
            if (k >= n_sys) break;
            int64_t* si = sys_i64 + k * POSI_SI_COUNT;
            double* sf = sys_f64 + k * POSI_SF_COUNT;
            int64_t* bi = body_i64 + k * nmax * POSI_BI_COUNT;
            double* bf = body_f64 + k * nmax * POSI_BF_COUNT;
            double* ro = roche ? roche + k * nmax * nmax : nullptr;
            double* ia = body_ias ? body_ias + k * nmax * POSI_IAS_COUNT : nullptr;
            orc::load(s, nmax, si, sf, bi, bf, tables, ro, ia);
#ifdef ORACLE_DUAL
            if (orc::g_dual_seed) orc::dual_seed(s, orc::g_dual_seed + (size_t)k * nmax * POSI_BF_COUNT * orc::ND);
#endif
            int64_t done = 0, rc = POSI_OK;
            if (op == ORACLE_ITERATE) {
                if (init_physical) rc = orc::initialize_physical_values(s);
                while (rc == POSI_OK && done < max_steps && !s.fatal()) {
                    bool rec = false;
                    rc = s.integrator == POSI_INTEGRATOR_IAS15 ? orc::ias15_iterate(s, &rec) : orc::iterate(s, &rec);
                    if (rc == POSI_OK || rc == POSI_COMPLETED) ++done;
                }
                if (rc == POSI_COMPLETED) s.status = (s.status & ~int64_t(POSI_SYS_FATAL_MASK)) | POSI_SYS_COMPLETED;
            } else if (op == ORACLE_GRAVITY) {
                orc::gravity_calculate_acceleration(s, arg);
            } else if (op == ORACLE_ADDITIONAL_EFFECTS) {
                orc::inertial_to_heliocentric(s);
                orc::calculate_additional_effects(s, t_arg, (arg & 1) != 0, (arg & 2) != 0, (arg & 4) != 0,
                                                  s.coords == POSI_JACOBI ? 1 : 2);
            } else if (op == ORACLE_INITIALIZE) {
                rc = orc::initialize_physical_values(s);
            }
            orc::store(s, nmax, si, sf, bi, bf, ro, ia);
#ifdef ORACLE_DUAL
            if (orc::g_dual_out) orc::dual_tangents(s, orc::g_dual_out + (size_t)k * nmax * POSI_BF_COUNT * orc::ND);
#endif
            if (steps_done) steps_done[k] = done;
            if (result) result[k] = rc;
        }
    };
    if (nthreads == 1) {
        worker();
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; ++t) th.emplace_back(worker);
        for (auto& t : th) t.join();
    }
    return 0;
}

// Attach (buf != NULL) or detach the historic-record buffer of the calling
// thread: room for `capacity` body records of 20 doubles; *len receives the
// count written so far on each call with len != NULL.
void oracle_history(double* buf, int64_t capacity, int64_t* len) {
    if (len) *len = orc::g_hist_len;
    if (buf != orc::g_hist || !buf) {
        orc::g_hist = buf;
        orc::g_hist_cap = buf ? capacity : 0;
        orc::g_hist_len = 0;
    }
}

#ifdef ORACLE_DUAL
// Seeds (inputs) and tangents (outputs) of the next oracle_run calls, both
// [n_sys][nmax][POSI_BF_COUNT][directions] or NULL; returns the directions
// every value carries.
int oracle_dual_io(const double* seed, double* out) {
    orc::g_dual_seed = seed;
    orc::g_dual_out = out;
    return orc::ND;
}
#endif

#ifdef ORACLE_COUNT_FLOPS
// Flop counters of the calling thread since the last reset: {all, divisions, square roots}.
void oracle_flops(int64_t* out, int reset) {
    out[0] = orc::g_flops; out[1] = orc::g_divs; out[2] = orc::g_sqrts;
    if (reset) { orc::g_flops = 0; orc::g_divs = 0; orc::g_sqrts = 0; }
}
#endif

double oracle_constant(int which) {
    switch (which) {
        case 0: return orc::G;
        case 1: return orc::SPEED_OF_LIGHT_2;
        case 2: return orc::DBL_EPSILON_2;
        default: return 0.;
    }
}

}  // extern "C"
