// whfast_device.cuh -- FP64 device code of the WHFast + tidal-effects step.
//
// Mapping: one group of G lanes (G = 2, 4, 8, 16 or 32; G >= n) integrates one
// independent system; lane j owns body j (reference particle order, the host
// at any index).  Each lane keeps its body's state in registers for the whole
// launch; the per-planet constants of a half kick live in shared memory.
//
// This header is compiled twice.
//
// POSI_EXACT=1 (with -fmad=false) keeps the reference's operation order and
// reproduces the Rust FP64 results bit for bit.  Cross-body work goes through
// a small per-group exchange area in shared memory: reductions over bodies
// (host back-reactions, midpoint convergence, democratic-heliocentric sums)
// are folded column-wise -- every lane writes its body's contributions, then
// lane c folds column c over the bodies in index order, the reference's own
// order -- and the Jacobi recurrences, sequential by nature, run in every lane.
//
// POSI_EXACT=0 (with -fmad=true) is the throughput build.  A 32-lane FP64
// instruction holds an SMSP's FP64 pipe for the same time whatever its active
// mask, so it minimises FP64 instructions per lane: divisions become products
// with reciprocals computed once per launch or per half kick, the Jacobi
// transforms are shuffle prefix / suffix scans over mass constants of the
// launch, gravity uses rsqrt, and the host back-reactions collapse to
// momentum sums (the host's tidal, flattening and GR acceleration is
// -sum_p (m_p/m_host) a_p).  Results stay within 1e-12 relative per step of the
// reference order.
//
// In both builds, position-only and parameter-only terms are evaluated once
// per half kick instead of once per midpoint iteration (the reference
// recomputes the same values, so this changes no bit).
//
// Reference: src/integrator/whfast.rs (step, midpoint, Kepler, transforms),
// src/particles/universe.rs (gravity, heliocentric, additional effects),
// src/effects/tides/{common,constant_time_lag}.rs,
// src/effects/rotational_flattening/{common,oblate_spheroid}.rs,
// src/effects/general_relativity.rs (Kidder 1995), src/effects/evolution.rs,
// src/tools.rs:840-907, src/constants.rs.

#pragma once
#include <cstdint>

#include "../../include/posidonius_gb300.h"
#include "adjoint_record.h"

#ifndef POSI_EXACT
#error "POSI_EXACT must be defined (1: reference operation order, 0: fast)"
#endif

#if POSI_EXACT
#define POSI_NS posi_exact
#else
#define POSI_NS posi_fast
#endif

namespace POSI_NS {

// ---------------------------------------------------------------------------
// src/constants.rs:20-61 -- the same literal expressions, folded at compile time
// ---------------------------------------------------------------------------
constexpr double kPI = 3.141592653589793;
constexpr double kDAY = 24. * 3600.;
constexpr double kM_SUN = 1.9818e30;
constexpr double kG_SI = 6.67428e-11;
constexpr double kAU = 1.49597870700e11;
constexpr double kC = (2.99792458e8 / kAU) * kDAY;
constexpr double kC2 = kC * kC;
constexpr double kG = kG_SI / (kAU * kAU * kAU) * kM_SUN * (kDAY * kDAY);
constexpr double kK2 = kG;
constexpr double kMAX_DISTANCE_2 = 100. * 100.;
constexpr double kDBL_EPSILON_2 = 2.2204460492503131e-16 * 2.2204460492503131e-16;
constexpr double kMINUS_3K2 = -3.0 * kK2;
constexpr double kFA = kG / kC2;
constexpr double kTWO_PI = 2. * kPI;
constexpr double kR_SUN = 6.957e8 / kAU;
constexpr double kSUN_DYN_FREQ_2 = kK2 / (kR_SUN * kR_SUN * kR_SUN);
constexpr double kSMOOTHING_DYN_TIDE = 1.0e-5 * 86400.;

// y^(-3/2) for the dynamical tide's mean motion (the reference's
// powf(-1.5)): 1 / (y sqrt(y)) carried to about 100 bits in double-double
// (sqrt's residual and the products' low parts by FMA) and rounded once, so
// the result is the correctly rounded power except in vanishingly rare cases.
__device__ __forceinline__ double pow_m1p5(double y) {
    const double s = sqrt(y);
    const double sl = fma(-s, s, y) / (2. * s);   // sqrt(y) = s + sl
    const double th = y * s;
    const double tl = fma(y, s, -th) + y * sl;    // y^1.5 = th + tl
    const double q = 1. / th;
    const double e = fma(-th, q, 1.) - tl * q;    // 1 - (th + tl) q
    return fma(q, e, q);
}
// Double-double helpers (Dekker / Knuth error-free transformations).
struct DD {
    double hi, lo;
};
// a <= b for a squared distance a and a squared threshold b (neither
// negative), decided on the bit patterns: the order of non-negative doubles
// is that of their bits read as integers.  A NaN on either side gives false,
// as the floating-point comparison does.
__device__ __forceinline__ bool sq_le(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long kInf = 0x7ff0000000000000LL;
    return ia <= ib && ib <= kInf && ia <= kInf;
}
// a > b on the same terms
__device__ __forceinline__ bool sq_gt(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long kInf = 0x7ff0000000000000LL;
    return ia > ib && ia <= kInf && ib <= kInf;
}

__device__ __forceinline__ DD dd_two_sum(double a, double b) {
    const double s = a + b;
    const double bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DD dd_quick(double a, double b) {
    const double s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
    DD s = dd_two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return dd_quick(s.hi, s.lo);
}
__device__ __forceinline__ DD dd_mul(DD a, DD b) {
    const double p = a.hi * b.hi;
    double e = fma(a.hi, b.hi, -p);
    e += a.hi * b.lo + a.lo * b.hi;
    return dd_quick(p, e);
}
__device__ __forceinline__ DD dd_mul_d(DD a, double b) {
    const double p = a.hi * b;
    double e = fma(a.hi, b, -p);
    e += a.lo * b;
    return dd_quick(p, e);
}

// ln 2 split in two doubles (the nearest double and the remainder)
constexpr double kLN2_HI = 0x1.62e42fefa39efp-1;
constexpr double kLN2_LO = 0x1.abc9e3b39803fp-56;

// e^x for the disk model (the reference's f64::exp), carried to about 100
// bits and rounded once: x = k ln 2 + r, r / 2^9 through the Taylor series of
// expm1 (double-double to the cubic term), nine doublings
// expm1(2y) = expm1(y) (2 + expm1(y)), then 2^k (1 + expm1(r)).
__device__ __forceinline__ double exp_dd(double x) {
    if (x != x) return x;
    if (x < -745.2) return 0.;
    if (x > 709.8) return __longlong_as_double(0x7ff0000000000000LL);
    const double k = rint(x * 1.4426950408889634);
    const double p = k * kLN2_HI;
    const double pe = fma(k, kLN2_HI, -p);   // k ln2_hi = p + pe exactly
    DD r = dd_two_sum(x, -p);
    r.lo -= pe;
    r.lo -= k * kLN2_LO;
    r = dd_quick(r.hi, r.lo);
    r.hi *= 1. / 512.;
    r.lo *= 1. / 512.;
    const double h = r.hi;
    const double tail = 1. / 24. + h * (1. / 120. + h * (1. / 720. + h * (1. / 5040. + h * (1. / 40320.))));
    const DD r2 = dd_mul(r, r);
    const DD r3 = dd_mul(r2, r);
    DD sm = dd_add(r, dd_mul_d(r2, 0.5));
    sm = dd_add(sm, dd_mul_d(r3, 1. / 6.));
    sm = dd_add(sm, DD{r3.hi * h * tail, 0.});
#pragma unroll
    for (int i = 0; i < 9; ++i) sm = dd_mul(sm, dd_add(DD{2., 0.}, sm));
    const DD e = dd_add(DD{1., 0.}, sm);
    return ldexp(e.hi + e.lo, (int)k);
}

// y^(-1/2) (the reference's powf(-0.5)): 1 / (sqrt(y) + its residual term),
// rounded once.
__device__ __forceinline__ double pow_m0p5(double y) {
    const double s = sqrt(y);
    const double sl = fma(-s, s, y) / (2. * s);
    const double q = 1. / s;
    const double e = fma(-s, q, 1.) - sl * q;
    return fma(q, e, q);
}

// src/constants.rs:71-74
constexpr double kBOLTZMANN = 1.380649e-23 / (kM_SUN * kAU * kAU) * kDAY * kDAY;
constexpr double kMASS_HYDROGEN = 1.672162841e-27 / kM_SUN;

constexpr int kNMAX_QUART = 64;
constexpr int kNMAX_NEWT = 32;
constexpr int kMIDPOINT_MIN = 3;
constexpr int kMIDPOINT_MAX = 10;
constexpr int kBISECTION_GUARD = 4096;
constexpr int kEVO_SHIFT = 10;

// LLVM's expansion of llvm.powi with a constant exponent (square-and-multiply
// from the low bit; the first factor is taken without multiplying by one).
template <int N>
__device__ __forceinline__ double powi(double x) {
    double res = 0.;
    bool have = false;
    double cur = x;
    unsigned v = (unsigned)N;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (v) {
            if (v & 1u) {
                if (have) res = res * cur; else { res = cur; have = true; }
            }
            v >>= 1;
            if (v) cur = cur * cur;
        }
    }
    return res;
}

// ---------------------------------------------------------------------------
// Device view of an ensemble (field-major SoA).
// ---------------------------------------------------------------------------
struct Dev {
    int64_t n_sys, nmax, stride;   // stride = n_sys * nmax
    double* bf;                    // [POSI_BF_COUNT][stride]
    int64_t* bi;                   // [POSI_BI_COUNT][stride]
    double* sf;                    // [POSI_SF_COUNT][n_sys]
    int64_t* si;                   // [POSI_SI_COUNT][n_sys]
    const double* roche;           // [n_sys][nmax][nmax]
    const double* tables;          // evolution tables
    const int32_t* list;           // systems of this launch
    int32_t n_list;
    int32_t* step_flags;           // per system: bit0 recovery trigger, bit1 historic trigger
    double* hist;                  // optional: [n_sys][nmax][HR_COUNT], last historic record
    double* rec;                   // optional: adjoint step records [step][POSI_REC_COUNT][stride]
    double* ias;                   // IAS15 systems: [POSI_IAS_COUNT][stride]
};

// Per-planet constants of one half kick, slot k of lane j at P[k * G + j].
enum {
    PC_X = 0, PC_Y, PC_Z, PC_D, PC_INV_D, PC_XD, PC_YD, PC_ZD,
    // constant-time-lag tides
    PC_OS, PC_OP, PC_OSD, PC_OPD, PC_OSPD, PC_OSDD, PC_OPDD, PC_C13, PC_CONS, PC_D8, PC_TERM1, PC_TERM2, PC_T12,
    // oblate flattening
    PC_MHK2F, PC_HMK2F, PC_R5H, PC_R5P, PC_D5, PC_N3D5, PC_F15D7, PC_CFS, PC_CFP, PC_COFS, PC_COFP,
    // Kidder GR
    PC_A, PC_B, PC_C, PC_DD, PC_E, PC_T1, PC_K2C, PC_K3C, PC_K4C, PC_K5C, PC_K6C, PC_A05, PC_P, PC_Q, PC_R3,
    PC_MRATIO, PC_MFM, PC_MU, PC_FM, PC_FM2, PC_NN0, PC_NN1, PC_NN2, PC_C6NN0, PC_C6NN1, PC_C6NN2,
    // tidal internals of the last evaluation (state: read by the historic dE/dt)
    PC_TD_DIST, PC_TD_VR, PC_TD_ORTHO, PC_TD_DPM, PC_TD_P0, PC_TD_P1, PC_TD_P2, PC_TD_V0, PC_TD_V1, PC_TD_V2,
    PC_TD_L0, PC_TD_L1, PC_TD_L2,
    PC_COUNT
};
#if !POSI_EXACT
// FAST keeps the Kidder GR constants in combined form (planet_constants):
// these slots take the place of the reference-order ones.
enum {
    PC_GR0 = PC_B, PC_GR1 = PC_C, PC_GR2 = PC_DD, PC_GO0 = PC_E, PC_GO1 = PC_T1, PC_GO2 = PC_K5C,
    PC_FMU = PC_FM, PC_FM2MU = PC_FM2
};
// Constants of a planet that hold for a whole launch when nothing evolves
// (masses, radii, Love numbers and dissipation factors fixed): set at load,
// or at each half kick of an evolving system (planet_launch_constants).
enum {
    PC_LT1 = PC_D8, PC_LT2 = PC_TERM1, PC_LCONS = PC_MHK2F,           // tides
    PC_LMGS = PC_HMK2F, PC_LMGSC2 = PC_R5H, PC_LT1C = PC_R5P, PC_LCC = PC_D5, PC_LB = PC_K6C,
    PC_LK5 = PC_A05, PC_LNDD = PC_P, PC_LK6 = PC_Q, PC_LQH = PC_R3, PC_LNEC = PC_MU,
    PC_LNPH = PC_NN0, PC_LR3H = PC_NN1, PC_LMA = PC_NN2, PC_LMB = PC_MFM  // Kidder GR
};
#endif

// Fields of one historic-snapshot record (src/integrator/output.rs:91-135).
enum { HR_T = 0, HR_DT, HR_ID, HR_PX, HR_PY, HR_PZ, HR_SX, HR_SY, HR_SZ, HR_VX, HR_VY, HR_VZ, HR_M, HR_R, HR_RG2,
       HR_K2, HR_SIGMA, HR_LAG, HR_DENERGY, HR_MIGRATION, HR_COUNT };

// Shared memory of one group: XS exchange slots of G doubles, the per-planet
// constants, a host card, column results and a few integers.
constexpr int kXS = 24;
constexpr int kCARD = 32;
constexpr int kSUMS = 32;
template <int G>
struct GroupSmem {
    static constexpr int doubles = kXS * G + PC_COUNT * G + kCARD + kSUMS;
    static constexpr int bytes = doubles * 8 + 32;  // + 8 ints
};

// host card slots
enum { HC_PX = 0, HC_PY, HC_PZ, HC_VX, HC_VY, HC_VZ, HC_SX, HC_SY, HC_SZ, HC_NSV2, HC_M, HC_MG, HC_R,
       HC_SIG, HC_K2, HC_K2F, HC_MOI, HC_AM, HC_SLX, HC_SLY, HC_SLZ,
       HC_LAG, HC_DFAC, HC_DSCALE,
       HC_DINNER, HC_DOUTER, HC_DLIFE, HC_DALPHA, HC_DSIG0, HC_DMU, HC_COUNT };
static_assert(HC_COUNT <= kCARD, "host card");

struct Body {
    double m, mg, R, rg2, moi;
    double r[3], v[3], a[3], L[3], S[3], nsv2;
    double ev[3], eL[3];
    double sig, k2, k2f;
    double aa[3], dl[3];
    double denergy, lag;
    int tk, fk, gk, evo;
    int wk;                              // wind: 1 Interaction
    double wind_k, wind_rsat, wind_rsat2;
    double diss_factor, diss_scale;      // ConstantTimeLag inputs (dynamical tide of a host)
    int dk;                              // disk effect kind
    double disk_p[6];                    // DiskProperties (a disk host)
    double dmts;                         // disk migration timescale of the last evaluation
    int64_t eoff, elen, eleft;
    // alternative (Jacobi / democratic-heliocentric / WHDS) coordinates
    double am, amg, ap[3], av[3], aacc[3];
};

template <int G>
struct Sys {
    // uniform per group
    int s, n, host, coords, lane;
    bool tides, flat, gr, evo, spin_on, wind, disk;
    int gr_impl;     // posi_gr_impl; grk(): Kidder1995, the per-planet formulation
    int gr_ignore;   // gravity terms the integrator leaves out (0 None, 1 WHFastOne, 2 WHFastTwo)
    bool dyn_host;   // the tidal host's evolution has a dynamical tide
    bool disk_on;    // disk effect with a disk host
    __device__ __forceinline__ bool grk() const { return gr && gr_impl == POSI_GR_KIDDER1995; }
    unsigned mask;
    double dt, half_dt, t, time_limit, last_hist, hist_period, last_rec, rec_period;
    int64_t iteration, n_hist, tw, status, fail_step, fail_pair, mid_iters;
    double* xs;
    double* pcs;
    double* card;
    double* sums;
    int* isc;
    // own body
    bool has, is_host;
    Body b;
    // adjoint step record of the current step (null: none)
    double* rp;
    int64_t rst;
    double kep_x;
    __device__ __forceinline__ void recw(int f, double v) const {
        if (rp && has) rp[(int64_t)f * rst] = v;
    }
#if !POSI_EXACT
    // mass-only constants of the launch
    double inv_m, inv_moi, inv_eta_excl, jac_c, eta_incl, kep_gm, gm_neg, whds_f, whds_w, dh_w;
    double inv_mtot, inv_hm;
    bool first_planet;
    // The per-planet constants of a half kick depend on the heliocentric
    // positions and on masses, radii and tidal parameters only.  Between the
    // closing half kick of one step and the opening half kick of the next
    // nothing moves, so without evolution the opening kick reuses them.
    bool pc_valid;   // P(PC_*) hold the constants of the current positions
    bool pc_reuse;   // this half kick reuses them
#endif

    __device__ __forceinline__ void sync() const {
        if (G > 1) __syncwarp(mask);
    }
    __device__ __forceinline__ double& X(int slot, int j) const { return xs[slot * G + j]; }
    __device__ __forceinline__ double& P(int slot) const { return pcs[slot * G + lane]; }
    __device__ __forceinline__ bool fatal() const { return (status & POSI_SYS_FATAL_MASK) != 0; }
    __device__ __forceinline__ bool planet() const { return has && !is_host; }
    __device__ static __forceinline__ bool dynamical_evo(int e) {
        return e == POSI_EVO_BOLMONT_MATHIS2016 || e == POSI_EVO_GALLET_BOLMONT2017;
    }

#if !POSI_EXACT
    // group collectives over the G lanes of this system
    __device__ __forceinline__ double gbcast(double v, int src) const {
        return G > 1 ? __shfl_sync(mask, v, src, G) : v;
    }
    __device__ __forceinline__ double gscan(double v) const {  // inclusive prefix in lane order
#pragma unroll
        for (int off = 1; off < G; off <<= 1) {
            const double y = __shfl_up_sync(mask, v, off, G);
            if (lane >= off) v += y;
        }
        return v;
    }
    __device__ __forceinline__ double gsum(double v) const {
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off, G);
        return v;
    }
#endif

    // ------------------------------------------------------------------
    // load / store
    // ------------------------------------------------------------------
    __device__ void load(const Dev& D, int sys, int lane_, unsigned mask_, double* smem) {
        rp = nullptr;
        rst = D.stride;
        kep_x = 0.;
        s = sys;
        lane = lane_;
        mask = mask_;
        xs = smem;
        pcs = smem + kXS * G;
        card = pcs + PC_COUNT * G;
        sums = card + kCARD;
        isc = reinterpret_cast<int*>(sums + kSUMS);
        const int64_t ns = D.n_sys;
        n = (int)D.si[POSI_SI_N * ns + s];
        host = (int)D.si[POSI_SI_HOST * ns + s];
        coords = (int)D.si[POSI_SI_COORDS * ns + s];
        tides = D.si[POSI_SI_TIDES * ns + s] != 0;
        flat = D.si[POSI_SI_FLAT * ns + s] != 0;
        gr = D.si[POSI_SI_GR * ns + s] != 0;
        wind = D.si[POSI_SI_WIND * ns + s] != 0;
        disk = D.si[POSI_SI_DISK * ns + s] != 0;
        evo = D.si[POSI_SI_EVOLUTION * ns + s] != 0;
        gr_impl = (int)D.si[POSI_SI_GR_IMPL * ns + s];
        gr_ignore = coords == POSI_JACOBI ? 1 : 2;
        // whfast.rs:270-274: GR adds a spin torque only in Kidder1995
        spin_on = tides || flat || evo || grk();
        iteration = D.si[POSI_SI_ITERATION * ns + s];
        n_hist = D.si[POSI_SI_N_HIST * ns + s];
        tw = D.si[POSI_SI_TIMESTEP_WARNING * ns + s];
        status = D.si[POSI_SI_STATUS * ns + s];
        fail_step = D.si[POSI_SI_FAIL_STEP * ns + s];
        fail_pair = D.si[POSI_SI_FAIL_PAIR * ns + s];
        mid_iters = D.si[POSI_SI_LAST_MIDPOINT_ITERS * ns + s];
        dt = D.sf[POSI_SF_DT * ns + s];
        half_dt = D.sf[POSI_SF_HALF_DT * ns + s];
        t = D.sf[POSI_SF_TIME * ns + s];
        time_limit = D.sf[POSI_SF_TIME_LIMIT * ns + s];
        last_hist = D.sf[POSI_SF_LAST_HIST * ns + s];
        hist_period = D.sf[POSI_SF_HIST_PERIOD * ns + s];
        last_rec = D.sf[POSI_SF_LAST_REC * ns + s];
        rec_period = D.sf[POSI_SF_REC_PERIOD * ns + s];
        has = lane < n;
        is_host = lane == host;
        if (lane < 8) isc[lane] = 0;
        b.m = 0.; b.mg = 0.; b.R = 0.; b.moi = 0.;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            b.r[k] = 0.; b.v[k] = 0.; b.a[k] = 0.; b.L[k] = 0.; b.S[k] = 0.;
            b.ap[k] = 0.; b.av[k] = 0.; b.aacc[k] = 0.;
        }
        b.am = 0.; b.amg = 0.;
        if (has) {
            const int64_t st = D.stride;
            const int64_t o = (int64_t)s * D.nmax + lane;
            const double* F = D.bf + o;
            b.m = F[POSI_BF_MASS * st];
            b.mg = F[POSI_BF_MASS_G * st];
            b.R = F[POSI_BF_RADIUS * st];
            b.rg2 = F[POSI_BF_RG2 * st];
            b.moi = F[POSI_BF_MOI * st];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                b.r[k] = F[(POSI_BF_PX + k) * st];
                b.v[k] = F[(POSI_BF_VX + k) * st];
                b.a[k] = F[(POSI_BF_AX + k) * st];
                b.L[k] = F[(POSI_BF_LX + k) * st];
                b.S[k] = F[(POSI_BF_SX + k) * st];
                b.ev[k] = F[(POSI_BF_EVX + k) * st];
                b.eL[k] = F[(POSI_BF_ELX + k) * st];
                b.aa[k] = F[(POSI_BF_ADDAX + k) * st];
                b.dl[k] = F[(POSI_BF_DLX + k) * st];
            }
            b.nsv2 = F[POSI_BF_NSV2 * st];
            b.sig = F[POSI_BF_SIGMA * st];
            b.k2 = F[POSI_BF_K2 * st];
            b.k2f = F[POSI_BF_K2F * st];
            b.denergy = F[POSI_BF_DENERGY_DT * st];
            b.lag = F[POSI_BF_LAG_ANGLE * st];
#pragma unroll
            for (int k = 0; k < 13; ++k) P(PC_TD_DIST + k) = F[(POSI_BF_TD_DIST + k) * st];
            const int64_t* I = D.bi + o;
            b.tk = (int)I[POSI_BI_TIDES_KIND * st];
            b.fk = (int)I[POSI_BI_FLAT_KIND * st];
            b.gk = (int)I[POSI_BI_GR_KIND * st];
            b.wk = (int)I[POSI_BI_WIND_KIND * st];
            b.wind_k = F[POSI_BF_WIND_K * st];
            b.wind_rsat = F[POSI_BF_WIND_RSAT * st];
            b.wind_rsat2 = F[POSI_BF_WIND_RSAT2 * st];
            b.diss_factor = F[POSI_BF_DISS_FACTOR * st];
            b.diss_scale = F[POSI_BF_DISS_SCALE * st];
            b.dk = (int)I[POSI_BI_DISK_KIND * st];
#pragma unroll
            for (int k = 0; k < 6; ++k) b.disk_p[k] = F[(POSI_BF_DISK_INNER + k) * st];
            b.dmts = F[POSI_BF_DISK_MTS * st];
            b.evo = (int)I[POSI_BI_EVO_TYPE * st];
            b.eoff = I[POSI_BI_EVO_OFFSET * st];
            b.elen = I[POSI_BI_EVO_LEN * st];
            b.eleft = I[POSI_BI_EVO_LEFT * st];
            if (b.elen <= 0) b.evo = POSI_EVO_NON_EVOLVING;
        }
        if (is_host) {
            isc[5] = (tides && dynamical_evo(b.evo)) ? 1 : 0;
            isc[6] = (disk && b.dk == POSI_EFFECT_CENTRAL) ? 1 : 0;
        }
        sync();
        dyn_host = isc[5] != 0;
        disk_on = isc[6] != 0;
#if !POSI_EXACT
        mass_constants();
        if (!evo) launch_constants();
        pc_valid = false;
        pc_reuse = false;
#endif
    }

    __device__ void store(const Dev& D) const {
        const int64_t ns = D.n_sys;
        if (lane == 0) {
            D.si[POSI_SI_ITERATION * ns + s] = iteration;
            D.si[POSI_SI_N_HIST * ns + s] = n_hist;
            D.si[POSI_SI_TIMESTEP_WARNING * ns + s] = tw;
            D.si[POSI_SI_STATUS * ns + s] = status;
            D.si[POSI_SI_FAIL_STEP * ns + s] = fail_step;
            D.si[POSI_SI_FAIL_PAIR * ns + s] = fail_pair;
            D.si[POSI_SI_LAST_MIDPOINT_ITERS * ns + s] = mid_iters;
            D.sf[POSI_SF_TIME * ns + s] = t;
            D.sf[POSI_SF_LAST_HIST * ns + s] = last_hist;
            D.sf[POSI_SF_LAST_REC * ns + s] = last_rec;
        }
        if (!has) return;
        const int64_t st = D.stride;
        const int64_t o = (int64_t)s * D.nmax + lane;
        double* F = D.bf + o;
        F[POSI_BF_RADIUS * st] = b.R;
        F[POSI_BF_RG2 * st] = b.rg2;
        F[POSI_BF_MOI * st] = b.moi;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            F[(POSI_BF_PX + k) * st] = b.r[k];
            F[(POSI_BF_VX + k) * st] = b.v[k];
            F[(POSI_BF_AX + k) * st] = b.a[k];
            F[(POSI_BF_LX + k) * st] = b.L[k];
            F[(POSI_BF_SX + k) * st] = b.S[k];
            F[(POSI_BF_EVX + k) * st] = b.ev[k];
            F[(POSI_BF_ELX + k) * st] = b.eL[k];
            F[(POSI_BF_ADDAX + k) * st] = b.aa[k];
            F[(POSI_BF_DLX + k) * st] = b.dl[k];
        }
        F[POSI_BF_NSV2 * st] = b.nsv2;
        F[POSI_BF_DENERGY_DT * st] = b.denergy;
        F[POSI_BF_LAG_ANGLE * st] = b.lag;
        F[POSI_BF_DISK_MTS * st] = b.dmts;
#pragma unroll
        for (int k = 0; k < 13; ++k) F[(POSI_BF_TD_DIST + k) * st] = P(PC_TD_DIST + k);
        D.bi[POSI_BI_EVO_LEFT * st + o] = b.eleft;
    }

    __device__ void set_fatal(int code, int i, int j) {
        if (fatal()) return;
        status = (status & ~(int64_t)POSI_SYS_FATAL_MASK) | code;
        fail_step = iteration;
        fail_pair = (int64_t)i * 1024 + j;
    }

    // Column fold: for c in [0, ncol) starting from init (0 if null),
    // sums[c] = (((init + X(base+c, j0)) + X(base+c, j1)) + ...) over the
    // bodies in index order, the host skipped (skip_host) or visited first
    // (host_first).  Lane l evaluates columns l, l+G, ...
    __device__ void colfold(int base, int ncol, const double* init, bool skip_host, bool host_first) {
        sync();
        for (int c = lane; c < ncol; c += G) {
            double acc = init ? init[c] : 0.;
            if (host_first) acc += X(base + c, host);
            for (int j = 0; j < n; ++j) {
                if ((skip_host || host_first) && j == host) continue;
                acc += X(base + c, j);
            }
            sums[c] = acc;
        }
        sync();
    }

#if !POSI_EXACT
    // Mass-only constants of the launch: Jacobi prefix masses (host first,
    // then the other bodies in index order), reciprocals, Kepler GM.
    __device__ void mass_constants() {
        const double own_m = planet() ? b.m : 0.;
        const double own_mg = planet() ? b.mg : 0.;
        const double hm = gbcast(has ? b.m : 0., host);
        const double hmg = gbcast(has ? b.mg : 0., host);
        const double incl_m = gscan(own_m);
        const double incl_mg = gscan(own_mg);
        const double tot_m = gbcast(incl_m, G - 1);
        const double eta_excl = hm + (incl_m - own_m);
        eta_incl = hm + incl_m;
        inv_eta_excl = planet() ? 1. / eta_excl : 0.;
        jac_c = planet() ? b.m / eta_incl : 0.;
        kep_gm = hmg + incl_mg;
        inv_mtot = 1. / (hm + tot_m);
        inv_hm = 1. / hm;
        inv_m = has ? 1. / b.m : 0.;
        inv_moi = (has && b.moi != 0.) ? 1. / b.moi : 0.;
        gm_neg = -kG * b.m;
        whds_f = (hm + b.m) * inv_hm;             // (m0 + m) / m0
        whds_w = planet() ? b.m / (hm + b.m) : 0.;
        dh_w = planet() ? b.m * inv_hm : 0.;
        const int p0 = host == 0 ? 1 : 0;
        first_planet = lane == p0;
    }
#endif

    // ------------------------------------------------------------------
    // src/effects/evolution.rs:446-546 + src/tools.rs:840-907
    // ------------------------------------------------------------------
    __device__ double interp(const Dev& D, double target, int which) {
        // Evolver::idx()
        const int64_t i0 = b.eleft > kEVO_SHIFT ? b.eleft - kEVO_SHIFT : 0;
        const double* x = D.tables + b.eoff + i0;
        const double* y = D.tables + b.eoff + (int64_t)which * b.elen + i0;
        const int64_t nd = b.elen - i0;
        int64_t left, right, pos = -1;
        for (int64_t k = 0; k < nd; ++k) {
            if (x[k] > target) { pos = k; break; }
        }
        if (pos < 0) { left = nd - 1; right = nd - 1; }
        else if (pos == 0) { left = 0; right = 0; }
        else { left = pos - 1; right = pos; }
        double ty;
        if (left == right) {
            ty = y[left];
        } else {
            const double xl = x[left];
            const double pct = (target - xl) / (x[right] - xl);
            ty = y[left] * (1. - pct) + y[right] * pct;
        }
        b.eleft += left;
        return ty;
    }

    __device__ void evolve_non_spin(const Dev& D, double tt) {
        if (b.evo == POSI_EVO_NON_EVOLVING) return;
        const double nr = interp(D, tt, 1);
        double ng = b.rg2;
        if (b.evo == POSI_EVO_BARAFFE2015 || b.evo == POSI_EVO_LECONTE2011 || b.evo == POSI_EVO_LECONTE_CHABRIER2013)
            ng = interp(D, tt, 2);
        if (nr != b.R || ng != b.rg2) {
            b.R = nr;
            b.rg2 = ng;
            b.moi = b.m * b.rg2 * powi<2>(b.R);
#if !POSI_EXACT
            inv_moi = b.moi != 0. ? 1. / b.moi : 0.;
#endif
        }
        // The love-number update of the reference writes to a copy; only the
        // table index moves.
        if (b.tk != POSI_EFFECT_DISABLED && b.evo == POSI_EVO_LECONTE_CHABRIER2013) (void)interp(D, tt, 3);
    }

    // src/particles/universe.rs:305-316 with src/particles/common.rs:3-14
    __device__ void spin_and_evolving(const Dev& D, double tt, bool evolution) {
        if (has) {
            if (evolution && evo) evolve_non_spin(D, tt);
            if (b.moi == 0.) {
                isc[1] = 1;
            } else {
#if POSI_EXACT
                b.S[0] = b.L[0] / b.moi;
                b.S[1] = b.L[1] / b.moi;
                b.S[2] = b.L[2] / b.moi;
#else
                b.S[0] = b.L[0] * inv_moi;
                b.S[1] = b.L[1] * inv_moi;
                b.S[2] = b.L[2] * inv_moi;
#endif
                b.nsv2 = powi<2>(b.S[0]) + powi<2>(b.S[1]) + powi<2>(b.S[2]);
            }
            // src/effects/evolution.rs:548-567 (the dynamical-tide table's 4th
            // column is the inverse tidal Q factor, src/effects/evolution.rs:487-512)
            if (evolution && evo) {
                if (dynamical_evo(b.evo)) {
                    const double inverse_tidal_q_factor = interp(D, tt, 3);
                    const double epsilon_squared = b.nsv2 / kSUN_DYN_FREQ_2;
                    b.lag = 3.0 * epsilon_squared * inverse_tidal_q_factor / 4.0;
                } else {
                    b.lag = 0.;
                }
            }
        }
    }

    // src/effects/disk.rs:154-268: the disk's force on this planet
    // (migration, eccentricity and inclination damping; Alibert et al. 2013)
    // from its heliocentric position (x, y, z), velocity (u, v, w), distance d
    // and squared speed nv2; the host's values and DiskProperties from the card
    __device__ void disk_force(double x, double y, double z, double u, double v, double w, double d, double nv2,
                               double F[3]) {
        const double hm = card[HC_M], hmg = card[HC_MG];
        const double sma = (b.mg + hmg) * d / (2.0 * (b.mg + hmg) - d * nv2);
        // DiskProperties::calculate_migration_timescale
        const double keplerian_frequency = sqrt(hmg / powi<3>(d));
        const double disk_temperature = 280.0 * pow_m0p5(d) * hm;
        const double speed_of_sound_squared = kBOLTZMANN * disk_temperature / (card[HC_DMU] * kMASS_HYDROGEN);
        const double viscosity = card[HC_DALPHA] * speed_of_sound_squared / keplerian_frequency;
        const double gas_radial_velocity = -3.0 * viscosity / (2.0 * sma);
        const double initial_density = card[HC_DSIG0] * (1. / d) * exp_dd(-1.0 * d / card[HC_DOUTER]) *
                                       (1.0 - sqrt(card[HC_DINNER] / d));
        double density = 0.;
        if (d > card[HC_DINNER]) density = initial_density * exp_dd(-t / card[HC_DLIFE]);
        const double yy = 2.0 * density * powi<2>(sma) / b.m;
        const double a_dot = gas_radial_velocity * (yy < 1.0 ? yy : 1.0);   // f64::min(1.0, yy)
        const double migration_timescale = -sma / a_dot;
        b.dmts = migration_timescale;
        const double factor_migration = -b.m / migration_timescale;
        const double ecc_timescale = 0.1 * migration_timescale;
        const double factor_ecc = -b.m * 2.0 / ecc_timescale;
        const double factor_inc = -b.m * 2.0 / ecc_timescale;
        const double sp = 1.0 / (d * d) * (x * u + y * v + z * w);
        F[0] = factor_migration * u + factor_ecc * sp * x + 0.0;
        F[1] = factor_migration * v + factor_ecc * sp * y + 0.0;
        F[2] = factor_migration * w + factor_ecc * sp * z + factor_inc * w;
    }

    // src/effects/tides/constant_time_lag.rs:20-93 with src/tools.rs:251-285:
    // the host's dissipation factor for this planet when the host's dynamical
    // tide is excited, else its own (x: heliocentric position, v: heliocentric
    // velocity; the host's values from the card)
    __device__ double host_sigma_for(double x, double y, double z, double u, double v, double w) const {
        const double host_norm_spin_vector = sqrt(card[HC_NSV2]);
        const double gm = card[HC_MG] + b.mg;
        const double hx = y * w - z * v;
        const double hy = z * u - x * w;
        const double hz = x * v - y * u;
        const double h2 = hx * hx + hy * hy + hz * hz;   // powf(2.): the exact square, rounded once
        const double v2 = u * u + v * v + w * w;
        const double r = sqrt(x * x + y * y + z * z);
        const double sv = h2 / gm;
        const double temp = 1. + sv * (v2 / gm - 2. / r);
        const double ecc = temp <= 0. ? 0. : sqrt(temp);
        const double peri = sv / (1. + ecc);
        const double mean_motion = sqrt(gm) * pow_m1p5(peri / (1.0 - ecc));
        double half = fabs(host_norm_spin_vector - mean_motion);
        if (!(half < host_norm_spin_vector)) return card[HC_SIG];
        if (half < kSMOOTHING_DYN_TIDE) half = kSMOOTHING_DYN_TIDE;
        const double inv = 1. / half;
        return card[HC_DSCALE] * (2.0 * kK2 / (3.0 * powi<5>(card[HC_R])) * card[HC_LAG] * inv + card[HC_DFAC]);
    }

    __device__ void zero_inertia_check() {
        sync();
        if (isc[1]) set_fatal(POSI_SYS_ZERO_INERTIA, 0, 0);
        sync();
    }

    // ------------------------------------------------------------------
    // Per-planet constants of a half kick (after the spin/evolution update
    // of its first midpoint iteration, so that evolved radii are used).
    // ------------------------------------------------------------------
    __device__ __forceinline__ void record_tidal_internals(double d, double vr, double ortho, double dpm, double x,
                                                           double y, double z, double vx, double vy, double vz,
                                                           double lx, double ly, double lz) {
        P(PC_TD_DIST) = d; P(PC_TD_VR) = vr; P(PC_TD_ORTHO) = ortho; P(PC_TD_DPM) = dpm;
        P(PC_TD_P0) = x; P(PC_TD_P1) = y; P(PC_TD_P2) = z;
        P(PC_TD_V0) = vx; P(PC_TD_V1) = vy; P(PC_TD_V2) = vz;
        P(PC_TD_L0) = lx; P(PC_TD_L1) = ly; P(PC_TD_L2) = lz;
    }

    // src/effects/tides/common.rs:263-279, in the reference's operation order,
    // from the tidal internals of the last evaluation and the current spin.
    __device__ void tides_denergy_dt() {
        if (!(planet() && b.tk == POSI_EFFECT_ORBITING)) return;
        const double d = P(PC_TD_DIST), vr = P(PC_TD_VR);
        const double x = P(PC_TD_P0), y = P(PC_TD_P1), z = P(PC_TD_P2);
        const double vx = P(PC_TD_V0), vy = P(PC_TD_V1), vz = P(PC_TD_V2);
        const double sx = b.S[0], sy = b.S[1], sz = b.S[2];
        const double factor2 = P(PC_TD_ORTHO) / d;
        b.denergy = -((1.0 / d * (P(PC_TD_DPM) + factor2 * vr)) * (x * vx + y * vy + z * vz)
                      + factor2 * ((sy * z - sz * y - vx) * vx + (sz * x - sx * z - vy) * vy + (sx * y - sy * x - vz) * vz))
                    - (P(PC_TD_L0) * sx + P(PC_TD_L1) * sy + P(PC_TD_L2) * sz);
    }

    // src/integrator/output.rs:91-135: the record of one historic snapshot.
    __device__ void write_history_record(const Dev& D) const {
        if (!D.hist || !has) return;
        double* R = D.hist + ((int64_t)s * D.nmax + lane) * HR_COUNT;
        R[HR_T] = t; R[HR_DT] = dt; R[HR_ID] = (double)lane;
        R[HR_PX] = b.r[0]; R[HR_PY] = b.r[1]; R[HR_PZ] = b.r[2];
        R[HR_SX] = b.S[0]; R[HR_SY] = b.S[1]; R[HR_SZ] = b.S[2];
        R[HR_VX] = b.v[0]; R[HR_VY] = b.v[1]; R[HR_VZ] = b.v[2];
        R[HR_M] = b.m; R[HR_R] = b.R; R[HR_RG2] = b.rg2;
        R[HR_K2] = b.tk != POSI_EFFECT_DISABLED ? b.k2 : 0.;
        R[HR_SIGMA] = b.sig; R[HR_LAG] = b.lag; R[HR_DENERGY] = b.denergy; R[HR_MIGRATION] = b.dmts;
    }

    // Heliocentric position of a planet, its distance and unit vector: fixed
    // for a whole half kick, needed from the first evaluation on.
    __device__ void set_geometry(double x, double y, double z) {
        P(PC_X) = x;
        P(PC_Y) = y;
        P(PC_Z) = z;
#if POSI_EXACT
        const double d = sqrt(powi<2>(x) + powi<2>(y) + powi<2>(z));
        const double inv_d = 1. / d;
#else
        const double d2 = powi<2>(x) + powi<2>(y) + powi<2>(z);
        const double inv_d = rsqrt(d2);
        const double d = d2 * inv_d;
#endif
        P(PC_D) = d;
        P(PC_INV_D) = inv_d;
        P(PC_XD) = x * inv_d;
        P(PC_YD) = y * inv_d;
        P(PC_ZD) = z * inv_d;
    }

#if !POSI_EXACT
    // FAST: the distance-free factors of the constants once per launch
    // (planet_launch_constants), the powers of 1 / d once per half kick.
    __device__ void planet_launch_constants(double hm, double hmg, double hR, double hsig, double hk2,
                                            double hk2f) {
        if (tides && b.tk == POSI_EFFECT_ORBITING) {
            // src/effects/tides/constant_time_lag.rs:229-264, :266-307
            const double hm2 = hm * hm, m2 = b.m * b.m;
            const double term1 = m2 * powi<10>(hR) * hsig;
            const double term2 = hm2 * powi<10>(b.R) * b.sig;
            P(PC_LT1) = 4.5 * term1;
            P(PC_LT2) = 4.5 * term2;
            P(PC_LCONS) = kMINUS_3K2 * (m2 * powi<5>(hR) * hk2 + hm2 * powi<5>(b.R) * b.k2);
            P(PC_TERM2) = term2;
            P(PC_T12) = term1 + term2;
        }
        if (flat && b.fk == POSI_EFFECT_ORBITING) {
            // src/effects/rotational_flattening/oblate_spheroid.rs:12-60
            // factor_star = cfs |Omega_host|^2, ortho_star = cofs (r . Omega_host(previous))
            P(PC_CFS) = b.m * hk2f * powi<5>(hR) * (1. / 6.);
            P(PC_CFP) = hm * b.k2f * powi<5>(b.R) * (1. / 6.);
        }
        if (grk() && b.gk == POSI_EFFECT_ORBITING) {
            // src/effects/general_relativity.rs:98, :187-298, :300-456.
            // The first- and second-order terms are one polynomial in |v|^2
            // and v_r^2:
            //   radial = A (GR0 + |v|^2 (GR1 + K2C |v|^2 - K4C v_r^2) + v_r^2 (GR2 + K3C v_r^2)),
            //   ortho  = v_r (GO0 + GO1 |v|^2 + GO2 v_r^2),
            // GR0 = T1 - C, GR1 = B - K5C, GR2 = -(DD + K6C), GO0 = E - A05 Q,
            // GO1 = A05 P, GO2 = -A05 R3 in the terms of the reference's two
            // orders; with mgd = (mg_host + mg) / d and A = -mgd / (c^2 d)
            // every one is a launch constant times a power of mgd and A.
            const double mgs = hmg + b.mg;
            const double imgs = 1. / mgs;
            const double f = hmg * b.mg * (imgs * imgs);
            const double f2 = f * f;
            P(PC_LMGS) = mgs;
            P(PC_LMGSC2) = -mgs * (1. / kC2);
            P(PC_LT1C) = (3.0 / 4.0) * (12.0 + 29.0 * f);   // T1 / mgd^2
            P(PC_LCC) = 2.0 * (2.0 + f);                     // C / mgd
            P(PC_LB) = 1.0 + 3.0 * f;                        // B
            P(PC_LK5) = 0.5 * f * (13.0 - 4.0 * f);          // K5C / mgd
            P(PC_LNDD) = -1.5 * f;                           // -DD
            P(PC_LK6) = 2.0 + 25.0 * f + 2.0 * f2;           // K6C / mgd
            P(PC_LQH) = 0.5 * (4.0 + 41.0 * f + 8.0 * f2);   // Q / (2 mgd)
            P(PC_LNEC) = -2.0 * (2.0 - f);                   // -E / (-A)
            P(PC_LNPH) = -0.5 * (f * (15.0 + 4.0 * f));      // -P / 2
            P(PC_LR3H) = 0.5 * (3.0 * f * (3.0 + 2.0 * f));  // R3 / 2
            P(PC_K2C) = f * (3.0 - 4.0 * f);
            P(PC_K3C) = (15.0 / 8.0) * f * (1.0 - 3.0 * f);
            P(PC_K4C) = (3.0 / 2.0) * f * (3.0 - 4.0 * f);
            const double M = hm + b.m;
            const double iM = 1. / M;
            const double mu = (hm * b.m) * iM;
            // ((m_host - m) / M) M (L_p / m - L_h / m_h) = LMA S_p - LMB L_h
            P(PC_LMA) = (hm - b.m) * b.moi * inv_m;
            P(PC_LMB) = (hm - b.m) * inv_hm;
            // Kidder 1995 eq. 2.4a / 2.4b: the orbital angular momentum
            // mu (r x v) enters the torques scaled by these
            P(PC_FMU) = (2. + (3. / 2.) * b.m * inv_hm) * mu;
            P(PC_FM2MU) = (2. + (3. / 2.) * hm * inv_m) * mu;
        }
        P(PC_MRATIO) = b.m * hm == 0. ? 0. : b.m * inv_hm;
    }

    // the launch constants from the host's values, at load (every lane of
    // the group takes part)
    __device__ void launch_constants() {
        const double hR = gbcast(has ? b.R : 0., host), hsig = gbcast(has ? b.sig : 0., host);
        const double hk2 = gbcast(has ? b.k2 : 0., host), hk2f = gbcast(has ? b.k2f : 0., host);
        const double hm = gbcast(has ? b.m : 0., host), hmg = gbcast(has ? b.mg : 0., host);
        if (planet()) planet_launch_constants(hm, hmg, hR, hsig, hk2, hk2f);
    }

    __device__ void planet_constants() {
        if (evo)
            planet_launch_constants(card[HC_M], card[HC_MG], card[HC_R], card[HC_SIG], card[HC_K2], card[HC_K2F]);
        const double id = P(PC_INV_D);
        const double id2 = id * id, id5 = id2 * id2 * id, id7 = id5 * id2;
        if (tides && b.tk == POSI_EFFECT_ORBITING) {
            const double o_s = P(PC_LT1) * id7;
            const double o_p = P(PC_LT2) * id7;
            P(PC_OS) = o_s;
            P(PC_OP) = o_p;
            P(PC_OSD) = o_s * id;
            P(PC_OPD) = o_p * id;
            P(PC_CONS) = P(PC_LCONS) * id7;
            P(PC_OSPD) = (o_s + o_p) * id;
            const double d = P(PC_D);
            P(PC_OSDD) = o_s * d;
            P(PC_OPDD) = o_p * d;
            P(PC_C13) = -13.5 * (id7 * id);
        }
        if (flat && b.fk == POSI_EFFECT_ORBITING) {
            P(PC_N3D5) = -3. * id5;
            P(PC_F15D7) = 15. * id7;
            P(PC_COFS) = -6. * P(PC_CFS) * id5;
            P(PC_COFP) = -6. * P(PC_CFP) * id5;
        }
        if (grk() && b.gk == POSI_EFFECT_ORBITING) {
            const double mgd = P(PC_LMGS) * id;
            const double A = P(PC_LMGSC2) * id2;
            P(PC_A) = A;
            P(PC_GR0) = mgd * (P(PC_LT1C) * mgd - P(PC_LCC));
            P(PC_GR1) = P(PC_LB) - P(PC_LK5) * mgd;
            P(PC_GR2) = P(PC_LNDD) - P(PC_LK6) * mgd;
            P(PC_GO0) = A * (P(PC_LQH) * mgd + P(PC_LNEC));
            P(PC_GO1) = A * P(PC_LNPH);
            P(PC_GO2) = A * P(PC_LR3H);
            const double id6 = 6. * id;
            P(PC_C6NN0) = id6 * P(PC_XD);
            P(PC_C6NN1) = id6 * P(PC_YD);
            P(PC_C6NN2) = id6 * P(PC_ZD);
        }
    }
#else
    __device__ void planet_constants() {
        const double hm = card[HC_M], hmg = card[HC_MG], hR = card[HC_R], hsig = card[HC_SIG];
        const double hk2 = card[HC_K2], hk2f = card[HC_K2F];
        const double d = P(PC_D);
        const double inv_d = P(PC_INV_D);
        if (tides && b.tk == POSI_EFFECT_ORBITING) {
            // src/effects/tides/constant_time_lag.rs:229-264, :266-307
            const double d7 = powi<7>(d);
            const double o_s = 4.5 * powi<2>(b.m) * powi<10>(hR) * hsig / d7;
            const double o_p = 4.5 * powi<2>(hm) * powi<10>(b.R) * b.sig / d7;
            P(PC_OS) = o_s;
            P(PC_OP) = o_p;
            P(PC_OSD) = o_s / d;
            P(PC_OPD) = o_p / d;
            const double hm2 = hm * hm;
            const double m2 = b.m * b.m;
            P(PC_CONS) = kMINUS_3K2 / powi<7>(d) * (m2 * powi<5>(hR) * hk2 + hm2 * powi<5>(b.R) * b.k2);
            const double d8 = powi<8>(d);
            P(PC_D8) = d8;
            const double term1 = m2 * powi<10>(hR) * hsig;
            const double term2 = hm2 * powi<10>(b.R) * b.sig;
            P(PC_TERM1) = term1;
            P(PC_TERM2) = term2;
        }
        if (flat && b.fk == POSI_EFFECT_ORBITING) {
            // src/effects/rotational_flattening/oblate_spheroid.rs:12-60
            P(PC_MHK2F) = b.m * hk2f;
            P(PC_HMK2F) = hm * b.k2f;
            P(PC_R5H) = powi<5>(hR);
            P(PC_R5P) = powi<5>(b.R);
            P(PC_D5) = powi<5>(d);
            P(PC_N3D5) = -3. / powi<5>(d);
            P(PC_F15D7) = 15. / powi<7>(d);
        }
        if (grk() && b.gk == POSI_EFFECT_ORBITING) {
            // src/effects/general_relativity.rs:98, :187-298, :300-456
            const double f = hmg * b.mg / powi<2>(hmg + b.mg);
            const double mgs = hmg + b.mg;
            const double d2 = powi<2>(d);
            const double mgd = mgs / d;
            const double f2 = powi<2>(f);
            const double A = -mgs / (d2 * kC2);
            P(PC_A) = A;
            P(PC_B) = 1.0 + 3.0 * f;
            P(PC_C) = 2.0 * (2.0 + f) * mgs / d;
            P(PC_DD) = 1.5 * f;
            P(PC_E) = mgs / (d2 * kC2) * 2.0 * (2.0 - f);
            P(PC_T1) = (3.0 / 4.0) * (12.0 + 29.0 * f) * (powi<2>(mgs) / d2);
            P(PC_K2C) = f * (3.0 - 4.0 * f);
            P(PC_K3C) = (15.0 / 8.0) * f * (1.0 - 3.0 * f);
            P(PC_K4C) = (3.0 / 2.0) * f * (3.0 - 4.0 * f);
            P(PC_K5C) = 0.5 * f * (13.0 - 4.0 * f) * mgd;
            P(PC_K6C) = (2.0 + 25.0 * f + 2.0 * f2) * mgd;
            P(PC_A05) = A * (-0.5);
            P(PC_P) = f * (15.0 + 4.0 * f);
            P(PC_Q) = (4.0 + 41.0 * f + 8.0 * f2) * mgd;
            P(PC_R3) = 3.0 * f * (3.0 + 2.0 * f);
            P(PC_MRATIO) = b.m / hm;
            const double M = hm + b.m;
            const double mf = (hm - b.m) / M;
            P(PC_MFM) = mf * M;
            P(PC_MU) = (hm * b.m) / M;
            P(PC_FM) = 2. + (3. / 2.) * b.m / hm;
            P(PC_FM2) = 2. + (3. / 2.) * hm / b.m;
            const double n0 = P(PC_X) / d, n1 = P(PC_Y) / d, n2 = P(PC_Z) / d;
            P(PC_NN0) = n0;
            P(PC_NN1) = n1;
            P(PC_NN2) = n2;
            P(PC_C6NN0) = 6. * n0;
            P(PC_C6NN1) = 6. * n1;
            P(PC_C6NN2) = 6. * n2;
        }
    }
#endif


    // src/effects/wind.rs:72-91 (Bolmont & Mathis 2016 eq. 14): the spin-down
    // torque of an interacting body, from the spin of this evaluation
    __device__ void wind_torque(double w[3]) const {
        w[0] = w[1] = w[2] = 0.;
        if (!(wind && has && b.wk == 1)) return;
        const double threshold = sqrt(b.nsv2);
        const double ww = threshold >= b.wind_rsat ? b.wind_rsat2 : b.nsv2;
#pragma unroll
        for (int k = 0; k < 3; ++k) w[k] = -1. * b.wind_k * b.S[k] * ww * sqrt(b.R / kR_SUN * 1. / b.m);
    }

    // ------------------------------------------------------------------
    // General relativity after REBOUNDx gr.c (src/effects/general_relativity.rs
    // :461-898): Anderson1975 (a central body, in Jacobi coordinates) and
    // Newhall1983 (every pair of bodies).  Every lane publishes its body in
    // the exchange slots and evaluates its own output; the sequential parts
    // (Jacobi recurrences, the host's sums, the convergence test) are run by
    // every lane over the shared slots in the reference's order, so that all
    // lanes agree and the arithmetic is the reference's.  g: this body's GR
    // acceleration (the host's included); bodies outside the effect get zero.
    // ------------------------------------------------------------------
    enum { GX_R = 0, GX_V = 3, GX_A = 6, GX_M = 9, GX_K = 10, GX_W = 11, GX_O = 14, GX_END = 17 };
    static_assert(GX_END <= kXS, "exchange slots");

    __device__ void gr_nbody(double g[3]) {
        const int ignore = gr_ignore;
        sync();
        if (has) {
#pragma unroll
            for (int k = 0; k < 3; ++k) { X(GX_R + k, lane) = b.r[k]; X(GX_V + k, lane) = b.v[k]; }
            X(GX_M, lane) = b.m;
            X(GX_K, lane) = (double)b.gk;
        }
        // :661-697 the gravity accelerations plus the host terms the
        // integrator ignored: host inertial position minus the body's
        // heliocentric (GR) position
        const int np = ignore == 1 ? 1 : (ignore == 2 ? n - 1 : 0);
        const int rank = lane < host ? lane : lane - 1;   // position among the other bodies
        double na[3] = {b.a[0], b.a[1], b.a[2]};
        if (planet() && rank < np) {
            const double dx = card[HC_PX] - P(PC_X), dy = card[HC_PY] - P(PC_Y), dz = card[HC_PZ] - P(PC_Z);
            const double r2 = powi<2>(dx) + powi<2>(dy) + powi<2>(dz);
            const double r = sqrt(r2);
            const double prefac = kG / (r2 * r);
            const double pms = prefac * card[HC_M];
            const double pmp = prefac * b.m;
            na[0] += pms * dx; na[1] += pms * dy; na[2] += pms * dz;
            X(GX_W + 0, lane) = pmp * dx; X(GX_W + 1, lane) = pmp * dy; X(GX_W + 2, lane) = pmp * dz;
        }
        sync();
        if (is_host) {
            for (int j = 0, rk = 0; j < n; ++j) {
                if (j == host) continue;
                if (rk++ >= np) break;
#pragma unroll
                for (int k = 0; k < 3; ++k) na[k] -= X(GX_W + k, j);
            }
        }
        sync();
        if (has) {
#pragma unroll
            for (int k = 0; k < 3; ++k) X(GX_A + k, lane) = na[k];
        }
        sync();
        g[0] = g[1] = g[2] = 0.;
        if (gr_impl == POSI_GR_ANDERSON1975) gr_anderson1975(g);
        else gr_newhall1983(g);
    }

    __device__ __forceinline__ bool gr_orbiting(int j) const { return X(GX_K, j) == (double)POSI_EFFECT_ORBITING; }

    // :461-535 with the Jacobi transforms :537-634
    __device__ void gr_anderson1975(double g[3]) {
        const double m0 = X(GX_M, host);
        double eta = m0;
        double sr[3], sv[3], sa[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sr[k] = eta * X(GX_R + k, host);
            sv[k] = eta * X(GX_V + k, host);
            sa[k] = eta * X(GX_A + k, host);
        }
        double jp[3] = {0., 0., 0.}, jv[3] = {0., 0., 0.}, ja[3] = {0., 0., 0.};
        for (int j = 0; j < n; ++j) {
            if (j == host || !gr_orbiting(j)) continue;
            const double mj = X(GX_M, j);
            const double ei = 1. / eta;
            eta += mj;
            const double pme = eta * ei;
            double p[3], v[3], a[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                p[k] = X(GX_R + k, j) - sr[k] * ei;
                v[k] = X(GX_V + k, j) - sv[k] * ei;
                a[k] = X(GX_A + k, j) - sa[k] * ei;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                sr[k] = sr[k] * pme + mj * p[k];
                sv[k] = sv[k] * pme + mj * v[k];
                sa[k] = sa[k] * pme + mj * a[k];
            }
            if (j == lane) {
#pragma unroll
                for (int k = 0; k < 3; ++k) { jp[k] = p[k]; jv[k] = v[k]; ja[k] = a[k]; }
            }
        }
        const double mtot = eta;
        const bool own = planet() && b.gk == POSI_EFFECT_ORBITING;
        if (own) {
            const double mu = card[HC_MG];
            double vi[3] = {jv[0], jv[1], jv[2]};
            double vi2 = powi<2>(jv[0]) + powi<2>(jv[1]) + powi<2>(jv[2]);
            const double ri = sqrt(powi<2>(jp[0]) + powi<2>(jp[1]) + powi<2>(jp[2]));
            double fa = (0.5 * vi2 + 3. * mu / ri) / kC2;
            for (int q = 0; q < 10; ++q) {
                const double o0 = vi[0], o1 = vi[1], o2 = vi[2];
                vi[0] = jv[0] / (1. - fa);
                vi[1] = jv[1] / (1. - fa);
                vi[2] = jv[2] / (1. - fa);
                vi2 = vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2];
                fa = (0.5 * vi2 + 3. * mu / ri) / kC2;
                const double dvx = vi[0] - o0, dvy = vi[1] - o1, dvz = vi[2] - o2;
                if ((dvx * dvx + dvy * dvy + dvz * dvz) / vi2 < kDBL_EPSILON_2) break;
            }
            const double fb = (mu / ri - 1.5 * vi2) * mu / (ri * ri * ri) / kC2;
            const double rdotrdot = jp[0] * jv[0] + jp[1] * jv[1] + jp[2] * jv[2];
            const double vd0 = ja[0] + fb * jp[0], vd1 = ja[1] + fb * jp[1], vd2 = ja[2] + fb * jp[2];
            const double vdotvdot = vi[0] * vd0 + vi[1] * vd1 + vi[2] * vd2;
            const double fd = (vdotvdot - 3. * mu / (ri * ri * ri) * rdotrdot) / kC2;
#pragma unroll
            for (int k = 0; k < 3; ++k) ja[k] = fb * (1. - fa) * jp[k] - fa * ja[k] - fd * vi[k];
        }
        sync();
        if (own) {
#pragma unroll
            for (int k = 0; k < 3; ++k) X(GX_W + k, lane) = ja[k];
        }
        sync();
        // Jacobi -> inertial, the Jacobi star acceleration zero
        eta = mtot;
        double s2[3] = {eta * 0., eta * 0., eta * 0.};
        for (int j = n - 1; j >= 0; --j) {
            if (j == host || !gr_orbiting(j)) continue;
            const double mj = X(GX_M, j);
            const double ei = 1. / eta;
#pragma unroll
            for (int k = 0; k < 3; ++k) s2[k] = (s2[k] - mj * X(GX_W + k, j)) * ei;
            if (j == lane) {
#pragma unroll
                for (int k = 0; k < 3; ++k) g[k] = X(GX_W + k, j) + s2[k];
            }
            eta -= mj;
#pragma unroll
            for (int k = 0; k < 3; ++k) s2[k] *= eta;
        }
        if (is_host) {
            const double mi = 1. / eta;
#pragma unroll
            for (int k = 0; k < 3; ++k) g[k] = s2[k] * mi;
        }
    }

    // :702-898: reference order of bodies is the host, then the others in
    // index order.  rs between two bodies exists only where one of them is in
    // the effect (zero otherwise, as in the reference).
    __device__ __forceinline__ int gr_ord(int t) const { return t == 0 ? host : (t - 1 < host ? t - 1 : t); }
    __device__ __forceinline__ bool gr_on(int j) const { return X(GX_K, j) != (double)POSI_EFFECT_DISABLED; }
    __device__ __forceinline__ double gr_dist(int a, int c, double d[3]) const {
#pragma unroll
        for (int k = 0; k < 3; ++k) d[k] = X(GX_R + k, a) - X(GX_R + k, c);
        return sqrt(powi<2>(d[0]) + powi<2>(d[1]) + powi<2>(d[2]));
    }
    __device__ __forceinline__ double gr_rs(int a, int c) const {
        if (a == c || !(gr_on(a) || gr_on(c))) return 0.;
        double d[3];
        return gr_dist(a, c, d);
    }

    __device__ void gr_newhall1983(double g[3]) {
        const int i = lane;
        double ac[3] = {0., 0., 0.};
        if (has) {
            const double vix = X(GX_V + 0, i), viy = X(GX_V + 1, i), viz = X(GX_V + 2, i);
            for (int tj = 0; tj < n; ++tj) {
                const int j = gr_ord(tj);
                if (j == i || !(gr_on(i) || gr_on(j))) continue;
                double d[3];
                const double rij = gr_dist(i, j, d);
                const double dxij = d[0], dyij = d[1], dzij = d[2];
                const double rij2 = powi<2>(rij);
                const double rij3 = rij2 * rij;
                double a1 = 0.;
                for (int tk = 0; tk < n; ++tk) {
                    const int k = gr_ord(tk);
                    if (k != i) a1 += (4. / kC2) * kG * X(GX_M, k) / gr_rs(i, k);
                }
                double a2 = 0.;
                for (int tl = 0; tl < n; ++tl) {
                    const int l = gr_ord(tl);
                    if (l != j) a2 += (1. / kC2) * kG * X(GX_M, l) / gr_rs(l, j);
                }
                const double vjx = X(GX_V + 0, j), vjy = X(GX_V + 1, j), vjz = X(GX_V + 2, j);
                const double vi2 = powi<2>(vix) + powi<2>(viy) + powi<2>(viz);
                const double a3 = -vi2 / kC2;
                const double vj2 = powi<2>(vjx) + powi<2>(vjy) + powi<2>(vjz);
                const double a4 = -2. * vj2 / kC2;
                const double a5 = (4. / kC2) * (vix * vjx + viy * vjy + viz * vjz);
                const double a6_0 = dxij * vjx + dyij * vjy + dzij * vjz;
                const double a6 = (3. / (2. * kC2)) * powi<2>(a6_0) / rij2;
                const double f1 = a1 + a2 + a3 + a4 + a5 + a6;
                const double gm = kG * X(GX_M, j);
                ac[0] += gm * dxij * f1 / rij3;
                ac[1] += gm * dyij * f1 / rij3;
                ac[2] += gm * dzij * f1 / rij3;
                const double dvx = vix - vjx, dvy = viy - vjy, dvz = viz - vjz;
                const double f2 = dxij * (4. * vix - 3. * vjx) + dyij * (4. * viy - 3. * vjy) + dzij * (4. * viz - 3. * vjz);
                ac[0] += gm * f2 * dvx / rij3 / kC2;
                ac[1] += gm * f2 * dvy / rij3 / kC2;
                ac[2] += gm * f2 * dvz / rij3 / kC2;
            }
        }
        // substitution loop: a_new in GX_W, a_old in GX_O
        sync();
        if (has) {
#pragma unroll
            for (int k = 0; k < 3; ++k) X(GX_W + k, lane) = 0.;
        }
        double an[3] = {0., 0., 0.};
        for (int it = 0; it < 10; ++it) {
            sync();
            if (has) {
#pragma unroll
                for (int k = 0; k < 3; ++k) X(GX_O + k, lane) = X(GX_W + k, lane);
            }
            sync();
            if (has) {
                double nc[3] = {0., 0., 0.};
                for (int tj = 0; tj < n; ++tj) {
                    const int j = gr_ord(tj);
                    if (j == i || !(gr_on(i) || gr_on(j))) continue;
                    double d[3];
                    const double rij = gr_dist(i, j, d);
                    const double dxij = d[0], dyij = d[1], dzij = d[2];
                    const double rij2 = powi<2>(rij);
                    const double rij3 = rij2 * rij;
                    const double sx = X(GX_A + 0, j) + X(GX_O + 0, j);
                    const double sy = X(GX_A + 1, j) + X(GX_O + 1, j);
                    const double sz = X(GX_A + 2, j) + X(GX_O + 2, j);
                    const double dot = dxij * sx + dyij * sy + dzij * sz;
                    const double gm = kG * X(GX_M, j);
                    nc[0] += (gm * dxij / rij3) * dot / (2. * kC2) + (7. / (2. * kC2)) * kG * X(GX_M, j) * sx / rij;
                    nc[1] += (gm * dyij / rij3) * dot / (2. * kC2) + (7. / (2. * kC2)) * kG * X(GX_M, j) * sy / rij;
                    nc[2] += (gm * dzij / rij3) * dot / (2. * kC2) + (7. / (2. * kC2)) * kG * X(GX_M, j) * sz / rij;
                }
#pragma unroll
                for (int k = 0; k < 3; ++k) an[k] = ac[k] + nc[k];
            }
            sync();
            if (has) {
#pragma unroll
                for (int k = 0; k < 3; ++k) X(GX_W + k, lane) = an[k];
            }
            sync();
            // the reference's test: a component's relative change counts only
            // where |a| < 1e-30, otherwise the previous value stays
            double maxdev = 0., dx = 0., dy = 0., dz = 0.;
            for (int t = 0; t < n; ++t) {
                const int j = gr_ord(t);
                if (!gr_on(j)) continue;
                const double nx = X(GX_W + 0, j), ny = X(GX_W + 1, j), nz = X(GX_W + 2, j);
                if (fabs(nx) < 1.0e-30) dx = fabs(nx - X(GX_O + 0, j)) / nx;
                if (fabs(ny) < 1.0e-30) dy = fabs(ny - X(GX_O + 1, j)) / ny;
                if (fabs(nz) < 1.0e-30) dz = fabs(nz - X(GX_O + 2, j)) / nz;
                if (dx > maxdev) maxdev = dx;
                if (dy > maxdev) maxdev = dy;
                if (dz > maxdev) maxdev = dz;
            }
            if (maxdev < 1.0e-30) break;
        }
        if (is_host || (planet() && b.gk == POSI_EFFECT_ORBITING)) {
            g[0] = an[0]; g[1] = an[1]; g[2] = an[2];
        }
    }

    // ------------------------------------------------------------------
    // One evaluation of src/particles/universe.rs:428-538 (after
    // inertial_to_heliocentric :318-351), it = midpoint iteration.
    // ------------------------------------------------------------------
#if POSI_EXACT
    // Contribution columns written per planet (host back-reactions):
    //  0-2 tidal force, 3-5 -torque on host (tides), 6-8 flattening force,
    //  9-11 -torque on host (flattening), 12-14 (m/M) a_1PN, 15-17 (m/M) a_2PN,
    //  18-20 (m/M) a_SO, 21-23 host dL/dt (GR).
    __device__ void additional_effects(const Dev& D, int it, bool evolution_now) {
        // host inertial velocity and the spin it had before this evaluation
        sync();
        if (is_host) {
            card[HC_VX] = b.v[0]; card[HC_VY] = b.v[1]; card[HC_VZ] = b.v[2];
            card[HC_SX] = b.S[0]; card[HC_SY] = b.S[1]; card[HC_SZ] = b.S[2];
        }
        if (lane == 0) isc[1] = 0;
        sync();
        double hv[3] = {0., 0., 0.}, vr = 0., nv2 = 0., nv = 0., rs_s = 0., rs_p = 0.;
        const double x = P(PC_X), y = P(PC_Y), z = P(PC_Z), d = P(PC_D);
        if (planet()) {
            hv[0] = b.v[0] - card[HC_VX];
            hv[1] = b.v[1] - card[HC_VY];
            hv[2] = b.v[2] - card[HC_VZ];
            vr = (x * hv[0] + y * hv[1] + z * hv[2]) / d;
            // the host's previous heliocentric velocity is zero (universe.rs:335-338)
            nv2 = powi<2>(hv[0] - 0.) + powi<2>(hv[1] - 0.) + powi<2>(hv[2] - 0.);
            nv = sqrt(nv2);
            // tides::initialize / rotational_flattening::initialize use the spin
            // computed before this evaluation
            rs_s = x * card[HC_SX] + y * card[HC_SY] + z * card[HC_SZ];
            rs_p = x * b.S[0] + y * b.S[1] + z * b.S[2];
        }
        spin_and_evolving(D, t, evolution_now);
        zero_inertia_check();
        if (fatal()) return;
        if (is_host) {
            card[HC_SX] = b.S[0]; card[HC_SY] = b.S[1]; card[HC_SZ] = b.S[2];
            card[HC_NSV2] = b.nsv2; card[HC_R] = b.R; card[HC_MOI] = b.moi; card[HC_LAG] = b.lag;
        }
        sync();
        if (it == 0 && planet()) planet_constants();
        sync();

        const double hS0 = card[HC_SX], hS1 = card[HC_SY], hS2 = card[HC_SZ];
        const double hnsv2 = card[HC_NSV2];
        double at[3] = {0., 0., 0.}, af[3] = {0., 0., 0.}, ag[3] = {0., 0., 0.};
        double dt_[3] = {0., 0., 0.}, df[3] = {0., 0., 0.}, dg[3] = {0., 0., 0.};
        const int ncol = grk() ? 24 : (flat ? 12 : (tides ? 6 : 0));
        if (planet()) {
            for (int k = 0; k < ncol; ++k) X(k, lane) = 0.;
        }
        double* col = planet() ? &X(0, lane) : nullptr;
        if (planet()) {
            const double inv_m = 1. / b.m;
            if (tides && b.tk == POSI_EFFECT_ORBITING) {
                double o_s = P(PC_OS), osd = P(PC_OSD), term1 = P(PC_TERM1);
                const double o_p = P(PC_OP), opd = P(PC_OPD);
                if (dyn_host) {
                    // the host's dissipation factor for this planet, per evaluation
                    const double sh = host_sigma_for(x, y, z, hv[0], hv[1], hv[2]);
                    const double hR = card[HC_R];
                    o_s = 4.5 * powi<2>(b.m) * powi<10>(hR) * sh / powi<7>(d);
                    osd = o_s / d;
                    term1 = (b.m * b.m) * powi<10>(hR) * sh;
                }
                // radial component (constant_time_lag.rs:266-307)
                const double factor1 = -13.5 * vr / P(PC_D8);
                const double diss_pm = factor1 * P(PC_TERM2);
                const double radial = P(PC_CONS) + (diss_pm + factor1 * term1);
                // force (constant_time_lag.rs:309-332)
                const double factor3 = radial + (o_s + o_p) * vr / d;
                double F[3];
                F[0] = factor3 * x / d + osd * (hS1 * z - hS2 * y - hv[0]) + opd * (b.S[1] * z - b.S[2] * y - hv[0]);
                F[1] = factor3 * y / d + osd * (hS2 * x - hS0 * z - hv[1]) + opd * (b.S[2] * x - b.S[0] * z - hv[1]);
                F[2] = factor3 * z / d + osd * (hS0 * y - hS1 * x - hv[2]) + opd * (b.S[0] * y - b.S[1] * x - hv[2]);
                // tides/common.rs:312-370
                at[0] = inv_m * F[0]; at[1] = inv_m * F[1]; at[2] = inv_m * F[2];
                col[0 * G] = F[0]; col[1 * G] = F[1]; col[2 * G] = F[2];
                // torques (constant_time_lag.rs:171-204), tides/common.rs:223-261
                const double h0 = y * hv[2] - z * hv[1];
                const double h1 = z * hv[0] - x * hv[2];
                const double h2 = x * hv[1] - y * hv[0];
                const double inv_d = P(PC_INV_D);
                dt_[0] = -1.0 * (o_p * (d * b.S[0] - rs_p * x / d - inv_d * h0));
                dt_[1] = -1.0 * (o_p * (d * b.S[1] - rs_p * y / d - inv_d * h1));
                dt_[2] = -1.0 * (o_p * (d * b.S[2] - rs_p * z / d - inv_d * h2));
                col[3 * G] = -1.0 * (o_s * (d * hS0 - rs_s * x / d - inv_d * h0));
                col[4 * G] = -1.0 * (o_s * (d * hS1 - rs_s * y / d - inv_d * h1));
                col[5 * G] = -1.0 * (o_s * (d * hS2 - rs_s * z / d - inv_d * h2));
                record_tidal_internals(d, vr, o_p, diss_pm, x, y, z, hv[0], hv[1], hv[2], dt_[0], dt_[1], dt_[2]);
            }
            if (flat && b.fk == POSI_EFFECT_ORBITING) {
                // oblate_spheroid.rs:12-60
                const double d5 = P(PC_D5);
                const double fs = P(PC_MHK2F) * hnsv2 * P(PC_R5H) / 6.;
                const double ofs = -6. * fs * rs_s / (hnsv2 * d5);
                const double fp = P(PC_HMK2F) * b.nsv2 * P(PC_R5P) / 6.;
                const double ofp = -6. * fp * rs_p / (b.nsv2 * d5);
                const double radial = P(PC_N3D5) * (fp + fs) + P(PC_F15D7) * (fs * rs_s * rs_s / hnsv2 + fp * rs_p * rs_p / b.nsv2);
                // oblate_spheroid.rs:83-97, common.rs:203-237
                double F[3];
                F[0] = radial * x + ofp * b.S[0] + ofs * hS0;
                F[1] = radial * y + ofp * b.S[1] + ofs * hS1;
                F[2] = radial * z + ofp * b.S[2] + ofs * hS2;
                af[0] = inv_m * F[0]; af[1] = inv_m * F[1]; af[2] = inv_m * F[2];
                col[6 * G] = F[0]; col[7 * G] = F[1]; col[8 * G] = F[2];
                // oblate_spheroid.rs:62-81, common.rs:165-201
                df[0] = -1.0 * (ofp * (y * b.S[2] - z * b.S[1]));
                df[1] = -1.0 * (ofp * (z * b.S[0] - x * b.S[2]));
                df[2] = -1.0 * (ofp * (x * b.S[1] - y * b.S[0]));
                col[9 * G] = -1.0 * (ofs * (y * hS2 - z * hS1));
                col[10 * G] = -1.0 * (ofs * (z * hS0 - x * hS2));
                col[11 * G] = -1.0 * (ofs * (x * hS1 - y * hS0));
            }
            if (grk() && b.gk == POSI_EFFECT_ORBITING) {
                const double vr2 = powi<2>(vr);
                // first order (general_relativity.rs:187-239)
                const double radial1 = P(PC_A) * (P(PC_B) * nv2 - P(PC_C) - P(PC_DD) * vr2);
                const double ortho1 = P(PC_E) * vr * nv;
                double a1[3];
                a1[0] = radial1 * x / d + ortho1 * hv[0] / nv;
                a1[1] = radial1 * y / d + ortho1 * hv[1] / nv;
                a1[2] = radial1 * z / d + ortho1 * hv[2] / nv;
                // second order (:241-298)
                const double nv4 = powi<2>(nv2);
                const double vr4 = powi<2>(vr2);
                const double radial2 = P(PC_A) * (P(PC_T1) + P(PC_K2C) * nv4 + P(PC_K3C) * vr4 - P(PC_K4C) * vr2 * nv2 -
                                                  P(PC_K5C) * nv2 - P(PC_K6C) * vr2);
                const double ortho2 = P(PC_A05) * vr * (P(PC_P) * nv2 - P(PC_Q) - P(PC_R3) * vr2);
                double a2[3];
                a2[0] = radial2 * x / d + ortho2 * hv[0];
                a2[1] = radial2 * y / d + ortho2 * hv[1];
                a2[2] = radial2 * z / d + ortho2 * hv[2];
                // spin-orbit (:300-456)
                const double hmoi = card[HC_MOI], hm = card[HC_M];
                const double sL0 = hmoi * hS0, sL1 = hmoi * hS1, sL2 = hmoi * hS2;
                const double pL0 = b.moi * b.S[0], pL1 = b.moi * b.S[1], pL2 = b.moi * b.S[2];
                const double nn0 = P(PC_NN0), nn1 = P(PC_NN1), nn2 = P(PC_NN2);
                const double mfM = P(PC_MFM);
                const double msx = mfM * (pL0 / b.m - sL0 / hm);
                const double msy = mfM * (pL1 / b.m - sL1 / hm);
                const double msz = mfM * (pL2 / b.m - sL2 / hm);
                const double e1x = 6. * nn0 * ((nn1 * hv[2] - nn2 * hv[1]) * (2. * (sL0 + pL0) + msx));
                const double e1y = 6. * nn1 * ((nn2 * hv[0] - nn0 * hv[2]) * (2. * (sL1 + pL1) + msy));
                const double e1z = 6. * nn2 * ((nn0 * hv[1] - nn1 * hv[0]) * (2. * (sL2 + pL2) + msz));
                const double e7x = 7. * (sL0 + pL0) + 3. * msx;
                const double e7y = 7. * (sL1 + pL1) + 3. * msy;
                const double e7z = 7. * (sL2 + pL2) + 3. * msz;
                const double e2x = hv[1] * e7z - hv[2] * e7y;
                const double e2y = hv[2] * e7x - hv[0] * e7z;
                const double e2z = hv[0] * e7y - hv[1] * e7x;
                const double e3sx = 3. * (sL0 + pL0) + msx;
                const double e3sy = 3. * (sL1 + pL1) + msy;
                const double e3sz = 3. * (sL2 + pL2) + msz;
                const double e3x = 3. * vr * (nn1 * e3sz - nn2 * e3sy);
                const double e3y = 3. * vr * (nn2 * e3sx - nn0 * e3sz);
                const double e3z = 3. * vr * (nn0 * e3sy - nn1 * e3sx);
                double a3[3];
                a3[0] = kFA * (e1x - e2x + e3x);
                a3[1] = kFA * (e1y - e2y + e3y);
                a3[2] = kFA * (e1z - e2z + e3z);
                ag[0] = a1[0] + a2[0] + a3[0];
                ag[1] = a1[1] + a2[1] + a3[1];
                ag[2] = a1[2] + a2[2] + a3[2];
                const double mratio = P(PC_MRATIO);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    col[(12 + k) * G] = mratio * a1[k];
                    col[(15 + k) * G] = mratio * a2[k];
                    col[(18 + k) * G] = mratio * a3[k];
                }
                // Kidder 1995 eq. 2.4a / 2.4b
                const double mu = P(PC_MU), fm = P(PC_FM), fm2 = P(PC_FM2);
                const double lo0 = mu * (y * hv[2] - z * hv[1]);
                const double lo1 = mu * (z * hv[0] - x * hv[2]);
                const double lo2 = mu * (x * hv[1] - y * hv[0]);
                const double h1x = fm * (lo1 * sL2 - lo2 * sL1);
                const double h1y = fm * (lo2 * sL0 - lo0 * sL2);
                const double h1z = fm * (lo0 * sL1 - lo1 * sL0);
                const double h2x = pL1 * sL2 - pL2 * sL1;
                const double h2y = pL2 * sL0 - pL0 * sL2;
                const double h2z = pL0 * sL1 - pL1 * sL0;
                const double sp = nn0 * pL0 + nn1 * pL1 + nn2 * pL2;
                const double h3x = 3. * sp * (nn1 * sL2 - nn2 * sL1);
                const double h3y = 3. * sp * (nn2 * sL0 - nn0 * sL2);
                const double h3z = 3. * sp * (nn0 * sL1 - nn1 * sL0);
                col[21 * G] = kFA * (h1x - h2x + h3x);
                col[22 * G] = kFA * (h1y - h2y + h3y);
                col[23 * G] = kFA * (h1z - h2z + h3z);
                const double q1x = fm2 * (lo1 * pL2 - lo2 * pL1);
                const double q1y = fm2 * (lo2 * pL0 - lo0 * pL2);
                const double q1z = fm2 * (lo0 * pL1 - lo1 * pL0);
                const double q2x = sL1 * pL2 - sL2 * pL1;
                const double q2y = sL2 * pL0 - sL0 * pL2;
                const double q2z = sL0 * pL1 - sL1 * pL0;
                const double ss = nn0 * sL0 + nn1 * sL1 + nn2 * sL2;
                const double q3x = 3. * ss * (nn1 * pL2 - nn2 * pL1);
                const double q3y = 3. * ss * (nn2 * pL0 - nn0 * pL2);
                const double q3z = 3. * ss * (nn0 * pL1 - nn1 * pL0);
                dg[0] = kFA * (q1x - q2x + q3x);
                dg[1] = kFA * (q1y - q2y + q3y);
                dg[2] = kFA * (q1z - q2z + q3z);
            }
        }
        double ad[3] = {0., 0., 0.}, fdisk[3] = {0., 0., 0.};
        if (disk_on && planet() && b.dk == POSI_EFFECT_ORBITING) {
            disk_force(x, y, z, hv[0], hv[1], hv[2], d, nv2, fdisk);
            const double factor1 = 1. / b.m;
#pragma unroll
            for (int k = 0; k < 3; ++k) ad[k] = factor1 * fdisk[k];
        }
        // host back-reactions: fold the contribution columns in body order
        if (ncol > 0) colfold(0, ncol, nullptr, true, false);
        if (is_host) {
            const double factor2 = 1. / card[HC_M];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (tides) {
                    at[k] = -1.0 * factor2 * sums[k];
                    dt_[k] = sums[3 + k];
                    // the host's tides output and its (zero) heliocentric
                    // copies (tides/common.rs:202-261)
                    P(PC_TD_L0 + k) = sums[3 + k];
                    P(PC_TD_P0 + k) = 0.;
                    P(PC_TD_V0 + k) = 0.;
                    P(PC_TD_DIST) = 0.;
                    P(PC_TD_VR) = 0.;
                }
                if (flat) { af[k] = -1.0 * factor2 * sums[6 + k]; df[k] = sums[9 + k]; }
                if (grk()) {
                    ag[k] = -1.0 * sums[12 + k] + -1.0 * sums[15 + k] + -1.0 * sums[18 + k];
                    dg[k] = sums[21 + k];
                }
            }
        }
        if (disk_on) {
            // src/effects/disk.rs:205-268: the host's force is minus the sum
            // of the planets' forces, in body order
            sync();
            if (has) {
#pragma unroll
                for (int k = 0; k < 3; ++k) X(k, lane) = fdisk[k];
            }
            colfold(0, 3, nullptr, true, false);
            if (is_host) {
                const double factor2 = 1. / card[HC_M];
#pragma unroll
                for (int k = 0; k < 3; ++k) ad[k] = -1.0 * factor2 * sums[k];
            }
        }
        if (gr && !grk()) gr_nbody(ag);
        sync();
        if (has) {
            // universe.rs:580-614 (disabled effects contribute their zero outputs)
            if (spin_on && (tides || flat || grk() || wind)) {
                double dw[3];
                wind_torque(dw);
#pragma unroll
                for (int k = 0; k < 3; ++k) b.dl[k] = dt_[k] + df[k] + dg[k] + dw[k];
            }
            // universe.rs:540-567
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                double acc = 0.;
                if (tides) acc += at[k];
                if (disk) acc += ad[k];
                if (flat) acc += af[k];
                if (gr) acc += ag[k];
                b.aa[k] = acc;
            }
        }
    }
#else
    // FAST: six contribution columns per planet -- (m/M) a_add (the host's
    // additional acceleration is minus their sum) and the torque the planet
    // exerts on the host's spin (tides + flattening + GR).
    __device__ void additional_effects(const Dev& D, int it, bool evolution_now) {
        sync();
        if (is_host) {
            card[HC_VX] = b.v[0]; card[HC_VY] = b.v[1]; card[HC_VZ] = b.v[2];
            card[HC_SX] = b.S[0]; card[HC_SY] = b.S[1]; card[HC_SZ] = b.S[2];
        }
        if (lane == 0) isc[1] = 0;
        sync();
        double hv0 = 0., hv1 = 0., hv2 = 0., vr = 0., nv2 = 0., rs_s = 0., rs_p = 0.;
        const double x = P(PC_X), y = P(PC_Y), z = P(PC_Z);
        if (planet()) {
            hv0 = b.v[0] - card[HC_VX];
            hv1 = b.v[1] - card[HC_VY];
            hv2 = b.v[2] - card[HC_VZ];
            vr = P(PC_XD) * hv0 + P(PC_YD) * hv1 + P(PC_ZD) * hv2;
            nv2 = hv0 * hv0 + hv1 * hv1 + hv2 * hv2;
            rs_s = x * card[HC_SX] + y * card[HC_SY] + z * card[HC_SZ];
            rs_p = x * b.S[0] + y * b.S[1] + z * b.S[2];
        }
        spin_and_evolving(D, t, evolution_now);
        zero_inertia_check();
        if (fatal()) return;
        if (is_host) {
            card[HC_SX] = b.S[0]; card[HC_SY] = b.S[1]; card[HC_SZ] = b.S[2];
            card[HC_NSV2] = b.nsv2; card[HC_R] = b.R; card[HC_MOI] = b.moi; card[HC_LAG] = b.lag;
            card[HC_SLX] = b.moi * b.S[0]; card[HC_SLY] = b.moi * b.S[1]; card[HC_SLZ] = b.moi * b.S[2];
        }
        sync();
        if (it == 0 && planet() && !pc_reuse) planet_constants();
        sync();
        const double hS0 = card[HC_SX], hS1 = card[HC_SY], hS2 = card[HC_SZ];
        double aa0 = 0., aa1 = 0., aa2 = 0., dl0 = 0., dl1 = 0., dl2 = 0.;  // own outputs
        double th0 = 0., th1 = 0., th2 = 0.;                               // torque on the host
        if (planet()) {
            const double xd = P(PC_XD), yd = P(PC_YD), zd = P(PC_ZD);
            const double S0 = b.S[0], S1 = b.S[1], S2 = b.S[2];
            // r x v_rel (tidal torques, GR orbital angular momentum)
            const double h0 = y * hv2 - z * hv1;
            const double h1 = z * hv0 - x * hv2;
            const double h2 = x * hv1 - y * hv0;
            // S_p x r and S_h x r (tidal force, flattening torques)
            double cS0 = 0., cS1 = 0., cS2 = 0., chS0 = 0., chS1 = 0., chS2 = 0.;
            if ((tides && b.tk == POSI_EFFECT_ORBITING) || (flat && b.fk == POSI_EFFECT_ORBITING)) {
                cS0 = S1 * z - S2 * y; cS1 = S2 * x - S0 * z; cS2 = S0 * y - S1 * x;
                chS0 = hS1 * z - hS2 * y; chS1 = hS2 * x - hS0 * z; chS2 = hS0 * y - hS1 * x;
            }
            if (tides && b.tk == POSI_EFFECT_ORBITING) {
                double osd = P(PC_OSD), t12 = P(PC_T12), ospd = P(PC_OSPD), os_ = P(PC_OS), osdd = P(PC_OSDD);
                const double opd = P(PC_OPD);
                if (dyn_host) {
                    // the host's dissipation factor for this planet, per evaluation
                    const double sh = host_sigma_for(x, y, z, hv0, hv1, hv2);
                    const double id = P(PC_INV_D), id2 = id * id, id7 = id2 * id2 * id2 * id;
                    const double term1 = (b.m * b.m) * powi<10>(card[HC_R]) * sh;
                    os_ = 4.5 * term1 * id7;
                    osd = os_ * id;
                    ospd = (os_ + P(PC_OP)) * id;
                    osdd = os_ * P(PC_D);
                    t12 = term1 + P(PC_TERM2);
                }
                const double factor1 = vr * P(PC_C13);
                const double radial = P(PC_CONS) + factor1 * t12;
                const double factor3 = radial + ospd * vr;
                // osd (S_h x r - v) + opd (S_p x r - v)
                const double F0 = factor3 * xd + (osd * chS0 + opd * cS0) - ospd * hv0;
                const double F1 = factor3 * yd + (osd * chS1 + opd * cS1) - ospd * hv1;
                const double F2 = factor3 * zd + (osd * chS2 + opd * cS2) - ospd * hv2;
                aa0 += inv_m * F0; aa1 += inv_m * F1; aa2 += inv_m * F2;
                const double qp = P(PC_OP) * rs_p, qs = os_ * rs_s;
                const double opdd = P(PC_OPDD);
                dl0 -= opdd * S0 - qp * xd - opd * h0;
                dl1 -= opdd * S1 - qp * yd - opd * h1;
                dl2 -= opdd * S2 - qp * zd - opd * h2;
                th0 -= osdd * hS0 - qs * xd - osd * h0;
                th1 -= osdd * hS1 - qs * yd - osd * h1;
                th2 -= osdd * hS2 - qs * zd - osd * h2;
                record_tidal_internals(P(PC_D), vr, P(PC_OP), factor1 * P(PC_TERM2), x, y, z, hv0, hv1, hv2, dl0, dl1,
                                       dl2);
            }
            if (flat && b.fk == POSI_EFFECT_ORBITING) {
                const double cfs = P(PC_CFS), cfp = P(PC_CFP);
                const double ofs = P(PC_COFS) * rs_s, ofp = P(PC_COFP) * rs_p;
                const double radial = P(PC_N3D5) * (cfp * b.nsv2 + cfs * card[HC_NSV2]) +
                                      P(PC_F15D7) * (cfs * rs_s * rs_s + cfp * rs_p * rs_p);
                const double F0 = radial * x + ofp * S0 + ofs * hS0;
                const double F1 = radial * y + ofp * S1 + ofs * hS1;
                const double F2 = radial * z + ofp * S2 + ofs * hS2;
                aa0 += inv_m * F0; aa1 += inv_m * F1; aa2 += inv_m * F2;
                // -ofp (r x S_p), -ofs (r x S_h)
                dl0 += ofp * cS0; dl1 += ofp * cS1; dl2 += ofp * cS2;
                th0 += ofs * chS0; th1 += ofs * chS1; th2 += ofs * chS2;
            }
            if (grk() && b.gk == POSI_EFFECT_ORBITING) {
                const double vr2 = vr * vr;
                // first + second order (the combined constants of planet_constants)
                const double rad = P(PC_A) * (P(PC_GR0) + nv2 * (P(PC_GR1) + P(PC_K2C) * nv2 - P(PC_K4C) * vr2) +
                                              vr2 * (P(PC_GR2) + P(PC_K3C) * vr2));
                const double ort = vr * (P(PC_GO0) + P(PC_GO1) * nv2 + P(PC_GO2) * vr2);
                aa0 += rad * xd; aa0 += ort * hv0;
                aa1 += rad * yd; aa1 += ort * hv1;
                aa2 += rad * zd; aa2 += ort * hv2;
                // spin-orbit
                const double sL0 = card[HC_SLX], sL1 = card[HC_SLY], sL2 = card[HC_SLZ];
                const double pL0 = b.moi * S0, pL1 = b.moi * S1, pL2 = b.moi * S2;
                const double nn0 = xd, nn1 = yd, nn2 = zd;
                // ((m_h - m) / M) M (L_p / m - L_h / m_h) from the spins
                const double ma = P(PC_LMA), mb = P(PC_LMB);
                const double msx = ma * S0 - mb * sL0, msy = ma * S1 - mb * sL1, msz = ma * S2 - mb * sL2;
                const double t0 = sL0 + pL0, t1 = sL1 + pL1, t2 = sL2 + pL2;
                // (n x v)_k = (r x v)_k / d, the 6 n_k / d of planet_constants
                const double e1x = P(PC_C6NN0) * (h0 * (2. * t0 + msx));
                const double e1y = P(PC_C6NN1) * (h1 * (2. * t1 + msy));
                const double e1z = P(PC_C6NN2) * (h2 * (2. * t2 + msz));
                // -v x (7 t + 3 ms) + 3 v_r n x (3 t + ms) = a x t + 3 q x ms
                // with q = v_r n - v and a = 7 q + 2 v_r n
                const double q0 = vr * nn0 - hv0, q1 = vr * nn1 - hv1, q2 = vr * nn2 - hv2;
                const double vr2x = 2. * vr;
                const double a0 = 7. * q0 + vr2x * nn0, a1 = 7. * q1 + vr2x * nn1, a2 = 7. * q2 + vr2x * nn2;
                aa0 += kFA * (e1x + (a1 * t2 - a2 * t1) + 3. * (q1 * msz - q2 * msy));
                aa1 += kFA * (e1y + (a2 * t0 - a0 * t2) + 3. * (q2 * msx - q0 * msz));
                aa2 += kFA * (e1z + (a0 * t1 - a1 * t0) + 3. * (q0 * msy - q1 * msx));
                // Kidder 1995 eq. 2.4a / 2.4b.  With L_o = mu (r x v) the
                // torques are fm (L_o x S_h) - (L_p x S_h) + 3 (n.L_p) (n x S_h)
                // on the host and fm2 (L_o x L_p) + (L_p x S_h) + 3 (n.S_h) (n x L_p)
                // on the planet; the cross product is linear in its first
                // argument, so each is one cross product of a combined vector.
                const double sp3 = 3. * (nn0 * pL0 + nn1 * pL1 + nn2 * pL2);
                const double ss3 = 3. * (nn0 * sL0 + nn1 * sL1 + nn2 * sL2);
                const double fmu = P(PC_FMU), fm2mu = P(PC_FM2MU);
                const double ws0 = fmu * h0 - pL0 + sp3 * nn0;
                const double ws1 = fmu * h1 - pL1 + sp3 * nn1;
                const double ws2 = fmu * h2 - pL2 + sp3 * nn2;
                const double wp0 = fm2mu * h0 - sL0 + ss3 * nn0;
                const double wp1 = fm2mu * h1 - sL1 + ss3 * nn1;
                const double wp2 = fm2mu * h2 - sL2 + ss3 * nn2;
                th0 += kFA * (ws1 * sL2 - ws2 * sL1);
                th1 += kFA * (ws2 * sL0 - ws0 * sL2);
                th2 += kFA * (ws0 * sL1 - ws1 * sL0);
                dl0 += kFA * (wp1 * pL2 - wp2 * pL1);
                dl1 += kFA * (wp2 * pL0 - wp0 * pL2);
                dl2 += kFA * (wp0 * pL1 - wp1 * pL0);
            }
            if (disk_on && b.dk == POSI_EFFECT_ORBITING) {
                // the host's share enters through the (m/M) a columns below
                double F[3];
                disk_force(x, y, z, hv0, hv1, hv2, P(PC_D), nv2, F);
                aa0 += inv_m * F[0]; aa1 += inv_m * F[1]; aa2 += inv_m * F[2];
            }
            const double mr = P(PC_MRATIO);
            X(0, lane) = mr * aa0; X(1, lane) = mr * aa1; X(2, lane) = mr * aa2;
            X(3, lane) = th0; X(4, lane) = th1; X(5, lane) = th2;
        }
        if (tides || flat || grk() || disk_on) colfold(0, 6, nullptr, true, false);
        if (is_host && (tides || flat || grk() || disk_on)) {
            aa0 = -sums[0]; aa1 = -sums[1]; aa2 = -sums[2];
            dl0 = sums[3]; dl1 = sums[4]; dl2 = sums[5];
        }
        if (gr && !grk()) {
            // Anderson1975 / Newhall1983: every body's GR acceleration, the host's included
            double g[3] = {0., 0., 0.};
            gr_nbody(g);
            aa0 += g[0]; aa1 += g[1]; aa2 += g[2];
        }
        if (has) {
            if (spin_on && (tides || flat || grk() || wind)) {
                double dw[3];
                wind_torque(dw);
                b.dl[0] = dl0 + dw[0]; b.dl[1] = dl1 + dw[1]; b.dl[2] = dl2 + dw[2];
            }
            b.aa[0] = aa0; b.aa[1] = aa1; b.aa[2] = aa2;
        }
    }
#endif

    // ------------------------------------------------------------------
    // src/integrator/whfast.rs:322-466 implicit midpoint with Kahan sums
    // ------------------------------------------------------------------
    __device__ void integrate_velocity_dependent_forces(const Dev& D, double hdt, bool evolution, int rbase = -1) {
        // heliocentric positions are fixed during the iterations
        sync();
        if (is_host) { card[HC_PX] = b.r[0]; card[HC_PY] = b.r[1]; card[HC_PZ] = b.r[2];
                       card[HC_M] = b.m; card[HC_MG] = b.mg; card[HC_R] = b.R; card[HC_SIG] = b.sig;
                       card[HC_K2] = b.k2; card[HC_K2F] = b.k2f;
                       card[HC_DFAC] = b.diss_factor; card[HC_DSCALE] = b.diss_scale;
                       for (int k = 0; k < 6; ++k) card[HC_DINNER + k] = b.dk == POSI_EFFECT_CENTRAL ? b.disk_p[k] : 0.; }
        sync();
#if POSI_EXACT
        if (planet()) set_geometry(b.r[0] - card[HC_PX], b.r[1] - card[HC_PY], b.r[2] - card[HC_PZ]);
#else
        pc_reuse = pc_valid && !evo;
        if (planet() && !pc_reuse) set_geometry(b.r[0] - card[HC_PX], b.r[1] - card[HC_PY], b.r[2] - card[HC_PZ]);
#endif
        double ov[3], oL[3], fv[3], fL[3], dvc[3] = {0., 0., 0.}, dLc[3] = {0., 0., 0.};
#pragma unroll
        for (int k = 0; k < 3; ++k) { ov[k] = b.v[k]; oL[k] = b.L[k]; fv[k] = ov[k]; fL[k] = oL[k]; }
        bool converged = false;
        int iters = 0;
        for (int it = 0; it < kMIDPOINT_MAX; ++it) {
            iters = it + 1;
            double pv[3], pL[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) { pv[k] = fv[k]; pL[k] = fL[k]; }
            if (rbase >= 0) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    recw(rbase + 1 + 9 * it + k, b.v[k]);
                    recw(rbase + 4 + 9 * it + k, b.L[k]);
                    recw(rbase + 7 + 9 * it + k, b.S[k]);
                }
            }
            additional_effects(D, it, evolution && it == 0);
            if (fatal()) return;
            if (has) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    dvc[k] = hdt * b.aa[k] - b.ev[k];
                    fv[k] = ov[k] + dvc[k];
                    if (spin_on) {
                        dLc[k] = hdt * b.dl[k] - b.eL[k];
                        fL[k] = oL[k] + dLc[k];
                    }
                }
            }
            if (it >= kMIDPOINT_MIN - 1) {
                // whfast.rs:424-451
                sync();
                if (has) {
                    const double dvx = fv[0] - pv[0], dvy = fv[1] - pv[1], dvz = fv[2] - pv[2];
                    X(0, lane) = powi<2>(dvx) + powi<2>(dvy) + powi<2>(dvz);
                    X(1, lane) = powi<2>(fv[0]) + powi<2>(fv[1]) + powi<2>(fv[2]);
                    const double dsx = fL[0] - pL[0], dsy = fL[1] - pL[1], dsz = fL[2] - pL[2];
                    X(2, lane) = powi<2>(dsx) + powi<2>(dsy) + powi<2>(dsz);
                    X(3, lane) = powi<2>(fL[0]) + powi<2>(fL[1]) + powi<2>(fL[2]);
                }
                colfold(0, spin_on ? 4 : 2, nullptr, false, false);
                const double dv2 = sums[0], fv2 = sums[1];
                bool conv;
#if POSI_EXACT
                if (spin_on) conv = dv2 / fv2 < kDBL_EPSILON_2 && sums[2] / sums[3] < kDBL_EPSILON_2;
                else conv = dv2 / fv2 < kDBL_EPSILON_2;
#else
                // a / b < eps^2 as a < eps^2 b (b >= 0; b = 0 fails both ways)
                conv = dv2 < kDBL_EPSILON_2 * fv2 && (!spin_on || sums[2] < kDBL_EPSILON_2 * sums[3]);
#endif
                if (conv) { converged = true; break; }
            }
            if (has) {
#pragma unroll
                for (int k = 0; k < 3; ++k) {
#if POSI_EXACT
                    b.v[k] = 0.5 * (ov[k] + fv[k]);
                    if (spin_on) b.L[k] = 0.5 * (oL[k] + fL[k]);
#else
                    // the midpoint as the start plus half the increment
                    b.v[k] = ov[k] + 0.5 * dvc[k];
                    if (spin_on) b.L[k] = oL[k] + 0.5 * dLc[k];
#endif
                }
            }
        }
        mid_iters = iters;
        if (rbase >= 0) recw(rbase, (double)iters);
        if (!converged) status |= POSI_SYS_WARN_NONCONVERGED;
        if (has) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                b.v[k] = fv[k];
                b.ev[k] = (b.v[k] - ov[k]) - dvc[k];
                if (spin_on) {
                    b.L[k] = fL[k];
                    b.eL[k] = (b.L[k] - oL[k]) - dLc[k];
                }
            }
        }
    }

    // ------------------------------------------------------------------
    // Coordinate transforms (whfast.rs:881-1155)
    // ------------------------------------------------------------------
#if POSI_EXACT
    // slots: 0 m, 1 mg, 2-4 r, 5-7 v (inertial)
    __device__ void inertial_to_alternative() {
        sync();
        if (has) {
            X(0, lane) = b.m; X(1, lane) = b.mg;
            X(2, lane) = b.r[0]; X(3, lane) = b.r[1]; X(4, lane) = b.r[2];
            X(5, lane) = b.v[0]; X(6, lane) = b.v[1]; X(7, lane) = b.v[2];
        }
        sync();
        if (coords == POSI_JACOBI) {
            // :889-933, sequential in every lane
            const double m0 = X(0, host);
            double eta = m0;
            double s0 = eta * X(2, host), s1 = eta * X(3, host), s2 = eta * X(4, host);
            double u0 = eta * X(5, host), u1 = eta * X(6, host), u2 = eta * X(7, host);
            for (int j = 0; j < n; ++j) {
                if (j == host) continue;
                const double mj = X(0, j);
                const double ei = 1. / eta;
                eta += mj;
                const double pme = eta * ei;
                const double p0 = X(2, j) - s0 * ei, p1 = X(3, j) - s1 * ei, p2 = X(4, j) - s2 * ei;
                const double w0 = X(5, j) - u0 * ei, w1 = X(6, j) - u1 * ei, w2 = X(7, j) - u2 * ei;
                if (j == lane) {
                    b.am = mj; b.amg = X(1, j);
                    b.ap[0] = p0; b.ap[1] = p1; b.ap[2] = p2;
                    b.av[0] = w0; b.av[1] = w1; b.av[2] = w2;
                }
                s0 = s0 * pme + mj * p0; s1 = s1 * pme + mj * p1; s2 = s2 * pme + mj * p2;
                u0 = u0 * pme + mj * w0; u1 = u1 * pme + mj * w1; u2 = u2 * pme + mj * w2;
            }
            if (is_host) {
                const double mtot_i = 1. / eta;
                b.am = eta;
                b.ap[0] = s0 * mtot_i; b.ap[1] = s1 * mtot_i; b.ap[2] = s2 * mtot_i;
                b.av[0] = u0 * mtot_i; b.av[1] = u1 * mtot_i; b.av[2] = u2 * mtot_i;
            }
        } else {
            // :973-1023 -- sums over host first, then the others in order
            sync();
            if (has) {
                X(8, lane) = b.r[0] * b.m; X(9, lane) = b.r[1] * b.m; X(10, lane) = b.r[2] * b.m;
                X(11, lane) = b.v[0] * b.m; X(12, lane) = b.v[1] * b.m; X(13, lane) = b.v[2] * b.m;
                X(14, lane) = b.m; X(15, lane) = b.mg;
            }
            colfold(8, 8, nullptr, false, true);
            const double mtot = sums[6];
            const double st0 = sums[0] / mtot, st1 = sums[1] / mtot, st2 = sums[2] / mtot;
            const double sv0 = sums[3] / mtot, sv1 = sums[4] / mtot, sv2 = sums[5] / mtot;
            if (is_host) {
                b.am = mtot; b.amg = sums[7];
                b.ap[0] = st0; b.ap[1] = st1; b.ap[2] = st2;
                b.av[0] = sv0; b.av[1] = sv1; b.av[2] = sv2;
            } else if (has) {
                const double hr0 = X(2, host), hr1 = X(3, host), hr2 = X(4, host);
                b.ap[0] = b.r[0] - hr0; b.ap[1] = b.r[1] - hr1; b.ap[2] = b.r[2] - hr2;
                b.av[0] = b.v[0] - sv0; b.av[1] = b.v[1] - sv1; b.av[2] = b.v[2] - sv2;
                b.am = b.m; b.amg = b.mg;
                if (coords == POSI_WHDS) {
                    const double hm = X(0, host);
                    const double factor = (hm + b.m) / hm;
                    b.av[0] *= factor; b.av[1] *= factor; b.av[2] *= factor;
                }
            }
        }
        sync();
    }

    // slots: 0 m, 2-4 alt r, 5-7 alt v (host: barycentre)
    __device__ void alternative_to_inertial() {
        sync();
        if (has) {
            X(0, lane) = b.m;
            X(2, lane) = b.ap[0]; X(3, lane) = b.ap[1]; X(4, lane) = b.ap[2];
            X(5, lane) = b.av[0]; X(6, lane) = b.av[1]; X(7, lane) = b.av[2];
        }
        if (is_host) card[HC_AM] = b.am;
        sync();
        if (coords == POSI_JACOBI) {
            // :1034-1080, reverse order, sequential in every lane
            double eta = card[HC_AM];
            double s0 = eta * X(2, host), s1 = eta * X(3, host), s2 = eta * X(4, host);
            double u0 = eta * X(5, host), u1 = eta * X(6, host), u2 = eta * X(7, host);
            for (int j = n - 1; j >= 0; --j) {
                if (j == host) continue;
                const double mj = X(0, j);
                const double ei = 1. / eta;
                s0 = (s0 - mj * X(2, j)) * ei; s1 = (s1 - mj * X(3, j)) * ei; s2 = (s2 - mj * X(4, j)) * ei;
                u0 = (u0 - mj * X(5, j)) * ei; u1 = (u1 - mj * X(6, j)) * ei; u2 = (u2 - mj * X(7, j)) * ei;
                if (j == lane) {
                    b.r[0] = X(2, j) + s0; b.r[1] = X(3, j) + s1; b.r[2] = X(4, j) + s2;
                    b.v[0] = X(5, j) + u0; b.v[1] = X(6, j) + u1; b.v[2] = X(7, j) + u2;
                }
                eta -= mj;
                s0 *= eta; s1 *= eta; s2 *= eta;
                u0 *= eta; u1 *= eta; u2 *= eta;
            }
            if (is_host) {
                const double mtot_i = 1. / eta;
                b.r[0] = s0 * mtot_i; b.r[1] = s1 * mtot_i; b.r[2] = s2 * mtot_i;
                b.v[0] = u0 * mtot_i; b.v[1] = u1 * mtot_i; b.v[2] = u2 * mtot_i;
            }
        } else {
            // :1090-1155
            const double mtot = card[HC_AM];
            const double hm = X(0, host);
            const bool whds = coords == POSI_WHDS;
            sync();
            if (planet()) {
                X(8, lane) = -(b.ap[0] * b.m / mtot);
                X(9, lane) = -(b.ap[1] * b.m / mtot);
                X(10, lane) = -(b.ap[2] * b.m / mtot);
                const double factor = whds ? b.m / (hm + b.m) : b.m / hm;
                X(11, lane) = -(b.av[0] * factor);
                X(12, lane) = -(b.av[1] * factor);
                X(13, lane) = -(b.av[2] * factor);
            }
            double init[6];
            init[0] = X(2, host); init[1] = X(3, host); init[2] = X(4, host);
            init[3] = X(5, host); init[4] = X(6, host); init[5] = X(7, host);
            colfold(8, 6, init, true, false);
            const double sp0 = sums[0], sp1 = sums[1], sp2 = sums[2];
            if (is_host) {
                b.r[0] = sp0; b.r[1] = sp1; b.r[2] = sp2;
                b.v[0] = sums[3]; b.v[1] = sums[4]; b.v[2] = sums[5];
            } else if (has) {
                b.r[0] = b.ap[0] + sp0; b.r[1] = b.ap[1] + sp1; b.r[2] = b.ap[2] + sp2;
                if (whds) {
                    const double factor = (hm + b.m) / hm;
                    b.v[0] = b.av[0] / factor + init[3];
                    b.v[1] = b.av[1] / factor + init[4];
                    b.v[2] = b.av[2] / factor + init[5];
                } else {
                    b.v[0] = b.av[0] + init[3];
                    b.v[1] = b.av[1] + init[4];
                    b.v[2] = b.av[2] + init[5];
                }
            }
        }
        sync();
    }

    // :495-556
    __device__ void jump_step(double hdt) {
        if (coords == POSI_JACOBI) return;
        sync();
        if (is_host) card[HC_M] = b.m;
        const bool whds = coords == POSI_WHDS;
        sync();
        const double m0 = card[HC_M];
        if (planet()) {
            if (whds) {
                const double factor = m0 + b.m;
                X(8, lane) = b.m * b.av[0] / factor; X(9, lane) = b.m * b.av[1] / factor; X(10, lane) = b.m * b.av[2] / factor;
            } else {
                X(8, lane) = b.m * b.av[0]; X(9, lane) = b.m * b.av[1]; X(10, lane) = b.m * b.av[2];
            }
        }
        colfold(8, 3, nullptr, true, false);
        if (planet()) {
            if (whds) {
                const double factor = m0 + b.m;
                b.ap[0] += hdt * (sums[0] - (b.m * b.av[0] / factor));
                b.ap[1] += hdt * (sums[1] - (b.m * b.av[1] / factor));
                b.ap[2] += hdt * (sums[2] - (b.m * b.av[2] / factor));
            } else {
                b.ap[0] += hdt * sums[0] / m0;
                b.ap[1] += hdt * sums[1] / m0;
                b.ap[2] += hdt * sums[2] / m0;
            }
        }
        sync();
    }

    // :558-625 (Jacobi also :935-963 inertial_to_jacobi_acc)
    __device__ void interaction_step(double fdt) {
        if (coords == POSI_JACOBI) {
            sync();
            if (has) {
                X(0, lane) = b.m;
                X(2, lane) = b.a[0]; X(3, lane) = b.a[1]; X(4, lane) = b.a[2];
            }
            sync();
            double eta = X(0, host);
            double s0 = eta * X(2, host), s1 = eta * X(3, host), s2 = eta * X(4, host);
            double eta_own = 0.;
            int k_own = -1, k = 0;
            for (int j = 0; j < n; ++j) {
                if (j == host) continue;
                const double mj = X(0, j);
                const double ei = 1. / eta;
                eta += mj;
                const double pme = eta * ei;
                const double a0 = X(2, j) - s0 * ei, a1 = X(3, j) - s1 * ei, a2 = X(4, j) - s2 * ei;
                if (j == lane) { b.aacc[0] = a0; b.aacc[1] = a1; b.aacc[2] = a2; eta_own = eta; k_own = k; }
                s0 = s0 * pme + mj * a0; s1 = s1 * pme + mj * a1; s2 = s2 * pme + mj * a2;
                ++k;
            }
            if (is_host) {
                const double mtot_i = 1. / eta;
                b.aacc[0] = s0 * mtot_i; b.aacc[1] = s1 * mtot_i; b.aacc[2] = s2 * mtot_i;
            }
            if (planet()) {
                const double softening = 1e-12;
                b.av[0] += fdt * b.aacc[0];
                b.av[1] += fdt * b.aacc[1];
                b.av[2] += fdt * b.aacc[2];
                if (k_own > 0) {
                    const double rj2i = 1. / (powi<2>(b.ap[0]) + powi<2>(b.ap[1]) + powi<2>(b.ap[2]) + softening);
                    const double rji = sqrt(rj2i);
                    const double rj3im = rji * rj2i * kG * eta_own;
                    const double prefac = fdt * rj3im;
                    b.av[0] += prefac * b.ap[0];
                    b.av[1] += prefac * b.ap[1];
                    b.av[2] += prefac * b.ap[2];
                }
            }
            sync();
        } else if (coords == POSI_DEMOCRATIC_HELIOCENTRIC) {
            if (planet()) {
                b.av[0] += fdt * b.a[0]; b.av[1] += fdt * b.a[1]; b.av[2] += fdt * b.a[2];
            }
        } else {
            sync();
            if (is_host) card[HC_M] = b.m;
            sync();
            const double m0 = card[HC_M];
            if (planet()) {
                const double factor = m0 + b.m;
                b.av[0] += fdt * factor * b.a[0] / m0;
                b.av[1] += fdt * factor * b.a[1] / m0;
                b.av[2] += fdt * factor * b.a[2] / m0;
            }
            sync();
        }
    }
#else
    // FAST transforms: prefix / suffix scans over the lanes (bodies in index
    // order; the host, first in the Jacobi order, is added separately).
    __device__ void inertial_to_alternative() {
        if (coords == POSI_JACOBI) {
            const double own[6] = {planet() ? b.m * b.r[0] : 0., planet() ? b.m * b.r[1] : 0., planet() ? b.m * b.r[2] : 0.,
                                   planet() ? b.m * b.v[0] : 0., planet() ? b.m * b.v[1] : 0., planet() ? b.m * b.v[2] : 0.};
            const double hmv[6] = {b.m * b.r[0], b.m * b.r[1], b.m * b.r[2], b.m * b.v[0], b.m * b.v[1], b.m * b.v[2]};
            double res[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const double hk = gbcast(hmv[k], host);
                const double incl = gscan(own[k]);
                const double tot = hk + gbcast(incl, G - 1);
                if (is_host) res[k] = tot * inv_mtot;
                else res[k] = (k < 3 ? b.r[k] : b.v[k - 3]) - (hk + (incl - own[k])) * inv_eta_excl;
            }
            b.ap[0] = res[0]; b.ap[1] = res[1]; b.ap[2] = res[2];
            b.av[0] = res[3]; b.av[1] = res[4]; b.av[2] = res[5];
            b.am = is_host ? 1. / inv_mtot : b.m;
            b.amg = b.mg;
        } else {
            double bar[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) bar[k] = gsum(b.m * (k < 3 ? b.r[k] : b.v[k - 3])) * inv_mtot;
            const double hr0 = gbcast(b.r[0], host), hr1 = gbcast(b.r[1], host), hr2 = gbcast(b.r[2], host);
            if (is_host) {
                b.ap[0] = bar[0]; b.ap[1] = bar[1]; b.ap[2] = bar[2];
                b.av[0] = bar[3]; b.av[1] = bar[4]; b.av[2] = bar[5];
            } else {
                const double f = coords == POSI_WHDS ? whds_f : 1.;
                b.ap[0] = b.r[0] - hr0; b.ap[1] = b.r[1] - hr1; b.ap[2] = b.r[2] - hr2;
                b.av[0] = (b.v[0] - bar[3]) * f; b.av[1] = (b.v[1] - bar[4]) * f; b.av[2] = (b.v[2] - bar[5]) * f;
            }
            b.am = b.m;
            b.amg = b.mg;
        }
    }

    // with_v = false: positions only (the pair loop needs nothing else;
    // the velocities follow from the same alternative coordinates later)
    __device__ void alternative_to_inertial(bool with_v = true) {
        if (coords == POSI_JACOBI) {
            // R_(k-1) = R_total - sum_(i >= k) (m_i / eta_i) r'_i
            const int nk = with_v ? 6 : 3;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                if (k >= nk) break;
                const double a = k < 3 ? b.ap[k] : b.av[k - 3];
                const double own = jac_c * a;
                const double incl = gscan(own);
                const double tot = gbcast(incl, G - 1);
                const double R = gbcast(a, host);
                const double res = is_host ? R - tot : a + (R - (tot - incl + own));
                if (k < 3) b.r[k] = res; else b.v[k - 3] = res;
            }
        } else {
            const bool whds = coords == POSI_WHDS;
            const double w = whds ? whds_w : dh_w;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double sp = gsum(planet() ? b.ap[k] * b.m : 0.) * inv_mtot;
                const double R = gbcast(b.ap[k], host);
                const double rh = R - sp;
                b.r[k] = is_host ? rh : b.ap[k] + rh;
                if (with_v) {
                    const double sv = gsum(planet() ? b.av[k] * w : 0.);
                    const double V = gbcast(b.av[k], host);
                    b.v[k] = is_host ? V - sv : (whds ? b.av[k] / whds_f : b.av[k]) + V;
                }
            }
        }
    }

    __device__ void jump_step(double hdt) {
        if (coords == POSI_JACOBI) return;
        const bool whds = coords == POSI_WHDS;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double own = planet() ? b.av[k] * (whds ? whds_w : b.m) : 0.;
            const double p = gsum(own);
            if (planet()) b.ap[k] += whds ? hdt * (p - own) : hdt * p * inv_hm;
        }
    }

    __device__ void interaction_step(double fdt) {
        if (coords == POSI_JACOBI) {
            const double hmA[3] = {b.m * b.a[0], b.m * b.a[1], b.m * b.a[2]};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const double own = planet() ? b.m * b.a[k] : 0.;
                const double hk = gbcast(hmA[k], host);
                const double incl = gscan(own);
                b.aacc[k] = b.a[k] - (hk + (incl - own)) * inv_eta_excl;
            }
            if (planet()) {
                b.av[0] += fdt * b.aacc[0];
                b.av[1] += fdt * b.aacc[1];
                b.av[2] += fdt * b.aacc[2];
                if (!first_planet) {
                    const double r2 = b.ap[0] * b.ap[0] + b.ap[1] * b.ap[1] + b.ap[2] * b.ap[2] + 1e-12;
                    const double ri = rsqrt(r2);
                    const double prefac = fdt * (ri * ri * ri) * kG * eta_incl;
                    b.av[0] += prefac * b.ap[0];
                    b.av[1] += prefac * b.ap[1];
                    b.av[2] += prefac * b.ap[2];
                }
            }
        } else if (planet()) {
            const double f = coords == POSI_WHDS ? fdt * whds_f : fdt;
            b.av[0] += f * b.a[0]; b.av[1] += f * b.a[1]; b.av[2] += f * b.a[2];
        }
    }
#endif

    // :835-876
    __device__ static void stiefel_gs3(double beta, double x, double gs[4]) {
        const double x2 = powi<2>(x);
        double z = beta * x2;
        int nq = 0;
        // |z| > 0.1 on the bit patterns (the same decision, off the FP64 pipe)
        while (sq_gt(fabs(z), 0.1)) { z = z / 4.; nq += 1; }
        // 1/k!, k = 0..13
        const double if0 = 1., if1 = 1., if2 = 1. / 2., if3 = 1. / 6., if4 = 1. / 24., if5 = 1. / 120.,
                     if6 = 1. / 720., if7 = 1. / 5040., if8 = 1. / 40320., if9 = 1. / 362880.,
                     if10 = 1. / 3628800., if11 = 1. / 39916800., if12 = 1. / 479001600., if13 = 1. / 6227020800.;
        double c_odd = if13, c_even = if12;
        c_odd = if11 - z * c_odd; c_even = if10 - z * c_even;
        c_odd = if9 - z * c_odd; c_even = if8 - z * c_even;
        c_odd = if7 - z * c_odd; c_even = if6 - z * c_even;
        c_odd = if5 - z * c_odd; c_even = if4 - z * c_even;
        c_odd = if3 - z * c_odd; c_even = if2 - z * c_even;
        double cs3 = c_odd, cs2 = c_even;
        double cs1 = if1 - z * c_odd, cs0 = if0 - z * c_even;
        while (nq > 0) {
            cs3 = (cs2 + cs0 * cs3) * 0.25;
            cs2 = cs1 * cs1 * 0.5;
            cs1 = cs0 * cs1;
            cs0 = 2. * cs0 * cs0 - 1.;
            nq -= 1;
        }
        gs[0] = cs0;
        gs[1] = cs1 * x;
        gs[2] = cs2 * x2;
        gs[3] = cs3 * (x2 * x);
    }

    // :676-833
    __device__ void kepler_individual_step(double mass_g, double kdt) {
        const double p0 = b.ap[0], p1 = b.ap[1], p2 = b.ap[2];
        const double w0 = b.av[0], w1 = b.av[1], w2 = b.av[2];
#if POSI_EXACT
        const double r0 = sqrt(powi<2>(p0) + powi<2>(p1) + powi<2>(p2));
        const double r0i = 1. / r0;
#else
        const double r02 = powi<2>(p0) + powi<2>(p1) + powi<2>(p2);
        const double r0i = rsqrt(r02);
        const double r0 = r02 * r0i;
#endif
        const double v2 = powi<2>(w0) + powi<2>(w1) + powi<2>(w2);
        const double beta = 2. * mass_g * r0i - v2;
        const double eta0 = p0 * w0 + p1 * w1 + p2 * w2;
        const double zeta0 = mass_g - beta * r0;
        double x, gs[4];
        double invperiod = 0., x_per_period = 0.;
        bool xpp_nan;
#if POSI_EXACT
        if (beta > 0.) {
            const double sqrt_beta = sqrt(beta);
            invperiod = sqrt_beta * beta / (kTWO_PI * mass_g);
            x_per_period = kTWO_PI / sqrt_beta;
            xpp_nan = isnan(x_per_period);
            if (fabs(kdt) * invperiod > 1. && tw == 0) {
                status |= POSI_SYS_WARN_TIMESTEP;
                isc[2] = 1;
            }
            const double dtr0i = kdt * r0i;
            x = dtr0i * (1. - dtr0i * eta0 * 0.5 * r0i);
        } else {
            x = 0.;
            xpp_nan = true;
        }
#else
        // The period tests without their divisions (invperiod and
        // x_per_period are formed only on the rare bisection path below):
        // |dt| / P > 1 as |dt| sqrt(beta) beta > 2 pi GM, and the first
        // Newton step's jump against 1 % of 2 pi / sqrt(beta) as
        // |jump| sqrt(beta) > 0.02 pi.  The starting value is the series
        // inversion of r0 X + eta0 G2(X) + zeta0 G3(X) = dt to fourth order
        // in u = dt / r0 (G2 = X^2/2 - beta X^4/24, G3 = X^3/6 + ...): its
        // error is O(u^5), about 1e-5 relative at 2 pi dt / P = 0.2, so the
        // first Newton step already lands within 1e-8 and the loop stops
        // after one more evaluation (the reference's second-order value
        // needs three).
        if (beta > 0.) {
            xpp_nan = false;
            // |dt| sqrt(beta) beta > 2 pi GM squared (both sides positive):
            // sqrt(beta) only where the iterations need the period
            const double tpg = kTWO_PI * mass_g;
            if (kdt * kdt * (beta * beta * beta) > tpg * tpg && tw == 0) {
                status |= POSI_SYS_WARN_TIMESTEP;
                isc[2] = 1;
            }
            const double u = kdt * r0i;
            const double a2 = -0.5 * eta0 * r0i;
            const double a3 = (0.5 * eta0 * eta0 * r0i - zeta0 * (1. / 6.)) * r0i;
            const double a4 = -(eta0 * a3 + 0.5 * eta0 * a2 * a2 + 0.5 * zeta0 * a2 - eta0 * beta * (1. / 24.)) * r0i;
            x = u * (1. + u * (a2 + u * (a3 + u * a4)));
        } else {
            x = 0.;
            xpp_nan = true;
        }
#endif
        int converged = 0;
        double old_x = x;
        stiefel_gs3(beta, x, gs);
        double e = eta0 * gs[1] + zeta0 * gs[2];
        double ri;
#if POSI_EXACT
        ri = 1. / (r0 + e);
        x = ri * (x * e - eta0 * gs[2] - zeta0 * gs[3] + kdt);
        const bool jumped = !xpp_nan && fabs(x - old_x) > 0.01 * x_per_period;
#else
        // Halley's step from the series start of a bound orbit (cubic: a
        // start within 4e-6 of the root lands within 1e-17 of it, below the
        // rounding of x), then the G-functions at the new x by a second-order
        // Taylor step (dG0 = -beta G1, dG1 = G0, dG2 = G1, dG3 = G2 per unit
        // x).  Starts further off go on with the Newton iterations below; an
        // unbound orbit (no series start) takes Newton's first step.
        if (!(beta > 0.)) {
            ri = 1. / (r0 + e);
            x = ri * (x * e - eta0 * gs[2] - zeta0 * gs[3] + kdt);
        } else {
            const double fx = r0 * x + eta0 * gs[2] + zeta0 * gs[3] - kdt;
            const double fp = r0 + e;
            const double fpp = eta0 * gs[0] + zeta0 * gs[1];
            const double dx = (2. * fx * fp) / (2. * fp * fp - fx * fpp);
            x = x - dx;
            if (fabs(dx) <= 4e-6 * fabs(x)) {
                const double tt = -dx, th = 0.5 * tt * tt;
                const double g0 = gs[0], g1 = gs[1], g2 = gs[2], g3 = gs[3];
                gs[0] = g0 - beta * (g1 * tt + g0 * th);
                gs[1] = g1 + g0 * tt - beta * g1 * th;
                gs[2] = g2 + g1 * tt + g0 * th;
                gs[3] = g3 + g2 * tt + g1 * th;
                converged = 1;
                e = eta0 * gs[1] + zeta0 * gs[2];
                ri = 1. / (r0 + e);
            }
        }
        const bool jumped = !converged && !xpp_nan && fabs(x - old_x) * sqrt(beta) > 0.02 * kPI;
#endif
        if (converged) {
            // Halley's step converged
        } else if (jumped) {
            x = beta * kdt / mass_g;
            double prev_x[kNMAX_QUART + 1];
            for (int k = 0; k <= kNMAX_QUART; ++k) prev_x[k] = 0.;
            bool done = false;
            for (int n_lag = 1; n_lag < kNMAX_QUART && !done; ++n_lag) {
                stiefel_gs3(beta, x, gs);
                const double f = r0 * x + eta0 * gs[2] + zeta0 * gs[3] - kdt;
                const double fp = r0 + eta0 * gs[1] + zeta0 * gs[2];
                const double fpp = eta0 * gs[0] + zeta0 * gs[1];
                const double denom = fp + sqrt(fabs(16. * fp * fp - 20. * f * fpp));
                x = (x * denom - 5. * f) / denom;
                for (int k = 1; k < n_lag; ++k) {
                    if (x == prev_x[k]) { converged = 1; done = true; break; }
                }
                if (!done) prev_x[n_lag] = x;
            }
            e = eta0 * gs[1] + zeta0 * gs[2];
            ri = 1. / (r0 + e);
        } else {
            double old_x2;
            for (int k = 1; k < kNMAX_NEWT; ++k) {
                old_x2 = old_x;
                old_x = x;
                stiefel_gs3(beta, x, gs);
                e = eta0 * gs[1] + zeta0 * gs[2];
                ri = 1. / (r0 + e);
                x = ri * (x * e - eta0 * gs[2] - zeta0 * gs[3] + kdt);
#if POSI_EXACT
                if (x == old_x || x == old_x2) { converged = 1; break; }
#else
                // quadratic convergence: after a step below 1e-10 |x| the
                // root is off by the step's square times the contraction
                // (below 1e-20 relative), so stop there and move the G
                // functions to the new root by their derivatives (dG_n/dx =
                // G_(n-1), dG_0/dx = -beta G_1; second-order error about the
                // step's square): the drift stays a smooth function of x.
                if (x == old_x || x == old_x2) { converged = 1; break; }
                if (fabs(x - old_x) <= 1e-10 * fabs(x)) {
                    const double dx = x - old_x;
                    const double g0 = gs[0], g1 = gs[1], g2 = gs[2];
                    gs[0] = g0 - beta * g1 * dx;
                    gs[1] = g1 + g0 * dx;
                    gs[2] = g2 + g1 * dx;
                    gs[3] = gs[3] + g2 * dx;
                    e = eta0 * gs[1] + zeta0 * gs[2];
                    ri = 1. / (r0 + e);
                    converged = 1;
                    break;
                }
#endif
            }
        }
        if (converged == 0) {
            double x_min, x_max;
#if !POSI_EXACT
            if (beta > 0.) {
                const double sqrt_beta = sqrt(beta);
                invperiod = sqrt_beta * beta / (kTWO_PI * mass_g);
                x_per_period = kTWO_PI / sqrt_beta;
            }
#endif
            if (beta > 0.) {
                x_min = x_per_period * floor(kdt * invperiod);
                x_max = x_min + x_per_period;
            } else {
                const double h2 = r0 * r0 * v2 - eta0 * eta0;
                const double q = h2 / mass_g / (1. + sqrt(1. - h2 * beta / (mass_g * mass_g)));
                const double vq = sqrt(h2) / q;
                x_min = 1. / (vq + r0 / kdt);
                x_max = kdt / q;
            }
            x = (x_max + x_min) / 2.;
            for (int guard = 0;; ++guard) {
                stiefel_gs3(beta, x, gs);
                const double sres = r0 * x + eta0 * gs[2] + zeta0 * gs[3] - kdt;
                if (sres >= 0.) x_max = x; else x_min = x;
                x = (x_max + x_min) / 2.;
                if (fabs(x_max - x_min) / x_max <= 1e-15) break;
                if (guard >= kBISECTION_GUARD) { isc[3] = 1; break; }
            }
            e = eta0 * gs[1] + zeta0 * gs[2];
            ri = 1. / (r0 + e);
        }
        if (isnan(ri)) { ri = 0.; gs[1] = 0.; gs[2] = 0.; gs[3] = 0.; }
        kep_x = x;
        const double f = -mass_g * gs[2] * r0i;
        const double g = kdt - mass_g * gs[3];
        const double fd = -mass_g * gs[1] * r0i * ri;
        const double gd = -mass_g * gs[2] * ri;
        b.ap[0] += f * p0 + g * w0;
        b.ap[1] += f * p1 + g * w1;
        b.ap[2] += f * p2 + g * w2;
        b.av[0] += fd * p0 + gd * w0;
        b.av[1] += fd * p1 + gd * w1;
        b.av[2] += fd * p2 + gd * w2;
    }

    // :628-672
    __device__ void kepler_steps(double kdt) {
        sync();
#if POSI_EXACT
        if (has) X(1, lane) = b.amg;
#endif
        if (is_host) card[HC_MG] = b.mg;
        if (lane == 0) { isc[2] = 0; isc[3] = 0; }
        sync();
        if (planet()) {
            double gm;
            if (coords == POSI_JACOBI) {
#if POSI_EXACT
                gm = card[HC_MG];
                for (int j = 0; j < n; ++j) {
                    if (j == host) continue;
                    gm += X(1, j);
                    if (j == lane) break;
                }
#else
                gm = kep_gm;
#endif
            } else if (coords == POSI_DEMOCRATIC_HELIOCENTRIC) {
                gm = card[HC_MG];
            } else {
                gm = card[HC_MG] + b.amg;
            }
            kepler_individual_step(gm, kdt);
        }
        if (is_host) {
            b.ap[0] += kdt * b.av[0];
            b.ap[1] += kdt * b.av[1];
            b.ap[2] += kdt * b.av[2];
        }
        sync();
        if (isc[2]) tw += 1;
        if (isc[3]) set_fatal(POSI_SYS_BISECTION_LIMIT, 0, 0);
        sync();
    }

    // src/particles/universe.rs:198-303
    __device__ void gravity(const Dev& D, int ignore_terms) {
        sync();
        if (has) {
#if POSI_EXACT
            X(0, lane) = b.m;
#else
            X(0, lane) = gm_neg;
#endif
            X(2, lane) = b.r[0]; X(3, lane) = b.r[1]; X(4, lane) = b.r[2];
            X(5, lane) = b.R;
        }
        if (lane == 0) isc[0] = 0x7fffffff;
        sync();
        int code = 0, ev_pair = 0x7fffffff;
        double acc0 = 0., acc1 = 0., acc2 = 0.;
#if POSI_EXACT
        if (has) {
            const int i = lane, mm = host;
            const double* ro = D.roche + (int64_t)s * D.nmax * D.nmax + (int64_t)i * D.nmax;
            for (int j = 0; j < n; ++j) {
                if (i == j) continue;
                const double dx = b.r[0] - X(2, j);
                const double dy = b.r[1] - X(3, j);
                const double dz = b.r[2] - X(4, j);
                const double distance_2 = dx * dx + dy * dy + dz * dz;
                if (i < j && code == 0) {
                    if (distance_2 <= powi<2>(ro[j])) { code = POSI_SYS_ROCHE; ev_pair = i * 1024 + j; }
                    else if (distance_2 <= powi<2>(b.R + X(5, j))) { code = POSI_SYS_COLLISION; ev_pair = i * 1024 + j; }
                    else if (kMAX_DISTANCE_2 > 0. && i == mm && distance_2 > kMAX_DISTANCE_2) { code = POSI_SYS_EJECTED; ev_pair = i * 1024 + j; }
                }
                if (ignore_terms == 1 &&
                    ((i == mm && mm == 0 && j == 1) || (i == mm && mm > 0 && j == 0) ||
                     (j == mm && mm == 0 && i == 1) || (j == mm && mm > 0 && i == 0)))
                    continue;
                if (ignore_terms == 2 && (i == mm || j == mm)) continue;
                const double distance = sqrt(distance_2);
                const double prefact = -kG / (distance * distance * distance) * X(0, j);
                acc0 += prefact * dx;
                acc1 += prefact * dy;
                acc2 += prefact * dz;
            }
            if (code) atomicMin(&isc[0], ev_pair);
        }
#else
        // Each unordered pair once: in round r lane k takes the pair
        // (k, k + r mod n), adds its own term and hands the partner's to lane
        // k + r by a shuffle; in the round r = n / 2 (n even) both lanes of
        // a pair take their own term.  A lane checks the pairs it takes (the
        // lower one in the round r = n / 2) and keeps its least (i, j).
        {
            const int mm = host;
            const int64_t rbase = (int64_t)s * D.nmax * D.nmax;
            for (int r = 1; 2 * r <= n; ++r) {
                const bool hand = 2 * r < n;
                double rx = 0., ry = 0., rz = 0.;
                if (has) {
                    int j = lane + r;
                    if (j >= n) j -= n;
                    const double dx = b.r[0] - X(2, j);
                    const double dy = b.r[1] - X(3, j);
                    const double dz = b.r[2] - X(4, j);
                    const double distance_2 = dx * dx + dy * dy + dz * dz;
                    if (hand || lane < j) {
                        const int lo = lane < j ? lane : j, hi = lane < j ? j : lane;
                        const int pair = lo * 1024 + hi;
                        if (pair < ev_pair) {
                            const double ro = D.roche[rbase + (int64_t)lo * D.nmax + hi];
                            int c = 0;
                            // the same tests on the bit patterns (sq_le), off the FP64 pipe
                            if (sq_le(distance_2, powi<2>(ro))) c = POSI_SYS_ROCHE;
                            else if (sq_le(distance_2, powi<2>(b.R + X(5, j)))) c = POSI_SYS_COLLISION;
                            else if (kMAX_DISTANCE_2 > 0. && lo == mm && sq_gt(distance_2, kMAX_DISTANCE_2)) c = POSI_SYS_EJECTED;
                            if (c) { code = c; ev_pair = pair; }
                        }
                    }
                    const int i = lane;
                    const bool skip =
                        (ignore_terms == 1 &&
                         ((i == mm && mm == 0 && j == 1) || (i == mm && mm > 0 && j == 0) ||
                          (j == mm && mm == 0 && i == 1) || (j == mm && mm > 0 && i == 0))) ||
                        (ignore_terms == 2 && (i == mm || j == mm));
                    if (!skip) {
                        const double ri = rsqrt(distance_2);
                        const double ri3 = ri * ri * ri;
                        const double prefact = ri3 * X(0, j);
                        acc0 += prefact * dx;
                        acc1 += prefact * dy;
                        acc2 += prefact * dz;
                        if (hand) {
                            const double pk = -(ri3 * gm_neg);
                            rx = pk * dx; ry = pk * dy; rz = pk * dz;
                        }
                    }
                }
                if (hand) {
                    int src = lane - r;
                    if (src < 0) src += n;
                    if (!has) src = lane;
                    const double gx = __shfl_sync(mask, rx, src, G);
                    const double gy = __shfl_sync(mask, ry, src, G);
                    const double gz = __shfl_sync(mask, rz, src, G);
                    if (has) { acc0 += gx; acc1 += gy; acc2 += gz; }
                }
            }
            if (code) atomicMin(&isc[0], ev_pair);
        }
#endif
        sync();
        const int first = isc[0];
        if (first != 0x7fffffff) {
            // the reference panics at the first offending pair in (i, j) order,
            // before it stores any acceleration
#if POSI_EXACT
            if (has && lane == first / 1024) isc[4] = code;
#else
            if (has && code && ev_pair == first) isc[4] = code;
#endif
            sync();
            set_fatal(isc[4], first / 1024, first % 1024);
        } else if (has) {
            b.a[0] = acc0; b.a[1] = acc1; b.a[2] = acc2;
        }
        sync();
    }

    // ------------------------------------------------------------------
    // src/integrator/whfast.rs:235-305 one step; returns false once the
    // system is frozen (completed or fatal)
    // ------------------------------------------------------------------
    __device__ bool iterate(const Dev& D) {
        const bool first = last_hist < 0.;
        const bool hist_trig = last_hist + hist_period <= t;
        const bool rec_trig = last_rec + rec_period <= t;
        if (first || hist_trig) {
            spin_and_evolving(D, t, true);
            zero_inertia_check();
            if (fatal()) return false;
            if (tides) tides_denergy_dt();
            write_history_record(D);
            if (!first) last_hist += hist_period; else last_hist = 0.;
            n_hist += 1;
        }
        const int ignore = coords == POSI_JACOBI ? 1 : 2;
        if (rp) {
            recw(posi_rec::SV_TRIG, (first || hist_trig) ? 1. : 0.);
#pragma unroll
            for (int k = 0; k < 3; ++k) recw(posi_rec::SV_R0 + k, b.r[k]);
        }
        integrate_velocity_dependent_forces(D, half_dt, true, rp ? posi_rec::SV_H1 : -1);
        if (fatal()) return false;
#if !POSI_EXACT
        pc_valid = false;  // the drifts move every body
#endif
        inertial_to_alternative();
        if (rp)
#pragma unroll
            for (int k = 0; k < 3; ++k) { recw(posi_rec::SV_RJA + k, b.ap[k]); recw(posi_rec::SV_VJA + k, b.av[k]); }
        kepler_steps(half_dt);
        if (rp && planet()) recw(posi_rec::SV_X1, kep_x);
        jump_step(half_dt);
        if (rp)
#pragma unroll
            for (int k = 0; k < 3; ++k) { recw(posi_rec::SV_RJB + k, b.ap[k]); recw(posi_rec::SV_VJB + k, b.av[k]); }
#if POSI_EXACT
        alternative_to_inertial();
#else
        // the velocities only where the step stops here (the state of a
        // stopped system is the transformed one)
        alternative_to_inertial(false);
#endif
        if (rp)
#pragma unroll
            for (int k = 0; k < 3; ++k) recw(posi_rec::SV_RG + k, b.r[k]);
#if POSI_EXACT
        if (fatal()) return false;
        gravity(D, ignore);
        if (fatal()) return false;
#else
        if (!fatal()) gravity(D, ignore);
        if (fatal()) {
            alternative_to_inertial(true);
            return false;
        }
#endif
        interaction_step(dt);
        jump_step(half_dt);
        if (rp)
#pragma unroll
            for (int k = 0; k < 3; ++k) recw(posi_rec::SV_VJC + k, b.av[k]);
        kepler_steps(half_dt);
        if (rp && planet()) recw(posi_rec::SV_X2, kep_x);
        alternative_to_inertial();
        if (rp)
#pragma unroll
            for (int k = 0; k < 3; ++k) recw(posi_rec::SV_R2 + k, b.r[k]);
        if (fatal()) return false;
        integrate_velocity_dependent_forces(D, half_dt, false, rp ? posi_rec::SV_H2 : -1);
        if (fatal()) return false;
#if !POSI_EXACT
        pc_valid = true;
#endif
        t += dt;
        iteration += 1;
        if (lane == 0 && D.step_flags) D.step_flags[s] = (rec_trig || first ? 1 : 0) | ((first || hist_trig) ? 2 : 0);
        if (t + dt > time_limit) {
            status = (status & ~(int64_t)POSI_SYS_FATAL_MASK) | POSI_SYS_COMPLETED;
            return false;
        }
        return true;
    }
};

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
template <int G>
__device__ __forceinline__ bool group_setup(const Dev& D, int& sys, int& lane, unsigned& mask, double*& smem) {
    extern __shared__ double shm[];
    const int tid = threadIdx.x;
    const int gib = tid / G;
    lane = tid % G;
    const int gid = blockIdx.x * (blockDim.x / G) + gib;
    const int in_warp = (tid % 32) / G;
    mask = (G >= 32) ? 0xffffffffu : (((1u << G) - 1u) << (in_warp * G));
    smem = shm + (size_t)gib * (GroupSmem<G>::bytes / 8);
    if (gid >= D.n_list) return false;
    sys = D.list[gid];
    return true;
}

// n_steps WHFast steps of one system by its lane group (fewer when it
// completes or freezes), state loaded from and stored to the device view.
template <int G, bool REC>
__device__ __forceinline__ void run_steps(const Dev& D, int sys, int lane, unsigned mask, double* smem,
                                          int64_t n_steps) {
    Sys<G> S;
    S.load(D, sys, lane, mask, smem);
    S.rp = nullptr;
    S.rst = D.stride;
    int64_t k = 0;
    if (!S.fatal()) {
        for (; k < n_steps; ++k) {
            // with REC, step k's record (the adjoint re-integration of a chunk)
            if (REC) S.rp = D.rec + k * posi_rec::SV_COUNT * D.stride + (int64_t)sys * D.nmax + lane;
            if (!S.iterate(D)) {
                // a completed step keeps its record; an abandoned one does not
                if ((S.status & POSI_SYS_FATAL_MASK) == POSI_SYS_COMPLETED) ++k;
                break;
            }
        }
    }
    if (REC) {
        // steps the system did not take: "no step" records (the reverse
        // sweep passes them through unchanged)
        for (; k < n_steps; ++k) {
            S.rp = D.rec + k * posi_rec::SV_COUNT * D.stride + (int64_t)sys * D.nmax + lane;
            S.recw(posi_rec::SV_TRIG, -1.);
            S.recw(posi_rec::SV_H1, 0.);
            S.recw(posi_rec::SV_H2, 0.);
        }
    }
    S.store(D);
}

// Advance each listed system by up to n_steps steps (the plain path launches
// it with one system and n_steps = 1; the batched path with many systems and
// many steps per launch).
template <int G, bool REC = false>
__global__ void __launch_bounds__(128) whfast_steps_kernel(Dev D, int64_t n_steps) {
    int sys, lane;
    unsigned mask;
    double* smem;
    if (!group_setup<G>(D, sys, lane, mask, smem)) return;
    run_steps<G, REC>(D, sys, lane, mask, smem, n_steps);
}

// The same steps under a balanced schedule: one 256-thread block per SM,
// eight warps (two per SMSP).  Warp slot w = blockIdx.x * 8 + warp runs job
// slot_job[w] -- the systems list[job * (32 / G) ...] of one warp -- for
// slot_steps[w] steps; job -1 leaves the slot idle.  A warp alone on its
// SMSP runs its FP64 work faster than two sharing one, so the host gives the
// jobs in such slots more steps and rotates the jobs between sub-launches.
template <int G>
__global__ void __launch_bounds__(posi::kSchedBlockThreads, 1)
whfast_sched_kernel(Dev D, const int32_t* slot_job, const int32_t* slot_steps) {
    extern __shared__ double shm[];
    const int tid = threadIdx.x;
    const int slot = blockIdx.x * (posi::kSchedBlockThreads / 32) + (tid >> 5);
    const int job = slot_job[slot];
    const int64_t n_steps = slot_steps[slot];
    if (job < 0 || n_steps <= 0) return;   // the whole warp
    const int gib = tid / G;
    const int lane = tid % G;
    const int in_warp = (tid % 32) / G;
    const unsigned mask = (G >= 32) ? 0xffffffffu : (((1u << G) - 1u) << (in_warp * G));
    double* smem = shm + (size_t)gib * (GroupSmem<G>::bytes / 8);
    const int64_t li = (int64_t)job * (32 / G) + in_warp;
    if (li >= D.n_list) return;            // the whole group
    run_steps<G, false>(D, D.list[li], lane, mask, smem, n_steps);
}

// src/integrator/whfast.rs:226-233 (the Roche radii are computed on the host)
template <int G>
__global__ void __launch_bounds__(128) init_physical_kernel(Dev D) {
    int sys, lane;
    unsigned mask;
    double* smem;
    if (!group_setup<G>(D, sys, lane, mask, smem)) return;
    Sys<G> S;
    S.load(D, sys, lane, mask, smem);
    S.spin_and_evolving(D, S.t, true);
    S.zero_inertia_check();
    S.store(D);
}

// src/particles/universe.rs:198-303
template <int G>
__global__ void __launch_bounds__(128) gravity_kernel(Dev D, int ignore_terms) {
    int sys, lane;
    unsigned mask;
    double* smem;
    if (!group_setup<G>(D, sys, lane, mask, smem)) return;
    Sys<G> S;
    S.load(D, sys, lane, mask, smem);
    S.gravity(D, ignore_terms);
    S.store(D);
}

// src/particles/universe.rs:318-351 + :428-538 (one evaluation)
template <int G>
__global__ void __launch_bounds__(128) additional_effects_kernel(Dev D, double t_eval, int evolution, int dl, int acc) {
    int sys, lane;
    unsigned mask;
    double* smem;
    if (!group_setup<G>(D, sys, lane, mask, smem)) return;
    Sys<G> S;
    S.load(D, sys, lane, mask, smem);
    (void)acc;
    S.spin_on = dl != 0;
    S.t = t_eval;
    S.sync();
    if (S.is_host) { S.card[HC_PX] = S.b.r[0]; S.card[HC_PY] = S.b.r[1]; S.card[HC_PZ] = S.b.r[2];
                     S.card[HC_M] = S.b.m; S.card[HC_MG] = S.b.mg; S.card[HC_R] = S.b.R; S.card[HC_SIG] = S.b.sig;
                     S.card[HC_K2] = S.b.k2; S.card[HC_K2F] = S.b.k2f;
                     S.card[HC_DFAC] = S.b.diss_factor; S.card[HC_DSCALE] = S.b.diss_scale;
                     for (int k = 0; k < 6; ++k) S.card[HC_DINNER + k] = S.b.dk == POSI_EFFECT_CENTRAL ? S.b.disk_p[k] : 0.; }
    S.sync();
    if (S.planet()) S.set_geometry(S.b.r[0] - S.card[HC_PX], S.b.r[1] - S.card[HC_PY], S.b.r[2] - S.card[HC_PZ]);
    S.additional_effects(D, 0, evolution != 0);
    S.store(D);
}

}  // namespace POSI_NS
