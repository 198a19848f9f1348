// adjoint_device.cuh -- reverse-mode (adjoint) WHFast step on the device.
//
// Differentiates K steps of src/integrator/whfast.rs:235-305 (Jacobi
// coordinates; constant-time-lag tides, oblate flattening and Kidder 1995 GR;
// non-evolving bodies) with respect to the state at the start of the steps
// (positions, velocities, spin angular momenta, spins) and to every body's
// tidal dissipation factor and Love number.
//
// Mapping as in the forward kernels: one group of G lanes per system, lane j
// owns body j.  Two kernels work on a chunk of K steps that starts from a
// checkpoint of the forward run:
//
//   adj_record_kernel  runs the K steps forward and writes, for every step,
//                      the intermediates its vector-Jacobian product needs
//                      (midpoint iterates, Jacobi coordinates, Kepler roots,
//                      gravity positions) to a record in HBM;
//   adj_reverse_kernel walks the records backwards and applies each step's
//                      vector-Jacobian product to the adjoint state it keeps
//                      in registers.
//
// Derivatives are those of the computed map: the implicit-midpoint loop is
// reversed iteration by iteration with the iteration count of the forward
// pass; the Kepler root is differentiated implicitly (adjoint_blocks.cuh); the
// Kahan compensation terms carry no derivative (their exact-arithmetic value
// is zero); the per-planet effect blocks use the generated sweeps of
// adjoint_effects.cuh.
#pragma once
#include <cstdint>

#include "../../include/posidonius_gb300.h"
#include "adjoint_effects.cuh"
#include "adjoint_record.h"

namespace posi_adj {

// Adjoint state fields.
enum { LM_R = 0, LM_V = 3, LM_L = 6, LM_S = 9, LM_COUNT = 12 };
// Parameter gradients.
enum { GD_SIGMA = 0, GD_K2 = 1, GD_COUNT = 2 };
// Error flags per system (posi_adjoint_flag).
enum { AE_KEPLER = POSI_ADJ_KEPLER, AE_ZERO_INERTIA = POSI_ADJ_ZERO_INERTIA };

struct AdjDev {
    int64_t n_sys, nmax, stride;
    const double* bf;       // [POSI_BF_COUNT][stride] state at the chunk start (SoA)
    const int64_t* bi;      // [POSI_BI_COUNT][stride]
    const double* sf;       // [POSI_SF_COUNT][n_sys]
    const int64_t* si;      // [POSI_SI_COUNT][n_sys]
    const int32_t* list;    // systems to run; a negative entry is skipped
    int32_t n_list;
    double* tape;           // [k][SV_COUNT][stride] step records
    double* lam;            // [LM_COUNT][stride]
    double* grad;           // [GD_COUNT][stride]
    int32_t* err;           // [n_sys]
};

constexpr int kAXS = 16;    // exchange slots of G doubles
constexpr int kACARD = 48;  // host card
constexpr int kASUMS = 16;
template <int G>
struct AdjSmem {
    // exchange, card, sums, masses, inclusive eta by order position, body by
    // order position, 1 / eta and eta_(p-1) / eta_p by order position
    static constexpr int doubles = kAXS * G + kACARD + kASUMS + 5 * G;
    static constexpr int bytes = doubles * 8;
};

enum { AC_PX = 0, AC_PY, AC_PZ, AC_VX, AC_VY, AC_VZ, AC_H0, AC_H1, AC_H2, AC_Q0, AC_Q1, AC_Q2,
       AC_LA0, AC_LA1, AC_LA2, AC_LD0, AC_LD1, AC_LD2, AC_M, AC_MG, AC_R, AC_MOI, AC_SIG, AC_K2, AC_K2F, AC_K,
       AC_SKIP, AC_COUNT };
static_assert(AC_COUNT <= kACARD, "card");

// Per-step record (adjoint_record.h).
using namespace posi_rec;
static_assert(kMidMax == kMIDPOINT_MAX, "record layout");

struct SaveRef {
    double* p;
    int64_t st;
    __device__ __forceinline__ double& operator()(int f) const { return p[(int64_t)f * st]; }
};

template <int G>
struct AdjSys {
    int s, n, host, lane, q;
    unsigned mask;
    bool tides, flat, gr, has, is_host;
    double dt, half_dt, t, last_hist, hist_period;
    double *xs, *card, *sums, *gm, *geta, *gord, *gieta, *gci;
    // own body constants
    double m, mg, R, moi, sig, k2, k2f, mr, kep_gm, eta_q, eta_prev, M, inv_moi;
    double iM, i_eta_prev, i_m, i_gmh;  // reciprocals of the Jacobi transforms' divisors
    int tk, fk, gk;
    // state
    double r[3], v[3], L[3], S[3], ev[3], eL[3];
    int32_t errf;

    __device__ __forceinline__ void sync() const { __syncwarp(mask); }
    __device__ __forceinline__ double& X(int slot, int j) const { return xs[slot * G + j]; }
    __device__ __forceinline__ bool planet() const { return has && !is_host; }
    __device__ __forceinline__ int ord(int k) const { return (int)gord[k]; }

    // sums[c] = sum over the non-host bodies of X(base + c, j)
    __device__ void colsum(int base, int ncol) {
        sync();
        for (int c = lane; c < ncol; c += G) {
            double acc = 0.;
            for (int j = 0; j < n; ++j)
                if (j != host) acc += X(base + c, j);
            sums[c] = acc;
        }
        sync();
    }

    __device__ void setup(const AdjDev& D, int sys, int lane_, unsigned mask_, double* smem) {
        s = sys;
        lane = lane_;
        mask = mask_;
        xs = smem;
        card = xs + kAXS * G;
        sums = card + kACARD;
        gm = sums + kASUMS;
        geta = gm + G;
        gord = geta + G;
        gieta = gord + G;
        gci = gieta + G;
        const int64_t ns = D.n_sys;
        n = (int)D.si[(int64_t)POSI_SI_N * ns + s];
        host = (int)D.si[(int64_t)POSI_SI_HOST * ns + s];
        tides = D.si[(int64_t)POSI_SI_TIDES * ns + s] != 0;
        flat = D.si[(int64_t)POSI_SI_FLAT * ns + s] != 0;
        gr = D.si[(int64_t)POSI_SI_GR * ns + s] != 0;
        dt = D.sf[(int64_t)POSI_SF_DT * ns + s];
        half_dt = D.sf[(int64_t)POSI_SF_HALF_DT * ns + s];
        t = D.sf[(int64_t)POSI_SF_TIME * ns + s];
        last_hist = D.sf[(int64_t)POSI_SF_LAST_HIST * ns + s];
        hist_period = D.sf[(int64_t)POSI_SF_HIST_PERIOD * ns + s];
        has = lane < n;
        is_host = lane == host;
        errf = 0;
        const int64_t st = D.stride;
        const int64_t k = (int64_t)s * D.nmax + lane;
        m = mg = R = moi = sig = k2 = k2f = inv_moi = 0.;
        tk = fk = gk = 0;
        if (has) {
            const double* F = D.bf + k;
            m = F[POSI_BF_MASS * st];
            mg = F[POSI_BF_MASS_G * st];
            R = F[POSI_BF_RADIUS * st];
            moi = F[POSI_BF_MOI * st];
            sig = F[POSI_BF_SIGMA * st];
            k2 = F[POSI_BF_K2 * st];
            k2f = F[POSI_BF_K2F * st];
            inv_moi = moi != 0. ? 1. / moi : 0.;
            tk = (int)D.bi[POSI_BI_TIDES_KIND * st + k];
            fk = (int)D.bi[POSI_BI_FLAT_KIND * st + k];
            gk = (int)D.bi[POSI_BI_GR_KIND * st + k];
        }
        // masses, Jacobi order (host first, then the others in index order)
        sync();
        gm[lane] = m;
        q = !has ? -1 : (is_host ? 0 : (lane < host ? lane + 1 : lane));
        if (has) gord[q] = (double)lane;
        sync();
        double acc = 0., acc_g = 0.;
        for (int p = 0; p < n; ++p) {
            const int j = ord(p);
            acc += gm[j];
            if (lane == 0) geta[p] = acc;
        }
        (void)acc_g;
        sync();
        M = geta[n - 1];
        eta_q = has ? geta[q] : 0.;
        eta_prev = (has && q > 0) ? geta[q - 1] : 0.;
        if (lane < n) {
            gieta[lane] = 1. / geta[lane];
            gci[lane] = lane > 0 ? geta[lane - 1] / geta[lane] : 0.;
        }
        iM = 1. / M;
        i_eta_prev = eta_prev != 0. ? 1. / eta_prev : 0.;
        i_m = has ? 1. / m : 0.;
        i_gmh = 1. / gm[host];
        // Kepler GM: host mass_g plus the mass_g of the bodies up to this one in Jacobi order
        sync();
        X(0, lane) = mg;
        sync();
        kep_gm = 0.;
        if (planet()) {
            kep_gm = X(0, host);
            for (int p = 1; p <= q; ++p) kep_gm += X(0, ord(p));
        }
        sync();
        if (is_host) {
            card[AC_M] = m; card[AC_MG] = mg; card[AC_R] = R; card[AC_MOI] = moi;
            card[AC_SIG] = sig; card[AC_K2] = k2; card[AC_K2F] = k2f;
        }
        sync();
        mr = planet() ? m / card[AC_M] : 0.;
    }

    __device__ void load_state(const double* F, int64_t st) {
        for (int c = 0; c < 3; ++c) {
            r[c] = F[(POSI_BF_PX + c) * st];
            v[c] = F[(POSI_BF_VX + c) * st];
            L[c] = F[(POSI_BF_LX + c) * st];
            S[c] = F[(POSI_BF_SX + c) * st];
            ev[c] = F[(POSI_BF_EVX + c) * st];
            eL[c] = F[(POSI_BF_ELX + c) * st];
        }
    }
    __device__ __forceinline__ void spin_of(const double Lc[3], double out[3]) {
        if (has && moi != 0.) {
            const double im = inv_moi;
            out[0] = Lc[0] * im; out[1] = Lc[1] * im; out[2] = Lc[2] * im;
        } else {
            out[0] = out[1] = out[2] = 0.;
            if (has) errf |= AE_ZERO_INERTIA;
        }
    }

    // ---- additional effects (src/particles/universe.rs:428-538) ----
    // Per-planet block values fixed during a half kick (the heliocentric
    // position and the tidal parameters), from the host card.
    struct Pre {
        double t[adj_tides_NPRE], f[adj_flat_NPRE], g[adj_gr_NPRE];
    };
    __device__ __forceinline__ bool tides_on() const { return tides && tk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool flat_on() const { return flat && fk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool gr_on() const { return gr && gk == POSI_EFFECT_ORBITING; }

    __device__ __forceinline__ void helio(const double pos[3], double x[3]) const {
        x[0] = pos[0] - card[AC_PX]; x[1] = pos[1] - card[AC_PY]; x[2] = pos[2] - card[AC_PZ];
    }
    __device__ void pre_fwd(const double pos[3], Pre& pr) const {
        if (!planet()) return;
        double x[3];
        helio(pos, x);
        const double hm = card[AC_M], hR = card[AC_R], hmg = card[AC_MG], hmoi = card[AC_MOI], hk2f = card[AC_K2F];
        if (tides_on()) adj_tides_pre(x[0], x[1], x[2], sig, card[AC_SIG], k2, card[AC_K2], R, hR, hm, m, pr.t);
        if (flat_on()) adj_flat_pre(x[0], x[1], x[2], R, hR, hk2f, hm, k2f, m, pr.f);
        if (gr_on()) adj_gr_pre(x[0], x[1], x[2], hm, hmg, hmoi, m, mg, moi, pr.g);
    }

    // One evaluation: spins Sc = Lc / I, the r.Omega products from Sp;
    // outputs a_add, dL/dt.
    __device__ void effects_fwd(const Pre& pr, const double vc[3], const double Lc[3], const double Sp[3], double a[3],
                                double dl[3], double Sc[3]) {
        spin_of(Lc, Sc);
        sync();
        if (is_host) {
            card[AC_VX] = vc[0]; card[AC_VY] = vc[1]; card[AC_VZ] = vc[2];
            card[AC_H0] = Sc[0]; card[AC_H1] = Sc[1]; card[AC_H2] = Sc[2];
            card[AC_Q0] = Sp[0]; card[AC_Q1] = Sp[1]; card[AC_Q2] = Sp[2];
        }
        sync();
        a[0] = a[1] = a[2] = 0.;
        dl[0] = dl[1] = dl[2] = 0.;
        double th[3] = {0., 0., 0.};
        if (planet()) {
            const double h0 = vc[0] - card[AC_VX], h1 = vc[1] - card[AC_VY], h2 = vc[2] - card[AC_VZ];
            const double H0 = card[AC_H0], H1 = card[AC_H1], H2 = card[AC_H2];
            const double Q0 = card[AC_Q0], Q1 = card[AC_Q1], Q2 = card[AC_Q2];
            const double hm = card[AC_M], hR = card[AC_R], hmg = card[AC_MG], hmoi = card[AC_MOI],
                         hk2f = card[AC_K2F];
            double out[9];
            if (tides_on()) {
                adj_tides_iter(pr.t, h0, h1, h2, Sc[0], Sc[1], Sc[2], H0, H1, H2, Sp[0], Sp[1], Sp[2], Q0, Q1, Q2, R, hR,
                               hm, m, out);
                for (int c = 0; c < 3; ++c) { a[c] += out[c]; dl[c] += out[3 + c]; th[c] += out[6 + c]; }
            }
            if (flat_on()) {
                adj_flat_iter(pr.f, h0, h1, h2, Sc[0], Sc[1], Sc[2], H0, H1, H2, Sp[0], Sp[1], Sp[2], Q0, Q1, Q2, R, hR,
                              hk2f, hm, k2f, m, out);
                for (int c = 0; c < 3; ++c) { a[c] += out[c]; dl[c] += out[3 + c]; th[c] += out[6 + c]; }
            }
            if (gr_on()) {
                adj_gr_iter(pr.g, h0, h1, h2, Sc[0], Sc[1], Sc[2], H0, H1, H2, Sp[0], Sp[1], Sp[2], Q0, Q1, Q2, hm, hmg,
                            hmoi, m, mg, moi, out);
                for (int c = 0; c < 3; ++c) { a[c] += out[c]; dl[c] += out[3 + c]; th[c] += out[6 + c]; }
            }
            for (int c = 0; c < 3; ++c) {
                X(c, lane) = mr * a[c];
                X(3 + c, lane) = th[c];
            }
        }
        colsum(0, 6);
        if (is_host) {
            for (int c = 0; c < 3; ++c) { a[c] = -sums[c]; dl[c] = sums[3 + c]; }
        }
        sync();
    }

    // Bpre: adjoints of the pre values, accumulated over the iterations.
    struct Bpre {
        double t[adj_tides_NPRE], f[adj_flat_NPRE], g[adj_gr_NPRE];
        __device__ void zero() {
            for (int k = 0; k < adj_tides_NPRE; ++k) t[k] = 0.;
            for (int k = 0; k < adj_flat_NPRE; ++k) f[k] = 0.;
            for (int k = 0; k < adj_gr_NPRE; ++k) g[k] = 0.;
        }
    };

    // VJP of one effects_fwd evaluation: adjoints la, ld of (a, dl) in;
    // adjoints of vc, Sc, Sp out (assigned); the pre adjoints accumulated.
    __device__ void effects_vjp(const Pre& pr, Bpre& bp, const double vc[3], const double Sc[3], const double Sp[3],
                                const double la[3], const double ld[3], double lvc[3], double lSc[3], double lSp[3]) {
        sync();
        if (is_host) {
            card[AC_VX] = vc[0]; card[AC_VY] = vc[1]; card[AC_VZ] = vc[2];
            card[AC_H0] = Sc[0]; card[AC_H1] = Sc[1]; card[AC_H2] = Sc[2];
            card[AC_Q0] = Sp[0]; card[AC_Q1] = Sp[1]; card[AC_Q2] = Sp[2];
            card[AC_LA0] = la[0]; card[AC_LA1] = la[1]; card[AC_LA2] = la[2];
            card[AC_LD0] = ld[0]; card[AC_LD1] = ld[1]; card[AC_LD2] = ld[2];
        }
        sync();
        for (int c = 0; c < 3; ++c) lvc[c] = lSc[c] = lSp[c] = 0.;
        if (planet()) {
            const double h0 = vc[0] - card[AC_VX], h1 = vc[1] - card[AC_VY], h2 = vc[2] - card[AC_VZ];
            const double H0 = card[AC_H0], H1 = card[AC_H1], H2 = card[AC_H2];
            const double Q0 = card[AC_Q0], Q1 = card[AC_Q1], Q2 = card[AC_Q2];
            const double hm = card[AC_M], hR = card[AC_R], hmg = card[AC_MG], hmoi = card[AC_MOI],
                         hk2f = card[AC_K2F];
            double bout[9], bin[15];
            for (int c = 0; c < 3; ++c) {
                bout[c] = la[c] - mr * card[AC_LA0 + c];
                bout[3 + c] = ld[c];
                bout[6 + c] = card[AC_LD0 + c];
            }
            for (int k = 0; k < 15; ++k) bin[k] = 0.;
            if (tides_on())
                adj_tides_iter_vjp(pr.t, h0, h1, h2, Sc[0], Sc[1], Sc[2], H0, H1, H2, Sp[0], Sp[1], Sp[2], Q0, Q1, Q2, R,
                                   hR, hm, m, bout, bin, bp.t);
            if (flat_on())
                adj_flat_iter_vjp(pr.f, h0, h1, h2, Sc[0], Sc[1], Sc[2], H0, H1, H2, Sp[0], Sp[1], Sp[2], Q0, Q1, Q2, R,
                                  hR, hk2f, hm, k2f, m, bout, bin, bp.f);
            if (gr_on())
                adj_gr_iter_vjp(pr.g, h0, h1, h2, Sc[0], Sc[1], Sc[2], H0, H1, H2, Sp[0], Sp[1], Sp[2], Q0, Q1, Q2, hm,
                                hmg, hmoi, m, mg, moi, bout, bin, bp.g);
            for (int c = 0; c < 3; ++c) {
                lvc[c] = bin[c];
                lSc[c] = bin[3 + c];
                lSp[c] = bin[9 + c];
                X(c, lane) = -bin[c];
                X(3 + c, lane) = bin[6 + c];
                X(6 + c, lane) = bin[12 + c];
            }
        }
        colsum(0, 9);
        if (is_host) {
            for (int c = 0; c < 3; ++c) {
                lvc[c] = sums[c];
                lSc[c] = sums[3 + c];
                lSp[c] = sums[6 + c];
            }
        }
        sync();
    }

    // VJP of the pre values of a half kick: position adjoint and parameter
    // gradients accumulated (the host's from the sums over its planets).
    __device__ void pre_vjp(const double pos[3], const Bpre& bp, double lpos[3], double& gsig, double& gk2) {
        sync();
        double bin[7] = {0., 0., 0., 0., 0., 0., 0.};
        if (planet()) {
            double x[3];
            helio(pos, x);
            const double hm = card[AC_M], hR = card[AC_R], hmg = card[AC_MG], hmoi = card[AC_MOI],
                         hk2f = card[AC_K2F];
            if (tides_on())
                adj_tides_pre_vjp(x[0], x[1], x[2], sig, card[AC_SIG], k2, card[AC_K2], R, hR, hm, m, bp.t, bin);
            if (flat_on()) adj_flat_pre_vjp(x[0], x[1], x[2], R, hR, hk2f, hm, k2f, m, bp.f, bin);
            if (gr_on()) adj_gr_pre_vjp(x[0], x[1], x[2], hm, hmg, hmoi, m, mg, moi, bp.g, bin);
            for (int c = 0; c < 3; ++c) {
                lpos[c] += bin[c];
                X(c, lane) = -bin[c];
            }
            gsig += bin[3];
            gk2 += bin[5];
            X(3, lane) = bin[4];
            X(4, lane) = bin[6];
        }
        colsum(0, 5);
        if (is_host) {
            for (int c = 0; c < 3; ++c) lpos[c] += sums[c];
            gsig += sums[3];
            gk2 += sums[4];
        }
        sync();
    }

    // src/integrator/whfast.rs:322-466 with the iterates saved for the VJP.
    __device__ void midpoint_fwd(double hdt, const SaveRef& sv, int base, bool save) {
        sync();
        if (is_host) { card[AC_PX] = r[0]; card[AC_PY] = r[1]; card[AC_PZ] = r[2]; }
        sync();
        Pre pr;
        pre_fwd(r, pr);
        double v0[3], L0[3], vc[3], Lc[3], Sp[3], vf[3], Lf[3], pv[3], pL[3], a[3], dl[3], Sc[3];
        double dvc[3] = {0., 0., 0.}, dLc[3] = {0., 0., 0.};
        for (int c = 0; c < 3; ++c) {
            v0[c] = v[c]; L0[c] = L[c]; vc[c] = v[c]; Lc[c] = L[c]; Sp[c] = S[c]; vf[c] = v[c]; Lf[c] = L[c];
        }
        int K = kMIDPOINT_MAX;
        for (int i = 0; i < kMIDPOINT_MAX; ++i) {
            for (int c = 0; c < 3; ++c) {
                if (save) {
                    sv(base + 1 + 9 * i + c) = vc[c];
                    sv(base + 4 + 9 * i + c) = Lc[c];
                    sv(base + 7 + 9 * i + c) = Sp[c];
                }
                pv[c] = vf[c]; pL[c] = Lf[c];
            }
            effects_fwd(pr, vc, Lc, Sp, a, dl, Sc);
            for (int c = 0; c < 3; ++c) {
                dvc[c] = hdt * a[c] - ev[c];
                vf[c] = v0[c] + dvc[c];
                dLc[c] = hdt * dl[c] - eL[c];
                Lf[c] = L0[c] + dLc[c];
            }
            if (i >= kMIDPOINT_MIN - 1) {
                sync();
                if (has) {
                    double d0 = 0., f0 = 0., d1 = 0., f1 = 0.;
                    for (int c = 0; c < 3; ++c) {
                        d0 += (vf[c] - pv[c]) * (vf[c] - pv[c]);
                        f0 += vf[c] * vf[c];
                        d1 += (Lf[c] - pL[c]) * (Lf[c] - pL[c]);
                        f1 += Lf[c] * Lf[c];
                    }
                    X(0, lane) = d0; X(1, lane) = f0; X(2, lane) = d1; X(3, lane) = f1;
                }
                sync();
                double s0 = 0., s1 = 0., s2 = 0., s3 = 0.;
                for (int j = 0; j < n; ++j) { s0 += X(0, j); s1 += X(1, j); s2 += X(2, j); s3 += X(3, j); }
                sync();
                // a / b < eps^2 as a < eps^2 b, the FAST kernel's form of the test
                if (s0 < kDBL_EPSILON_2 * s1 && (s3 == 0. || s2 < kDBL_EPSILON_2 * s3)) { K = i + 1; break; }
            }
            for (int c = 0; c < 3; ++c) {
                vc[c] = 0.5 * (v0[c] + vf[c]);
                Lc[c] = 0.5 * (L0[c] + Lf[c]);
                Sp[c] = Sc[c];
            }
        }
        if (save) sv(base) = (double)K;
        for (int c = 0; c < 3; ++c) {
            v[c] = vf[c];
            L[c] = Lf[c];
            S[c] = Sc[c];
            ev[c] = (v[c] - v0[c]) - dvc[c];
            eL[c] = (L[c] - L0[c]) - dLc[c];
        }
    }

    // VJP of midpoint_fwd: (lv, lL, lS) adjoints of the output on entry, of
    // the input on exit; lr accumulates the position adjoint.
    __device__ void midpoint_vjp(double hdt, const SaveRef& sv, int base, const double pos[3], double lv[3],
                                 double lL[3], double lS[3], double lr[3], double& gsig, double& gk2) {
        sync();
        if (is_host) { card[AC_PX] = pos[0]; card[AC_PY] = pos[1]; card[AC_PZ] = pos[2]; }
        sync();
        Pre pr;
        pre_fwd(pos, pr);
        Bpre bp;
        bp.zero();
        double lvf[3], lLf[3], lSn[3], lv0[3] = {0., 0., 0.}, lL0[3] = {0., 0., 0.};
        for (int c = 0; c < 3; ++c) { lvf[c] = lv[c]; lLf[c] = lL[c]; lSn[c] = lS[c]; }
        // the iteration count is group-uniform: every lane takes the host's
        // (clamped: a record is never trusted to bound a loop)
        sync();
        if (is_host) {
            const double kr = sv(base);
            card[AC_K] = (kr >= 0. && kr <= (double)kMIDPOINT_MAX) ? kr : 0.;
        }
        sync();
        const int K = (int)card[AC_K];
        for (int i = K - 1; i >= 0; --i) {
            double la[3], ld[3], vc[3], Sc[3], Sp[3], Lc[3];
            for (int c = 0; c < 3; ++c) {
                lv0[c] += lvf[c];
                lL0[c] += lLf[c];
                la[c] = hdt * lvf[c];
                ld[c] = hdt * lLf[c];
                vc[c] = has ? sv(base + 1 + 9 * i + c) : 0.;
                Lc[c] = has ? sv(base + 4 + 9 * i + c) : 0.;
                Sp[c] = has ? sv(base + 7 + 9 * i + c) : 0.;
            }
            spin_of(Lc, Sc);
            double lvc[3], lSc[3], lSp[3];
            effects_vjp(pr, bp, vc, Sc, Sp, la, ld, lvc, lSc, lSp);
            const double im = has ? inv_moi : 0.;
            for (int c = 0; c < 3; ++c) {
                lSc[c] += lSn[c];
                const double lLc = lSc[c] * im;
                if (i > 0) {
                    lv0[c] += 0.5 * lvc[c];
                    lvf[c] = 0.5 * lvc[c];
                    lL0[c] += 0.5 * lLc;
                    lLf[c] = 0.5 * lLc;
                    lSn[c] = lSp[c];
                } else {
                    lv0[c] += lvc[c];
                    lL0[c] += lLc;
                    lSn[c] = lSp[c];
                }
            }
        }
        pre_vjp(pos, bp, lr, gsig, gk2);
        for (int c = 0; c < 3; ++c) { lv[c] = lv0[c]; lL[c] = lL0[c]; lS[c] = lSn[c]; }
    }

    // ---- Jacobi coordinates (src/integrator/whfast.rs:889-963, 1034-1080) ----
    // w -> Jacobi w (own component); slots base..base+2 are used.
    __device__ void jacobi_fwd(const double w[3], double wj[3], int base) {
        sync();
        for (int c = 0; c < 3; ++c) X(base + c, lane) = w[c];
        sync();
        if (has) {
            const int upto = is_host ? n : q;
            double Rs[3] = {0., 0., 0.};
            for (int p = 0; p < upto; ++p) {
                const int j = ord(p);
                for (int c = 0; c < 3; ++c) Rs[c] += gm[j] * X(base + c, j);
            }
            for (int c = 0; c < 3; ++c) wj[c] = is_host ? Rs[c] * iM : w[c] - Rs[c] * i_eta_prev;
        }
        sync();
    }
    // transpose of jacobi_fwd
    __device__ void jacobi_fwd_T(const double lwj[3], double lw[3], int base) {
        sync();
        for (int c = 0; c < 3; ++c) X(base + c, lane) = lwj[c];
        sync();
        if (has) {
            double acc[3];
            for (int c = 0; c < 3; ++c) acc[c] = X(base + c, host) * iM;
            for (int p = n - 1; p >= 1; --p) {
                if (p <= q && !is_host) break;
                const int j = ord(p);
                for (int c = 0; c < 3; ++c) acc[c] -= X(base + c, j) * gieta[p - 1];
            }
            for (int c = 0; c < 3; ++c) lw[c] = (is_host ? 0. : lwj[c]) + m * acc[c];
        }
        sync();
    }
    // Jacobi w -> w
    __device__ void jacobi_inv(const double wj[3], double w[3], int base) {
        sync();
        for (int c = 0; c < 3; ++c) X(base + c, lane) = wj[c];
        sync();
        if (has) {
            double Rs[3];
            for (int c = 0; c < 3; ++c) Rs[c] = M * X(base + c, host);
            const int low = is_host ? 1 : q;
            for (int p = n - 1; p >= low; --p) {
                const int j = ord(p);
                const double ci = gci[p];
                for (int c = 0; c < 3; ++c) Rs[c] = (Rs[c] - gm[j] * X(base + c, j)) * ci;
            }
            for (int c = 0; c < 3; ++c) w[c] = is_host ? Rs[c] * i_m : wj[c] + Rs[c] * i_eta_prev;
        }
        sync();
    }
    // transpose of jacobi_inv
    __device__ void jacobi_inv_T(const double lw[3], double lwj[3], int base) {
        sync();
        for (int c = 0; c < 3; ++c) X(base + c, lane) = lw[c];
        sync();
        if (has) {
            double A[3];
            for (int c = 0; c < 3; ++c) A[c] = X(base + c, host) * i_gmh;
            const int upto = is_host ? n - 1 : q;
            for (int p = 1; p <= upto; ++p) {
                const int j = ord(p);
                const double ci = gci[p];
                for (int c = 0; c < 3; ++c) {
                    A[c] += X(base + c, j) * gieta[p - 1];
                    if (p == q) lwj[c] = lw[c] - gm[j] * ci * A[c];
                    A[c] *= ci;
                }
            }
            if (is_host)
                for (int c = 0; c < 3; ++c) lwj[c] = M * A[c];
        }
        sync();
    }

    // ---- gravity (src/particles/universe.rs:198-303, WHFastOne skip) ----
    __device__ __forceinline__ bool skipped(int i, int j) const {
        const int p0 = host == 0 ? 1 : 0;
        return (i == host && j == p0) || (j == host && i == p0);
    }
    __device__ void gravity_fwd(const double pos[3], double a[3]) {
        sync();
        for (int c = 0; c < 3; ++c) X(c, lane) = pos[c];
        sync();
        a[0] = a[1] = a[2] = 0.;
        if (has) {
            for (int j = 0; j < n; ++j) {
                if (j == lane || skipped(lane, j)) continue;
                const double rj[3] = {X(0, j), X(1, j), X(2, j)};
                gravity_pair(pos, rj, gm[j], a);
            }
        }
        sync();
    }
    __device__ void gravity_vjp(const double pos[3], const double la[3], double lpos[3]) {
        sync();
        for (int c = 0; c < 3; ++c) { X(c, lane) = pos[c]; X(3 + c, lane) = la[c]; }
        sync();
        lpos[0] = lpos[1] = lpos[2] = 0.;
        if (has) {
            for (int j = 0; j < n; ++j) {
                if (j == lane || skipped(lane, j)) continue;
                const double rj[3] = {X(0, j), X(1, j), X(2, j)};
                const double laj[3] = {X(3, j), X(4, j), X(5, j)};
                gravity_pair_vjp(pos, rj, m, gm[j], la, laj, lpos);
            }
        }
        sync();
    }

    // ---- one step ----
    __device__ bool trigger_now() {
        const bool first = last_hist < 0.;
        const bool ht = last_hist + hist_period <= t;
        if (first || ht) {
            last_hist = first ? 0. : last_hist + hist_period;
            return true;
        }
        return false;
    }

    // One forward step; with save, everything the reverse sweep needs is
    // written to the step's record (lanes without a body write nothing).
    __device__ void step_fwd(const SaveRef& sv, bool trig, bool save) {
        save = save && has;
        if (save) sv(SV_TRIG) = trig ? 1. : 0.;
        if (trig) spin_of(L, S);  // first / historic snapshot: spins refreshed (whfast.rs:240-247)
        if (save) for (int c = 0; c < 3; ++c) sv(SV_R0 + c) = r[c];
        midpoint_fwd(half_dt, sv, SV_H1, save);
        // part 1: Jacobi, Kepler drift, back to inertial positions
        double rj[3], vj[3];
        jacobi_fwd(r, rj, 0);
        jacobi_fwd(v, vj, 3);
        if (save) for (int c = 0; c < 3; ++c) { sv(SV_RJA + c) = rj[c]; sv(SV_VJA + c) = vj[c]; }
        if (planet()) {
            const KeplerScalars ks = kepler_scalars(kep_gm, rj, vj);
            bool ok = false;
            const double X1 = kepler_solve(ks, half_dt, &ok);
            if (!ok) errf |= AE_KEPLER;
            if (save) sv(SV_X1) = X1;
            double r1[3], v1[3];
            kepler_apply(kep_gm, half_dt, rj, vj, ks, X1, r1, v1);
            for (int c = 0; c < 3; ++c) { rj[c] = r1[c]; vj[c] = v1[c]; }
        } else if (is_host) {
            for (int c = 0; c < 3; ++c) rj[c] += half_dt * vj[c];
        }
        if (save) for (int c = 0; c < 3; ++c) { sv(SV_RJB + c) = rj[c]; sv(SV_VJB + c) = vj[c]; }
        double rg[3];
        jacobi_inv(rj, rg, 0);
        if (save) for (int c = 0; c < 3; ++c) sv(SV_RG + c) = rg[c];
        // gravity, interaction kick
        double a[3], aj[3];
        gravity_fwd(rg, a);
        jacobi_fwd(a, aj, 6);
        if (has)
            for (int c = 0; c < 3; ++c) vj[c] += dt * aj[c];
        if (planet() && q >= 2) {
            double dv[3];
            jacobi_indirect(dt * kG * eta_q, rj, dv);
            for (int c = 0; c < 3; ++c) vj[c] += dv[c];
        }
        if (save) for (int c = 0; c < 3; ++c) sv(SV_VJC + c) = vj[c];
        // part 2: Kepler drift, back to inertial
        if (planet()) {
            const KeplerScalars ks = kepler_scalars(kep_gm, rj, vj);
            bool ok = false;
            const double X2 = kepler_solve(ks, half_dt, &ok);
            if (!ok) errf |= AE_KEPLER;
            if (save) sv(SV_X2) = X2;
            double r1[3], v1[3];
            kepler_apply(kep_gm, half_dt, rj, vj, ks, X2, r1, v1);
            for (int c = 0; c < 3; ++c) { rj[c] = r1[c]; vj[c] = v1[c]; }
        } else if (is_host) {
            for (int c = 0; c < 3; ++c) rj[c] += half_dt * vj[c];
        }
        jacobi_inv(rj, r, 0);
        jacobi_inv(vj, v, 3);
        if (save) for (int c = 0; c < 3; ++c) sv(SV_R2 + c) = r[c];
        midpoint_fwd(half_dt, sv, SV_H2, save);
        t += dt;
    }

    // Adjoint of one step: lam (r, v, L, S) of the output -> of the input.
    __device__ void step_vjp(const SaveRef& sv, double lr[3], double lv[3], double lL[3], double lS[3],
                             double& gsig, double& gk2) {
        // a step the forward run did not take (the system was frozen): the
        // adjoint passes through unchanged
        sync();
        if (is_host) card[AC_SKIP] = sv(SV_TRIG) < 0. ? 1. : 0.;
        sync();
        if (card[AC_SKIP] != 0.) return;
        double r0[3], rjA[3], vjA[3], rjB[3], rg[3], vjC[3], r2[3], X1 = 0., X2 = 0.;
        bool trig = false;
        for (int c = 0; c < 3; ++c) r0[c] = rjA[c] = vjA[c] = rjB[c] = rg[c] = vjC[c] = r2[c] = 0.;
        if (has) {
            trig = sv(SV_TRIG) != 0.;
            for (int c = 0; c < 3; ++c) {
                r0[c] = sv(SV_R0 + c); rjA[c] = sv(SV_RJA + c); vjA[c] = sv(SV_VJA + c); rjB[c] = sv(SV_RJB + c);
                rg[c] = sv(SV_RG + c); vjC[c] = sv(SV_VJC + c); r2[c] = sv(SV_R2 + c);
            }
            if (planet()) { X1 = sv(SV_X1); X2 = sv(SV_X2); }
        }
        // second half kick (positions r2)
        double lpos[3] = {lr[0], lr[1], lr[2]};
        midpoint_vjp(half_dt, sv, SV_H2, r2, lv, lL, lS, lpos, gsig, gk2);
        // (r2, v) = inverse Jacobi of (rjD, vjD)
        double lrj[3], lvj[3];
        jacobi_inv_T(lpos, lrj, 0);
        jacobi_inv_T(lv, lvj, 3);
        // Kepler drift 2
        if (planet()) {
            double a0[3], b0[3];
            kepler_vjp(kep_gm, half_dt, rjB, vjC, X2, lrj, lvj, a0, b0);
            for (int c = 0; c < 3; ++c) { lrj[c] = a0[c]; lvj[c] = b0[c]; }
        } else if (is_host) {
            for (int c = 0; c < 3; ++c) lvj[c] += half_dt * lrj[c];
        }
        // interaction: vjC = vjB + dt aj + indirect(rjB)
        double laj[3];
        for (int c = 0; c < 3; ++c) laj[c] = has ? dt * lvj[c] : 0.;
        if (planet() && q >= 2) jacobi_indirect_vjp(dt * kG * eta_q, rjB, lvj, lrj);
        double la[3], lrg[3];
        jacobi_fwd_T(laj, la, 6);
        gravity_vjp(rg, la, lrg);
        double tmp[3];
        jacobi_inv_T(lrg, tmp, 0);
        for (int c = 0; c < 3; ++c) lrj[c] += tmp[c];
        // Kepler drift 1
        if (planet()) {
            double a0[3], b0[3];
            kepler_vjp(kep_gm, half_dt, rjA, vjA, X1, lrj, lvj, a0, b0);
            for (int c = 0; c < 3; ++c) { lrj[c] = a0[c]; lvj[c] = b0[c]; }
        } else if (is_host) {
            for (int c = 0; c < 3; ++c) lvj[c] += half_dt * lrj[c];
        }
        // (rjA, vjA) = Jacobi of (r0, v after the first half kick)
        double lr0[3];
        jacobi_fwd_T(lrj, lr0, 0);
        jacobi_fwd_T(lvj, lv, 3);
        // first half kick (positions r0)
        midpoint_vjp(half_dt, sv, SV_H1, r0, lv, lL, lS, lr0, gsig, gk2);
        if (trig && has) {
            const double im = moi != 0. ? 1. / moi : 0.;
            for (int c = 0; c < 3; ++c) { lL[c] += lS[c] * im; lS[c] = 0.; }
        }
        for (int c = 0; c < 3; ++c) lr[c] = lr0[c];
    }
};

template <int G>
__device__ __forceinline__ bool adj_group_setup(const AdjDev& D, int& sys, int& lane, unsigned& mask,
                                                double*& smem) {
    extern __shared__ double shm[];
    const int tid = threadIdx.x;
    const int gib = tid / G;
    lane = tid % G;
    const int gid = blockIdx.x * (blockDim.x / G) + gib;
    const int in_warp = (tid % 32) / G;
    mask = (G >= 32) ? 0xffffffffu : (((1u << G) - 1u) << (in_warp * G));
    smem = shm + (size_t)gib * (AdjSmem<G>::bytes / 8);
    if (gid >= D.n_list) return false;
    sys = D.list[gid];
    return sys >= 0;  // a negative entry is a system left out of the run
}

// Forward K steps from the chunk's start state, writing every step's record.
template <int G>
__global__ void __launch_bounds__(128) adj_record_kernel(AdjDev D, int64_t k_steps) {
    int sys, lane;
    unsigned mask;
    double* smem;
    if (!adj_group_setup<G>(D, sys, lane, mask, smem)) return;
    AdjSys<G> A;
    A.setup(D, sys, lane, mask, smem);
    const int64_t st = D.stride;
    const int64_t k = (int64_t)sys * D.nmax + lane;
    if (A.has) A.load_state(D.bf + k, st);
    for (int64_t i = 0; i < k_steps; ++i) {
        const bool trig = A.trigger_now();
        const SaveRef sv{D.tape + i * SV_COUNT * st + k, st};
        A.step_fwd(sv, trig, true);
    }
    A.sync();
    if (A.errf) atomicOr(&D.err[sys], A.errf);
}

// Reverse sweep over the K recorded steps of a chunk.
template <int G>
__global__ void __launch_bounds__(128) adj_reverse_kernel(AdjDev D, int64_t k_steps) {
    int sys, lane;
    unsigned mask;
    double* smem;
    if (!adj_group_setup<G>(D, sys, lane, mask, smem)) return;
    AdjSys<G> A;
    A.setup(D, sys, lane, mask, smem);
    const int64_t st = D.stride;
    const int64_t k = (int64_t)sys * D.nmax + lane;
    double lr[3] = {0., 0., 0.}, lv[3] = {0., 0., 0.}, lL[3] = {0., 0., 0.}, lS[3] = {0., 0., 0.};
    double gsig = 0., gk2 = 0.;
    if (A.has) {
        for (int c = 0; c < 3; ++c) {
            lr[c] = D.lam[(LM_R + c) * st + k];
            lv[c] = D.lam[(LM_V + c) * st + k];
            lL[c] = D.lam[(LM_L + c) * st + k];
            lS[c] = D.lam[(LM_S + c) * st + k];
        }
        gsig = D.grad[GD_SIGMA * st + k];
        gk2 = D.grad[GD_K2 * st + k];
    }
    for (int64_t i = k_steps - 1; i >= 0; --i) {
        const SaveRef sv{D.tape + i * SV_COUNT * st + k, st};
        A.step_vjp(sv, lr, lv, lL, lS, gsig, gk2);
    }
    if (A.has) {
        for (int c = 0; c < 3; ++c) {
            D.lam[(LM_R + c) * st + k] = lr[c];
            D.lam[(LM_V + c) * st + k] = lv[c];
            D.lam[(LM_L + c) * st + k] = lL[c];
            D.lam[(LM_S + c) * st + k] = lS[c];
        }
        D.grad[GD_SIGMA * st + k] = gsig;
        D.grad[GD_K2 * st + k] = gk2;
    }
    A.sync();
    if (A.errf) atomicOr(&D.err[sys], A.errf);
}

}  // namespace posi_adj
