// ias15_device.cuh -- FP64 device code of the IAS15 integrator
// (src/integrator/ias15.rs), included by ias15_impl.cuh inside the namespace
// of whfast_device.cuh and compiled in both arithmetic modes.
//
// Mapping: the WHFast kernel's lane groups (G = 2 to 32 lanes, the smallest
// that holds the system; lane j owns body j).  A lane keeps its body's
// Gauss-Radau coefficients b and g (7 sets of 3 components, and the same for
// the spin angular momentum), their
// compensated-summation terms and the step's initial state in local arrays;
// the predictions e, the last accepted br / er (and their spin forms) and
// csx / csv / css stay in the per-body IAS15 array in HBM ([POSI_IAS_COUNT]
// [stride]), read and written once per step.  Each of the seven substeps of a
// predictor-corrector iteration is one force evaluation of the WHFast path
// (gravity without ignored terms, heliocentric geometry, the additional
// effects with evolution at the substep time).  The maxima of the error
// estimates are taken by lane 0 over the bodies in index order from the group
// exchange slots, so the reference's order-dependent step-size rule
// (ias15.rs:1121-1124 compares the torque maximum against the acceleration
// maximum) is reproduced exactly.
//
// EXACT keeps the reference's operation order and matches the CPU oracle bit
// for bit; FAST lets the compiler contract FMAs in the same expressions.

// Gauss-Radau spacings, their differences h[j] - h[k] and the b <-> g
// conversion constants of the reference (ias15.rs:485-528), as exact doubles.
__constant__ double kIAS_H[8] = {
    0x0.0p+0, 0x1.cce7242fd9812p-5, 0x1.7122082358d27p-3,
    0x1.6916742f0c9c5p-2, 0x1.18248525f4802p-1, 0x1.77ea65770fa49p-1,
    0x1.c548c982467cdp-1, 0x1.f47d94f4d2bb2p-1,
};
__constant__ double kIAS_R[28] = {
    0x1.cce7242fd9812p-5, 0x1.7122082358d27p-3, 0x1.fbd07e2ec4e45p-4,
    0x1.6916742f0c9c5p-2, 0x1.2f798fa9116c3p-2, 0x1.610ae03ac0664p-3,
    0x1.18248525f4802p-1, 0x1.f6ac25c5edd01p-2, 0x1.77b8063a3c970p-2,
    0x1.8e652c39b8c7cp-3, 0x1.77ea65770fa49p-1, 0x1.5b1bf334120c8p-1,
    0x1.1ba1e36e39700p-1, 0x1.86be56bf12acdp-2, 0x1.7f1781446c91fp-3,
    0x1.c548c982467cdp-1, 0x1.a87a573f48e4cp-1, 0x1.6900477970483p-1,
    0x1.10bd8f6ac02eap-1, 0x1.5a4888b8a3f96p-2, 0x1.3579902cdb60ep-3,
    0x1.f47d94f4d2bb2p-1, 0x1.d7af22b1d5231p-1, 0x1.983512ebfc868p-1,
    0x1.3ff25add4c6cfp-1, 0x1.b8b21f9dbc761p-2, 0x1.f24cbdf70c5a2p-3,
    0x1.79a65b9461f2ap-4,
};
// FAST: the reciprocals of kIAS_R (a product instead of a division in the
// substep updates; one rounding more than the reference's division)
__constant__ double kIAS_RINV[28] = {
    1. / 0x1.cce7242fd9812p-5, 1. / 0x1.7122082358d27p-3, 1. / 0x1.fbd07e2ec4e45p-4,
    1. / 0x1.6916742f0c9c5p-2, 1. / 0x1.2f798fa9116c3p-2, 1. / 0x1.610ae03ac0664p-3,
    1. / 0x1.18248525f4802p-1, 1. / 0x1.f6ac25c5edd01p-2, 1. / 0x1.77b8063a3c970p-2,
    1. / 0x1.8e652c39b8c7cp-3, 1. / 0x1.77ea65770fa49p-1, 1. / 0x1.5b1bf334120c8p-1,
    1. / 0x1.1ba1e36e39700p-1, 1. / 0x1.86be56bf12acdp-2, 1. / 0x1.7f1781446c91fp-3,
    1. / 0x1.c548c982467cdp-1, 1. / 0x1.a87a573f48e4cp-1, 1. / 0x1.6900477970483p-1,
    1. / 0x1.10bd8f6ac02eap-1, 1. / 0x1.5a4888b8a3f96p-2, 1. / 0x1.3579902cdb60ep-3,
    1. / 0x1.f47d94f4d2bb2p-1, 1. / 0x1.d7af22b1d5231p-1, 1. / 0x1.983512ebfc868p-1,
    1. / 0x1.3ff25add4c6cfp-1, 1. / 0x1.b8b21f9dbc761p-2, 1. / 0x1.f24cbdf70c5a2p-3,
    1. / 0x1.79a65b9461f2ap-4,
};
__constant__ double kIAS_C[21] = {
    -0x1.cce7242fd9812p-5, 0x1.4c4b384151c1ep-7, -0x1.e45bd12f4f32cp-3,
    -0x1.d4b3379a1992dp-9, 0x1.7f2161e152586p-4, -0x1.2da22e635a1aep-1,
    0x1.007370e57b89dp-9, -0x1.c08e5e7efcf23p-5, 0x1.a9dcc2e57fbbfp-2,
    -0x1.22e359c4a74d8p+0, -0x1.7893e98a2a997p-10, 0x1.595cd739ee74fp-5,
    -0x1.70bdf2d91dd44p-2, 0x1.4009e0866d488p+0, -0x1.ded88c802f1fcp+0,
    0x1.4d64672378b3dp-10, -0x1.3d865cb429919p-5, 0x1.71a0161ae20fep-2,
    -0x1.7785b93619434p+0, 0x1.73fc45dfb9889p+1, -0x1.60be78a0a92f1p+1,
};
__constant__ double kIAS_D[21] = {
    0x1.cce7242fd9812p-5, 0x1.9ee7bd5f24900p-9, 0x1.e45bd12f4f32cp-3,
    0x1.757f83047d1ecp-13, 0x1.7722d9e44e93cp-5, 0x1.2da22e635a1aep-1,
    0x1.50392d238405bp-17, 0x1.144b8b5c061cdp-7, 0x1.039e6f5c0b72fp-2,
    0x1.22e359c4a74d8p+0, 0x1.2eab281d37645p-21, 0x1.9106110af09c6p-10,
    0x1.90baa1e56027dp-4, 0x1.c0216120faaf2p-1, 0x1.ded88c802f1fcp+0,
    0x1.107669a72b0ebp-25, 0x1.21b6dca35a7eap-12, 0x1.27255aa2a25aap-5,
    0x1.27498c3d6d930p-1, 0x1.1fd1c1aad40f1p+1, 0x1.60be78a0a92f1p+1,
};
constexpr double kIAS_EPSILON = 1e-6;        // src/constants.rs:13
constexpr double kIAS_SAFETY_FACTOR = 0.25;  // src/constants.rs:17

// ias15.rs:1471-1476 compensated add
__device__ __forceinline__ void ias_add_cs(double& p, double& csp, double inp) {
    const double y = inp - csp;
    const double np = p + y;
    csp = (np - p) - y;
    p = np;
}

// ias15.rs:1453-1461: seventh root by 20 Newton steps from 1
__device__ __forceinline__ double ias_sqrt7(double a) {
    double x = 1.;
    for (int k = 0; k < 20; ++k) {
        const double x6 = x * x * x * x * x * x;
        x += (a / x6 - x) / 7.;
    }
    return x;
}

__device__ __forceinline__ double ias_max(double a, double b) { return a > b ? a : b; }
// f64::is_normal: neither zero, subnormal, infinite nor NaN
__device__ __forceinline__ bool ias_normal(double a) {
    const double m = fabs(a);
    return m >= 2.2250738585072014e-308 && m <= 1.7976931348623157e308;
}

// The per-lane IAS15 state of one body.
struct IasLane {
    double b[21], sb[21];      // b_j component c at 3j + c
    double g[21], sg[21];
    double csb[21], cssb[21];
    double x0[3], v0[3], a0[3], l0[3], dl0[3], at[3], dlt[3];
    double csx[3], csv[3], css[3];
};

template <int G>
struct Ias15 {
    Sys<G>& S;
    const Dev& D;
    double* F;       // this body's IAS15 fields (stride D.stride)
    int64_t st;
    bool ispin;      // ias15.rs:499-501: the spin angular momenta are integrated
    double dt_last;  // time_step_last_success
    int64_t max_exceeded;
    IasLane L;

    __device__ Ias15(Sys<G>& s_, const Dev& d_) : S(s_), D(d_) {
        st = D.stride;
        F = D.ias + (int64_t)S.s * D.nmax + S.lane;
        ispin = S.tides || S.flat || S.evo || S.grk();
        const int64_t ns = D.n_sys;
        dt_last = D.sf[POSI_SF_IAS_DT_LAST * ns + S.s];
        max_exceeded = D.si[POSI_SI_IAS_MAX_EXCEEDED * ns + S.s];
        for (int k = 0; k < 21; ++k) { L.b[k] = 0.; L.sb[k] = 0.; }
        for (int k = 0; k < 3; ++k) { L.csx[k] = 0.; L.csv[k] = 0.; L.css[k] = 0.; }
        if (S.has) {
            for (int k = 0; k < 21; ++k) {
                L.b[k] = F[(POSI_IAS_B + k) * st];
                L.sb[k] = F[(POSI_IAS_SB + k) * st];
            }
            for (int k = 0; k < 3; ++k) {
                L.csx[k] = F[(POSI_IAS_CSX + k) * st];
                L.csv[k] = F[(POSI_IAS_CSV + k) * st];
                L.css[k] = F[(POSI_IAS_CSS + k) * st];
            }
        }
    }

    __device__ void store() {
        const int64_t ns = D.n_sys;
        if (S.lane == 0) {
            D.sf[POSI_SF_DT * ns + S.s] = S.dt;
            D.sf[POSI_SF_IAS_DT_LAST * ns + S.s] = dt_last;
            D.si[POSI_SI_IAS_MAX_EXCEEDED * ns + S.s] = max_exceeded;
        }
        if (!S.has) return;
        for (int k = 0; k < 21; ++k) {
            F[(POSI_IAS_B + k) * st] = L.b[k];
            F[(POSI_IAS_SB + k) * st] = L.sb[k];
        }
        for (int k = 0; k < 3; ++k) {
            F[(POSI_IAS_CSX + k) * st] = L.csx[k];
            F[(POSI_IAS_CSV + k) * st] = L.csv[k];
            F[(POSI_IAS_CSS + k) * st] = L.css[k];
        }
    }

    // ias15.rs:1342-1451 predict_next_step (this lane's body)
    __device__ void predict_next_step(double ratio) {
        if (!S.has) return;
        const int nblk = ispin ? 2 : 1;
        for (int q = 0; q < nblk; ++q) {
            double* B = q == 0 ? L.b : L.sb;
            const int E = q == 0 ? POSI_IAS_E : POSI_IAS_SE;
            const int BR = q == 0 ? POSI_IAS_BR : POSI_IAS_SBR;
            const int ER = q == 0 ? POSI_IAS_ER : POSI_IAS_SER;
            if (ratio > 20.) {
                for (int k = 0; k < 21; ++k) { F[(E + k) * st] = 0.; B[k] = 0.; }
                continue;
            }
            const double q1 = ratio, q2 = q1 * q1, q3 = q1 * q2, q4 = q2 * q2, q5 = q2 * q3, q6 = q3 * q3,
                         q7 = q3 * q4;
            for (int c = 0; c < 3; ++c) {
                double br[7], be[7], e[7];
                for (int j = 0; j < 7; ++j) {
                    br[j] = F[(BR + 3 * j + c) * st];
                    be[j] = br[j] - F[(ER + 3 * j + c) * st];
                }
                // Everhart's eqs. 13
                e[0] = q1 * (br[6] * 7.0 + br[5] * 6.0 + br[4] * 5.0 + br[3] * 4.0 + br[2] * 3.0 + br[1] * 2.0 + br[0]);
                e[1] = q2 * (br[6] * 21.0 + br[5] * 15.0 + br[4] * 10.0 + br[3] * 6.0 + br[2] * 3.0 + br[1]);
                e[2] = q3 * (br[6] * 35.0 + br[5] * 20.0 + br[4] * 10.0 + br[3] * 4.0 + br[2]);
                e[3] = q4 * (br[6] * 35.0 + br[5] * 15.0 + br[4] * 5.0 + br[3]);
                e[4] = q5 * (br[6] * 21.0 + br[5] * 6.0 + br[4]);
                e[5] = q6 * (br[6] * 7.0 + br[5]);
                e[6] = q7 * br[6];
                for (int j = 0; j < 7; ++j) {
                    F[(E + 3 * j + c) * st] = e[j];
                    B[3 * j + c] = e[j] + be[j];
                }
            }
        }
    }

    // g_j from b (Everhart's eqs. 7, ias15.rs:567-583)
    __device__ static double g_from_b(const double* b, int c, int j) {
        if (j == 6) return b[18 + c];
        double acc = b[18 + c] * kIAS_D[15 + j];
        for (int m = 5; m > j; --m) acc = acc + b[3 * m + c] * kIAS_D[m * (m - 1) / 2 + j];
        return acc + b[3 * j + c];
    }

    // one substep's update of g_j and b_0..b_j of component c
    // (ias15.rs:710-1001); returns the change of g_j
    __device__ static double update(double at, double a0, double* g, double* b, double* csb, int c, int j) {
        const double zero = 0.;
        double gk = at, cs = zero;
        ias_add_cs(gk, cs, -a0);
        ias_add_cs(gk, cs, zero);
        const double old = g[3 * j + c];
        const int base = j * (j + 1) / 2;
#if POSI_EXACT
        double v = gk / kIAS_R[base];
        for (int m = 0; m < j; ++m) v = (v - g[3 * m + c]) / kIAS_R[base + 1 + m];
#else
        double v = gk * kIAS_RINV[base];
        for (int m = 0; m < j; ++m) v = (v - g[3 * m + c]) * kIAS_RINV[base + 1 + m];
#endif
        g[3 * j + c] = v;
        const double tmp = v - old;
        const int cb = j * (j - 1) / 2;
        for (int m = 0; m < j; ++m) ias_add_cs(b[3 * m + c], csb[3 * m + c], tmp * kIAS_C[cb + m]);
        ias_add_cs(b[3 * j + c], csb[3 * j + c], tmp);
        return tmp;
    }

    // gravity without ignored terms, heliocentric geometry and the additional
    // effects at the substep time, then a += a_add (ias15.rs:690-700)
    __device__ bool evaluate(double t_eval) {
        S.gravity(D, 0);
        if (S.fatal()) return false;
        S.t = t_eval;
        S.sync();
        if (S.is_host) {
            Sys<G>& s = S;
            s.card[HC_PX] = s.b.r[0]; s.card[HC_PY] = s.b.r[1]; s.card[HC_PZ] = s.b.r[2];
            s.card[HC_M] = s.b.m; s.card[HC_MG] = s.b.mg; s.card[HC_R] = s.b.R; s.card[HC_SIG] = s.b.sig;
            s.card[HC_K2] = s.b.k2; s.card[HC_K2F] = s.b.k2f;
            s.card[HC_DFAC] = s.b.diss_factor; s.card[HC_DSCALE] = s.b.diss_scale;
            for (int k = 0; k < 6; ++k) s.card[HC_DINNER + k] = s.b.dk == POSI_EFFECT_CENTRAL ? s.b.disk_p[k] : 0.;
        }
        S.sync();
#if !POSI_EXACT
        S.pc_reuse = false;
#endif
        if (S.planet()) S.set_geometry(S.b.r[0] - S.card[HC_PX], S.b.r[1] - S.card[HC_PY], S.b.r[2] - S.card[HC_PZ]);
        S.additional_effects(D, 0, true);
        if (S.fatal()) return false;
        if (S.has)
            for (int k = 0; k < 3; ++k) S.b.a[k] += S.b.aa[k];
        return true;
    }

    // ias15.rs:480-1339: one accepted step (rejected tries are redone);
    // false when the system froze in a force evaluation
    __device__ bool integrator() {
        Body& bd = S.b;
        for (int guard = 0; guard < 64; ++guard) {
            for (int c = 0; c < 3; ++c) {
                L.x0[c] = bd.r[c]; L.v0[c] = bd.v[c]; L.a0[c] = bd.a[c];
                if (ispin) { L.dl0[c] = bd.dl[c]; L.l0[c] = bd.L[c]; }
                L.at[c] = 0.; L.dlt[c] = 0.;
            }
            for (int k = 0; k < 21; ++k) { L.csb[k] = 0.; L.cssb[k] = 0.; }
            for (int c = 0; c < 3; ++c)
                for (int j = 0; j < 7; ++j) {
                    L.g[3 * j + c] = g_from_b(L.b, c, j);
                    if (ispin) L.sg[3 * j + c] = g_from_b(L.sb, c, j);
                }
            const double t_beginning = S.t;
            double pce = 1e300, pce_last = 2.;
            int iterations = 0;
            for (;;) {
                if (pce < 1e-16) break;
                if (iterations > 2 && pce_last <= pce) break;
                if (iterations >= 12) {
                    max_exceeded += 1;
                    break;
                }
                pce_last = pce;
                pce = 0.;
                iterations += 1;
                for (int sub = 1; sub < 8; ++sub) {
                    const double h = kIAS_H[sub];
                    double sp[9];
                    sp[0] = S.dt * h;
                    double sv[8];
                    sv[0] = S.dt * h;
#if POSI_EXACT
                    sp[1] = sp[0] * sp[0] / 2.;
                    sp[2] = sp[1] * h / 3.;
                    sp[3] = sp[2] * h / 2.;
                    sp[4] = 3. * sp[3] * h / 5.;
                    sp[5] = 2. * sp[4] * h / 3.;
                    sp[6] = 5. * sp[5] * h / 7.;
                    sp[7] = 3. * sp[6] * h / 4.;
                    sp[8] = 7. * sp[7] * h / 9.;
                    sv[1] = sv[0] * h / 2.;
                    sv[2] = 2. * sv[1] * h / 3.;
                    sv[3] = 3. * sv[2] * h / 4.;
                    sv[4] = 4. * sv[3] * h / 5.;
                    sv[5] = 5. * sv[4] * h / 6.;
                    sv[6] = 6. * sv[5] * h / 7.;
                    sv[7] = 7. * sv[6] * h / 8.;
#else
                    // the same factors with products by the reciprocals
                    sp[1] = sp[0] * sp[0] * 0.5;
                    sp[2] = sp[1] * h * (1. / 3.);
                    sp[3] = sp[2] * h * 0.5;
                    sp[4] = sp[3] * h * (3. / 5.);
                    sp[5] = sp[4] * h * (2. / 3.);
                    sp[6] = sp[5] * h * (5. / 7.);
                    sp[7] = sp[6] * h * 0.75;
                    sp[8] = sp[7] * h * (7. / 9.);
                    sv[1] = sv[0] * h * 0.5;
                    sv[2] = sv[1] * h * (2. / 3.);
                    sv[3] = sv[2] * h * 0.75;
                    sv[4] = sv[3] * h * 0.8;
                    sv[5] = sv[4] * h * (5. / 6.);
                    sv[6] = sv[5] * h * (6. / 7.);
                    sv[7] = sv[6] * h * 0.875;
#endif
                    if (S.has) {
                        for (int c = 0; c < 3; ++c) {
                            // Everhart's eq. 9 (positions) and 10 (velocities, spins)
                            double acc = sp[8] * L.b[18 + c];
                            for (int j = 5; j >= 0; --j) acc = acc + sp[j + 2] * L.b[3 * j + c];
                            acc = acc + sp[1] * L.a0[c];
                            acc = acc + sp[0] * L.v0[c];
                            bd.r[c] = (-L.csx[c] + acc) + L.x0[c];
                            double va = -L.csv[c];
                            for (int j = 6; j >= 0; --j) va = va + sv[j + 1] * L.b[3 * j + c];
                            va = va + sv[0] * L.a0[c];
                            bd.v[c] = va + L.v0[c];
                            if (ispin) {
                                double la = -L.css[c];
                                for (int j = 6; j >= 0; --j) la = la + sv[j + 1] * L.sb[3 * j + c];
                                la = la + sv[0] * L.dl0[c];
                                bd.L[c] = la + L.l0[c];
                            }
                        }
                    }
                    if (!evaluate(t_beginning + sp[0])) {
                        S.t = t_beginning;
                        return false;
                    }
                    const int j = sub - 1;
                    double m_ak = 0., m_b6 = 0., m_dl = 0., m_sb6 = 0.;
                    if (S.has) {
                        for (int c = 0; c < 3; ++c) {
                            L.at[c] = bd.a[c];
                            if (ispin) L.dlt[c] = bd.dl[c];
                            const double tmp = update(L.at[c], L.a0[c], L.g, L.b, L.csb, c, j);
                            double stmp = 0.;
                            if (ispin) stmp = update(L.dlt[c], L.dl0[c], L.sg, L.sb, L.cssb, c, j);
                            if (sub == 7) {
                                const double ak = fabs(L.at[c]);
                                if (ias_normal(ak) && ak > m_ak) m_ak = ak;
                                const double b6 = fabs(tmp);
                                if (ias_normal(b6) && b6 > m_b6) m_b6 = b6;
                                if (ispin) {
                                    const double dk = fabs(L.dlt[c]);
                                    if (ias_normal(dk) && dk > m_dl) m_dl = dk;
                                    const double sb6 = fabs(stmp);
                                    if (ias_normal(sb6) && sb6 > m_sb6) m_sb6 = sb6;
                                }
                            }
                        }
                    }
                    if (sub == 7) {
                        // global error estimate (ias15.rs:1009-1061): maxima over
                        // every body and component (order-free)
                        S.sync();
                        S.X(0, S.lane) = m_ak; S.X(1, S.lane) = m_b6; S.X(2, S.lane) = m_dl; S.X(3, S.lane) = m_sb6;
                        S.sync();
                        double a = 0., b6 = 0., dl = 0., sb6 = 0.;
                        for (int i = 0; i < S.n; ++i) {
                            a = fmax(a, S.X(0, i)); b6 = fmax(b6, S.X(1, i));
                            dl = fmax(dl, S.X(2, i)); sb6 = fmax(sb6, S.X(3, i));
                        }
                        S.sync();
                        pce = ias_max(b6, sb6) / ias_max(a, dl);
                    }
                }
            }
            S.t = t_beginning;
            // new step size (ias15.rs:1065-1225): lane 0 folds the bodies in
            // index order
            const double dt_done = S.dt;
            S.sync();
            if (S.has) {
                const double v2 = bd.v[0] * bd.v[0] + bd.v[1] * bd.v[1] + bd.v[2] * bd.v[2];
                const double x2 = bd.r[0] * bd.r[0] + bd.r[1] * bd.r[1] + bd.r[2] * bd.r[2];
                bool skip;
                if (ispin) {
                    const double dl2 = bd.dl[0] * bd.dl[0] + bd.dl[1] * bd.dl[1] + bd.dl[2] * bd.dl[2];
                    const double l2 = bd.L[0] * bd.L[0] + bd.L[1] * bd.L[1] + bd.L[2] * bd.L[2];
                    skip = fabs(v2 * S.dt * S.dt / x2) < 1e-16 && fabs(dl2 * S.dt * S.dt / l2) < 1e-16;
                } else {
                    skip = fabs(v2 * S.dt * S.dt / x2) < 1e-16;
                }
                S.X(0, S.lane) = skip ? 1. : 0.;
                for (int c = 0; c < 3; ++c) {
                    S.X(1 + c, S.lane) = fabs(L.at[c]);
                    S.X(4 + c, S.lane) = fabs(L.b[18 + c]);
                    S.X(7 + c, S.lane) = fabs(L.dlt[c]);
                    S.X(10 + c, S.lane) = fabs(L.sb[18 + c]);
                }
            }
            S.sync();
            if (S.lane == 0) {
                double maxak = 0., maxb6 = 0., maxdl = 0., maxsb6 = 0.;
                for (int i = 0; i < S.n; ++i) {
                    if (S.X(0, i) != 0.) continue;
                    for (int c = 0; c < 3; ++c) {
                        const double ak = S.X(1 + c, i);
                        if (ias_normal(ak) && ak > maxak) maxak = ak;
                        const double b6 = S.X(4 + c, i);
                        if (ias_normal(b6) && b6 > maxb6) maxb6 = b6;
                        if (ispin) {
                            const double dk = S.X(7 + c, i);
                            if (ias_normal(dk) && dk > maxak) maxdl = dk;  // sic: against maxak
                            const double sb6 = S.X(10 + c, i);
                            if (ias_normal(sb6) && sb6 > maxsb6) maxsb6 = sb6;
                        }
                    }
                }
                const double err = ias_max(maxb6, maxsb6) / ias_max(maxak, maxdl);
                double dt_new;
                if (ias_normal(err)) dt_new = ias_sqrt7(kIAS_EPSILON / err) * dt_done;
                else dt_new = dt_done / kIAS_SAFETY_FACTOR;
                S.sums[0] = dt_new;
            }
            S.sync();
            double dt_new = S.sums[0];
            S.sync();
            if (fabs(dt_new / dt_done) < kIAS_SAFETY_FACTOR) {
                // rejected: back to the step's start with the smaller step
                for (int c = 0; c < 3; ++c) {
                    bd.r[c] = L.x0[c]; bd.v[c] = L.v0[c]; bd.a[c] = L.a0[c];
                    if (ispin) { bd.dl[c] = L.dl0[c]; bd.L[c] = L.l0[c]; }
                }
                S.dt = dt_new;
                if (dt_last != 0.) predict_next_step(S.dt / dt_last);
                continue;
            }
            if (fabs(dt_new / dt_done) > 1.0) {
                if (dt_new / dt_done > 1. / kIAS_SAFETY_FACTOR) dt_new = dt_done / kIAS_SAFETY_FACTOR;
            }
            S.dt = dt_new;
            // Everhart's eqs. 11-12, compensated
            if (S.has) {
                const double dt2 = dt_done * dt_done;
#if POSI_EXACT
                const double xdiv[7] = {6., 12., 20., 30., 42., 56., 72.};
                const double vdiv[7] = {2., 3., 4., 5., 6., 7., 8.};
#else
                // products by the reciprocals
                const double xmul[7] = {1. / 6., 1. / 12., 1. / 20., 1. / 30., 1. / 42., 1. / 56., 1. / 72.};
                const double vmul[7] = {0.5, 1. / 3., 0.25, 0.2, 1. / 6., 1. / 7., 0.125};
#endif
                for (int c = 0; c < 3; ++c) {
                    double x = L.x0[c], cx = L.csx[c];
#if POSI_EXACT
                    for (int j = 6; j >= 0; --j) ias_add_cs(x, cx, L.b[3 * j + c] / xdiv[j] * dt2);
#else
                    for (int j = 6; j >= 0; --j) ias_add_cs(x, cx, L.b[3 * j + c] * xmul[j] * dt2);
#endif
                    ias_add_cs(x, cx, L.a0[c] / 2. * dt2);
                    ias_add_cs(x, cx, L.v0[c] * dt_done);
                    L.csx[c] = cx;
                    double v = L.v0[c], cv = L.csv[c];
#if POSI_EXACT
                    for (int j = 6; j >= 0; --j) ias_add_cs(v, cv, L.b[3 * j + c] / vdiv[j] * dt_done);
#else
                    for (int j = 6; j >= 0; --j) ias_add_cs(v, cv, L.b[3 * j + c] * vmul[j] * dt_done);
#endif
                    ias_add_cs(v, cv, L.a0[c] * dt_done);
                    L.csv[c] = cv;
                    bd.r[c] = x;
                    bd.v[c] = v;
                    if (ispin) {
                        double l = L.l0[c], cl = L.css[c];
#if POSI_EXACT
                        for (int j = 6; j >= 0; --j) ias_add_cs(l, cl, L.sb[3 * j + c] / vdiv[j] * dt_done);
#else
                        for (int j = 6; j >= 0; --j) ias_add_cs(l, cl, L.sb[3 * j + c] * vmul[j] * dt_done);
#endif
                        ias_add_cs(l, cl, L.dl0[c] * dt_done);
                        L.css[c] = cl;
                        bd.L[c] = l;
                    }
                }
                // er = e, br = b, ser = se, sbr = sb
                for (int k = 0; k < 21; ++k) {
                    F[(POSI_IAS_ER + k) * st] = F[(POSI_IAS_E + k) * st];
                    F[(POSI_IAS_BR + k) * st] = L.b[k];
                    F[(POSI_IAS_SER + k) * st] = F[(POSI_IAS_SE + k) * st];
                    F[(POSI_IAS_SBR + k) * st] = L.sb[k];
                }
            }
            S.t += dt_done;
            dt_last = dt_done;
            predict_next_step(S.dt / dt_done);
            return true;
        }
        // a step rejected 64 times in a row (each try at most a quarter of the
        // last) is a step below 1e-38 of the first: treated as non-convergence
        S.set_fatal(POSI_SYS_BISECTION_LIMIT, 0, 0);
        return false;
    }

    // ias15.rs:420-463 Integrator::iterate; false once the system is frozen
    __device__ bool iterate() {
        const bool first = S.last_hist < 0.;
        const bool hist_trig = S.last_hist + S.hist_period <= S.t;
        const bool rec_trig = S.last_rec + S.rec_period <= S.t;
        if (first || hist_trig) {
            S.spin_and_evolving(D, S.t, true);
            S.zero_inertia_check();
            if (S.fatal()) return false;
            if (S.tides) S.tides_denergy_dt();
            S.write_history_record(D);
            S.last_hist = S.t;
            S.n_hist += 1;
        }
        if (!evaluate(S.t)) return false;
        if (!integrator()) return false;
        S.iteration += 1;
        if (S.lane == 0 && D.step_flags) D.step_flags[S.s] = (rec_trig || first ? 1 : 0) | ((first || hist_trig) ? 2 : 0);
        if (S.t + S.dt > S.time_limit) {
            S.status = (S.status & ~(int64_t)POSI_SYS_FATAL_MASK) | POSI_SYS_COMPLETED;
            return false;
        }
        return true;
    }
};

// Advance each listed IAS15 system by up to n_steps steps.
template <int G>
__global__ void __launch_bounds__(128) ias15_steps_kernel(Dev D, int64_t n_steps) {
    int sys, lane;
    unsigned mask;
    double* smem;
    if (!group_setup<G>(D, sys, lane, mask, smem)) return;
    Sys<G> S;
    S.load(D, sys, lane, mask, smem);
    S.gr_ignore = 0;     // IgnoreGravityTerms::None
    S.spin_on = true;    // dangular_momentum_dt = true in every evaluation
    Ias15<G> I(S, D);
    if (!S.fatal())
        for (int64_t k = 0; k < n_steps; ++k)
            if (!I.iterate()) break;
    S.store(D);
    I.store();
}
