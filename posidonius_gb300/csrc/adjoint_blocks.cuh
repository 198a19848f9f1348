// adjoint_blocks.cuh -- scalar building blocks of the WHFast adjoint.
//
// Host-and-device functions (the tests compile them for the CPU as well):
// Stumpff functions c0..c5, the universal-variable Kepler drift of one body
// (src/integrator/whfast.rs:676-876) as a forward map with its
// vector-Jacobian product, and the Jacobi interaction term.
//
// The Kepler drift maps (r0, v0) to (r1, v1) through the root X of
// F(X) = r0 X + eta0 G2(beta, X) + zeta0 G3(beta, X) - dt = 0 with
// G_n(beta, X) = X^n c_n(beta X^2).  Its VJP differentiates the converged
// root implicitly (dX = -dF / F_X, F_X = r) using dG_n/dX = G_(n-1) and
// dG_n/dbeta = (n G_(n+2) - X G_(n+1)) / 2, so it costs one evaluation of the
// G functions and no iteration.
#pragma once
#include <cmath>
#include <cstdint>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace posi_adj {

// src/constants.rs (same literal expressions)
constexpr double kPI = 3.141592653589793;
constexpr double kDAY = 24. * 3600.;
constexpr double kM_SUN = 1.9818e30;
constexpr double kG_SI = 6.67428e-11;
constexpr double kAU = 1.49597870700e11;
constexpr double kC = (2.99792458e8 / kAU) * kDAY;
constexpr double kC2 = kC * kC;
constexpr double kG = kG_SI / (kAU * kAU * kAU) * kM_SUN * (kDAY * kDAY);
constexpr double kK2 = kG;
constexpr double kFA = kG / kC2;
constexpr double kDBL_EPSILON_2 = 2.2204460492503131e-16 * 2.2204460492503131e-16;
constexpr int kMIDPOINT_MIN = 3;
constexpr int kMIDPOINT_MAX = 10;
constexpr int kKEPLER_MAX_NEWTON = 64;
constexpr double kJACOBI_SOFTENING = 1e-12;

// c_n(z) = sum_k (-z)^k / (2k + n)!, n = 0..5.  Small |z|: the series; larger
// |z|: quarter z until it is small, double back c0..c3 with the half-angle
// identities, and take c4, c5 from c_n = 1/n! - z c_(n+2).
__host__ __device__ __forceinline__ void stumpff6(double z, double c[6]) {
    // 1/n! for n = 0..19
    const double f[20] = {1., 1., 1. / 2., 1. / 6., 1. / 24., 1. / 120., 1. / 720., 1. / 5040., 1. / 40320.,
                          1. / 362880., 1. / 3628800., 1. / 39916800., 1. / 479001600., 1. / 6227020800.,
                          1. / 87178291200., 1. / 1307674368000., 1. / 20922789888000., 1. / 355687428096000.,
                          1. / 6402373705728000., 1. / 121645100408832000.};
    double zz = z;
    int n = 0;
    while (fabs(zz) > 0.1 && n < 64) {
        zz *= 0.25;
        ++n;
    }
    // series with 7 terms (|z| <= 0.1: error below 0.1^7 / 14! relative)
    for (int k = 0; k < 6; ++k) {
        double s = f[k + 12];
        for (int j = 5; j >= 0; --j) s = f[k + 2 * j] - zz * s;
        c[k] = s;
    }
    if (n == 0) return;
    double c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3];
    for (int k = 0; k < n; ++k) {
        c3 = (c2 + c0 * c3) * 0.25;
        c2 = c1 * c1 * 0.5;
        c1 = c0 * c1;
        c0 = 2. * c0 * c0 - 1.;
    }
    c[0] = c0; c[1] = c1; c[2] = c2; c[3] = c3;
    c[4] = (0.5 - c2) / z;
    c[5] = (1. / 6. - c3) / z;
}

// G_n(beta, X), n = 0..5
__host__ __device__ __forceinline__ void gfun6(double beta, double X, double G[6]) {
    double c[6];
    stumpff6(beta * X * X, c);
    double p = 1.;
    for (int k = 0; k < 6; ++k) {
        G[k] = p * c[k];
        p *= X;
    }
}

struct KeplerScalars {
    double r0, v2, beta, eta0, zeta0;
};

__host__ __device__ __forceinline__ KeplerScalars kepler_scalars(double mu, const double r[3], const double v[3]) {
    KeplerScalars s;
    s.r0 = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    s.v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    s.beta = 2. * mu / s.r0 - s.v2;
    s.eta0 = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
    s.zeta0 = mu - s.beta * s.r0;
    return s;
}

// c0..c3 only (the solver's iterations need no more): the series with the
// same truncation, quartering and doubling as stumpff6.
__host__ __device__ __forceinline__ void stumpff4(double z, double c[4]) {
    const double f[20] = {1., 1., 1. / 2., 1. / 6., 1. / 24., 1. / 120., 1. / 720., 1. / 5040., 1. / 40320.,
                          1. / 362880., 1. / 3628800., 1. / 39916800., 1. / 479001600., 1. / 6227020800.,
                          1. / 87178291200., 1. / 1307674368000., 1. / 20922789888000., 1. / 355687428096000.,
                          1. / 6402373705728000., 1. / 121645100408832000.};
    double zz = z;
    int n = 0;
    while (fabs(zz) > 0.1 && n < 64) {
        zz *= 0.25;
        ++n;
    }
    for (int k = 0; k < 4; ++k) {
        double s = f[k + 12];
        for (int j = 5; j >= 0; --j) s = f[k + 2 * j] - zz * s;
        c[k] = s;
    }
    for (int k = 0; k < n; ++k) {
        c[3] = (c[2] + c[0] * c[3]) * 0.25;
        c[2] = c[1] * c[1] * 0.5;
        c[1] = c[0] * c[1];
        c[0] = 2. * c[0] * c[0] - 1.;
    }
}

// Root of Kepler's equation in universal variables, r0 X + eta0 G2(X) +
// zeta0 G3(X) = dt, by Newton's method.  Elliptic orbits start from the
// series inversion of the equation to fourth order in u = dt / r0 (G2 = X^2/2
// - beta X^4/24 + ..., G3 = X^3/6 + ...; the reference's second-order value,
// src/integrator/whfast.rs:716-720, extended by two terms): its error is
// O(u^5), below 1e-8 relative for drifts under a tenth of an orbit.  Newton's
// convergence is quadratic with a contraction far below one here, so after
// a step below 1e-8 |X| the root is off by less than the step's square,
// below rounding, and the loop stops; *ok = false when it did not converge.
// Unbound orbits start from 0.
__host__ __device__ __forceinline__ double kepler_solve(const KeplerScalars& s, double dt, bool* ok) {
    double X = 0.;
    if (s.beta > 0.) {
        const double ir0 = 1. / s.r0;
        const double u = dt * ir0;
        const double a2 = -0.5 * s.eta0 * ir0;
        const double a3 = (0.5 * s.eta0 * s.eta0 * ir0 - s.zeta0 * (1. / 6.)) * ir0;
        const double a4 = -(s.eta0 * a3 + 0.5 * s.eta0 * a2 * a2 + 0.5 * s.zeta0 * a2 - s.eta0 * s.beta * (1. / 24.)) * ir0;
        X = u * (1. + u * (a2 + u * (a3 + u * a4)));
    }
    *ok = false;
    for (int it = 0; it < kKEPLER_MAX_NEWTON; ++it) {
        double c[4];
        stumpff4(s.beta * X * X, c);
        const double X2 = X * X;
        const double G1 = X * c[1], G2 = X2 * c[2], G3 = X2 * X * c[3];
        const double F = s.r0 * X + s.eta0 * G2 + s.zeta0 * G3 - dt;
        const double Fp = s.r0 + s.eta0 * G1 + s.zeta0 * G2;
        const double dX = F / Fp;
        X -= dX;
        if (fabs(dX) <= 1e-8 * fabs(X) || dX == 0.) {
            *ok = true;
            break;
        }
    }
    return X;
}

// (r1, v1) of the drift, given the root X.
__host__ __device__ __forceinline__ void kepler_apply(double mu, double dt, const double r[3], const double v[3],
                                                      const KeplerScalars& s, double X, double r1[3], double v1[3]) {
    double c[4], G[4];
    stumpff4(s.beta * X * X, c);
    G[0] = c[0]; G[1] = X * c[1]; G[2] = X * X * c[2]; G[3] = X * X * X * c[3];
    const double rr = s.r0 + s.eta0 * G[1] + s.zeta0 * G[2];
    const double f = -mu * G[2] / s.r0;
    const double g = dt - mu * G[3];
    const double fd = -mu * G[1] / (s.r0 * rr);
    const double gd = -mu * G[2] / rr;
    for (int k = 0; k < 3; ++k) {
        r1[k] = r[k] + (f * r[k] + g * v[k]);
        v1[k] = v[k] + (fd * r[k] + gd * v[k]);
    }
}

// Vector-Jacobian product of the drift: (lr1, lv1) -> (lr0, lv0) (assigned).
__host__ __device__ __forceinline__ void kepler_vjp(double mu, double dt, const double r[3], const double v[3],
                                                    double X, const double lr1[3], const double lv1[3], double lr0[3],
                                                    double lv0[3]) {
    const KeplerScalars s = kepler_scalars(mu, r, v);
    double G[6];
    gfun6(s.beta, X, G);
    const double r0 = s.r0;
    const double rr = r0 + s.eta0 * G[1] + s.zeta0 * G[2];
    // the two reciprocals every quotient below needs
    const double ir0 = 1. / r0, irr = 1. / rr;
    const double f = -mu * G[2] * ir0;
    const double g = dt - mu * G[3];
    const double fd = -mu * G[1] * (ir0 * irr);
    const double gd = -mu * G[2] * irr;
    double lf = 0., lg = 0., lfd = 0., lgd = 0.;
    for (int k = 0; k < 3; ++k) {
        lr0[k] = lr1[k] * (1. + f) + fd * lv1[k];
        lv0[k] = g * lr1[k] + (1. + gd) * lv1[k];
        lf += lr1[k] * r[k];
        lg += lr1[k] * v[k];
        lfd += lv1[k] * r[k];
        lgd += lv1[k] * v[k];
    }
    double lG1 = 0., lG2 = 0., lG3 = 0., lr0s = 0., lrr = 0., leta = 0., lzeta = 0., lbeta = 0.;
    // f = -mu G2 / r0
    lG2 += -mu * ir0 * lf;
    lr0s += mu * G[2] * (ir0 * ir0) * lf;
    // g = dt - mu G3
    lG3 += -mu * lg;
    // fd = -mu G1 / (r0 rr)
    lG1 += -mu * (ir0 * irr) * lfd;
    lr0s += mu * G[1] * (ir0 * ir0 * irr) * lfd;
    lrr += mu * G[1] * (ir0 * irr * irr) * lfd;
    // gd = -mu G2 / rr
    lG2 += -mu * irr * lgd;
    lrr += mu * G[2] * (irr * irr) * lgd;
    // rr = r0 + eta0 G1 + zeta0 G2
    lr0s += lrr;
    leta += G[1] * lrr;
    lG1 += s.eta0 * lrr;
    lzeta += G[2] * lrr;
    lG2 += s.zeta0 * lrr;
    // G_n(beta, X)
    const double dG1b = 0.5 * (G[3] - X * G[2]);
    const double dG2b = 0.5 * (2. * G[4] - X * G[3]);
    const double dG3b = 0.5 * (3. * G[5] - X * G[4]);
    const double lX = G[0] * lG1 + G[1] * lG2 + G[2] * lG3;
    lbeta += dG1b * lG1 + dG2b * lG2 + dG3b * lG3;
    // implicit root: F(X; r0, eta0, zeta0, beta) = 0, F_X = rr
    const double w = lX * irr;
    const double Fb = s.eta0 * dG2b + s.zeta0 * dG3b;
    lr0s += -X * w;
    leta += -G[2] * w;
    lzeta += -G[3] * w;
    lbeta += -Fb * w;
    // zeta0 = mu - beta r0
    lbeta += -r0 * lzeta;
    lr0s += -s.beta * lzeta;
    // beta = 2 mu / r0 - v2
    lr0s += -2. * mu * (ir0 * ir0) * lbeta;
    const double lv2 = -lbeta;
    const double lr0i = lr0s * ir0;
    for (int k = 0; k < 3; ++k) {
        lr0[k] += v[k] * leta + r[k] * lr0i;
        lv0[k] += r[k] * leta + 2. * v[k] * lv2;
    }
}

// Jacobian-vector product of the drift: tangent (dr, dv) of the start ->
// tangent (dr1, dv1) of the end, at the converged root X (same derivatives as
// kepler_vjp, applied forwards).
__host__ __device__ __forceinline__ void kepler_jvp(double mu, double dt, const double r[3], const double v[3],
                                                    double X, const double dr[3], const double dv[3], double dr1[3],
                                                    double dv1[3]) {
    const KeplerScalars s = kepler_scalars(mu, r, v);
    double G[6];
    gfun6(s.beta, X, G);
    const double r0 = s.r0;
    const double rr = r0 + s.eta0 * G[1] + s.zeta0 * G[2];
    const double ir0 = 1. / r0, irr = 1. / rr;
    const double f = -mu * G[2] * ir0;
    const double g = dt - mu * G[3];
    const double fd = -mu * G[1] * (ir0 * irr);
    const double gd = -mu * G[2] * irr;
    const double dr0s = (r[0] * dr[0] + r[1] * dr[1] + r[2] * dr[2]) * ir0;
    const double dv2 = 2. * (v[0] * dv[0] + v[1] * dv[1] + v[2] * dv[2]);
    const double dbeta = -2. * mu * (ir0 * ir0) * dr0s - dv2;
    const double deta = dr[0] * v[0] + dr[1] * v[1] + dr[2] * v[2] + r[0] * dv[0] + r[1] * dv[1] + r[2] * dv[2];
    const double dzeta = -s.beta * dr0s - r0 * dbeta;
    const double dG1b = 0.5 * (G[3] - X * G[2]);
    const double dG2b = 0.5 * (2. * G[4] - X * G[3]);
    const double dG3b = 0.5 * (3. * G[5] - X * G[4]);
    const double Fb = s.eta0 * dG2b + s.zeta0 * dG3b;
    const double dX = -(X * dr0s + G[2] * deta + G[3] * dzeta + Fb * dbeta) * irr;
    const double dG1 = G[0] * dX + dG1b * dbeta;
    const double dG2 = G[1] * dX + dG2b * dbeta;
    const double dG3 = G[2] * dX + dG3b * dbeta;
    const double drr = dr0s + deta * G[1] + s.eta0 * dG1 + dzeta * G[2] + s.zeta0 * dG2;
    const double df = -mu * (dG2 * r0 - G[2] * dr0s) * (ir0 * ir0);
    const double dg = -mu * dG3;
    const double den = r0 * rr, iden = ir0 * irr;
    const double dfd = -mu * (dG1 * den - G[1] * (dr0s * rr + r0 * drr)) * (iden * iden);
    const double dgd = -mu * (dG2 * rr - G[2] * drr) * (irr * irr);
    for (int k = 0; k < 3; ++k) {
        dr1[k] = dr[k] + df * r[k] + f * dr[k] + dg * v[k] + g * dv[k];
        dv1[k] = dv[k] + dfd * r[k] + fd * dr[k] + dgd * v[k] + gd * dv[k];
    }
}

// Jacobi interaction term of planet i > 0 (src/integrator/whfast.rs:566-592):
// v += dt G eta r / (|r|^2 + softening)^(3/2).
__host__ __device__ __forceinline__ void jacobi_indirect(double dt_g_eta, const double r[3], double dv[3]) {
    const double s2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + kJACOBI_SOFTENING;
    const double inv_s = 1. / sqrt(s2);
    const double p = dt_g_eta * inv_s * inv_s * inv_s;
    for (int k = 0; k < 3; ++k) dv[k] = p * r[k];
}

__host__ __device__ __forceinline__ void jacobi_indirect_vjp(double dt_g_eta, const double r[3], const double lv[3],
                                                             double lr[3]) {
    const double s2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + kJACOBI_SOFTENING;
    const double inv_s = 1. / sqrt(s2);
    const double inv_s3 = inv_s * inv_s * inv_s;
    const double rl = r[0] * lv[0] + r[1] * lv[1] + r[2] * lv[2];
    for (int k = 0; k < 3; ++k) lr[k] += dt_g_eta * (lv[k] * inv_s3 - 3. * r[k] * rl * inv_s3 / s2);
}

// Newtonian pair term of body i from body j: a_i += -G m_j (r_i - r_j) / d^3,
// and its VJP for the pair: lr_i += -G K (m_j la_i - m_i la_j),
// K u = u / d^3 - 3 D (D . u) / d^5, D = r_i - r_j.
__host__ __device__ __forceinline__ void gravity_pair(const double ri[3], const double rj[3], double mj,
                                                      double a[3]) {
    const double D0 = ri[0] - rj[0], D1 = ri[1] - rj[1], D2 = ri[2] - rj[2];
    const double d2 = D0 * D0 + D1 * D1 + D2 * D2;
    const double inv_d = 1. / sqrt(d2);
    const double p = -kG * mj * inv_d * inv_d * inv_d;
    a[0] += p * D0;
    a[1] += p * D1;
    a[2] += p * D2;
}

__host__ __device__ __forceinline__ void gravity_pair_vjp(const double ri[3], const double rj[3], double mi, double mj,
                                                          const double lai[3], const double laj[3], double lr[3]) {
    const double D[3] = {ri[0] - rj[0], ri[1] - rj[1], ri[2] - rj[2]};
    const double d2 = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
    const double inv_d = 1. / sqrt(d2);
    const double inv_d3 = inv_d * inv_d * inv_d;
    double u[3];
    for (int k = 0; k < 3; ++k) u[k] = mj * lai[k] - mi * laj[k];
    const double du = D[0] * u[0] + D[1] * u[1] + D[2] * u[2];
    for (int k = 0; k < 3; ++k) lr[k] += -kG * (u[k] * inv_d3 - 3. * D[k] * du * inv_d3 / d2);
}

}  // namespace posi_adj
