// large_device.cuh -- WHFast for one system of many bodies (FP64).
//
// The batched kernels map a system onto one lane group (at most 32 bodies).
// A system of hundreds or thousands of bodies -- a star, tidally active
// planets and a swarm of small massive bodies -- runs here instead: one
// persistent cooperative grid (one block per SM) integrates it for K steps.
//
// * Thread i owns body i for the whole launch (its state in registers).  The
//   host body's state is kept, redundantly and identically, by every thread,
//   so that the implicit-midpoint loop needs no broadcast.
// * Reductions over bodies (host back-reactions, midpoint convergence,
//   barycentre and momentum sums of the democratic-heliocentric transforms)
//   are block sums written to a per-block slot and added in block order by
//   every thread after a grid barrier: deterministic, run to run.
// * Gravity (src/particles/universe.rs:198-303, all ordered pairs, WHFastTwo
//   skip of the host) spreads the O(N^2) pair loop over every thread of the
//   grid: thread t sums body (t mod N) over the t / N-th slice of the partner
//   bodies; the slices are added in order.  The collision, Roche and
//   ejection checks of the same loop report the first offending pair in the
//   reference's (i, j) order.
// * Grid barriers are counters in global memory with a bounded wait: a wait
//   that runs out sets an error flag and every thread leaves the kernel.
//
// Coordinates: democratic heliocentric (src/integrator/whfast.rs:495-530,
// 965-1024, 1082-1155).  Effects: constant-time-lag tides, oblate
// flattening, Kidder GR for orbiting bodies of a central host, in the FAST
// formulation (the generated blocks of adjoint_effects.cuh); non-evolving
// bodies.  Kepler drift: universal variables (adjoint_blocks.cuh).
#pragma once
#include <cstdint>

#include "../../include/posidonius_gb300.h"
#include "adjoint_effects.cuh"

namespace posi_many {

using namespace posi_adj;

constexpr int kBlock = 256;
constexpr double kMAX_DISTANCE_2 = 100. * 100.;
constexpr long long kBarrierSpinLimit = 1LL << 25;  // x 64 ns sleeps: about 2 s

enum { BP_SLOTS = 16 };  // per-block partial sums
enum { LE_BARRIER = 1, LE_KEPLER = 2, LE_ZERO_INERTIA = 4 };

struct LDev {
    int64_t n;
    double* bf;             // [POSI_BF_COUNT][n]
    const int64_t* bi;      // [POSI_BI_COUNT][n]
    double* sf;             // [POSI_SF_COUNT]
    int64_t* si;            // [POSI_SI_COUNT]
    const double* roche;    // [n][n] (symmetric)
    double* pos;            // [3][n] positions for the pair loop
    double* gpart;          // [nchunk][3][n] partial accelerations
    double* bpart;          // [gridDim.x][BP_SLOTS]
    unsigned* bar;          // [2] arrival count, generation
    int* err;               // error flags (LE_*)
    unsigned long long* bad;  // first failing pair: min over (i n + j) * 4 + code; all ones if none
    int nchunk;
};

// Sum of v over the block into slot s of this block's partial row; called by
// every thread of the block with its own contribution (0 when it has none).
__device__ __forceinline__ void block_partial(double* bpart, double (&vals)[BP_SLOTS], int nslots, double* shm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < nslots; ++k) {
        double x = vals[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) shm[warp * BP_SLOTS + k] = x;
    }
    __syncthreads();
    if (threadIdx.x < nslots) {
        double acc = 0.;
        for (int w = 0; w < kBlock / 32; ++w) acc += shm[w * BP_SLOTS + threadIdx.x];
        bpart[(size_t)blockIdx.x * BP_SLOTS + threadIdx.x] = acc;
    }
    __syncthreads();
}

// Totals of the block partials, in block order (every thread, same result).
__device__ __forceinline__ void block_totals(const double* bpart, double* out, int nslots) {
    for (int k = 0; k < nslots; ++k) out[k] = 0.;
    for (unsigned b = 0; b < gridDim.x; ++b)
        for (int k = 0; k < nslots; ++k) out[k] += __ldcg(&bpart[(size_t)b * BP_SLOTS + k]);
}

// Grid-wide barrier with a bounded wait.  Returns false (and flags the error)
// when the wait ran out; callers then leave the kernel.
__device__ bool grid_barrier(const LDev& D) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = D.bar + 1;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(D.bar, 1u) + 1u;
        int ok = 1;
        if (arrived == gridDim.x) {
            D.bar[0] = 0u;
            __threadfence();
            atomicAdd(D.bar + 1, 1u);
        } else {
            long long spins = 0;
            while (*gen == g) {
                if (++spins > kBarrierSpinLimit || (*(volatile int*)D.err & LE_BARRIER)) {
                    ok = 0;
                    atomicOr(D.err, LE_BARRIER);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

struct BodyConst {
    double m, mg, R, moi, sig, k2, k2f;
    int tk, fk, gk;
};

__device__ __forceinline__ BodyConst load_const(const LDev& D, int64_t i) {
    BodyConst c;
    const int64_t n = D.n;
    c.m = D.bf[POSI_BF_MASS * n + i];
    c.mg = D.bf[POSI_BF_MASS_G * n + i];
    c.R = D.bf[POSI_BF_RADIUS * n + i];
    c.moi = D.bf[POSI_BF_MOI * n + i];
    c.sig = D.bf[POSI_BF_SIGMA * n + i];
    c.k2 = D.bf[POSI_BF_K2 * n + i];
    c.k2f = D.bf[POSI_BF_K2F * n + i];
    c.tk = (int)D.bi[POSI_BI_TIDES_KIND * n + i];
    c.fk = (int)D.bi[POSI_BI_FLAT_KIND * n + i];
    c.gk = (int)D.bi[POSI_BI_GR_KIND * n + i];
    return c;
}

struct BodyState {
    double r[3], v[3], L[3], S[3], ev[3], eL[3];
};

__device__ __forceinline__ void load_state(const LDev& D, int64_t i, BodyState& b) {
    const int64_t n = D.n;
    for (int c = 0; c < 3; ++c) {
        b.r[c] = D.bf[(POSI_BF_PX + c) * n + i];
        b.v[c] = D.bf[(POSI_BF_VX + c) * n + i];
        b.L[c] = D.bf[(POSI_BF_LX + c) * n + i];
        b.S[c] = D.bf[(POSI_BF_SX + c) * n + i];
        b.ev[c] = D.bf[(POSI_BF_EVX + c) * n + i];
        b.eL[c] = D.bf[(POSI_BF_ELX + c) * n + i];
    }
}

struct Large {
    const LDev& D;
    int64_t n, i;
    int host;
    bool has, is_host, planet;
    bool tides, flat, gr;
    double dt, half_dt, t, time_limit, last_hist, hist_period;
    BodyConst c, hc;        // own and host constants
    BodyState b, h;         // own and host state (host: redundant copy)
    double a[3];            // gravity acceleration (own)
    double* shm;
    double Mtot;

    __device__ Large(const LDev& D_, double* shm_) : D(D_), shm(shm_) {}

    __device__ __forceinline__ bool tides_on() const { return tides && c.tk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool flat_on() const { return flat && c.fk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool gr_on() const { return gr && c.gk == POSI_EFFECT_ORBITING; }

    __device__ static void spin_of(const BodyConst& k, const double L[3], double S[3]) {
        if (k.moi != 0.) {
            const double im = 1. / k.moi;
            for (int q = 0; q < 3; ++q) S[q] = L[q] * im;
        } else {
            for (int q = 0; q < 3; ++q) S[q] = 0.;
        }
    }

    // ---- implicit midpoint (src/integrator/whfast.rs:322-466) ----
    __device__ bool midpoint(double hdt) {
        double x[3] = {0., 0., 0.};
        Pre pr;
        if (planet) {
            for (int q = 0; q < 3; ++q) x[q] = b.r[q] - h.r[q];
            if (tides_on()) adj_tides_pre(x[0], x[1], x[2], c.sig, hc.sig, c.k2, hc.k2, c.R, hc.R, hc.m, c.m, pr.t);
            if (flat_on()) adj_flat_pre(x[0], x[1], x[2], c.R, hc.R, hc.k2f, hc.m, c.k2f, c.m, pr.f);
            if (gr_on()) adj_gr_pre(x[0], x[1], x[2], hc.m, hc.mg, hc.moi, c.m, c.mg, c.moi, pr.g);
        }
        const double mr = planet ? c.m / hc.m : 0.;
        // own and host: original, current, previous-final, previous spin
        double v0[3], L0[3], vc[3], Lc[3], vf[3], Lf[3], pv[3], pL[3], Sp[3], Sc[3], dvc[3], dLc[3];
        double hv0[3], hL0[3], hvc[3], hLc[3], hvf[3], hLf[3], hpv[3], hpL[3], hSp[3], hSc[3], hdvc[3], hdLc[3];
        for (int q = 0; q < 3; ++q) {
            v0[q] = vc[q] = vf[q] = b.v[q]; L0[q] = Lc[q] = Lf[q] = b.L[q]; Sp[q] = b.S[q];
            hv0[q] = hvc[q] = hvf[q] = h.v[q]; hL0[q] = hLc[q] = hLf[q] = h.L[q]; hSp[q] = h.S[q];
            dvc[q] = dLc[q] = hdvc[q] = hdLc[q] = 0.;
        }
        for (int it = 0; it < kMIDPOINT_MAX; ++it) {
            for (int q = 0; q < 3; ++q) { pv[q] = vf[q]; pL[q] = Lf[q]; hpv[q] = hvf[q]; hpL[q] = hLf[q]; }
            spin_of(c, Lc, Sc);
            spin_of(hc, hLc, hSc);
            double aa[3] = {0., 0., 0.}, dl[3] = {0., 0., 0.}, th[3] = {0., 0., 0.};
            if (planet) {
                const double h0 = vc[0] - hvc[0], h1 = vc[1] - hvc[1], h2 = vc[2] - hvc[2];
                double out[9];
                if (tides_on()) {
                    adj_tides_iter(pr.t, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0], Sp[1], Sp[2],
                                   hSp[0], hSp[1], hSp[2], c.R, hc.R, hc.m, c.m, out);
                    for (int q = 0; q < 3; ++q) { aa[q] += out[q]; dl[q] += out[3 + q]; th[q] += out[6 + q]; }
                }
                if (flat_on()) {
                    adj_flat_iter(pr.f, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0], Sp[1], Sp[2],
                                  hSp[0], hSp[1], hSp[2], c.R, hc.R, hc.k2f, hc.m, c.k2f, c.m, out);
                    for (int q = 0; q < 3; ++q) { aa[q] += out[q]; dl[q] += out[3 + q]; th[q] += out[6 + q]; }
                }
                if (gr_on()) {
                    adj_gr_iter(pr.g, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0], Sp[1], Sp[2],
                                hSp[0], hSp[1], hSp[2], hc.m, hc.mg, hc.moi, c.m, c.mg, c.moi, out);
                    for (int q = 0; q < 3; ++q) { aa[q] += out[q]; dl[q] += out[3 + q]; th[q] += out[6 + q]; }
                }
            }
            double vals[BP_SLOTS] = {};
            for (int q = 0; q < 3; ++q) { vals[q] = mr * aa[q]; vals[3 + q] = th[q]; }
            block_partial(D.bpart, vals, 6, shm);
            if (!grid_barrier(D)) return false;
            double tot[6];
            block_totals(D.bpart, tot, 6);
            // the host's outputs, computed by every thread
            double haa[3], hdl[3];
            for (int q = 0; q < 3; ++q) { haa[q] = -tot[q]; hdl[q] = tot[3 + q]; }
            if (is_host)
                for (int q = 0; q < 3; ++q) { aa[q] = haa[q]; dl[q] = hdl[q]; }
            for (int q = 0; q < 3; ++q) {
                dvc[q] = hdt * aa[q] - b.ev[q];
                vf[q] = v0[q] + dvc[q];
                dLc[q] = hdt * dl[q] - b.eL[q];
                Lf[q] = L0[q] + dLc[q];
                hdvc[q] = hdt * haa[q] - h.ev[q];
                hvf[q] = hv0[q] + hdvc[q];
                hdLc[q] = hdt * hdl[q] - h.eL[q];
                hLf[q] = hL0[q] + hdLc[q];
            }
            if (it >= kMIDPOINT_MIN - 1) {
                double cv[BP_SLOTS] = {};
                if (has) {
                    for (int q = 0; q < 3; ++q) {
                        cv[0] += (vf[q] - pv[q]) * (vf[q] - pv[q]);
                        cv[1] += vf[q] * vf[q];
                        cv[2] += (Lf[q] - pL[q]) * (Lf[q] - pL[q]);
                        cv[3] += Lf[q] * Lf[q];
                    }
                }
                block_partial(D.bpart, cv, 4, shm);
                if (!grid_barrier(D)) return false;
                double s4[4];
                block_totals(D.bpart, s4, 4);
                if (s4[0] / s4[1] < kDBL_EPSILON_2 && (s4[3] == 0. || s4[2] / s4[3] < kDBL_EPSILON_2)) break;
            }
            for (int q = 0; q < 3; ++q) {
                vc[q] = 0.5 * (v0[q] + vf[q]);
                Lc[q] = 0.5 * (L0[q] + Lf[q]);
                Sp[q] = Sc[q];
                hvc[q] = 0.5 * (hv0[q] + hvf[q]);
                hLc[q] = 0.5 * (hL0[q] + hLf[q]);
                hSp[q] = hSc[q];
            }
        }
        for (int q = 0; q < 3; ++q) {
            b.v[q] = vf[q]; b.L[q] = Lf[q]; b.S[q] = Sc[q];
            b.ev[q] = (vf[q] - v0[q]) - dvc[q];
            b.eL[q] = (Lf[q] - L0[q]) - dLc[q];
            h.v[q] = hvf[q]; h.L[q] = hLf[q]; h.S[q] = hSc[q];
            h.ev[q] = (hvf[q] - hv0[q]) - hdvc[q];
            h.eL[q] = (hLf[q] - hL0[q]) - hdLc[q];
        }
        if (is_host) b = h;
        return true;
    }

    struct Pre {
        double t[adj_tides_NPRE], f[adj_flat_NPRE], g[adj_gr_NPRE];
    };

    // ---- gravity over all ordered pairs, with the pair checks ----
    __device__ bool gravity() {
        const int64_t nn = n;
        if (has)
            for (int q = 0; q < 3; ++q) D.pos[q * nn + i] = b.r[q];
        if (!grid_barrier(D)) return false;
        const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        const int64_t gi = tid % nn, chunk = tid / nn;
        if (chunk < D.nchunk) {
            const int64_t j0 = chunk * nn / D.nchunk, j1 = (chunk + 1) * nn / D.nchunk;
            const double xi = __ldcg(&D.pos[gi]), yi = __ldcg(&D.pos[nn + gi]), zi = __ldcg(&D.pos[2 * nn + gi]);
            const double Ri = D.bf[POSI_BF_RADIUS * nn + gi];
            double ax = 0., ay = 0., az = 0.;
            unsigned long long bad = ~0ull;
            for (int64_t j = j0; j < j1; ++j) {
                if (j == gi) continue;
                const double dx = xi - __ldcg(&D.pos[j]), dy = yi - __ldcg(&D.pos[nn + j]),
                             dz = zi - __ldcg(&D.pos[2 * nn + j]);
                const double d2 = dx * dx + dy * dy + dz * dz;
                if (gi < j && bad == ~0ull) {
                    const double rr = D.roche[gi * nn + j];
                    const double Rs = Ri + D.bf[POSI_BF_RADIUS * nn + j];
                    const unsigned long long key = (unsigned long long)(gi * nn + j) * 4ull;
                    if (d2 <= rr * rr) bad = key + POSI_SYS_ROCHE;
                    else if (d2 <= Rs * Rs) bad = key + POSI_SYS_COLLISION;
                    else if (gi == host && d2 > kMAX_DISTANCE_2) bad = key + POSI_SYS_EJECTED;
                }
                if (gi == host || j == host) continue;  // WHFastTwo
                const double inv_d = rsqrt(d2);
                const double p = -kG * D.bf[POSI_BF_MASS * nn + j] * (inv_d * inv_d * inv_d);
                ax += p * dx; ay += p * dy; az += p * dz;
            }
            D.gpart[(chunk * 3 + 0) * nn + gi] = ax;
            D.gpart[(chunk * 3 + 1) * nn + gi] = ay;
            D.gpart[(chunk * 3 + 2) * nn + gi] = az;
            if (bad != ~0ull) atomicMin(D.bad, bad);
        }
        if (!grid_barrier(D)) return false;
        if (has) {
            for (int q = 0; q < 3; ++q) {
                double acc = 0.;
                for (int k = 0; k < D.nchunk; ++k) acc += __ldcg(&D.gpart[(k * 3 + q) * nn + i]);
                a[q] = acc;
            }
        }
        return true;
    }

    // sums over all bodies (host included) of m * w, for 1 or 2 vectors
    __device__ bool msum(const double w1[3], const double* w2, bool with_host, double out[6]) {
        double vals[BP_SLOTS] = {};
        const bool take = has && (with_host || !is_host);
        for (int q = 0; q < 3; ++q) {
            vals[q] = take ? c.m * w1[q] : 0.;
            vals[3 + q] = (take && w2) ? c.m * w2[q] : 0.;
        }
        block_partial(D.bpart, vals, w2 ? 6 : 3, shm);
        if (!grid_barrier(D)) return false;
        block_totals(D.bpart, out, w2 ? 6 : 3);
        return true;
    }

    // ---- one step (src/integrator/whfast.rs:235-305), democratic heliocentric ----
    __device__ bool step() {
        const bool first = last_hist < 0.;
        if (first || last_hist + hist_period <= t) {
            spin_of(c, b.L, b.S);
            spin_of(hc, h.L, h.S);
            last_hist = first ? 0. : last_hist + hist_period;
        }
        if (!midpoint(half_dt)) return false;
        // inertial -> democratic heliocentric (barycentre and its velocity)
        double tot[6];
        if (!msum(b.r, b.v, true, tot)) return false;
        double Rc[3], Vc[3];
        for (int q = 0; q < 3; ++q) { Rc[q] = tot[q] / Mtot; Vc[q] = tot[3 + q] / Mtot; }
        double x[3] = {0., 0., 0.}, u[3] = {0., 0., 0.};
        if (planet)
            for (int q = 0; q < 3; ++q) { x[q] = b.r[q] - h.r[q]; u[q] = b.v[q] - Vc[q]; }
        // Kepler drift, barycentre drift, jump
        if (!drift(x, u, Rc, Vc)) return false;
        // back to inertial
        if (!to_inertial(x, u, Rc, Vc)) return false;
        if (!gravity()) return false;
        if (__ldcg(D.bad) != ~0ull) return false;  // frozen at the first failing pair
        // interaction: u += dt a (inertial accelerations)
        if (planet)
            for (int q = 0; q < 3; ++q) u[q] += dt * a[q];
        if (!jump(x, u)) return false;
        if (!kepler(x, u)) return false;
        for (int q = 0; q < 3; ++q) Rc[q] += half_dt * Vc[q];
        if (!to_inertial(x, u, Rc, Vc)) return false;
        if (!midpoint(half_dt)) return false;
        t += dt;
        return true;
    }

    __device__ bool kepler(double x[3], double u[3]) {
        if (planet) {
            const KeplerScalars ks = kepler_scalars(hc.mg, x, u);
            bool ok = false;
            const double X = kepler_solve(ks, half_dt, &ok);
            if (!ok) atomicOr(D.err, LE_KEPLER);
            double r1[3], v1[3];
            kepler_apply(hc.mg, half_dt, x, u, ks, X, r1, v1);
            for (int q = 0; q < 3; ++q) { x[q] = r1[q]; u[q] = v1[q]; }
        }
        return true;
    }

    // src/integrator/whfast.rs:507-530: x += dt/2 * sum_p m_p u_p / m_host
    __device__ bool jump(double x[3], double u[3]) {
        double P[6];
        if (!msum(u, nullptr, false, P)) return false;
        if (planet)
            for (int q = 0; q < 3; ++q) x[q] += half_dt * P[q] / hc.m;
        return true;
    }

    __device__ bool drift(double x[3], double u[3], double Rc[3], const double Vc[3]) {
        kepler(x, u);
        for (int q = 0; q < 3; ++q) Rc[q] += half_dt * Vc[q];
        return jump(x, u);
    }

    // src/integrator/whfast.rs:1082-1155
    __device__ bool to_inertial(const double x[3], const double u[3], const double Rc[3], const double Vc[3]) {
        double tot[6];
        if (!msum(x, u, false, tot)) return false;
        for (int q = 0; q < 3; ++q) {
            h.r[q] = Rc[q] - tot[q] / Mtot;
            h.v[q] = Vc[q] - tot[3 + q] / hc.m;
        }
        if (planet)
            for (int q = 0; q < 3; ++q) { b.r[q] = x[q] + h.r[q]; b.v[q] = u[q] + Vc[q]; }
        if (is_host)
            for (int q = 0; q < 3; ++q) { b.r[q] = h.r[q]; b.v[q] = h.v[q]; }
        return true;
    }
};

__global__ void __launch_bounds__(kBlock) large_steps_kernel(LDev D, int64_t n_steps) {
    __shared__ double shm[(kBlock / 32) * BP_SLOTS];
    Large S(D, shm);
    S.n = D.n;
    S.i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    S.host = (int)D.si[POSI_SI_HOST];
    S.has = S.i < S.n;
    S.is_host = S.has && S.i == S.host;
    S.planet = S.has && !S.is_host;
    S.tides = D.si[POSI_SI_TIDES] != 0;
    S.flat = D.si[POSI_SI_FLAT] != 0;
    S.gr = D.si[POSI_SI_GR] != 0;
    S.dt = D.sf[POSI_SF_DT];
    S.half_dt = D.sf[POSI_SF_HALF_DT];
    S.t = D.sf[POSI_SF_TIME];
    S.time_limit = D.sf[POSI_SF_TIME_LIMIT];
    S.last_hist = D.sf[POSI_SF_LAST_HIST];
    S.hist_period = D.sf[POSI_SF_HIST_PERIOD];
    S.a[0] = S.a[1] = S.a[2] = 0.;
    S.hc = load_const(D, S.host);
    load_state(D, S.host, S.h);
    if (S.has) {
        S.c = load_const(D, S.i);
        load_state(D, S.i, S.b);
    } else {
        S.c = S.hc;
        S.b = S.h;
    }
    // total mass, in block order
    {
        double vals[BP_SLOTS] = {};
        vals[0] = S.has ? S.c.m : 0.;
        block_partial(D.bpart, vals, 1, shm);
        if (!grid_barrier(D)) return;
        double tot[1];
        block_totals(D.bpart, tot, 1);
        S.Mtot = tot[0];
    }
    const bool live = (D.si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK) == 0;
    int64_t done = 0;
    bool ok = true;
    if (live) {
        for (int64_t k = 0; k < n_steps; ++k) {
            ok = S.step();
            if (!ok) break;
            ++done;
            if (S.t + S.dt > S.time_limit) break;
        }
    }
    if (__ldcg(D.err) & LE_BARRIER) return;  // state left as it was: the launch failed
    if (S.has) {
        const int64_t n = S.n, i = S.i;
        for (int q = 0; q < 3; ++q) {
            D.bf[(POSI_BF_PX + q) * n + i] = S.b.r[q];
            D.bf[(POSI_BF_VX + q) * n + i] = S.b.v[q];
            D.bf[(POSI_BF_LX + q) * n + i] = S.b.L[q];
            D.bf[(POSI_BF_SX + q) * n + i] = S.b.S[q];
            D.bf[(POSI_BF_EVX + q) * n + i] = S.b.ev[q];
            D.bf[(POSI_BF_ELX + q) * n + i] = S.b.eL[q];
            D.bf[(POSI_BF_AX + q) * n + i] = S.a[q];
        }
        D.bf[POSI_BF_NSV2 * n + i] = S.b.S[0] * S.b.S[0] + S.b.S[1] * S.b.S[1] + S.b.S[2] * S.b.S[2];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && live) {
        D.sf[POSI_SF_TIME] = S.t;
        D.sf[POSI_SF_LAST_HIST] = S.last_hist;
        D.si[POSI_SI_ITERATION] += done;
        const unsigned long long key = __ldcg(D.bad);
        if (key != ~0ull) {
            D.si[POSI_SI_STATUS] = (D.si[POSI_SI_STATUS] & ~(int64_t)POSI_SYS_FATAL_MASK) | (int64_t)(key & 3ull);
            D.si[POSI_SI_FAIL_STEP] = D.si[POSI_SI_ITERATION];
            D.si[POSI_SI_FAIL_PAIR] = (int64_t)(key >> 2);
        } else if (S.t + S.dt > S.time_limit) {
            D.si[POSI_SI_STATUS] = (D.si[POSI_SI_STATUS] & ~(int64_t)POSI_SYS_FATAL_MASK) | POSI_SYS_COMPLETED;
        }
    }
}

}  // namespace posi_many
