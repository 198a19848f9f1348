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
// * large_steps_kernel<NT> with NT > 0 carries forward-mode tangents of the
//   state along NT directions (derivatives with respect to initial state,
//   dissipation factors and Love numbers); NT = 0 is the plain integration.
//
// Coordinates: democratic heliocentric (src/integrator/whfast.rs:495-530,
// 965-1024, 1082-1155).  Effects: constant-time-lag tides, oblate
// flattening, Kidder GR for orbiting bodies of a central host, in the FAST
// formulation (the generated blocks of adjoint_effects.cuh); non-evolving
// bodies.  Kepler drift: universal variables (adjoint_blocks.cuh).
#pragma once
#include <cstdint>

#include <cuda/atomic>

#include "../../include/posidonius_gb300.h"
#include "adjoint_effects.cuh"

namespace posi_many {

using namespace posi_adj;

constexpr int kBlock = 256;
constexpr double kMAX_DISTANCE_2 = 100. * 100.;
constexpr long long kBarrierWaitCycles = 4000000000LL;  // about 2 s at the maximum SM clock

// Value slots of a reduction: 16 in the plain engine; with NT tangent
// directions a reduction carries 10 + 6 NT values.  Partial rows are BP_ROW
// doubles apart whatever the count.
enum { BP_SLOTS = 16, BP_ROW = 40 };
constexpr int kMaxTangents = 4;
constexpr int slots_for(int nt) { return nt == 0 ? BP_SLOTS : 10 + 6 * nt; }
static_assert(slots_for(kMaxTangents) <= BP_ROW, "partial row too short");
enum { LE_BARRIER = 1, LE_KEPLER = 2, LE_ZERO_INERTIA = 4 };
enum { SEED_SIGMA = POSI_SEED_SIGMA, SEED_K2 = POSI_SEED_K2 };  // parameters a tangent direction can perturb

struct LDev {
    int64_t n;
    double* bf;             // [POSI_BF_COUNT][n]
    const int64_t* bi;      // [POSI_BI_COUNT][n]
    double* sf;             // [POSI_SF_COUNT]
    int64_t* si;            // [POSI_SI_COUNT]
    const double* roche;    // [n][n] (symmetric)
    double* pos;            // [3][n] positions for the pair loop
    double* gpart;          // [nchunk][3 (1 + NT)][n] partial accelerations (and their tangents)
    double* bpart;          // [gridDim.x][BP_ROW]
    double* tot;            // [BP_ROW] totals of the last reduction
    unsigned* bar;          // [2] arrival count, generation
    int* err;               // error flags (LE_*)
    unsigned long long* bad;  // first failing pair: min over (i n + j) * 4 + code; all ones if none
    int nchunk;
    int per_block;          // bodies per block: body i is thread i % per_block of block i / per_block
    // tangent directions (the tangent kernels only)
    double* tan;            // [NT][12][n] tangents of r, v, L, S; read at launch, written back at the end
    double* dpos;           // [NT][3][n] position tangents for the pair loop
    int seed_body[kMaxTangents];   // body whose parameter direction k perturbs by a unit rate, or -1
    int seed_param[kMaxTangents];  // SEED_SIGMA (dissipation factor) or SEED_K2 (Love number)
};

// Sum of vals over the block into this block's partial row.  Only warps
// that own bodies (active = the warp has a body) add: a warp's FP64 add holds
// its SMSP's FP64 pipe 64 cycles, so the trees of empty warps would cost as
// much as real ones; empty warps contribute zeros.
template <int NS>
__device__ __forceinline__ void block_partial(double* bpart, const double (&vals)[NS], int nslots, double* shm,
                                              bool warp_active) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp_active) {
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            if (k < nslots) {
                double x = vals[k];
                for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
                if (lane == 0) shm[warp * BP_ROW + k] = x;
            }
        }
    }
    __syncthreads();
    // the warps that own bodies are the first ones of the block
    const int nw = __syncthreads_count(warp_active && lane == 0);
    if (threadIdx.x < nslots && nw > 0) {
        double acc = shm[threadIdx.x];
        for (int w = 1; w < nw; ++w) acc += shm[w * BP_ROW + threadIdx.x];
        bpart[(size_t)blockIdx.x * BP_ROW + threadIdx.x] = acc;
    }
    __syncthreads();
}

// Grid-wide barrier with a bounded wait: thread 0 of each block arrives with
// a release-acquire add on the arrival count; the last block resets it and
// releases the generation, the others poll it with acquire loads.  Returns
// false (and flags the error) when the wait ran out; callers then leave the
// kernel.
__device__ bool grid_barrier(const LDev& D) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> count(D.bar[0]), gen(D.bar[1]);
        cuda::atomic_ref<int, cuda::thread_scope_device> err(*D.err);
        const unsigned g = gen.load(cuda::memory_order_relaxed);
        int ok = 1;
        if (count.fetch_add(1u, cuda::memory_order_acq_rel) + 1u == gridDim.x) {
            count.store(0u, cuda::memory_order_relaxed);
            gen.fetch_add(1u, cuda::memory_order_release);
        } else {
            const long long start = clock64();
            while (gen.load(cuda::memory_order_relaxed) == g) {
                if (clock64() - start > kBarrierWaitCycles || (err.load(cuda::memory_order_relaxed) & LE_BARRIER)) {
                    ok = 0;
                    err.fetch_or(LE_BARRIER, cuda::memory_order_relaxed);
                    break;
                }
                __nanosleep(20);
            }
            cuda::atomic_thread_fence(cuda::memory_order_acquire, cuda::thread_scope_device);
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// Grid-wide sum: every block writes its partial row and arrives; the last
// block to arrive adds the rows in block order (first warp, fixed butterfly),
// publishes the totals and releases the others, which then read them once per
// block.  One barrier, and only one block reads the partial rows.
template <int NS>
__device__ bool grid_reduce(const LDev& D, const double (&vals)[NS], int nslots, double* out, double* shm,
                            bool warp_active, unsigned rows) {
    __shared__ int last_s, ok_s;
    __shared__ unsigned gen_s;
    block_partial(D.bpart, vals, nslots, shm, warp_active);
    if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> count(D.bar[0]), gen(D.bar[1]);
        gen_s = gen.load(cuda::memory_order_relaxed);
        last_s = count.fetch_add(1u, cuda::memory_order_acq_rel) + 1u == gridDim.x;
    }
    __syncthreads();
    int ok = 1;
    if (last_s) {
        // slot k is added by warp k mod 8 (the warps sit on different
        // SMSPs); lane l takes rows l, l + 32, ... of the blocks that own
        // bodies (the other rows are zero), then a fixed butterfly
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int k = warp; k < nslots; k += kBlock / 32) {
            double x = 0.;
            for (unsigned b = lane; b < rows; b += 32) x += __ldcg(D.bpart + (size_t)b * BP_ROW + k);
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) D.tot[k] = x;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            cuda::atomic_ref<unsigned, cuda::thread_scope_device> count(D.bar[0]), gen(D.bar[1]);
            count.store(0u, cuda::memory_order_relaxed);
            gen.fetch_add(1u, cuda::memory_order_release);
        }
    } else if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> gen(D.bar[1]);
        cuda::atomic_ref<int, cuda::thread_scope_device> err(*D.err);
        const long long start = clock64();
        while (gen.load(cuda::memory_order_relaxed) == gen_s) {
            if (clock64() - start > kBarrierWaitCycles || (err.load(cuda::memory_order_relaxed) & LE_BARRIER)) {
                ok = 0;
                err.fetch_or(LE_BARRIER, cuda::memory_order_relaxed);
                break;
            }
            __nanosleep(20);
        }
        cuda::atomic_thread_fence(cuda::memory_order_acquire, cuda::thread_scope_device);
    }
    if (threadIdx.x == 0) {
        ok_s = ok;
        for (int k = 0; k < nslots; ++k) shm[(kBlock / 32) * BP_ROW + k] = __ldcg(D.tot + k);
    }
    __syncthreads();
    for (int k = 0; k < nslots; ++k) out[k] = shm[(kBlock / 32) * BP_ROW + k];
    const bool r = ok_s != 0;
    __syncthreads();
    return r;
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

// Tangents of one body's state along NT directions ([component][direction]).
template <int NT>
struct Tangents {
    static constexpr int A = NT > 0 ? NT : 1;
    double r[3][A], v[3][A], L[3][A], S[3][A];
};

// One thread of the engine.  NT = 0: the plain integration.  NT > 0: the
// same integration carrying the forward-mode derivatives (tangents) of every
// body's state along NT directions -- the derivative of the step map applied
// to the incoming tangents, plus the unit rate of change of the seeded
// parameter (a body's dissipation factor or Love number) where the seeded
// body's tides enter.  The primal arithmetic is the plain engine's, in the
// same order; the midpoint convergence tests only the primal values.  The
// compensated (Kahan) error terms of the kick carry no tangent.
template <int NT>
struct Large {
    static constexpr int A = NT > 0 ? NT : 1;   // extent of the direction index
    static constexpr int NS = slots_for(NT);    // value slots of the reductions
    const LDev& D;
    int64_t n, i;
    int host;
    bool has, is_host, planet;
    bool tides, flat, gr;
    double dt, half_dt, t, time_limit, last_hist, hist_period;
    BodyConst c, hc;        // own and host constants
    BodyState b, h;         // own and host state (host: redundant copy)
    double a[3];            // gravity acceleration (own)
    Tangents<NT> T, HT;     // own and host tangents (host: redundant copy)
    double da[3][A];        // tangent of the gravity acceleration
    double* shm;
    double Mtot, inv_M, inv_hm;
    bool warp_bodies;       // this thread's warp owns at least one body
    unsigned body_rows;     // blocks that own bodies (the partial rows that can be nonzero)

    __device__ Large(const LDev& D_, double* shm_) : D(D_), shm(shm_) {}

    __device__ __forceinline__ bool tides_on() const { return tides && c.tk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool flat_on() const { return flat && c.fk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool gr_on() const { return gr && c.gk == POSI_EFFECT_ORBITING; }

    // unit rate of the seeded parameter of direction k for body j
    __device__ __forceinline__ double seed(int k, int param, int64_t j) const {
        return (D.seed_body[k] == j && D.seed_param[k] == param) ? 1. : 0.;
    }

    __device__ static void spin_of(const BodyConst& k, const double L[3], double S[3]) {
        if (k.moi != 0.) {
            const double im = 1. / k.moi;
            for (int q = 0; q < 3; ++q) S[q] = L[q] * im;
        } else {
            for (int q = 0; q < 3; ++q) S[q] = 0.;
        }
    }

    __device__ static void dspin_of(const BodyConst& k, const double (&dL)[3][A], double (&dS)[3][A]) {
        const double im = k.moi != 0. ? 1. / k.moi : 0.;
        for (int q = 0; q < 3; ++q)
            for (int d = 0; d < NT; ++d) dS[q][d] = dL[q][d] * im;
    }

    struct Pre {
        double t[adj_tides_NPRE], f[adj_flat_NPRE], g[adj_gr_NPRE];
    };
    struct DPre {
        double t[adj_tides_NPRE * A], f[adj_flat_NPRE * A], g[adj_gr_NPRE * A];
    };

    // ---- implicit midpoint (src/integrator/whfast.rs:322-466) ----
    // With cm != nullptr the last convergence reduction also carries the sums
    // of m r and m v over all bodies at the final velocities (cm[0..5]), and
    // their tangents (dcm).
    __device__ bool midpoint(double hdt, double* cm, double (*dcm)[A]) {
        double x[3] = {0., 0., 0.};
        Pre pr;
        DPre dpr;
        if (planet) {
            for (int q = 0; q < 3; ++q) x[q] = b.r[q] - h.r[q];
            if (tides_on()) adj_tides_pre(x[0], x[1], x[2], c.sig, hc.sig, c.k2, hc.k2, c.R, hc.R, hc.m, c.m, pr.t);
            if (flat_on()) adj_flat_pre(x[0], x[1], x[2], c.R, hc.R, hc.k2f, hc.m, c.k2f, c.m, pr.f);
            if (gr_on()) adj_gr_pre(x[0], x[1], x[2], hc.m, hc.mg, hc.moi, c.m, c.mg, c.moi, pr.g);
            if constexpr (NT > 0) {
                // din[p * NT + d]: tangent d of pre input p (x, y, z, sig_p, sig_h, k2_p, k2_h)
                double din[7 * A], scratch[adj_gr_NPRE];
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) din[q * NT + d] = T.r[q][d] - HT.r[q][d];
                for (int d = 0; d < NT; ++d) {
                    din[3 * NT + d] = seed(d, SEED_SIGMA, i);
                    din[4 * NT + d] = seed(d, SEED_SIGMA, host);
                    din[5 * NT + d] = seed(d, SEED_K2, i);
                    din[6 * NT + d] = seed(d, SEED_K2, host);
                }
                if (tides_on())
                    adj_tides_pre_jvp<NT>(x[0], x[1], x[2], c.sig, hc.sig, c.k2, hc.k2, c.R, hc.R, hc.m, c.m, din,
                                          scratch, dpr.t);
                if (flat_on())
                    adj_flat_pre_jvp<NT>(x[0], x[1], x[2], c.R, hc.R, hc.k2f, hc.m, c.k2f, c.m, din, scratch, dpr.f);
                if (gr_on())
                    adj_gr_pre_jvp<NT>(x[0], x[1], x[2], hc.m, hc.mg, hc.moi, c.m, c.mg, c.moi, din, scratch, dpr.g);
            }
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
        // tangents: the originals stay in T / HT (v, L); the previous spin is
        // T.S / HT.S, advanced with the primal's Sp
        double tvf[3][A], tLf[3][A], tSc[3][A], thvf[3][A], thLf[3][A], thSc[3][A];
        if constexpr (NT > 0) {
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < NT; ++d) {
                    tvf[q][d] = T.v[q][d]; tLf[q][d] = T.L[q][d];
                    thvf[q][d] = HT.v[q][d]; thLf[q][d] = HT.L[q][d];
                    tSc[q][d] = T.S[q][d]; thSc[q][d] = HT.S[q][d];
                }
        }
        for (int it = 0; it < kMIDPOINT_MAX; ++it) {
            for (int q = 0; q < 3; ++q) { pv[q] = vf[q]; pL[q] = Lf[q]; hpv[q] = hvf[q]; hpL[q] = hLf[q]; }
            if (has) {
                spin_of(c, Lc, Sc);
                spin_of(hc, hLc, hSc);
                if constexpr (NT > 0) {
                    double tLc[3][A], thLc[3][A];
                    for (int q = 0; q < 3; ++q)
                        for (int d = 0; d < NT; ++d) {
                            tLc[q][d] = 0.5 * (T.L[q][d] + tLf[q][d]);
                            thLc[q][d] = 0.5 * (HT.L[q][d] + thLf[q][d]);
                        }
                    dspin_of(c, tLc, tSc);
                    dspin_of(hc, thLc, thSc);
                }
            }
            double aa[3] = {0., 0., 0.}, dl[3] = {0., 0., 0.}, th[3] = {0., 0., 0.};
            double taa[3][A], tdl[3][A], tth[3][A];
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) taa[q][d] = tdl[q][d] = tth[q][d] = 0.;
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
                if constexpr (NT > 0) {
                    // din[p * NT + d] over the 15 iteration inputs: relative
                    // velocity, spin, host spin, previous spin, previous host spin
                    double din[15 * A], dout[9 * A];
                    for (int q = 0; q < 3; ++q)
                        for (int d = 0; d < NT; ++d) {
                            din[q * NT + d] = 0.5 * (T.v[q][d] + tvf[q][d]) - 0.5 * (HT.v[q][d] + thvf[q][d]);
                            din[(3 + q) * NT + d] = tSc[q][d];
                            din[(6 + q) * NT + d] = thSc[q][d];
                            din[(9 + q) * NT + d] = T.S[q][d];
                            din[(12 + q) * NT + d] = HT.S[q][d];
                        }
                    auto add = [&]() {
                        for (int q = 0; q < 3; ++q)
                            for (int d = 0; d < NT; ++d) {
                                taa[q][d] += dout[q * NT + d];
                                tdl[q][d] += dout[(3 + q) * NT + d];
                                tth[q][d] += dout[(6 + q) * NT + d];
                            }
                    };
                    if (tides_on()) {
                        adj_tides_iter_jvp<NT>(pr.t, dpr.t, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0],
                                               Sp[1], Sp[2], hSp[0], hSp[1], hSp[2], c.R, hc.R, hc.m, c.m, din, out, dout);
                        add();
                    }
                    if (flat_on()) {
                        adj_flat_iter_jvp<NT>(pr.f, dpr.f, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0],
                                              Sp[1], Sp[2], hSp[0], hSp[1], hSp[2], c.R, hc.R, hc.k2f, hc.m, c.k2f, c.m,
                                              din, out, dout);
                        add();
                    }
                    if (gr_on()) {
                        adj_gr_iter_jvp<NT>(pr.g, dpr.g, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0],
                                            Sp[1], Sp[2], hSp[0], hSp[1], hSp[2], hc.m, hc.mg, hc.moi, c.m, c.mg, c.moi,
                                            din, out, dout);
                        add();
                    }
                }
            }
            double vals[NS] = {};
            for (int q = 0; q < 3; ++q) { vals[q] = mr * aa[q]; vals[3 + q] = th[q]; }
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) {
                        vals[6 + q * NT + d] = mr * taa[q][d];
                        vals[6 + (3 + q) * NT + d] = tth[q][d];
                    }
            double tot[NS];
            if (!grid_reduce(D, vals, 6 + 6 * NT, tot, shm, warp_bodies, body_rows)) return false;
            // the host's outputs, computed by every thread
            double haa[3], hdl[3];
            for (int q = 0; q < 3; ++q) { haa[q] = -tot[q]; hdl[q] = tot[3 + q]; }
            if (is_host)
                for (int q = 0; q < 3; ++q) { aa[q] = haa[q]; dl[q] = hdl[q]; }
            if (has) for (int q = 0; q < 3; ++q) {
                dvc[q] = hdt * aa[q] - b.ev[q];
                vf[q] = v0[q] + dvc[q];
                dLc[q] = hdt * dl[q] - b.eL[q];
                Lf[q] = L0[q] + dLc[q];
                hdvc[q] = hdt * haa[q] - h.ev[q];
                hvf[q] = hv0[q] + hdvc[q];
                hdLc[q] = hdt * hdl[q] - h.eL[q];
                hLf[q] = hL0[q] + hdLc[q];
            }
            if constexpr (NT > 0) {
                if (has)
                    for (int q = 0; q < 3; ++q)
                        for (int d = 0; d < NT; ++d) {
                            const double thaa = -tot[6 + q * NT + d], thdl = tot[6 + (3 + q) * NT + d];
                            if (is_host) { taa[q][d] = thaa; tdl[q][d] = thdl; }
                            tvf[q][d] = T.v[q][d] + hdt * taa[q][d];
                            tLf[q][d] = T.L[q][d] + hdt * tdl[q][d];
                            thvf[q][d] = HT.v[q][d] + hdt * thaa;
                            thLf[q][d] = HT.L[q][d] + hdt * thdl;
                        }
            }
            if (it >= kMIDPOINT_MIN - 1) {
                double cv[NS] = {};
                if (has) {
                    for (int q = 0; q < 3; ++q) {
                        cv[0] += (vf[q] - pv[q]) * (vf[q] - pv[q]);
                        cv[1] += vf[q] * vf[q];
                        cv[2] += (Lf[q] - pL[q]) * (Lf[q] - pL[q]);
                        cv[3] += Lf[q] * Lf[q];
                        cv[4 + q] = c.m * b.r[q];
                        cv[7 + q] = c.m * vf[q];
                    }
                    if constexpr (NT > 0)
                        if (cm)
                            for (int q = 0; q < 3; ++q)
                                for (int d = 0; d < NT; ++d) {
                                    cv[10 + q * NT + d] = c.m * T.r[q][d];
                                    cv[10 + (3 + q) * NT + d] = c.m * tvf[q][d];
                                }
                }
                const int ns = cm ? 10 + 6 * NT : 4;
                double s4[NS];
                if (!grid_reduce(D, cv, ns, s4, shm, warp_bodies, body_rows)) return false;
                if (cm) {
                    for (int q = 0; q < 6; ++q) cm[q] = s4[4 + q];
                    if constexpr (NT > 0)
                        for (int q = 0; q < 6; ++q)
                            for (int d = 0; d < NT; ++d) dcm[q][d] = s4[10 + q * NT + d];
                }
                if (s4[0] / s4[1] < kDBL_EPSILON_2 && (s4[3] == 0. || s4[2] / s4[3] < kDBL_EPSILON_2)) break;
            }
            if (has) for (int q = 0; q < 3; ++q) {
                vc[q] = 0.5 * (v0[q] + vf[q]);
                Lc[q] = 0.5 * (L0[q] + Lf[q]);
                Sp[q] = Sc[q];
                hvc[q] = 0.5 * (hv0[q] + hvf[q]);
                hLc[q] = 0.5 * (hL0[q] + hLf[q]);
                hSp[q] = hSc[q];
            }
            if constexpr (NT > 0) {
                if (has)
                    for (int q = 0; q < 3; ++q)
                        for (int d = 0; d < NT; ++d) { T.S[q][d] = tSc[q][d]; HT.S[q][d] = thSc[q][d]; }
            }
        }
        if (!has) return true;
        for (int q = 0; q < 3; ++q) {
            b.v[q] = vf[q]; b.L[q] = Lf[q]; b.S[q] = Sc[q];
            b.ev[q] = (vf[q] - v0[q]) - dvc[q];
            b.eL[q] = (Lf[q] - L0[q]) - dLc[q];
            h.v[q] = hvf[q]; h.L[q] = hLf[q]; h.S[q] = hSc[q];
            h.ev[q] = (hvf[q] - hv0[q]) - hdvc[q];
            h.eL[q] = (hLf[q] - hL0[q]) - hdLc[q];
        }
        if (is_host) b = h;
        if constexpr (NT > 0) {
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < NT; ++d) {
                    T.v[q][d] = tvf[q][d]; T.L[q][d] = tLf[q][d]; T.S[q][d] = tSc[q][d];
                    HT.v[q][d] = thvf[q][d]; HT.L[q][d] = thLf[q][d]; HT.S[q][d] = thSc[q][d];
                }
            if (is_host) T = HT;
        }
        return true;
    }

    // ---- gravity over all ordered pairs, with the pair checks ----
    // pos[] holds heliocentric positions published before the preceding
    // barrier (differences of heliocentric and of inertial positions agree);
    // the host sits at -shift (the jump moved every planet by +shift).  The
    // tangent of the pair term -G m_j d / |d|^3 along dd is
    // -G m_j (dd - 3 (d . dd) d / |d|^2) / |d|^3.
    __device__ bool gravity(const double shift[3], const double (&tshift)[3][A]) {
        const int64_t nn = n;
        constexpr int rows = 3 * (1 + NT);  // rows of one slice in gpart
        const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        const int64_t gi = tid % nn, chunk = tid / nn;
        if (chunk < D.nchunk) {
            const int64_t j0 = chunk * nn / D.nchunk, j1 = (chunk + 1) * nn / D.nchunk;
            double xi, yi, zi;
            if (gi == host) { xi = -shift[0]; yi = -shift[1]; zi = -shift[2]; }
            else { xi = __ldcg(&D.pos[gi]); yi = __ldcg(&D.pos[nn + gi]); zi = __ldcg(&D.pos[2 * nn + gi]); }
            double txi[3][A], tax[3][A];
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) {
                        txi[q][d] = gi == host ? -tshift[q][d] : __ldcg(&D.dpos[(d * 3 + q) * nn + gi]);
                        tax[q][d] = 0.;
                    }
            const double Ri = D.bf[POSI_BF_RADIUS * nn + gi];
            double ax = 0., ay = 0., az = 0.;
            unsigned long long bad = ~0ull;
            for (int64_t j = j0; j < j1; ++j) {
                if (j == gi) continue;
                double xj, yj, zj;
                if (j == host) { xj = -shift[0]; yj = -shift[1]; zj = -shift[2]; }
                else { xj = __ldcg(&D.pos[j]); yj = __ldcg(&D.pos[nn + j]); zj = __ldcg(&D.pos[2 * nn + j]); }
                const double dx = xi - xj, dy = yi - yj, dz = zi - zj;
                const double d2 = dx * dx + dy * dy + dz * dz;
                if (gi < j && bad == ~0ull) {
                    const double rr = D.roche[j * nn + gi];  // symmetric: coalesced across the warp
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
                if constexpr (NT > 0) {
                    const double i2 = inv_d * inv_d;
                    for (int d = 0; d < NT; ++d) {
                        const double ex = txi[0][d] - __ldcg(&D.dpos[(d * 3 + 0) * nn + j]);
                        const double ey = txi[1][d] - __ldcg(&D.dpos[(d * 3 + 1) * nn + j]);
                        const double ez = txi[2][d] - __ldcg(&D.dpos[(d * 3 + 2) * nn + j]);
                        const double s = 3. * (dx * ex + dy * ey + dz * ez) * i2;
                        tax[0][d] += p * (ex - s * dx);
                        tax[1][d] += p * (ey - s * dy);
                        tax[2][d] += p * (ez - s * dz);
                    }
                }
            }
            D.gpart[(chunk * rows + 0) * nn + gi] = ax;
            D.gpart[(chunk * rows + 1) * nn + gi] = ay;
            D.gpart[(chunk * rows + 2) * nn + gi] = az;
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) D.gpart[(chunk * rows + 3 + q * NT + d) * nn + gi] = tax[q][d];
            if (bad != ~0ull) atomicMin(D.bad, bad);
        }
        if (!grid_barrier(D)) return false;
        if (has) {
            for (int q = 0; q < 3; ++q) {
                double acc = 0.;
                for (int k = 0; k < D.nchunk; ++k) acc += __ldcg(&D.gpart[(k * rows + q) * nn + i]);
                a[q] = acc;
            }
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) {
                        double acc = 0.;
                        for (int k = 0; k < D.nchunk; ++k) acc += __ldcg(&D.gpart[(k * rows + 3 + q * NT + d) * nn + i]);
                        da[q][d] = acc;
                    }
        }
        return true;
    }

    // Kepler drift of a planet over half_dt, with the tangents (the implicit
    // derivative at the converged root).
    __device__ void kepler(double x[3], double u[3], double (&tx)[3][A], double (&tu)[3][A]) {
        if (planet) {
            const KeplerScalars ks = kepler_scalars(hc.mg, x, u);
            bool ok = false;
            const double X = kepler_solve(ks, half_dt, &ok);
            if (!ok) atomicOr(D.err, LE_KEPLER);
            double r1[3], v1[3];
            kepler_apply(hc.mg, half_dt, x, u, ks, X, r1, v1);
            if constexpr (NT > 0)
                for (int d = 0; d < NT; ++d) {
                    const double e0[3] = {tx[0][d], tx[1][d], tx[2][d]}, f0[3] = {tu[0][d], tu[1][d], tu[2][d]};
                    double e1[3], f1[3];
                    kepler_jvp(hc.mg, half_dt, x, u, X, e0, f0, e1, f1);
                    for (int q = 0; q < 3; ++q) { tx[q][d] = e1[q]; tu[q][d] = f1[q]; }
                }
            for (int q = 0; q < 3; ++q) { x[q] = r1[q]; u[q] = v1[q]; }
        }
    }

    // inertial positions and velocities from the heliocentric x, barycentric
    // u, the barycentre (Rc, Vc) and the sums S[0..2] = sum_p m_p x_p,
    // S[3..5] = sum_p m_p u_p (src/integrator/whfast.rs:1082-1155); tS[q][d]
    // holds the tangents of S (the linear map applied to the tangents)
    __device__ void to_inertial(const double x[3], const double u[3], const double Rc[3], const double Vc[3],
                                const double S[6], const double (&tx)[3][A], const double (&tu)[3][A],
                                const double (&tRc)[3][A], const double (&tVc)[3][A], const double (&tS)[6][A]) {
        if (!has) return;
        for (int q = 0; q < 3; ++q) {
            h.r[q] = Rc[q] - S[q] * inv_M;
            h.v[q] = Vc[q] - S[3 + q] * inv_hm;
        }
        if (planet)
            for (int q = 0; q < 3; ++q) { b.r[q] = x[q] + h.r[q]; b.v[q] = u[q] + Vc[q]; }
        if (is_host)
            for (int q = 0; q < 3; ++q) { b.r[q] = h.r[q]; b.v[q] = h.v[q]; }
        if constexpr (NT > 0) {
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < NT; ++d) {
                    HT.r[q][d] = tRc[q][d] - tS[q][d] * inv_M;
                    HT.v[q][d] = tVc[q][d] - tS[3 + q][d] * inv_hm;
                    if (planet) { T.r[q][d] = tx[q][d] + HT.r[q][d]; T.v[q][d] = tu[q][d] + tVc[q][d]; }
                    if (is_host) { T.r[q][d] = HT.r[q][d]; T.v[q][d] = HT.v[q][d]; }
                }
        }
    }

    // sums of m x and m u over the planets (and their tangents), optionally
    // publishing the positions for the pair loop
    __device__ bool planet_sums(const double x[3], const double u[3], const double (&tx)[3][A],
                                const double (&tu)[3][A], bool publish, double S[6], double (&tS)[6][A]) {
        double vals[NS] = {};
        if (planet) {
            for (int q = 0; q < 3; ++q) {
                if (publish) D.pos[q * n + i] = x[q];
                vals[q] = c.m * x[q];
                vals[3 + q] = c.m * u[q];
            }
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) {
                        if (publish) D.dpos[(d * 3 + q) * n + i] = tx[q][d];
                        vals[6 + q * NT + d] = c.m * tx[q][d];
                        vals[6 + (3 + q) * NT + d] = c.m * tu[q][d];
                    }
        }
        double tot[NS];
        if (!grid_reduce(D, vals, 6 + 6 * NT, tot, shm, warp_bodies, body_rows)) return false;
        for (int q = 0; q < 6; ++q) S[q] = tot[q];
        if constexpr (NT > 0)
            for (int q = 0; q < 6; ++q)
                for (int d = 0; d < NT; ++d) tS[q][d] = tot[6 + q * NT + d];
        return true;
    }

    // ---- one step (src/integrator/whfast.rs:235-305), democratic heliocentric ----
    // Eleven grid barriers: four per half kick (three midpoint iterations),
    // one for the jump and back-transform of the first drift (the positions
    // for the pair loop published before it), one for the pair loop, one
    // for the back-transform of the second drift.  The second jump uses the
    // planets' total momentum from the first: the interaction kick adds
    // dt sum_p m_p a_p, which is zero (the planets' mutual forces cancel and
    // the host's are left out of the kick).
    __device__ __forceinline__ bool step() {
        const bool first = last_hist < 0.;
        if (first || last_hist + hist_period <= t) {
            spin_of(c, b.L, b.S);
            spin_of(hc, h.L, h.S);
            if constexpr (NT > 0) {
                dspin_of(c, T.L, T.S);
                dspin_of(hc, HT.L, HT.S);
            }
            last_hist = first ? 0. : last_hist + hist_period;
        }
        double cm[6], tcm[6][A];
        if (!midpoint(half_dt, cm, tcm)) return false;
        // inertial -> democratic heliocentric
        double Rc[3], Vc[3], x[3] = {0., 0., 0.}, u[3] = {0., 0., 0.};
        double tRc[3][A], tVc[3][A], tx[3][A], tu[3][A];
        for (int q = 0; q < 3; ++q) { Rc[q] = cm[q] * inv_M; Vc[q] = cm[3 + q] * inv_M; }
        if (planet)
            for (int q = 0; q < 3; ++q) { x[q] = b.r[q] - h.r[q]; u[q] = b.v[q] - Vc[q]; }
        if constexpr (NT > 0)
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < NT; ++d) {
                    tRc[q][d] = tcm[q][d] * inv_M;
                    tVc[q][d] = tcm[3 + q][d] * inv_M;
                    tx[q][d] = planet ? T.r[q][d] - HT.r[q][d] : 0.;
                    tu[q][d] = planet ? T.v[q][d] - tVc[q][d] : 0.;
                }
        // part 1: Kepler drift (and the barycentre's), jump, back to inertial
        kepler(x, u, tx, tu);
        for (int q = 0; q < 3; ++q) Rc[q] += half_dt * Vc[q];
        if constexpr (NT > 0)
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < NT; ++d) tRc[q][d] += half_dt * tVc[q][d];
        double S[6], tS[6][A];
        if (!planet_sums(x, u, tx, tu, true, S, tS)) return false;
        double shift[3], tshift[3][A];
        for (int q = 0; q < 3; ++q) {
            shift[q] = half_dt * S[3 + q] * inv_hm;        // jump: dt/2 P / m_host
            S[q] += shift[q] * (Mtot - hc.m);              // sum_p m_p (x_p + shift)
        }
        const double P[3] = {S[3], S[4], S[5]};
        if (planet)
            for (int q = 0; q < 3; ++q) x[q] += shift[q];
        double tP[3][A];
        if constexpr (NT > 0)
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < NT; ++d) {
                    tshift[q][d] = half_dt * tS[3 + q][d] * inv_hm;
                    tS[q][d] += tshift[q][d] * (Mtot - hc.m);
                    tP[q][d] = tS[3 + q][d];
                    if (planet) tx[q][d] += tshift[q][d];
                }
        to_inertial(x, u, Rc, Vc, S, tx, tu, tRc, tVc, tS);
        // gravity and the interaction kick
        if (!gravity(shift, tshift)) return false;
        if (__ldcg(D.bad) != ~0ull) return false;  // frozen at the first failing pair
        if (planet)
            for (int q = 0; q < 3; ++q) u[q] += dt * a[q];
        // part 2: jump, Kepler drift, back to inertial
        if (planet)
            for (int q = 0; q < 3; ++q) x[q] += half_dt * P[q] * inv_hm;
        if constexpr (NT > 0)
            if (planet)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) {
                        tu[q][d] += dt * da[q][d];
                        tx[q][d] += half_dt * tP[q][d] * inv_hm;
                    }
        kepler(x, u, tx, tu);
        for (int q = 0; q < 3; ++q) Rc[q] += half_dt * Vc[q];
        if constexpr (NT > 0)
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < NT; ++d) tRc[q][d] += half_dt * tVc[q][d];
        if (!planet_sums(x, u, tx, tu, false, S, tS)) return false;
        to_inertial(x, u, Rc, Vc, S, tx, tu, tRc, tVc, tS);
        if (!midpoint(half_dt, nullptr, nullptr)) return false;
        t += dt;
        return true;
    }
};

template <int NT>
__global__ void __launch_bounds__(kBlock, 1) large_steps_kernel(LDev D, int64_t n_steps) {
    __shared__ double shm[(kBlock / 32 + 1) * BP_ROW];
    Large<NT> S(D, shm);
    S.n = D.n;
    // bodies spread over the blocks, at most one warp of bodies per SMSP
    // while the grid has room: the per-body work runs on as many SMSPs as it can
    S.i = threadIdx.x < D.per_block ? (int64_t)blockIdx.x * D.per_block + threadIdx.x : INT64_MAX;
    S.host = (int)D.si[POSI_SI_HOST];
    S.has = S.i < S.n;
    {
        const int64_t warp_first = (int64_t)blockIdx.x * D.per_block + (threadIdx.x & ~31);
        S.warp_bodies = (int)(threadIdx.x & ~31) < D.per_block && warp_first < S.n;
        S.body_rows = (unsigned)((S.n + D.per_block - 1) / D.per_block);
    }
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
    if constexpr (NT > 0) {
        const int64_t n = S.n, src = S.has ? S.i : S.host;
        for (int q = 0; q < 3; ++q)
            for (int d = 0; d < NT; ++d) {
                const double* base = D.tan + (size_t)d * 12 * n;
                S.HT.r[q][d] = base[(0 + q) * n + S.host];
                S.HT.v[q][d] = base[(3 + q) * n + S.host];
                S.HT.L[q][d] = base[(6 + q) * n + S.host];
                S.HT.S[q][d] = base[(9 + q) * n + S.host];
                S.T.r[q][d] = base[(0 + q) * n + src];
                S.T.v[q][d] = base[(3 + q) * n + src];
                S.T.L[q][d] = base[(6 + q) * n + src];
                S.T.S[q][d] = base[(9 + q) * n + src];
                S.da[q][d] = 0.;
            }
    }
    // total mass, in block order
    {
        double vals[Large<NT>::NS] = {};
        vals[0] = S.has ? S.c.m : 0.;
        double tot[1];
        if (!grid_reduce(D, vals, 1, tot, shm, S.warp_bodies, S.body_rows)) return;
        S.Mtot = tot[0];
        S.inv_M = 1. / S.Mtot;
        S.inv_hm = 1. / S.hc.m;
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
        if constexpr (NT > 0)
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < NT; ++d) {
                    double* base = D.tan + (size_t)d * 12 * n;
                    base[(0 + q) * n + i] = S.T.r[q][d];
                    base[(3 + q) * n + i] = S.T.v[q][d];
                    base[(6 + q) * n + i] = S.T.L[q][d];
                    base[(9 + q) * n + i] = S.T.S[q][d];
                }
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
