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
// * The bodies sit in the first blocks of the grid (the body blocks, 32
//   bodies each while the grid has blocks enough).  Reductions over bodies
//   (host back-reactions, midpoint convergence, barycentre and momentum sums
//   of the transforms) are block sums written to a per-block row and added
//   in block order after a barrier among the body blocks alone:
//   deterministic run to run, and cheaper than a barrier of the whole grid
//   (1.4 against 2.3 us on GB300).
// * Gravity (src/particles/universe.rs:198-303) spreads the O(N^2) pair loop
//   over every warp of the grid, over unordered pairs: the bodies form tiles
//   of 32, and one warp takes a pair of tiles (I <= J), lane l holding body
//   32 I + l while tile J's bodies rotate through the lanes by warp shuffles
//   and carry their own sums with them, so each pair's 1 / r^3 serves both
//   bodies.  Every body gets one partial sum per partner tile, added in tile
//   order (deterministic).  Two grid barriers per step frame it: the
//   positions published before, the partial sums after.  The blocks without
//   bodies wait at the first and leave when the body blocks have finished.
//   The collision, Roche and ejection checks of the same loop report the
//   first offending pair in the reference's (i, j) order; a pair reads the
//   Roche table's row i only when it is closer than the largest threshold of
//   body i's checks.
// * Barriers are counters in global memory with a bounded wait: a wait that
//   runs out sets an error flag and every thread leaves the kernel.
//
// * large_steps_kernel<NT> with NT > 0 carries forward-mode tangents of the
//   state along NT directions (derivatives with respect to initial state,
//   dissipation factors and Love numbers); NT = 0 is the plain integration.
//
// Coordinates: democratic heliocentric (src/integrator/whfast.rs:495-530,
// 965-1024, 1082-1155); Jacobi (:889-963, 1034-1080: the sequential
// recurrences as grid prefix scans) and WHDS (the scaled velocities, per-body
// jump and kick) in kernels of their own, without tangents.  Effects: constant-time-lag tides, oblate
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
// parts a tile pair of the pair loop is split into (a divisor of 32): halves
// measured best at 1024 bodies (131.6 us per step; quarters 132.7, eighths
// 138.0 -- more partial slots to gather -- and whole pairs 140.8)
constexpr int kPairSplit = 2;
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
    const double* roche;    // [n][n] Roche radii, row i for the pairs (i, j > i)
    const double* near2;    // [n] squared distance below which body i's pair checks can fire
    double* pos;            // [3][n] positions for the pair loop
    double* gpart;          // [ntile][3 (1 + NT)][n] partial accelerations (and their tangents), per partner tile
    double* bpart;          // [nbb][BP_ROW]
    double* tot;            // [BP_ROW] totals of the last reduction
    unsigned* bar;          // arrival count of the whole grid's barriers (zeroed before each launch)
    unsigned* bbar;         // the same among the body blocks
    int* ctl;               // set to 1 by the body blocks when they have finished (the others then leave)
    int* err;               // error flags (LE_*)
    unsigned long long* bad;  // first failing pair: min over (i n + j) * 4 + code; all ones if none
    int ntile;              // tiles of 32 bodies
    int nbb;                // body blocks (the first nbb blocks of the grid)
    int per_block;          // bodies per body block: body i is thread i % per_block of block i / per_block
    // tangent directions (the tangent kernels only)
    double* tan;            // [NT][12][n] tangents of r, v, L, S; read at launch, written back at the end
    double* dpos;           // [NT][3][n] position tangents for the pair loop
    int seed_body[kMaxTangents];   // body whose parameter direction k perturbs by a unit rate, or -1
    int seed_param[kMaxTangents];  // SEED_SIGMA (dissipation factor) or SEED_K2 (Love number)
};

// Sum of vals over the block into row blockIdx.x of bpart.  Only warps that
// own bodies (warp_active) add: a warp's FP64 add holds its SMSP's FP64 pipe
// 64 cycles whatever its active lanes, so the warps' sums are formed with
// the lanes spread over the slots -- eight slots at a time, lane 4 s + p adds
// the eight values 8p .. 8p + 7 of slot s as a pairwise tree, then the
// quarters pair up, ((q0 + q1) + (q2 + q3)) -- 9 FP64 adds per eight slots instead
// of 40 for shuffle trees.  The order of every slot's sum is fixed whatever
// the number of slots, so a reduction carrying tangent slots beside the
// primal ones gives the primal slots the same bits.
template <int NS>
__device__ __forceinline__ void block_partial(double* bpart, const double (&vals)[NS], int nslots, double* shm,
                                              bool warp_active) {
    __shared__ double tw[kBlock / 32][8 * 33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp_active) {
        const int s = lane >> 2, p = lane & 3;
#pragma unroll
        for (int c = 0; c < (NS + 7) / 8; ++c) {
            if (c * 8 < nslots) {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int k = c * 8 + q;
                    if (k < NS) tw[warp][q * 33 + lane] = k < nslots ? vals[k] : 0.;
                }
                __syncwarp();
                const double* t = &tw[warp][s * 33 + 8 * p];
                // a tree (depth 3, not a chain of 7): the adds wait on one another less
                double acc = ((t[0] + t[1]) + (t[2] + t[3])) + ((t[4] + t[5]) + (t[6] + t[7]));
                acc += __shfl_down_sync(0xffffffffu, acc, 1);
                acc += __shfl_down_sync(0xffffffffu, acc, 2);
                if (p == 0 && c * 8 + s < nslots) shm[warp * BP_ROW + c * 8 + s] = acc;
                __syncwarp();
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

// Per-block counts of the barriers passed (0: the whole grid's, 1: the body
// blocks'), zeroed by thread 0 at launch; only thread 0 touches them.
__device__ __forceinline__ unsigned& barrier_count(int which) {
    __shared__ unsigned counts[2];
    return counts[which];
}

// Barrier among `parts` blocks with a bounded wait.  The arrival count only
// grows during a launch (the host zeroes it before each): thread 0 of each
// block adds its arrival with a release reduction, whose result it does not
// wait for, then polls the count with acquire loads until the k-th barrier's
// k x parts arrivals are in (a signed difference, so the count may wrap).
// One trip to L2 and back on the critical path, where an arrive / reset /
// release-a-generation barrier takes three.  Returns false (and flags the
// error) when the wait ran out; callers then leave the kernel.
__device__ bool sync_blocks(const LDev& D, unsigned* ctr, unsigned parts, int which) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned& k = barrier_count(which);
        const unsigned target = (++k) * parts;
        cuda::atomic_ref<int, cuda::thread_scope_device> err(*D.err);
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(ctr) : "memory");
        int ok = 1;
        const long long start = clock64();
        for (;;) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
            if ((int)(v - target) >= 0) break;
            if (clock64() - start > kBarrierWaitCycles || (err.load(cuda::memory_order_relaxed) & LE_BARRIER)) {
                ok = 0;
                err.fetch_or(LE_BARRIER, cuda::memory_order_relaxed);
                break;
            }
            __nanosleep(20);
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// Barrier of the whole grid (the pair loop's), and of the body blocks alone.
__device__ __forceinline__ bool grid_barrier(const LDev& D) { return sync_blocks(D, D.bar, gridDim.x, 0); }
__device__ __forceinline__ bool body_barrier(const LDev& D) { return sync_blocks(D, D.bbar, (unsigned)D.nbb, 1); }

// Sum over the body blocks: every body block writes its partial row, the
// body blocks meet, and every one of them adds the rows itself in a fixed
// order (a tree per chunk of eight slots for up to 32 rows; beyond, warp
// k mod 8 takes slot k, lane l rows l, l + 32, ..., then a butterfly): the
// same bits in every block, one barrier and no second round trip through
// global memory.  The rows alternate between two buffers
// (seq, counted by each caller): a block running ahead writes the next
// reduction's row while a slower one may still read this one's.
template <int NS>
__device__ bool grid_reduce(const LDev& D, const double (&vals)[NS], int nslots, double* out, double* shm,
                            bool warp_active, unsigned rows, unsigned& seq) {
    double* buf = D.bpart + (size_t)(seq & 1u) * gridDim.x * BP_ROW;
    ++seq;
    block_partial(buf, vals, nslots, shm, warp_active);
    if (!body_barrier(D)) return false;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (rows <= 32) {
        // up to 32 rows: lane 4 s + p of a warp adds rows p, p + 4, ..., p + 28
        // of slot 8 c + s as a pairwise tree, then the four parts pair up,
        // ((0 + 1) + (2 + 3)) -- nine FP64 adds per chunk of eight slots, one
        // chunk per warp, where a shuffle tree takes five per slot; the order
        // of a slot's sum depends on the rows alone
        const int s8 = lane >> 2, p = lane & 3;
        for (int c = warp; c * 8 < nslots; c += kBlock / 32) {
            const int k = c * 8 + s8;
            double t[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const unsigned b = (unsigned)(4 * e + p);
                t[e] = (k < nslots && b < rows) ? __ldcg(buf + (size_t)b * BP_ROW + k) : 0.;
            }
            double x = ((t[0] + t[1]) + (t[2] + t[3])) + ((t[4] + t[5]) + (t[6] + t[7]));
            x += __shfl_down_sync(0xffffffffu, x, 1);
            x += __shfl_down_sync(0xffffffffu, x, 2);
            if (p == 0 && k < nslots) shm[(kBlock / 32) * BP_ROW + k] = x;
        }
    } else {
        for (int k = warp; k < nslots; k += kBlock / 32) {
            double x = 0.;
            for (unsigned b = lane; b < rows; b += 32) x += __ldcg(buf + (size_t)b * BP_ROW + k);
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) shm[(kBlock / 32) * BP_ROW + k] = x;
        }
    }
    __syncthreads();
    for (int k = 0; k < nslots; ++k) out[k] = shm[(kBlock / 32) * BP_ROW + k];
    __syncthreads();
    return true;
}

// Exclusive prefix over the bodies in index order, among the body blocks (body i is thread
// i % per_block of block i / per_block; only the one-role engine calls it):
// excl[k] = sum of vals[k] over the bodies before this thread's, tot[k] over
// all bodies, for nslots <= 8.  Warp shuffle scans, then the warps' totals in
// shared memory, then one barrier after which every block sums the partial
// rows of the blocks before it (one warp per slot, fixed butterfly); rows in
// alternating buffers, as grid_reduce's.
template <int NS>
__device__ bool grid_scan(const LDev& D, const double (&vals)[NS], int nslots, double* excl, double* tot, double* shm,
                          unsigned rows, unsigned& seq) {
    double* buf = D.bpart + (size_t)(seq & 1u) * gridDim.x * BP_ROW;
    ++seq;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NW = kBlock / 32;
    double wex[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        wex[k] = 0.;
        if (k < nslots) {
            double x = vals[k];
            for (int o = 1; o < 32; o <<= 1) {
                const double y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            const double ex = __shfl_up_sync(0xffffffffu, x, 1);
            wex[k] = lane == 0 ? 0. : ex;
            if (lane == 31) shm[warp * BP_ROW + k] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NS; ++k)
        if (k < nslots)
            for (int w = 0; w < warp; ++w) wex[k] += shm[w * BP_ROW + k];
    if (threadIdx.x < nslots) {
        double bt = 0.;
        for (int w = 0; w < NW; ++w) bt += shm[w * BP_ROW + threadIdx.x];
        buf[(size_t)blockIdx.x * BP_ROW + threadIdx.x] = bt;
    }
    if (!body_barrier(D)) return false;
    for (int k = warp; k < nslots; k += NW) {
        double pre = 0., all = 0.;
        for (unsigned b = lane; b < rows; b += 32) {
            const double x = __ldcg(buf + (size_t)b * BP_ROW + k);
            all += x;
            if (b < blockIdx.x) pre += x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            pre += __shfl_xor_sync(0xffffffffu, pre, o);
            all += __shfl_xor_sync(0xffffffffu, all, o);
        }
        if (lane == 0) { shm[NW * BP_ROW + k] = pre; shm[NW * BP_ROW + 8 + k] = all; }
    }
    __syncthreads();
    for (int k = 0; k < nslots; ++k) {
        excl[k] = shm[NW * BP_ROW + k] + wex[k];
        tot[k] = shm[NW * BP_ROW + 8 + k];
    }
    __syncthreads();
    return true;
}

struct BodyConst {
    double m, mg, R, moi, sig, k2, k2f;
    double inv_moi;  // 1 / moi (0 for a body without moment of inertia)
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
    c.inv_moi = c.moi != 0. ? 1. / c.moi : 0.;
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

// One lane of rotation of the partner tile's data and sums (lane l takes
// lane l + 1's).
template <int NT>
__device__ __forceinline__ void rotate_partner(int lane, double& xj, double& yj, double& zj, double& gmj,
                                               double& axj, double& ayj, double& azj,
                                               double (&txj)[3][NT > 0 ? NT : 1], double (&taj)[3][NT > 0 ? NT : 1]) {
    constexpr unsigned FULL = 0xffffffffu;
    const int src = (lane + 1) & 31;
    xj = __shfl_sync(FULL, xj, src); yj = __shfl_sync(FULL, yj, src); zj = __shfl_sync(FULL, zj, src);
    gmj = __shfl_sync(FULL, gmj, src);
    axj = __shfl_sync(FULL, axj, src); ayj = __shfl_sync(FULL, ayj, src); azj = __shfl_sync(FULL, azj, src);
    if constexpr (NT > 0)
        for (int q = 0; q < 3; ++q)
            for (int d = 0; d < NT; ++d) {
                txj[q][d] = __shfl_sync(FULL, txj[q][d], src);
                taj[q][d] = __shfl_sync(FULL, taj[q][d], src);
            }
}

// The pair loop of gravity (src/particles/universe.rs:198-303), run by every
// warp of the grid after the positions are published.  Bodies form tiles of
// 32; a warp takes one pair of tiles (I <= J), tile pairs spread over the
// blocks first so that a block's warps (one per SMSP) take different pairs.
// Lane l holds body i = 32 I + l; tile J's bodies start in lane order and
// rotate one lane per step through 32 steps (warp shuffles), carrying their
// own acceleration sums, so that each unordered pair (i < j) is evaluated
// once: -G m_j d / |d|^3 for i, +G m_i d / |d|^3 for j, with d = x_i - x_j.
// A diagonal tile (I = J) takes its 31 partners one-sided.  The pair skips of
// the reference (WHFastOne: the host and the first planet in Jacobi
// coordinates; WHFastTwo: every pair of the host otherwise) apply to the
// forces only; the collision, Roche and ejection checks run on every pair
// i < j -- the Roche table's row i (roche_radiuses[i][j], the reference's
// entry for i < j) is read only when the pair is closer than body i's largest
// threshold -- and the smallest (i n + j, check) key wins.  With NT tangent
// directions the same rotation carries the tangents: the pair term's tangent
// is -+ G m (dd - 3 (d . dd) d / |d|^2) / |d|^3, dd = dx_i - dx_j.  Partial
// sums go to gpart[partner tile][row][body]: every body receives one per
// tile.
template <int NT>
__device__ void pair_loop(const LDev& D, int host, int64_t p1, bool jac) {
    constexpr int AN = NT > 0 ? NT : 1;
    constexpr int rows = 3 * (1 + NT);
    const int64_t n = D.n;
    const int T = D.ntile;
    const int64_t npairs = (int64_t)T * (T + 1) / 2;
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    // a work item is a part of a tile pair: partner offsets
    // [32 h / kPairSplit, 32 (h + 1) / kPairSplit) (the diagonal pair from
    // 1), so that several items share an SMSP where one pair would leave a
    // lone warp; each part writes its own partial slot
    for (int64_t it = blockIdx.x + (int64_t)gridDim.x * wib; it < kPairSplit * npairs;
         it += (int64_t)gridDim.x * wpb) {
        const int h = (int)(it / npairs);
        const int64_t tp = it - h * npairs;
        int I = 0;
        int64_t r = tp;
        while (r >= T - I) { r -= T - I; ++I; }
        const int J = I + (int)r;
        const bool diag = I == J;
        const int64_t i = (int64_t)I * 32 + lane;
        const bool hi = i < n;
        double xi = 0., yi = 0., zi = 0., gmi = 0., Ri = 0., nr2 = 0.;
        double txi[3][AN] = {};
        if (hi) {
            xi = __ldcg(&D.pos[i]); yi = __ldcg(&D.pos[n + i]); zi = __ldcg(&D.pos[2 * n + i]);
            gmi = kG * D.bf[POSI_BF_MASS * n + i];
            Ri = D.bf[POSI_BF_RADIUS * n + i];
            nr2 = D.near2[i];
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) txi[q][d] = __ldcg(&D.dpos[(d * 3 + q) * n + i]);
        }
        // the partner tile: positions, masses and sums travel together (the
        // partner's index follows from the step: lane l holds 32 J + (l + k) mod 32)
        const int kb = h ? h * (32 / kPairSplit) : (diag ? 1 : 0), ke = (h + 1) * (32 / kPairSplit);
        const int64_t j0 = (int64_t)J * 32 + ((lane + kb) & 31);
        double xj = 0., yj = 0., zj = 0., gmj = 0.;
        double txj[3][AN] = {}, taj[3][AN] = {};
        double axj = 0., ayj = 0., azj = 0.;
        if (j0 < n) {
            xj = __ldcg(&D.pos[j0]); yj = __ldcg(&D.pos[n + j0]); zj = __ldcg(&D.pos[2 * n + j0]);
            gmj = kG * D.bf[POSI_BF_MASS * n + j0];
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) txj[q][d] = __ldcg(&D.dpos[(d * 3 + q) * n + j0]);
        }
        // distances compared as the bit patterns of non-negative doubles
        // (their order is the integers'), which keeps the gate off the FP64 pipe
        const long long nr2_bits = __double_as_longlong(nr2);
        double ax = 0., ay = 0., az = 0.;
        double tai[3][AN] = {};
        unsigned long long bad = ~0ull;
        for (int k = kb; k < ke; ++k) {
            const int64_t j = (int64_t)J * 32 + ((lane + k) & 31);
            if (hi && j < n) {
                const double dx = xi - xj, dy = yi - yj, dz = zi - zj;
                const double d2 = dx * dx + dy * dy + dz * dz;
                if (i < j && bad == ~0ull && (__double_as_longlong(d2) <= nr2_bits || i == host)) {
                    const double rr = D.roche[i * n + j];
                    const double Rs = Ri + D.bf[POSI_BF_RADIUS * n + j];
                    const unsigned long long key = (unsigned long long)(i * n + j) * 4ull;
                    if (d2 <= rr * rr) bad = key + POSI_SYS_ROCHE;
                    else if (d2 <= Rs * Rs) bad = key + POSI_SYS_COLLISION;
                    else if (i == host && d2 > kMAX_DISTANCE_2) bad = key + POSI_SYS_EJECTED;
                }
                const bool skip = jac ? ((i == host && j == p1) || (j == host && i == p1))  // WHFastOne
                                      : (i == host || j == host);                          // WHFastTwo
                if (!skip) {
                    const double inv_d = rsqrt(d2);
                    const double id3 = inv_d * inv_d * inv_d;
                    const double pi = -gmj * id3, pj = gmi * id3;
                    ax += pi * dx; ay += pi * dy; az += pi * dz;
                    if (!diag) { axj += pj * dx; ayj += pj * dy; azj += pj * dz; }
                    if constexpr (NT > 0) {
                        const double i2 = inv_d * inv_d;
                        for (int d = 0; d < NT; ++d) {
                            const double ex = txi[0][d] - txj[0][d];
                            const double ey = txi[1][d] - txj[1][d];
                            const double ez = txi[2][d] - txj[2][d];
                            const double s3 = 3. * (dx * ex + dy * ey + dz * ez) * i2;
                            const double cx = ex - s3 * dx, cy = ey - s3 * dy, cz = ez - s3 * dz;
                            tai[0][d] += pi * cx; tai[1][d] += pi * cy; tai[2][d] += pi * cz;
                            if (!diag) { taj[0][d] += pj * cx; taj[1][d] += pj * cy; taj[2][d] += pj * cz; }
                        }
                    }
                }
            }
            rotate_partner<NT>(lane, xj, yj, zj, gmj, axj, ayj, azj, txj, taj);
        }
        // after the part's rotations lane l holds the partner 32 J + (l + ke) mod 32;
        // partial slot kPairSplit K + h holds the sums over partner tile K's part h
        const int64_t sj = kPairSplit * (int64_t)J + h, si = kPairSplit * (int64_t)I + h;
        if (hi) {
            D.gpart[(sj * rows + 0) * n + i] = ax;
            D.gpart[(sj * rows + 1) * n + i] = ay;
            D.gpart[(sj * rows + 2) * n + i] = az;
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) D.gpart[(sj * rows + 3 + q * NT + d) * n + i] = tai[q][d];
        }
        const int64_t jw = (int64_t)J * 32 + ((lane + ke) & 31);
        if (!diag && jw < n) {
            D.gpart[(si * rows + 0) * n + jw] = axj;
            D.gpart[(si * rows + 1) * n + jw] = ayj;
            D.gpart[(si * rows + 2) * n + jw] = azj;
            if constexpr (NT > 0)
                for (int q = 0; q < 3; ++q)
                    for (int d = 0; d < NT; ++d) D.gpart[(si * rows + 3 + q * NT + d) * n + jw] = taj[q][d];
        }
        if (bad != ~0ull) atomicMin(D.bad, bad);
    }
}

// Tangent of one body's state along one direction.
struct Tangent {
    double r[3], v[3], L[3], S[3];
};

// One thread of the engine.  NT = 0: the plain integration.  NT > 0: the
// same integration carrying forward-mode derivatives (tangents) of every
// body's state along NT directions -- the derivative of the step map applied
// to the incoming tangents, plus the unit rate of change of the seeded
// parameter (a body's dissipation factor or Love number) where the seeded
// body's tides enter.
//
// Roles: a body is held by 1 + NT threads, one warp each.  Role 0 (dir = -1)
// integrates the primal state and alone contributes the primal sums; role
// r >= 1 repeats the primal arithmetic (identical, so every role holds the
// same primal state) and carries the tangent of direction dir = r - 1.  A
// warp's FP64 instructions cost the same whatever its active lanes, so
// spreading the directions over warps keeps each warp's work at one primal
// plus one tangent.  The midpoint convergence tests only primal values; the
// compensated (Kahan) error terms of the kick carry no tangent.
template <int NT>
struct Large {
    static constexpr int NS = slots_for(NT);    // value slots of the reductions
    const LDev& D;
    int64_t n, i;
    int host;
    int dir;                // tangent direction of this thread, -1: the primal role
    bool has, is_host, planet;
    bool tides, flat, gr;
    double dt, half_dt, t, time_limit, last_hist, hist_period;
    BodyConst c, hc;        // own and host constants
    BodyState b, h;         // own and host state (host: redundant copy)
    double a[3];            // gravity acceleration (own)
    Tangent T, HT;          // own and host tangents (host: redundant copy)
    double da[3];           // tangent of the gravity acceleration
    double* shm;
    double Mtot, inv_M, inv_hm;
    double kgm;             // GM of this body's Kepler drift
    // Jacobi coordinates (the one-role engine): masses before this body and
    // including it (host first, then index order), the first planet, and the
    // barycentre (the host's Jacobi coordinates)
    bool jac;
    double eta_ex, eta_in;
    int64_t p1;
    double Rb[3], Vb[3];
    bool warp_bodies;       // this thread's warp owns at least one body
    unsigned body_rows;     // blocks that own bodies (the partial rows that can be nonzero)
    unsigned rseq = 0;      // reductions and scans so far (their row buffer alternates)

    __device__ Large(const LDev& D_, double* shm_) : D(D_), shm(shm_) {}

    __device__ __forceinline__ bool tides_on() const { return tides && c.tk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool flat_on() const { return flat && c.fk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool gr_on() const { return gr && c.gk == POSI_EFFECT_ORBITING; }
    __device__ __forceinline__ bool tan_on() const { return NT > 0 && dir >= 0; }
    __device__ __forceinline__ bool primal_role() const { return dir < 0; }
    // reduction slot of tangent component q of this thread's direction
    __device__ __forceinline__ int tslot(int base, int q) const { return base + q * NT + dir; }

    // unit rate of this direction's seeded parameter for body j
    __device__ __forceinline__ double seed(int param, int64_t j) const {
        return (D.seed_body[dir] == j && D.seed_param[dir] == param) ? 1. : 0.;
    }

    __device__ static void spin_of(const BodyConst& k, const double L[3], double S[3]) {
        if (k.moi != 0.) {
            const double im = k.inv_moi;
            for (int q = 0; q < 3; ++q) S[q] = L[q] * im;
        } else {
            for (int q = 0; q < 3; ++q) S[q] = 0.;
        }
    }

    __device__ static void dspin_of(const BodyConst& k, const double dL[3], double dS[3]) {
        const double im = k.inv_moi;
        for (int q = 0; q < 3; ++q) dS[q] = dL[q] * im;
    }

    struct Pre {
        double t[adj_tides_NPRE], f[adj_flat_NPRE], g[adj_gr_NPRE];
    };

    // ---- implicit midpoint (src/integrator/whfast.rs:322-466) ----
    // With cm != nullptr the last convergence reduction also carries the sums
    // of m r and m v over all bodies at the final velocities (cm[0..5]), and
    // their tangents (tcm).
    // The position terms of the effect blocks (and their tangents): the
    // closing half kick of a step and the opening one of the next see the
    // same positions, so the second reuses the first's; a drift clears them.
    Pre prc, dprc;
    bool prc_ok = false;

    __device__ bool midpoint(double hdt, double* cm, double* tcm) {
        double x[3] = {0., 0., 0.};
        Pre& pr = prc;
        Pre& dpr = dprc;
        const bool tn = tan_on();
        if (planet && !prc_ok) {
            for (int q = 0; q < 3; ++q) x[q] = b.r[q] - h.r[q];
            if (tides_on()) adj_tides_pre(x[0], x[1], x[2], c.sig, hc.sig, c.k2, hc.k2, c.R, hc.R, hc.m, c.m, pr.t);
            if (flat_on()) adj_flat_pre(x[0], x[1], x[2], c.R, hc.R, hc.k2f, hc.m, c.k2f, c.m, pr.f);
            if (gr_on()) adj_gr_pre(x[0], x[1], x[2], hc.m, hc.mg, hc.moi, c.m, c.mg, c.moi, pr.g);
            if (tn) {
                // tangents of the pre inputs (x, y, z, sig_p, sig_h, k2_p, k2_h)
                double din[7], scratch[adj_gr_NPRE];
                for (int q = 0; q < 3; ++q) din[q] = T.r[q] - HT.r[q];
                din[3] = seed(SEED_SIGMA, i);
                din[4] = seed(SEED_SIGMA, host);
                din[5] = seed(SEED_K2, i);
                din[6] = seed(SEED_K2, host);
                if (tides_on())
                    adj_tides_pre_jvp<1>(x[0], x[1], x[2], c.sig, hc.sig, c.k2, hc.k2, c.R, hc.R, hc.m, c.m, din, scratch,
                                         dpr.t);
                if (flat_on())
                    adj_flat_pre_jvp<1>(x[0], x[1], x[2], c.R, hc.R, hc.k2f, hc.m, c.k2f, c.m, din, scratch, dpr.f);
                if (gr_on())
                    adj_gr_pre_jvp<1>(x[0], x[1], x[2], hc.m, hc.mg, hc.moi, c.m, c.mg, c.moi, din, scratch, dpr.g);
            }
        }
        prc_ok = true;
        const double mr = planet ? c.m * inv_hm : 0.;
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
        double tvf[3], tLf[3], tSc[3], thvf[3], thLf[3], thSc[3];
        for (int q = 0; q < 3; ++q) {
            tvf[q] = T.v[q]; tLf[q] = T.L[q]; thvf[q] = HT.v[q]; thLf[q] = HT.L[q];
            tSc[q] = T.S[q]; thSc[q] = HT.S[q];
        }
        for (int it = 0; it < kMIDPOINT_MAX; ++it) {
            for (int q = 0; q < 3; ++q) { pv[q] = vf[q]; pL[q] = Lf[q]; hpv[q] = hvf[q]; hpL[q] = hLf[q]; }
            if (has) {
                spin_of(c, Lc, Sc);
                spin_of(hc, hLc, hSc);
                if (tn) {
                    double tLc[3], thLc[3];
                    for (int q = 0; q < 3; ++q) {
                        tLc[q] = 0.5 * (T.L[q] + tLf[q]);
                        thLc[q] = 0.5 * (HT.L[q] + thLf[q]);
                    }
                    dspin_of(c, tLc, tSc);
                    dspin_of(hc, thLc, thSc);
                }
            }
            double aa[3] = {0., 0., 0.}, dl[3] = {0., 0., 0.}, th[3] = {0., 0., 0.};
            double taa[3] = {0., 0., 0.}, tdl[3] = {0., 0., 0.}, tth[3] = {0., 0., 0.};
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
                if (tn) {
                    // tangents of the 15 iteration inputs: relative velocity,
                    // spin, host spin, previous spin, previous host spin
                    double din[15], dout[9];
                    for (int q = 0; q < 3; ++q) {
                        din[q] = 0.5 * (T.v[q] + tvf[q]) - 0.5 * (HT.v[q] + thvf[q]);
                        din[3 + q] = tSc[q];
                        din[6 + q] = thSc[q];
                        din[9 + q] = T.S[q];
                        din[12 + q] = HT.S[q];
                    }
                    auto add = [&]() {
                        for (int q = 0; q < 3; ++q) { taa[q] += dout[q]; tdl[q] += dout[3 + q]; tth[q] += dout[6 + q]; }
                    };
                    if (tides_on()) {
                        adj_tides_iter_jvp<1>(pr.t, dpr.t, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0],
                                              Sp[1], Sp[2], hSp[0], hSp[1], hSp[2], c.R, hc.R, hc.m, c.m, din, out, dout);
                        add();
                    }
                    if (flat_on()) {
                        adj_flat_iter_jvp<1>(pr.f, dpr.f, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0],
                                             Sp[1], Sp[2], hSp[0], hSp[1], hSp[2], c.R, hc.R, hc.k2f, hc.m, c.k2f, c.m,
                                             din, out, dout);
                        add();
                    }
                    if (gr_on()) {
                        adj_gr_iter_jvp<1>(pr.g, dpr.g, h0, h1, h2, Sc[0], Sc[1], Sc[2], hSc[0], hSc[1], hSc[2], Sp[0],
                                           Sp[1], Sp[2], hSp[0], hSp[1], hSp[2], hc.m, hc.mg, hc.moi, c.m, c.mg, c.moi,
                                           din, out, dout);
                        add();
                    }
                }
            }
            // threads without a body leave their slots at zero and run no FP64
            // work of their own here: in a body block, a warp without bodies
            // shares its SMSP's FP64 pipe with a warp of bodies
            double vals[NS] = {};
            if (primal_role() && has)
                for (int q = 0; q < 3; ++q) { vals[q] = mr * aa[q]; vals[3 + q] = th[q]; }
            if (tn && has)
                for (int q = 0; q < 3; ++q) {
                    vals[tslot(6, q)] = mr * taa[q];
                    vals[tslot(6, 3 + q)] = tth[q];
                }
            // A planet's final values of this iteration need no reduction
            // (only the host's do), so without tangents the convergence sums
            // and the barycentre sums over the planets travel in the same
            // reduction as the host's back-reactions (slots 6-15), and every
            // thread adds the host's terms afterwards: one reduction per
            // iteration.  The tangent engine reduces them separately, adding
            // the host's terms the same way, so its primal state keeps the
            // plain engine's bits.
            const bool ctest = it >= kMIDPOINT_MIN - 1;
            constexpr bool kMerged = NT == 0;
            if (kMerged && ctest) {
                if (planet) {
                    double cvf[3], cLf[3];
                    for (int q = 0; q < 3; ++q) {
                        cvf[q] = v0[q] + (hdt * aa[q] - b.ev[q]);
                        cLf[q] = L0[q] + (hdt * dl[q] - b.eL[q]);
                        vals[6] += (cvf[q] - pv[q]) * (cvf[q] - pv[q]);
                        vals[7] += cvf[q] * cvf[q];
                        vals[8] += (cLf[q] - pL[q]) * (cLf[q] - pL[q]);
                        vals[9] += cLf[q] * cLf[q];
                        if (cm) vals[13 + q] = c.m * cvf[q];
                    }
                }
                if (cm && has)
                    for (int q = 0; q < 3; ++q) vals[10 + q] = c.m * b.r[q];
            }
            const int nred = kMerged && ctest ? (cm ? 16 : 10) : 6 + 6 * NT;
            double tot[NS];
            if (!grid_reduce(D, vals, nred, tot, shm, warp_bodies, body_rows, rseq)) return false;
            // the host's outputs and final values, computed by every thread
            // that holds a body (the block's first thread among them)
            double haa[3] = {0., 0., 0.}, hdl[3] = {0., 0., 0.};
            if (has)
                for (int q = 0; q < 3; ++q) {
                    haa[q] = -tot[q]; hdl[q] = tot[3 + q];
                    hdvc[q] = hdt * haa[q] - h.ev[q];
                    hvf[q] = hv0[q] + hdvc[q];
                    hdLc[q] = hdt * hdl[q] - h.eL[q];
                    hLf[q] = hL0[q] + hdLc[q];
                }
            if (is_host)
                for (int q = 0; q < 3; ++q) { aa[q] = haa[q]; dl[q] = hdl[q]; }
            if (has) for (int q = 0; q < 3; ++q) {
                dvc[q] = hdt * aa[q] - b.ev[q];
                vf[q] = v0[q] + dvc[q];
                dLc[q] = hdt * dl[q] - b.eL[q];
                Lf[q] = L0[q] + dLc[q];
            }
            if (tn && has)
                for (int q = 0; q < 3; ++q) {
                    const double thaa = -tot[tslot(6, q)], thdl = tot[tslot(6, 3 + q)];
                    if (is_host) { taa[q] = thaa; tdl[q] = thdl; }
                    tvf[q] = T.v[q] + hdt * taa[q];
                    tLf[q] = T.L[q] + hdt * tdl[q];
                    thvf[q] = HT.v[q] + hdt * thaa;
                    thLf[q] = HT.L[q] + hdt * thdl;
                }
            if (ctest) {
                // s4: the planets' convergence sums (0-3) and, with cm, the
                // sums of m r (4-6, host included) and of the planets' m v (7-9)
                double s4[NS];
                if (kMerged) {
                    for (int k = 0; k < 10; ++k) s4[k] = tot[6 + k];
                } else {
                    double cv[NS] = {};
                    if (has) {
                        if (primal_role())
                            for (int q = 0; q < 3; ++q) {
                                if (planet) {
                                    cv[0] += (vf[q] - pv[q]) * (vf[q] - pv[q]);
                                    cv[1] += vf[q] * vf[q];
                                    cv[2] += (Lf[q] - pL[q]) * (Lf[q] - pL[q]);
                                    cv[3] += Lf[q] * Lf[q];
                                    cv[7 + q] = c.m * vf[q];
                                }
                                cv[4 + q] = c.m * b.r[q];
                            }
                        if (tn && cm)
                            for (int q = 0; q < 3; ++q) {
                                cv[tslot(10, q)] = c.m * T.r[q];
                                cv[tslot(10, 3 + q)] = c.m * tvf[q];
                            }
                    }
                    const int ns = cm ? 10 + 6 * NT : 4;
                    if (!grid_reduce(D, cv, ns, s4, shm, warp_bodies, body_rows, rseq)) return false;
                    if (tn && cm)
                        for (int q = 0; q < 6; ++q) tcm[q] = s4[tslot(10, q)];
                }
                // the host's terms, added by the block's first thread (a body:
                // its copy of the host's state is current) and shared with the
                // convergence decision, so that every thread of the block takes
                // the same branch; the test compares a < eps b instead of
                // dividing (the sums of squares are not negative)
                const int nsh = cm ? 10 : 4;
                double* bc = shm + (kBlock / 32) * BP_ROW;
                __shared__ int converged_s;
                if (threadIdx.x == 0) {
                    double hc4[4] = {0., 0., 0., 0.};
                    for (int q = 0; q < 3; ++q) {
                        hc4[0] += (hvf[q] - hpv[q]) * (hvf[q] - hpv[q]);
                        hc4[1] += hvf[q] * hvf[q];
                        hc4[2] += (hLf[q] - hpL[q]) * (hLf[q] - hpL[q]);
                        hc4[3] += hLf[q] * hLf[q];
                    }
                    for (int k = 0; k < 4; ++k) bc[k] = s4[k] + hc4[k];
                    if (cm)
                        for (int q = 0; q < 3; ++q) {
                            bc[4 + q] = s4[4 + q];
                            bc[7 + q] = s4[7 + q] + hc.m * hvf[q];
                        }
                    converged_s = bc[0] < kDBL_EPSILON_2 * bc[1] && (bc[3] == 0. || bc[2] < kDBL_EPSILON_2 * bc[3]);
                }
                __syncthreads();
                const bool converged = converged_s != 0;
                if (cm)
                    for (int k = 0; k < nsh; ++k) s4[k] = bc[k];
                __syncthreads();
                if (cm)
                    for (int q = 0; q < 6; ++q) cm[q] = s4[4 + q];
                if (converged) break;
            }
            // the midpoints (v0 + vf) / 2 as v0 + dvc / 2 (vf = v0 + dvc): one
            // FMA instead of an add and a multiply, as in the batched FAST kernel
            if (has) for (int q = 0; q < 3; ++q) {
                vc[q] = v0[q] + 0.5 * dvc[q];
                Lc[q] = L0[q] + 0.5 * dLc[q];
                Sp[q] = Sc[q];
                hvc[q] = hv0[q] + 0.5 * hdvc[q];
                hLc[q] = hL0[q] + 0.5 * hdLc[q];
                hSp[q] = hSc[q];
            }
            if (tn && has)
                for (int q = 0; q < 3; ++q) { T.S[q] = tSc[q]; HT.S[q] = thSc[q]; }
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
        if (tn) {
            for (int q = 0; q < 3; ++q) {
                T.v[q] = tvf[q]; T.L[q] = tLf[q]; T.S[q] = tSc[q];
                HT.v[q] = thvf[q]; HT.L[q] = thLf[q]; HT.S[q] = thSc[q];
            }
            if (is_host) T = HT;
        }
        return true;
    }

    // ---- gravity: positions published, the pair loop over the whole grid,
    // partial sums gathered ----
    // pos[] holds the positions the pair loop reads: the planets' heliocentric
    // positions (democratic heliocentric: published before the jump, the host
    // then at -shift, since the jump moves every planet by +shift; WHDS:
    // after the jump, the host at the origin) or every body's inertial
    // position (Jacobi).  The host publishes its own entry here (and its
    // tangents, -tshift[d], in dpos[]); then the grid meets, runs pair_loop,
    // meets again, and each body adds its partial sums in tile order.
    __device__ bool gravity(const double shift[3], const double (&tshift)[NT > 0 ? NT : 1][3]) {
        if (is_host && !jac) {
            if (primal_role())
                for (int q = 0; q < 3; ++q) D.pos[q * n + i] = -shift[q];
            if constexpr (NT > 0)
                if (tan_on())
                    for (int q = 0; q < 3; ++q) D.dpos[(dir * 3 + q) * n + i] = -tshift[dir][q];
        }
        if (!grid_barrier(D)) return false;
        pair_loop<NT>(D, host, p1, jac);
        if (!grid_barrier(D)) return false;
        if (D.per_block == 32) {
            // the body block's 32 bodies are tile blockIdx.x: its eight warps
            // add the partial sums together -- warp w the partial slots
            // [w c, (w + 1) c), c = ceil(kPairSplit ntile / 8), in order -- and the
            // chunk sums are added in warp order: a fixed order whatever the
            // number of tangent rows, loads spread over the block instead of
            // one latency-bound chain per body
            __shared__ double gchunk[kBlock / 32][3][32];
            __shared__ double gfinal[3 * (1 + kMaxTangents)][32];
            constexpr int rows = 3 * (1 + NT);
            const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
            const int nslot = kPairSplit * D.ntile;  // kPairSplit partials per partner tile
            const int c = (nslot + kBlock / 32 - 1) / (kBlock / 32);
            const int64_t body = (int64_t)blockIdx.x * 32 + l, nn = n;
            const int k0 = w * c, k1 = min(nslot, (w + 1) * c);
            for (int rg = 0; rg < rows; rg += 3) {
                double v[3] = {0., 0., 0.};
                if (body < nn)
                    for (int k = k0; k < k1; ++k)
#pragma unroll
                        for (int q = 0; q < 3; ++q) v[q] += __ldcg(&D.gpart[((int64_t)k * rows + rg + q) * nn + body]);
#pragma unroll
                for (int q = 0; q < 3; ++q) gchunk[w][q][l] = v[q];
                __syncthreads();
                if (threadIdx.x < 96) {
                    const int q = threadIdx.x >> 5;
                    double acc = gchunk[0][q][l];
                    for (int ww = 1; ww < kBlock / 32; ++ww) acc += gchunk[ww][q][l];
                    gfinal[rg + q][l] = acc;
                }
                __syncthreads();
            }
            if (has) {
                for (int q = 0; q < 3; ++q) a[q] = gfinal[q][l];
                if (tan_on())
                    for (int q = 0; q < 3; ++q) da[q] = gfinal[3 + q * NT + dir][l];
            }
            __syncthreads();
        } else if (has) {
            // more than 32 bodies per block: each body adds its partial sums
            // in tile order, loaded eight tiles at a time
            constexpr int rows = 3 * (1 + NT);
            const int64_t nn = n;
            const int nq = tan_on() ? 6 : 3;
            for (int qq = 0; qq < nq; ++qq) {
                const int row = qq < 3 ? qq : 3 + (qq - 3) * NT + dir;
                const double* src = D.gpart + (int64_t)row * nn + i;
                const int64_t stride = (int64_t)rows * nn;
                double acc = 0.;
                const int nslot = kPairSplit * D.ntile;
                for (int kk = 0; kk < nslot; kk += 8) {
                    double v[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) v[e] = kk + e < nslot ? __ldcg(src + (int64_t)(kk + e) * stride) : 0.;
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (kk + e < nslot) acc += v[e];
                }
                if (qq < 3) a[qq] = acc; else da[qq - 3] = acc;
            }
        }
        return true;
    }

    // Kepler drift of a planet over half_dt, with the tangent (the implicit
    // derivative at the converged root).
    // The universal-variable drift of kepler_solve / kepler_apply with fewer
    // FP64 instructions on the body's chain: 1 / r0 from rsqrt, the
    // G-functions of the root from the last Newton iterate's by a
    // second-order Taylor step (the iterate is within 1e-8 of the root, so
    // the neglected third order is below 1e-24 relative), one reciprocal of
    // r instead of three divisions.
    __device__ void kepler(double x[3], double u[3], double tx[3], double tu[3]) {
        prc_ok = false;  // the drift moves the positions
        if (planet) {
            const double mu = kgm, dt = half_dt;
            const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
            const double ir0 = rsqrt(r2);
            const double r0 = r2 * ir0;
            const double v2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
            const double beta = 2. * mu * ir0 - v2;
            const double eta0 = x[0] * u[0] + x[1] * u[1] + x[2] * u[2];
            const double zeta0 = mu - beta * r0;
            double X = 0.;
            if (beta > 0.) {
                const double uu = dt * ir0;
                const double a2 = -0.5 * eta0 * ir0;
                const double a3 = (0.5 * eta0 * eta0 * ir0 - zeta0 * (1. / 6.)) * ir0;
                const double a4 = -(eta0 * a3 + 0.5 * eta0 * a2 * a2 + 0.5 * zeta0 * a2 - eta0 * beta * (1. / 24.)) * ir0;
                X = uu * (1. + uu * (a2 + uu * (a3 + uu * a4)));
            }
            bool ok = false;
            double G0 = 1., G1 = 0., G2 = 0., G3 = 0.;
            for (int it = 0; it < kKEPLER_MAX_NEWTON; ++it) {
                double c[4];
                stumpff4(beta * X * X, c);
                const double X2 = X * X;
                G0 = c[0]; G1 = X * c[1]; G2 = X2 * c[2]; G3 = X2 * X * c[3];
                const double F = r0 * X + eta0 * G2 + zeta0 * G3 - dt;
                const double Fp = r0 + eta0 * G1 + zeta0 * G2;
                const double dX = F / Fp;
                X -= dX;
                if (fabs(dX) <= 1e-8 * fabs(X) || dX == 0.) {
                    // dG0 = -beta G1, dG1 = G0, dG2 = G1, dG3 = G2 per unit X
                    const double e = -dX, e2h = 0.5 * e * e;
                    const double n0 = G0 - beta * (G1 * e + G0 * e2h);
                    const double n1 = G1 + G0 * e - beta * G1 * e2h;
                    const double n2 = G2 + G1 * e + G0 * e2h;
                    const double n3 = G3 + G2 * e + G1 * e2h;
                    G0 = n0; G1 = n1; G2 = n2; G3 = n3;
                    ok = true;
                    break;
                }
            }
            if (!ok) {
                atomicOr(D.err, LE_KEPLER);
                double c[4];
                stumpff4(beta * X * X, c);
                G0 = c[0]; G1 = X * c[1]; G2 = X * X * c[2]; G3 = X * X * X * c[3];
            }
            const double irr = 1. / (r0 + eta0 * G1 + zeta0 * G2);
            const double f = -mu * G2 * ir0;
            const double g = dt - mu * G3;
            const double fd = -mu * G1 * ir0 * irr;
            const double gd = -mu * G2 * irr;
            double r1[3], v1[3];
            for (int k = 0; k < 3; ++k) {
                r1[k] = x[k] + (f * x[k] + g * u[k]);
                v1[k] = u[k] + (fd * x[k] + gd * u[k]);
            }
            if (tan_on()) {
                double e1[3], f1[3];
                kepler_jvp(kgm, half_dt, x, u, X, tx, tu, e1, f1);
                for (int q = 0; q < 3; ++q) { tx[q] = e1[q]; tu[q] = f1[q]; }
            }
            for (int q = 0; q < 3; ++q) { x[q] = r1[q]; u[q] = v1[q]; }
        }
    }

    // inertial positions and velocities from the heliocentric x, barycentric
    // u, the barycentre (Rc, Vc) and the sums S[0..2] = sum_p m_p x_p,
    // S[3..5] = sum_p m_p u_p (src/integrator/whfast.rs:1082-1155); tS holds
    // the tangents of S (the linear map applied to the tangents)
    __device__ void to_inertial(const double x[3], const double u[3], const double Rc[3], const double Vc[3],
                                const double S[6], const double tx[3], const double tu[3], const double tRc[3],
                                const double tVc[3], const double tS[6]) {
        if (!has) return;
        for (int q = 0; q < 3; ++q) {
            h.r[q] = Rc[q] - S[q] * inv_M;
            h.v[q] = Vc[q] - S[3 + q] * inv_hm;
        }
        if (planet)
            for (int q = 0; q < 3; ++q) { b.r[q] = x[q] + h.r[q]; b.v[q] = u[q] + Vc[q]; }
        if (is_host)
            for (int q = 0; q < 3; ++q) { b.r[q] = h.r[q]; b.v[q] = h.v[q]; }
        if (tan_on()) {
            for (int q = 0; q < 3; ++q) {
                HT.r[q] = tRc[q] - tS[q] * inv_M;
                HT.v[q] = tVc[q] - tS[3 + q] * inv_hm;
                if (planet) { T.r[q] = tx[q] + HT.r[q]; T.v[q] = tu[q] + tVc[q]; }
                if (is_host) { T.r[q] = HT.r[q]; T.v[q] = HT.v[q]; }
            }
        }
    }

    // sums of m x and m u over the planets (and the tangents of every
    // direction, tS_all[d][q]), optionally publishing the positions for the
    // pair loop
    __device__ bool planet_sums(const double x[3], const double u[3], const double tx[3], const double tu[3],
                                bool publish, double S[6], double (&tS_all)[NT > 0 ? NT : 1][6]) {
        double vals[NS] = {};
        if (planet) {
            if (primal_role())
                for (int q = 0; q < 3; ++q) {
                    if (publish) D.pos[q * n + i] = x[q];
                    vals[q] = c.m * x[q];
                    vals[3 + q] = c.m * u[q];
                }
            if (tan_on())
                for (int q = 0; q < 3; ++q) {
                    if (publish) D.dpos[(dir * 3 + q) * n + i] = tx[q];
                    vals[tslot(6, q)] = c.m * tx[q];
                    vals[tslot(6, 3 + q)] = c.m * tu[q];
                }
        }
        double tot[NS];
        if (!grid_reduce(D, vals, 6 + 6 * NT, tot, shm, warp_bodies, body_rows, rseq)) return false;
        for (int q = 0; q < 6; ++q) S[q] = tot[q];
        if constexpr (NT > 0)
            for (int d = 0; d < NT; ++d)
                for (int q = 0; q < 6; ++q) tS_all[d][q] = tot[6 + q * NT + d];
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
    // Jacobi -> inertial (src/integrator/whfast.rs:1034-1080): the reference's
    // backward recurrence is R_(k-1) = R - sum over body k and the later ones
    // of (m / eta_incl) x, R the barycentre; one grid scan of those terms
    __device__ bool from_jacobi(const double x[3], const double u[3]) {
        double vals[NS] = {}, ex[NS], tot[NS];
        if (planet) {
            const double w = c.m / eta_in;
            for (int q = 0; q < 3; ++q) { vals[q] = w * x[q]; vals[3 + q] = w * u[q]; }
        }
        if (!grid_scan(D, vals, 6, ex, tot, shm, body_rows, rseq)) return false;
        for (int q = 0; q < 3; ++q) { h.r[q] = Rb[q] - tot[q]; h.v[q] = Vb[q] - tot[3 + q]; }
        if (planet)
            for (int q = 0; q < 3; ++q) {
                b.r[q] = x[q] + (Rb[q] - (tot[q] - ex[q]));
                b.v[q] = u[q] + (Vb[q] - (tot[3 + q] - ex[3 + q]));
            }
        if (is_host)
            for (int q = 0; q < 3; ++q) { b.r[q] = h.r[q]; b.v[q] = h.v[q]; }
        return true;
    }

    // ---- one step in Jacobi coordinates (the one-role engine) ----
    // The reference's sequential recurrences over the bodies (host first,
    // then index order) become grid scans: inertial -> Jacobi subtracts the
    // centre of mass of the bodies before (:889-933), the Jacobi
    // accelerations likewise (:935-963), the Kepler drift of body k uses the
    // cumulative GM of the bodies up to k (:640-645), the kick adds the
    // indirect term for every planet but the first (:558-592), and there is
    // no jump.  Summation order differs from the reference's (FAST).
    __device__ bool step_jacobi() {
        const bool first = last_hist < 0.;
        if (first || last_hist + hist_period <= t) {
            spin_of(c, b.L, b.S);
            spin_of(hc, h.L, h.S);
            last_hist = first ? 0. : last_hist + hist_period;
        }
        double cm[6], tcm[6] = {0., 0., 0., 0., 0., 0.};
        if (!midpoint(half_dt, cm, tcm)) return false;
        for (int q = 0; q < 3; ++q) { Rb[q] = cm[q] * inv_M; Vb[q] = cm[3 + q] * inv_M; }
        double x[3] = {0., 0., 0.}, u[3] = {0., 0., 0.}, tx[3] = {0., 0., 0.}, tu[3] = {0., 0., 0.};
        {
            double vals[NS] = {}, ex[NS], tot[NS];
            if (planet)
                for (int q = 0; q < 3; ++q) { vals[q] = c.m * b.r[q]; vals[3 + q] = c.m * b.v[q]; }
            if (!grid_scan(D, vals, 6, ex, tot, shm, body_rows, rseq)) return false;
            if (planet) {
                const double ie = 1. / eta_ex;
                for (int q = 0; q < 3; ++q) {
                    x[q] = b.r[q] - (hc.m * h.r[q] + ex[q]) * ie;
                    u[q] = b.v[q] - (hc.m * h.v[q] + ex[3 + q]) * ie;
                }
            }
        }
        kepler(x, u, tx, tu);
        for (int q = 0; q < 3; ++q) Rb[q] += half_dt * Vb[q];
        if (!from_jacobi(x, u)) return false;
        if (has && primal_role())
            for (int q = 0; q < 3; ++q) D.pos[q * n + i] = b.r[q];
        const double zero[3] = {0., 0., 0.};
        double tzero[NT > 0 ? NT : 1][3] = {};
        if (!gravity(zero, tzero)) return false;
        if (__ldcg(D.bad) != ~0ull) return false;  // frozen at the first failing pair
        {
            // Jacobi accelerations: planets' m a before this body, plus the host's
            double vals[NS] = {}, ex[NS], tot[NS];
            if (planet)
                for (int q = 0; q < 3; ++q) vals[q] = c.m * a[q];
            if (is_host)
                for (int q = 0; q < 3; ++q) vals[3 + q] = hc.m * a[q];
            if (!grid_scan(D, vals, 6, ex, tot, shm, body_rows, rseq)) return false;
            if (planet) {
                const double ie = 1. / eta_ex;
                for (int q = 0; q < 3; ++q) u[q] += dt * (a[q] - (tot[3 + q] + ex[q]) * ie);
                if (i != p1) {
                    const double rj2i = 1. / (x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + 1e-12);
                    const double rji = sqrt(rj2i);
                    const double prefac = dt * (rji * rj2i * kG * eta_in);
                    for (int q = 0; q < 3; ++q) u[q] += prefac * x[q];
                }
            }
        }
        kepler(x, u, tx, tu);
        for (int q = 0; q < 3; ++q) Rb[q] += half_dt * Vb[q];
        if (!from_jacobi(x, u)) return false;
        if (!midpoint(half_dt, nullptr, nullptr)) return false;
        t += dt;
        return true;
    }

    // ---- one step in WHDS coordinates (the one-role engine) ----
    // Heliocentric positions, barycentric velocities scaled by
    // (m0 + m) / m0 (src/integrator/whfast.rs:973-1023), the Kepler drift
    // with GM = G (m0 + m) (:648-652), a jump by dt/2 (p - m u / (m0 + m))
    // with p = sum m u / (m0 + m) (:521-556), the kick scaled by
    // (m0 + m) / m0 (:605-625) and the back-transform of :1090-1155.  The
    // second jump reuses p: the kick adds dt sum m a / m0 to it, zero
    // because the planets' mutual forces cancel and the host's are left out.
    // sums: S[0..2] = sum m x, S[3..5] = sum (m / (m0 + m)) u, S[6..8] =
    // sum m (m / (m0 + m)) u over the planets
    __device__ bool whds_sums(const double x[3], const double u[3], double wv, double S[9]) {
        double vals[NS] = {}, tot[NS];
        if (planet)
            for (int q = 0; q < 3; ++q) {
                vals[q] = c.m * x[q];
                vals[3 + q] = wv * u[q];
                vals[6 + q] = c.m * wv * u[q];
            }
        if (!grid_reduce(D, vals, 9, tot, shm, warp_bodies, body_rows, rseq)) return false;
        for (int q = 0; q < 9; ++q) S[q] = tot[q];
        return true;
    }

    __device__ void whds_to_inertial(const double x[3], const double u[3], const double Rc[3], const double Vc[3],
                                     const double Smx[3], const double P[3], double fac) {
        for (int q = 0; q < 3; ++q) {
            h.r[q] = Rc[q] - Smx[q] * inv_M;
            h.v[q] = Vc[q] - P[q];
        }
        if (planet)
            for (int q = 0; q < 3; ++q) { b.r[q] = x[q] + h.r[q]; b.v[q] = u[q] / fac + Vc[q]; }
        if (is_host)
            for (int q = 0; q < 3; ++q) { b.r[q] = h.r[q]; b.v[q] = h.v[q]; }
    }

    __device__ bool step_whds() {
        const bool first = last_hist < 0.;
        if (first || last_hist + hist_period <= t) {
            spin_of(c, b.L, b.S);
            spin_of(hc, h.L, h.S);
            last_hist = first ? 0. : last_hist + hist_period;
        }
        double cm[6], tcm[6] = {0., 0., 0., 0., 0., 0.};
        if (!midpoint(half_dt, cm, tcm)) return false;
        double Rc[3], Vc[3], x[3] = {0., 0., 0.}, u[3] = {0., 0., 0.}, tx[3] = {0., 0., 0.}, tu[3] = {0., 0., 0.};
        for (int q = 0; q < 3; ++q) { Rc[q] = cm[q] * inv_M; Vc[q] = cm[3 + q] * inv_M; }
        const double fac = planet ? (hc.m + c.m) * inv_hm : 1.;   // (m0 + m) / m0
        const double wv = planet ? c.m / (hc.m + c.m) : 0.;       // m / (m0 + m)
        if (planet)
            for (int q = 0; q < 3; ++q) { x[q] = b.r[q] - h.r[q]; u[q] = (b.v[q] - Vc[q]) * fac; }
        // part 1: Kepler drift (and the barycentre's), jump, back to inertial
        kepler(x, u, tx, tu);
        for (int q = 0; q < 3; ++q) Rc[q] += half_dt * Vc[q];
        double S[9];
        if (!whds_sums(x, u, wv, S)) return false;
        const double P[3] = {S[3], S[4], S[5]};
        double Smx[3];
        for (int q = 0; q < 3; ++q) Smx[q] = S[q] + half_dt * (P[q] * (Mtot - hc.m) - S[6 + q]);
        if (planet)
            for (int q = 0; q < 3; ++q) x[q] += half_dt * (P[q] - wv * u[q]);
        whds_to_inertial(x, u, Rc, Vc, Smx, P, fac);
        // heliocentric positions after the jump for the pair loop (the host
        // at the origin)
        if (planet && primal_role())
            for (int q = 0; q < 3; ++q) D.pos[q * n + i] = x[q];
        const double zero[3] = {0., 0., 0.};
        double tzero[NT > 0 ? NT : 1][3] = {};
        if (!gravity(zero, tzero)) return false;
        if (__ldcg(D.bad) != ~0ull) return false;  // frozen at the first failing pair
        // part 2: kick, jump, Kepler drift, back to inertial
        if (planet)
            for (int q = 0; q < 3; ++q) {
                u[q] += dt * fac * a[q];
                x[q] += half_dt * (P[q] - wv * u[q]);
            }
        kepler(x, u, tx, tu);
        for (int q = 0; q < 3; ++q) Rc[q] += half_dt * Vc[q];
        if (!whds_sums(x, u, wv, S)) return false;
        const double P2[3] = {S[3], S[4], S[5]};
        whds_to_inertial(x, u, Rc, Vc, S, P2, fac);
        if (!midpoint(half_dt, nullptr, nullptr)) return false;
        t += dt;
        return true;
    }

    __device__ __forceinline__ bool step() {
        constexpr int AN = NT > 0 ? NT : 1;
        const bool tn = tan_on();
        const bool first = last_hist < 0.;
        if (first || last_hist + hist_period <= t) {
            spin_of(c, b.L, b.S);
            spin_of(hc, h.L, h.S);
            if (tn) {
                dspin_of(c, T.L, T.S);
                dspin_of(hc, HT.L, HT.S);
            }
            last_hist = first ? 0. : last_hist + hist_period;
        }
        double cm[6], tcm[6] = {0., 0., 0., 0., 0., 0.};
        if (!midpoint(half_dt, cm, tcm)) return false;
        // inertial -> democratic heliocentric (the barycentre's terms and the
        // jump's shift only in threads that hold a body: a warp without
        // bodies shares a body warp's SMSP and its FP64 pipe)
        double Rc[3] = {0., 0., 0.}, Vc[3] = {0., 0., 0.}, x[3] = {0., 0., 0.}, u[3] = {0., 0., 0.};
        double tRc[3] = {0., 0., 0.}, tVc[3] = {0., 0., 0.}, tx[3] = {0., 0., 0.}, tu[3] = {0., 0., 0.};
        if (has)
            for (int q = 0; q < 3; ++q) { Rc[q] = cm[q] * inv_M; Vc[q] = cm[3 + q] * inv_M; }
        if (planet)
            for (int q = 0; q < 3; ++q) { x[q] = b.r[q] - h.r[q]; u[q] = b.v[q] - Vc[q]; }
        if (tn)
            for (int q = 0; q < 3; ++q) {
                tRc[q] = tcm[q] * inv_M;
                tVc[q] = tcm[3 + q] * inv_M;
                tx[q] = planet ? T.r[q] - HT.r[q] : 0.;
                tu[q] = planet ? T.v[q] - tVc[q] : 0.;
            }
        // part 1: Kepler drift (and the barycentre's), jump, back to inertial
        kepler(x, u, tx, tu);
        if (has)
            for (int q = 0; q < 3; ++q) Rc[q] += half_dt * Vc[q];
        if (tn)
            for (int q = 0; q < 3; ++q) tRc[q] += half_dt * tVc[q];
        double S[6], tS_all[AN][6];
        if (!planet_sums(x, u, tx, tu, true, S, tS_all)) return false;
        double shift[3] = {0., 0., 0.}, tshift[AN][3];
        if (has)
            for (int q = 0; q < 3; ++q) {
                shift[q] = half_dt * S[3 + q] * inv_hm;        // jump: dt/2 P / m_host
                S[q] += shift[q] * (Mtot - hc.m);              // sum_p m_p (x_p + shift)
            }
        const double P[3] = {S[3], S[4], S[5]};
        if (planet)
            for (int q = 0; q < 3; ++q) x[q] += shift[q];
        // every direction's shift (the pair loop needs them all), then this
        // thread's own sums
        if constexpr (NT > 0)
            for (int d = 0; d < NT; ++d)
                for (int q = 0; q < 3; ++q) tshift[d][q] = half_dt * tS_all[d][3 + q] * inv_hm;
        double tS[6] = {0., 0., 0., 0., 0., 0.}, tP[3] = {0., 0., 0.};
        if (tn) {
            for (int q = 0; q < 6; ++q) tS[q] = tS_all[dir][q];
            for (int q = 0; q < 3; ++q) {
                tS[q] += tshift[dir][q] * (Mtot - hc.m);
                tP[q] = tS[3 + q];
                if (planet) tx[q] += tshift[dir][q];
            }
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
        if (tn && planet)
            for (int q = 0; q < 3; ++q) {
                tu[q] += dt * da[q];
                tx[q] += half_dt * tP[q] * inv_hm;
            }
        kepler(x, u, tx, tu);
        if (has)
            for (int q = 0; q < 3; ++q) Rc[q] += half_dt * Vc[q];
        if (tn)
            for (int q = 0; q < 3; ++q) tRc[q] += half_dt * tVc[q];
        if (!planet_sums(x, u, tx, tu, false, S, tS_all)) return false;
        if (tn)
            for (int q = 0; q < 6; ++q) tS[q] = tS_all[dir][q];
        to_inertial(x, u, Rc, Vc, S, tx, tu, tRc, tVc, tS);
        if (!midpoint(half_dt, nullptr, nullptr)) return false;
        t += dt;
        return true;
    }
};

// Thread roles: block b holds bodies [b per_block, (b + 1) per_block); thread
// r per_block + l of the block is role r of body b per_block + l (r = 0..NT).
// CO: the coordinates (posi_coords); Jacobi and WHDS (NT = 0 only) are
// kernels of their own, so that the democratic-heliocentric one carries none
// of their code.
template <int NT, int CO = POSI_DEMOCRATIC_HELIOCENTRIC>
__global__ void __launch_bounds__(kBlock, 1) large_steps_kernel(LDev D, int64_t n_steps) {
    constexpr bool JAC = CO == POSI_JACOBI;
    static_assert(CO == POSI_DEMOCRATIC_HELIOCENTRIC || NT == 0, "Jacobi and WHDS carry no tangents");
    __shared__ double shm[(kBlock / 32 + 1) * BP_ROW];
    if (threadIdx.x == 0) barrier_count(0) = barrier_count(1) = 0;
    if ((int)blockIdx.x >= D.nbb) {
        // a block without bodies joins the pair loop of every step and leaves
        // once the body blocks have finished (ctl) or a pair has failed
        const int host = (int)D.si[POSI_SI_HOST];
        const int64_t p1 = host == 0 ? 1 : 0;
        for (;;) {
            if (!grid_barrier(D)) return;
            if (__ldcg(D.ctl) != 0) return;
            pair_loop<NT>(D, host, p1, JAC);
            if (!grid_barrier(D)) return;
            if (__ldcg(D.bad) != ~0ull) return;
        }
    }
    Large<NT> S(D, shm);
    S.n = D.n;
    const int roles = 1 + NT;
    const int role = (int)threadIdx.x / D.per_block;
    S.i = role < roles ? (int64_t)blockIdx.x * D.per_block + (int64_t)(threadIdx.x % D.per_block) : INT64_MAX;
    S.dir = NT > 0 && role >= 1 && role < roles ? role - 1 : -1;
    S.host = (int)D.si[POSI_SI_HOST];
    S.has = S.i < S.n;
    {
        const int w0 = (int)(threadIdx.x & ~31);
        const int64_t warp_first = (int64_t)blockIdx.x * D.per_block + (w0 % D.per_block);
        S.warp_bodies = w0 < D.per_block * roles && warp_first < S.n;
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
    S.da[0] = S.da[1] = S.da[2] = 0.;
    S.hc = load_const(D, S.host);
    load_state(D, S.host, S.h);
    if (S.has) {
        S.c = load_const(D, S.i);
        load_state(D, S.i, S.b);
    } else {
        S.c = S.hc;
        S.b = S.h;
    }
    for (int q = 0; q < 3; ++q) {
        S.T.r[q] = S.T.v[q] = S.T.L[q] = S.T.S[q] = 0.;
        S.HT.r[q] = S.HT.v[q] = S.HT.L[q] = S.HT.S[q] = 0.;
    }
    if (S.tan_on()) {
        const int64_t n = S.n, src = S.has ? S.i : S.host;
        const double* base = D.tan + (size_t)S.dir * 12 * n;
        for (int q = 0; q < 3; ++q) {
            S.HT.r[q] = base[(0 + q) * n + S.host];
            S.HT.v[q] = base[(3 + q) * n + S.host];
            S.HT.L[q] = base[(6 + q) * n + S.host];
            S.HT.S[q] = base[(9 + q) * n + S.host];
            S.T.r[q] = base[(0 + q) * n + src];
            S.T.v[q] = base[(3 + q) * n + src];
            S.T.L[q] = base[(6 + q) * n + src];
            S.T.S[q] = base[(9 + q) * n + src];
        }
    }
    // total mass, in block order
    {
        double vals[Large<NT>::NS] = {};
        vals[0] = S.has && S.primal_role() ? S.c.m : 0.;
        double tot[1];
        if (!grid_reduce(D, vals, 1, tot, shm, S.warp_bodies, S.body_rows, S.rseq)) return;
        S.Mtot = tot[0];
        S.inv_M = 1. / S.Mtot;
        S.inv_hm = 1. / S.hc.m;
    }
    S.jac = JAC;
    S.kgm = CO == POSI_WHDS ? S.hc.mg + (S.planet ? S.c.mg : 0.) : S.hc.mg;
    S.p1 = S.host == 0 ? 1 : 0;
    S.eta_ex = S.eta_in = S.hc.m;
    for (int q = 0; q < 3; ++q) S.Rb[q] = S.Vb[q] = 0.;
    if constexpr (JAC) {
        // the masses before each body and its cumulative GM (host first)
        double vals[Large<NT>::NS] = {}, ex[Large<NT>::NS], tot[Large<NT>::NS];
        if (S.planet) { vals[0] = S.c.m; vals[1] = S.c.mg; }
        if (!grid_scan(D, vals, 2, ex, tot, shm, S.body_rows, S.rseq)) return;
        S.eta_ex = S.hc.m + ex[0];
        S.eta_in = S.eta_ex + S.c.m;
        S.kgm = S.hc.mg + ex[1] + (S.planet ? S.c.mg : 0.);
    }
    const bool live = (D.si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK) == 0;
    int64_t done = 0;
    bool ok = true;
    if (live) {
        for (int64_t k = 0; k < n_steps; ++k) {
            if constexpr (JAC) ok = S.step_jacobi();
            else if constexpr (CO == POSI_WHDS) ok = S.step_whds();
            else ok = S.step();
            if (!ok) break;
            ++done;
            if (S.t + S.dt > S.time_limit) break;
        }
    }
    // the blocks without bodies wait for another pair loop: release them,
    // unless a failing pair (which every block reads after the last pair
    // loop) or a failed barrier has sent them away already
    if (!(__ldcg(D.err) & LE_BARRIER) && __ldcg(D.bad) == ~0ull) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(D.ctl, 1);
        grid_barrier(D);
    }
    if (__ldcg(D.err) & LE_BARRIER) return;  // state left as it was: the launch failed
    if (S.has && S.primal_role()) {
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
    if (S.has && S.tan_on()) {
        const int64_t n = S.n, i = S.i;
        double* base = D.tan + (size_t)S.dir * 12 * n;
        for (int q = 0; q < 3; ++q) {
            base[(0 + q) * n + i] = S.T.r[q];
            base[(3 + q) * n + i] = S.T.v[q];
            base[(6 + q) * n + i] = S.T.L[q];
            base[(9 + q) * n + i] = S.T.S[q];
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
