// posi_host.cu -- C ABI of the GB300 WHFast + tidal-effects path.
//
// Host side of the boundary declared in include/posidonius_gb300.h: case
// reading, device buffers (field-major SoA), host<->device transposes, the
// per-body-count buckets of the batched kernel and the CUDA-graph replay of
// its launches.  All floating-point work runs in the kernels of
// kernels_exact.cu / kernels_fast.cu; the only host arithmetic is the Roche
// radius table (libm pow, as src/particles/universe.rs:177-196 uses it) and
// the step-time bookkeeping of the plain path.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/posidonius_gb300.h"
#include "bincode.hpp"
#include "case_reader.hpp"
#include "json.hpp"
#include "kernels.h"
#include "snapshot.hpp"

#include <ctime>
#include <unistd.h>

using posi::DevView;
using posi::LaunchArgs;

namespace {

thread_local std::string g_last_error;

// AoS (row-major, rows x fields) <-> SoA (fields x rows) on the device.
template <typename T>
__global__ void aos_to_soa(const T* __restrict__ aos, T* __restrict__ soa, int64_t rows, int fields) {
    const int64_t total = rows * fields;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k / fields;
        const int f = (int)(k % fields);
        soa[(int64_t)f * rows + r] = aos[k];
    }
}
template <typename T>
__global__ void soa_to_aos(const T* __restrict__ soa, T* __restrict__ aos, int64_t rows, int fields) {
    const int64_t total = rows * fields;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = k / fields;
        const int f = (int)(k % fields);
        aos[k] = soa[(int64_t)f * rows + r];
    }
}

int grid_for(int64_t n) {
    int64_t b = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

#define CK(call)                                                        \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) {                                        \
            g_last_error = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return POSI_ERR_CUDA;                                       \
        }                                                               \
    } while (0)

}  // namespace

struct Bucket {
    int G;
    int32_t offset;  // into the system list
    int32_t count;
};

struct posi_batch {
    int64_t n_sys = 0, nmax = 0, stride = 0;
    int mode = POSI_MODE_EXACT;
    int mapping = POSI_MAP_AUTO;
    double* d_bf = nullptr;
    int64_t* d_bi = nullptr;
    double* d_sf = nullptr;
    int64_t* d_si = nullptr;
    double* d_roche = nullptr;
    double* d_tables = nullptr;
    int32_t* d_list = nullptr;
    int32_t* d_flags = nullptr;
    double* d_hist = nullptr;  // historic records (attached by the snapshot writer)
    // IAS15 batches (every system integrated by IAS15): the per-body
    // Gauss-Radau state [POSI_IAS_COUNT][stride]
    bool ias15 = false;
    double* d_ias = nullptr;
    void* d_stage = nullptr;  // AoS staging buffer
    size_t stage_bytes = 0;
    int64_t n_tables = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<Bucket> buckets;
    std::vector<int64_t> n_of;    // bodies per system
    std::vector<int64_t> key_of;  // ordering key: bodies, effect flags, coordinates
    std::vector<int32_t> host_list;
    std::map<int64_t, int> mapping_of_n;
    std::map<int64_t, double> tuned_ms_of_n;  // autotuner: best probe time per body count
    std::map<int64_t, std::array<double, 6>> probe_ms_of_n;  // every probe, by log2 of the lanes
    double last_ms = 0.;
    int64_t last_launches = 0;
    cudaGraphExec_t graph = nullptr;
    int64_t graph_steps = -1, graph_spl = -1;
    // balanced schedules of the captured graph (whfast_sched_kernel tables)
    bool balanced = true;
    int sms = 0;
    int32_t* d_sched = nullptr;
    // one stream per bucket: the buckets' launches of a chunk run side by
    // side (disjoint systems), forked from and joined back to `stream`
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> side_done;
    cudaEvent_t fork = nullptr;

    DevView view(int32_t list_offset, int32_t count) const {
        DevView v;
        v.n_sys = n_sys; v.nmax = nmax; v.stride = stride;
        v.bf = d_bf; v.bi = d_bi; v.sf = d_sf; v.si = d_si;
        v.roche = d_roche; v.tables = d_tables;
        v.list = d_list + list_offset; v.n_list = count;
        v.step_flags = d_flags;
        v.hist = d_hist;
        v.rec = nullptr;
        v.ias = d_ias;
        return v;
    }
    cudaError_t launch(const Bucket& bk, const LaunchArgs& a0, cudaStream_t on = nullptr) const {
        LaunchArgs a = a0;
        a.G = bk.G;
        if (ias15 && a.op == posi::OP_STEPS) a.op = posi::OP_IAS15_STEPS;
        DevView v = view(bk.offset, bk.count);
        cudaStream_t st = on ? on : stream;
        return mode == POSI_MODE_EXACT ? posi::launch_exact(v, a, st) : posi::launch_fast(v, a, st);
    }
};

struct posi_handle {
    posi_batch* b = nullptr;
    // host mirror of the system scalars (the device copy is authoritative)
    std::vector<int64_t> si;
    std::vector<double> sf;
    // the case document the run started from (recovery snapshots rewrite it)
    std::shared_ptr<posi::json::Value> doc;
    // historic snapshot file (src/integrator/output.rs:57-89)
    std::FILE* hist = nullptr;
};

namespace {

void free_batch(posi_batch* b) {
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (cudaStream_t st : b->side) cudaStreamDestroy(st);
    for (cudaEvent_t e : b->side_done) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    cudaFree(b->d_sched);
    cudaFree(b->d_bf); cudaFree(b->d_bi); cudaFree(b->d_sf); cudaFree(b->d_si);
    cudaFree(b->d_roche); cudaFree(b->d_tables); cudaFree(b->d_list); cudaFree(b->d_flags);
    cudaFree(b->d_stage);
    cudaFree(b->d_hist);
    cudaFree(b->d_ias);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int validate_system(const int64_t* si, int64_t nmax, std::string& err) {
    const int64_t n = si[POSI_SI_N], host = si[POSI_SI_HOST], coords = si[POSI_SI_COORDS];
    if (n < 1 || n > nmax) { err = "system body count out of range"; return POSI_ERR_ARG; }
    if (posi::group_size_for(n) == 0) { err = "too many bodies for the batched kernel"; return POSI_ERR_UNSUPPORTED; }
    if (host < 0 || host >= n) { err = "host index out of range"; return POSI_ERR_ARG; }
    if (coords < POSI_JACOBI || coords > POSI_WHDS) { err = "unknown coordinates type"; return POSI_ERR_ARG; }
    const int64_t integ = si[POSI_SI_INTEGRATOR];
    if (integ != POSI_INTEGRATOR_WHFAST && integ != POSI_INTEGRATOR_IAS15) { err = "unknown integrator"; return POSI_ERR_ARG; }
    return POSI_OK;
}

// Upload host AoS arrays into the device SoA array `dst` (rows x fields).
template <typename T>
int upload_aos(posi_batch* b, const T* host, T* dst, int64_t rows, int fields) {
    const size_t bytes = (size_t)rows * fields * sizeof(T);
    CK(cudaMemcpyAsync(b->d_stage, host, bytes, cudaMemcpyHostToDevice, b->stream));
    aos_to_soa<T><<<grid_for(rows * fields), 256, 0, b->stream>>>((const T*)b->d_stage, dst, rows, fields);
    CK(cudaGetLastError());
    return POSI_OK;
}

template <typename T>
int download_aos(const posi_batch* b, T* host, const T* src, int64_t rows, int fields) {
    const size_t bytes = (size_t)rows * fields * sizeof(T);
    soa_to_aos<T><<<grid_for(rows * fields), 256, 0, b->stream>>>(src, (T*)b->d_stage, rows, fields);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host, b->d_stage, bytes, cudaMemcpyDeviceToHost, b->stream));
    return POSI_OK;
}

// Systems are grouped by lanes per system (one body per lane); within a
// group they are ordered by body count, then effect flags and coordinates,
// so that the groups sharing a warp take the same branches.  `chosen` maps a
// body count to its lanes per system (the autotuner's choice); otherwise the
// smallest group that holds the system, or the caller's fixed mapping.
int build_buckets(posi_batch* b, const int64_t* sys_i64, const std::map<int64_t, int>* chosen = nullptr) {
    std::map<int, std::vector<int32_t>> by_g;
    b->n_of.resize(b->n_sys);
    b->key_of.resize(b->n_sys);
    for (int64_t s = 0; s < b->n_sys; ++s) {
        const int64_t* si = sys_i64 + s * POSI_SI_COUNT;
        const int64_t n = si[POSI_SI_N];
        b->n_of[s] = n;
        b->key_of[s] = (((n * 2 + si[POSI_SI_TIDES]) * 2 + si[POSI_SI_FLAT]) * 2 + si[POSI_SI_GR]) * 4 +
                       si[POSI_SI_COORDS];
        b->key_of[s] = b->key_of[s] * 2 + si[POSI_SI_EVOLUTION];
        int G = posi::group_size_for(n);
        if (chosen && chosen->count(n)) {
            G = chosen->at(n);
        } else if (b->mapping >= POSI_MAP_LANES2 && b->mapping <= POSI_MAP_WARP && b->mapping >= G) {
            G = b->mapping;
        }
        by_g[G].push_back((int32_t)s);
        b->mapping_of_n[n] = G;
    }
    std::vector<int32_t> list;
    b->buckets.clear();
    for (auto& kv : by_g) {
        std::stable_sort(kv.second.begin(), kv.second.end(),
                         [&](int32_t x, int32_t y) { return b->key_of[x] < b->key_of[y]; });
        Bucket bk;
        bk.G = kv.first;
        bk.offset = (int32_t)list.size();
        bk.count = (int32_t)kv.second.size();
        list.insert(list.end(), kv.second.begin(), kv.second.end());
        b->buckets.push_back(bk);
    }
    if (!b->d_list) CK(cudaMalloc(&b->d_list, (size_t)std::max<int64_t>(1, b->n_sys) * sizeof(int32_t)));
    CK(cudaMemcpyAsync(b->d_list, list.data(), list.size() * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    b->host_list = list;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        b->graph_steps = -1;
    }
    return POSI_OK;
}

// Balanced schedule of one bucket's launch of `steps` steps for
// whfast_sched_kernel: one 256-thread block per SM, eight warp slots each.
// With `jobs` warps of systems between one and two per SMSP, the first
// `light` blocks hold four jobs (one warp per SMSP) and the others eight (two
// per SMSP).  A lone warp runs kLoneSpeed times as many steps per unit time as
// one sharing its SMSP (measured on GB300: 104.8 against 169.2 us per step of
// the 8-body ensemble at 2432 and 4864 systems), so in every sub-launch the
// jobs in lone slots get that many more steps, and the jobs with the most
// steps left take the lone slots.
// table: per sub-launch, the job of every slot (-1: idle) then its steps.
// Returns false when the bucket needs no schedule.
bool build_schedule(int sms, int jobs, int64_t steps, std::vector<int32_t>& table, int& launches) {
    constexpr double kLoneSpeed = 1.6;
    // about this many sub-launches per launch of `steps` steps, at least 50
    // steps each: a sub-launch costs tens of microseconds (state load and
    // store, launch, the tail of its slowest slot), which a short launch
    // does not win back -- 20 steps in 17 sub-launches took 230 us per step
    // on the 8-body ensemble against 213 us for one plain launch
    const int64_t kSubLaunches = std::min<int64_t>(12, steps / 50);
    if (kSubLaunches < 2) return false;
    const int per = posi::kSchedBlockThreads / 32;
    const int slots = sms * per;
    if (sms <= 0 || jobs <= slots / 2 || jobs >= slots) return false;
    const int light = (slots - jobs) / (per / 2);
    if (light < 1) return false;
    const int64_t q = std::max<int64_t>(1, steps / kSubLaunches);
    const int64_t ql = std::max<int64_t>(1, (int64_t)std::llround(kLoneSpeed * (double)q));
    std::vector<int64_t> rem((size_t)jobs, steps);
    std::vector<int> order((size_t)jobs);
    table.clear();
    launches = 0;
    for (;;) {
        bool left = false;
        for (int64_t r : rem) left = left || r > 0;
        if (!left) break;
        for (int j = 0; j < jobs; ++j) order[(size_t)j] = j;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return rem[(size_t)x] > rem[(size_t)y]; });
        std::vector<int32_t> job((size_t)slots, -1), st((size_t)slots, 0);
        int k = 0;
        for (int blk = 0; blk < sms && k < jobs; ++blk) {
            const bool lone = blk < light;
            for (int w = 0; w < (lone ? per / 2 : per) && k < jobs; ++w) {
                const int j = order[(size_t)k++];
                const int64_t s = std::min(rem[(size_t)j], lone ? ql : q);
                if (s <= 0) continue;
                job[(size_t)(blk * per + w)] = j;
                st[(size_t)(blk * per + w)] = (int32_t)s;
                rem[(size_t)j] -= s;
            }
        }
        table.insert(table.end(), job.begin(), job.end());
        table.insert(table.end(), st.begin(), st.end());
        if (++launches > 100000) return false;
    }
    return true;
}

posi_batch* create_batch(int64_t n_sys, int64_t nmax, const int64_t* si, const double* sf, const int64_t* bi,
                         const double* bf, const double* tables, int64_t n_tables, const double* roche, int mode,
                         int mapping, int* status) {
    auto fail = [&](int code, posi_batch* b) -> posi_batch* {
        free_batch(b);
        if (status) *status = code;
        return nullptr;
    };
    if (n_sys < 1 || nmax < 1 || nmax > POSI_MAX_BODIES || !si || !sf || !bi || !bf) {
        g_last_error = "bad arguments";
        return fail(POSI_ERR_ARG, nullptr);
    }
    if (mode != POSI_MODE_EXACT && mode != POSI_MODE_FAST) { g_last_error = "unknown mode"; return fail(POSI_ERR_ARG, nullptr); }
    if (mapping == POSI_MAP_THREAD) {
        g_last_error = "POSI_MAP_THREAD (one thread per system) is not built; the batched kernels map a system "
                       "onto a lane group (POSI_MAP_AUTO, POSI_MAP_LANES2..POSI_MAP_WARP)";
        return fail(POSI_ERR_UNSUPPORTED, nullptr);
    }
    if (mapping != POSI_MAP_AUTO && mapping != POSI_MAP_LANES2 && mapping != POSI_MAP_LANES4 &&
        mapping != POSI_MAP_LANES8 && mapping != POSI_MAP_LANES16 && mapping != POSI_MAP_WARP) {
        g_last_error = "unknown mapping";
        return fail(POSI_ERR_ARG, nullptr);
    }
    for (int64_t s = 0; s < n_sys; ++s) {
        std::string err;
        int rc = validate_system(si + s * POSI_SI_COUNT, nmax, err);
        if (rc != POSI_OK) { g_last_error = err; return fail(rc, nullptr); }
        if (si[s * POSI_SI_COUNT + POSI_SI_INTEGRATOR] != si[POSI_SI_INTEGRATOR]) {
            g_last_error = "a batch holds systems of one integrator";
            return fail(POSI_ERR_UNSUPPORTED, nullptr);
        }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        g_last_error = "no CUDA device";
        return fail(POSI_ERR_CUDA, nullptr);
    }
    posi_batch* b = new posi_batch();
    b->n_sys = n_sys;
    b->nmax = nmax;
    b->stride = n_sys * nmax;
    b->mode = mode;
    b->mapping = mapping;
    b->n_tables = std::max<int64_t>(1, n_tables);
    b->ias15 = si[POSI_SI_INTEGRATOR] == POSI_INTEGRATOR_IAS15;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess) { g_last_error = cudaGetErrorString(e); return false; }
        return true;
    };
    if (!ok(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) || !ok(cudaEventCreate(&b->ev0)) ||
        !ok(cudaEventCreate(&b->ev1)))
        return fail(POSI_ERR_CUDA, b);
    if (!ok(mode == POSI_MODE_EXACT ? posi::prepare_exact() : posi::prepare_fast())) return fail(POSI_ERR_CUDA, b);
    {
        int dev = 0;
        if (!ok(cudaGetDevice(&dev)) || !ok(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev)))
            return fail(POSI_ERR_CUDA, b);
    }
    const size_t nb = (size_t)b->stride;
    b->stage_bytes = std::max({nb * POSI_BF_COUNT * sizeof(double), nb * POSI_BI_COUNT * sizeof(int64_t),
                               b->ias15 ? nb * POSI_IAS_COUNT * sizeof(double) : (size_t)0,
                               (size_t)n_sys * POSI_SF_COUNT * sizeof(double),
                               (size_t)n_sys * POSI_SI_COUNT * sizeof(int64_t), nb * nmax * sizeof(double)});
    if (!ok(cudaMalloc(&b->d_bf, nb * POSI_BF_COUNT * sizeof(double))) ||
        !ok(cudaMalloc(&b->d_bi, nb * POSI_BI_COUNT * sizeof(int64_t))) ||
        !ok(cudaMalloc(&b->d_sf, (size_t)n_sys * POSI_SF_COUNT * sizeof(double))) ||
        !ok(cudaMalloc(&b->d_si, (size_t)n_sys * POSI_SI_COUNT * sizeof(int64_t))) ||
        !ok(cudaMalloc(&b->d_roche, nb * nmax * sizeof(double))) ||
        !ok(cudaMalloc(&b->d_tables, (size_t)b->n_tables * sizeof(double))) ||
        !ok(cudaMalloc(&b->d_flags, (size_t)n_sys * sizeof(int32_t))) || !ok(cudaMalloc(&b->d_stage, b->stage_bytes)))
        return fail(POSI_ERR_CUDA, b);
    if (b->ias15 && (!ok(cudaMalloc(&b->d_ias, nb * POSI_IAS_COUNT * sizeof(double))) ||
                     !ok(cudaMemsetAsync(b->d_ias, 0, nb * POSI_IAS_COUNT * sizeof(double), b->stream))))
        return fail(POSI_ERR_CUDA, b);
    int rc;
    if ((rc = upload_aos<int64_t>(b, si, b->d_si, n_sys, POSI_SI_COUNT)) != POSI_OK ||
        (rc = upload_aos<double>(b, sf, b->d_sf, n_sys, POSI_SF_COUNT)) != POSI_OK ||
        (rc = upload_aos<int64_t>(b, bi, b->d_bi, b->stride, POSI_BI_COUNT)) != POSI_OK ||
        (rc = upload_aos<double>(b, bf, b->d_bf, b->stride, POSI_BF_COUNT)) != POSI_OK)
        return fail(rc, b);
    if (!ok(cudaStreamSynchronize(b->stream))) return fail(POSI_ERR_CUDA, b);
    if (roche) {
        if (!ok(cudaMemcpyAsync(b->d_roche, roche, nb * nmax * sizeof(double), cudaMemcpyHostToDevice, b->stream)))
            return fail(POSI_ERR_CUDA, b);
    } else if (!ok(cudaMemsetAsync(b->d_roche, 0, nb * nmax * sizeof(double), b->stream))) {
        return fail(POSI_ERR_CUDA, b);
    }
    if (tables && n_tables > 0) {
        if (!ok(cudaMemcpyAsync(b->d_tables, tables, (size_t)n_tables * sizeof(double), cudaMemcpyHostToDevice, b->stream)))
            return fail(POSI_ERR_CUDA, b);
    } else if (!ok(cudaMemsetAsync(b->d_tables, 0, (size_t)b->n_tables * sizeof(double), b->stream))) {
        return fail(POSI_ERR_CUDA, b);
    }
    if (!ok(cudaMemsetAsync(b->d_flags, 0, (size_t)n_sys * sizeof(int32_t), b->stream))) return fail(POSI_ERR_CUDA, b);
    if ((rc = build_buckets(b, si)) != POSI_OK) return fail(rc, b);
    if (!ok(cudaStreamSynchronize(b->stream))) return fail(POSI_ERR_CUDA, b);
    if (status) *status = POSI_OK;
    return b;
}

int run_op(posi_batch* b, const LaunchArgs& a) {
    for (const Bucket& bk : b->buckets) CK(b->launch(bk, a));
    CK(cudaStreamSynchronize(b->stream));
    return POSI_OK;
}

// src/particles/universe.rs:177-196 (libm pow, like Rust's f64::powf)
int compute_roche(posi_batch* b) {
    const size_t nb = (size_t)b->stride;
    std::vector<double> mass(nb), radius(nb), roche(nb * b->nmax, 0.);
    CK(cudaMemcpyAsync(mass.data(), b->d_bf + (size_t)POSI_BF_MASS * nb, nb * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaMemcpyAsync(radius.data(), b->d_bf + (size_t)POSI_BF_RADIUS * nb, nb * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    for (int64_t s = 0; s < b->n_sys; ++s) {
        const int64_t n = b->n_of[s];
        const size_t o = (size_t)s * b->nmax;
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = 0; j < n; ++j) {
                if (i == j) continue;
                const double ma = mass[o + i], mb = mass[o + j];
                double r;
                if (ma > mb) r = (radius[o + j] / 0.462) * std::pow(ma / mb, 1. / 3.);
                else r = (radius[o + i] / 0.462) * std::pow(mb / ma, 1. / 3.);
                roche[(o + i) * b->nmax + j] = r;
            }
    }
    CK(cudaMemcpyAsync(b->d_roche, roche.data(), roche.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return POSI_OK;
}

// The transposes and copies share one staging buffer; the stream orders them
// (a copy into or out of the buffer waits for the kernel before it), so one
// synchronisation at the end suffices.
int batch_get(const posi_batch* b, int64_t* si, double* sf, int64_t* bi, double* bf, double* roche) {
    int rc;
    if (si && (rc = download_aos<int64_t>(b, si, b->d_si, b->n_sys, POSI_SI_COUNT)) != POSI_OK) return rc;
    if (sf && (rc = download_aos<double>(b, sf, b->d_sf, b->n_sys, POSI_SF_COUNT)) != POSI_OK) return rc;
    if (bi && (rc = download_aos<int64_t>(b, bi, b->d_bi, b->stride, POSI_BI_COUNT)) != POSI_OK) return rc;
    if (bf && (rc = download_aos<double>(b, bf, b->d_bf, b->stride, POSI_BF_COUNT)) != POSI_OK) return rc;
    if (roche)
        CK(cudaMemcpyAsync(roche, b->d_roche, (size_t)b->stride * b->nmax * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return POSI_OK;
}

int batch_set(posi_batch* b, const int64_t* si, const double* sf, const int64_t* bi, const double* bf) {
    int rc;
    if (si && (rc = upload_aos<int64_t>(b, si, b->d_si, b->n_sys, POSI_SI_COUNT)) != POSI_OK) return rc;
    if (sf && (rc = upload_aos<double>(b, sf, b->d_sf, b->n_sys, POSI_SF_COUNT)) != POSI_OK) return rc;
    if (bi && (rc = upload_aos<int64_t>(b, bi, b->d_bi, b->stride, POSI_BI_COUNT)) != POSI_OK) return rc;
    if (bf && (rc = upload_aos<double>(b, bf, b->d_bf, b->stride, POSI_BF_COUNT)) != POSI_OK) return rc;
    CK(cudaStreamSynchronize(b->stream));
    return POSI_OK;
}

int refresh_mirror(posi_handle* h) {
    return batch_get(h->b, h->si.data(), h->sf.data(), nullptr, nullptr, nullptr);
}

posi_handle* make_handle(posi_batch* b, const int64_t* si, const double* sf) {
    posi_handle* h = new posi_handle();
    h->b = b;
    h->si.assign(si, si + POSI_SI_COUNT);
    h->sf.assign(sf, sf + POSI_SF_COUNT);
    return h;
}

}  // namespace

extern "C" {

const char* posi_version(void) { return "posidonius-gb300 0.1 (sm_103a, FP64)"; }

const char* posi_status_string(int status) {
    switch (status) {
        case POSI_OK: return "ok";
        case POSI_COMPLETED: return "Simulation completed";
        case POSI_ERR_ARG: return "bad argument";
        case POSI_ERR_IO: return "file missing or unreadable";
        case POSI_ERR_PARSE: return "malformed case";
        case POSI_ERR_UNSUPPORTED: return "unsupported case";
        case POSI_ERR_CUDA: return "CUDA error";
        case POSI_ERR_PHYSICS: return "physics event (collision, Roche limit, ejection)";
        case POSI_ERR_STATE: return "invalid state";
        default: return "unknown status";
    }
}

// Detail of the last error on this thread (not part of the reference surface).
const char* posi_last_error(void) { return g_last_error.c_str(); }

int posi_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

}  // extern "C"

namespace {
int load_case_file(const char* path, posi::FlatSystem& fs, posi::json::Value* doc_out = nullptr) {
    if (!path) return POSI_ERR_ARG;
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        g_last_error = std::string("cannot open ") + path;
        return POSI_ERR_IO;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    posi::json::Value doc;
    std::string err;
    // src/integrator/output.rs:178-191: a path whose extension is not
    // "json" holds a bincode snapshot
    if (posi::is_bincode_path(path)) {
        if (!posi::bincode_to_json(text, doc, err)) {
            g_last_error = err;
            return POSI_ERR_PARSE;
        }
    } else {
        posi::json::Parser parser(text.data(), text.size());
        if (!parser.parse(doc, err)) {
            g_last_error = "JSON: " + err;
            return POSI_ERR_PARSE;
        }
    }
    int rc = posi::read_case(doc, fs, err);
    if (rc != POSI_OK) g_last_error = err;
    if (rc == POSI_OK && doc_out) *doc_out = std::move(doc);
    return rc;
}
}  // namespace

extern "C" {

int posi_read_case(const char* path, int64_t* n, int64_t* n_tables, int64_t* sys_i64, double* sys_f64,
                   int64_t* body_i64, double* body_f64, double* tables, double* roche) {
    posi::FlatSystem fs;
    int rc = load_case_file(path, fs);
    if (rc != POSI_OK) return rc;
    if (n) *n = fs.n;
    if (n_tables) *n_tables = (int64_t)fs.tables.size();
    if (sys_i64) std::memcpy(sys_i64, fs.si.data(), fs.si.size() * sizeof(int64_t));
    if (sys_f64) std::memcpy(sys_f64, fs.sf.data(), fs.sf.size() * sizeof(double));
    if (body_i64) std::memcpy(body_i64, fs.bi.data(), fs.bi.size() * sizeof(int64_t));
    if (body_f64) std::memcpy(body_f64, fs.bf.data(), fs.bf.size() * sizeof(double));
    if (tables && !fs.tables.empty()) std::memcpy(tables, fs.tables.data(), fs.tables.size() * sizeof(double));
    if (roche) std::memcpy(roche, fs.roche.data(), fs.roche.size() * sizeof(double));
    return POSI_OK;
}

int posi_read_case_ias15(const char* path, double* body_ias) {
    posi::FlatSystem fs;
    int rc = load_case_file(path, fs);
    if (rc != POSI_OK) return rc;
    if (fs.si[POSI_SI_INTEGRATOR] != POSI_INTEGRATOR_IAS15) {
        g_last_error = "not an IAS15 case";
        return POSI_ERR_STATE;
    }
    if (body_ias) std::memcpy(body_ias, fs.ias.data(), fs.ias.size() * sizeof(double));
    return POSI_OK;
}

posi_handle* posi_universe_from_json(const char* path, int mode, int* status) {
    posi::FlatSystem fs;
    posi::json::Value doc;
    int rc = load_case_file(path, fs, &doc);
    if (rc != POSI_OK) {
        if (status) *status = rc;
        return nullptr;
    }
    posi_batch* b = create_batch(1, fs.n, fs.si.data(), fs.sf.data(), fs.bi.data(), fs.bf.data(),
                                 fs.tables.empty() ? nullptr : fs.tables.data(), (int64_t)fs.tables.size(),
                                 fs.roche.data(), mode, POSI_MAP_AUTO, status);
    if (!b) return nullptr;
    if (b->ias15 && (rc = posi_batch_set_ias15(b, fs.ias.data())) != POSI_OK) {
        free_batch(b);
        if (status) *status = rc;
        return nullptr;
    }
    posi_handle* h = make_handle(b, fs.si.data(), fs.sf.data());
    h->doc = std::make_shared<posi::json::Value>(std::move(doc));
    return h;
}

posi_handle* posi_universe_from_arrays(const int64_t* sys_i64, const double* sys_f64, const int64_t* body_i64,
                                       const double* body_f64, const double* tables, int64_t n_tables,
                                       const double* roche, int mode, int* status) {
    if (!sys_i64 || !sys_f64) { if (status) *status = POSI_ERR_ARG; return nullptr; }
    const int64_t n = sys_i64[POSI_SI_N];
    posi_batch* b = create_batch(1, n, sys_i64, sys_f64, body_i64, body_f64, tables, n_tables, roche, mode,
                                 POSI_MAP_AUTO, status);
    if (!b) return nullptr;
    return make_handle(b, sys_i64, sys_f64);
}

void posi_destroy(posi_handle* h) {
    if (!h) return;
    if (h->hist) std::fclose(h->hist);
    free_batch(h->b);
    delete h;
}

int posi_get_n_particles(const posi_handle* h, int64_t* n) {
    if (!h || !n) return POSI_ERR_ARG;
    *n = h->si[POSI_SI_N];
    return POSI_OK;
}

int posi_get_current_time(const posi_handle* h, double* t) {
    if (!h || !t) return POSI_ERR_ARG;
    *t = h->sf[POSI_SF_TIME];
    return POSI_OK;
}

int posi_get_n_historic_snapshots(const posi_handle* h, int64_t* n) {
    if (!h || !n) return POSI_ERR_ARG;
    *n = h->si[POSI_SI_N_HIST];
    return POSI_OK;
}

// src/integrator/whfast.rs:187-208 (the evolving-body table-range check of the
// reference does not apply: tables are read as they stand)
int posi_set_time_limit(posi_handle* h, double time_limit) {
    if (!h) return POSI_ERR_ARG;
    if (time_limit > 0. && h->sf[POSI_SF_TIME_LIMIT] != time_limit) {
        if (time_limit < h->sf[POSI_SF_TIME_LIMIT] && time_limit < h->sf[POSI_SF_TIME]) {
            g_last_error = "new time limit is smaller than the current time";
            return POSI_ERR_STATE;
        }
        h->sf[POSI_SF_TIME_LIMIT] = time_limit;
        // a completed run may continue under a larger limit
        if ((h->si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK) == POSI_SYS_COMPLETED)
            h->si[POSI_SI_STATUS] &= ~(int64_t)POSI_SYS_FATAL_MASK;
        return batch_set(h->b, h->si.data(), h->sf.data(), nullptr, nullptr);
    }
    return POSI_OK;
}

// src/integrator/whfast.rs:210-224
int posi_set_snapshot_periods(posi_handle* h, double historic_period, double recovery_period) {
    if (!h) return POSI_ERR_ARG;
    if (historic_period > 0.) h->sf[POSI_SF_HIST_PERIOD] = historic_period;
    if (recovery_period > 0.) h->sf[POSI_SF_REC_PERIOD] = recovery_period;
    return batch_set(h->b, nullptr, h->sf.data(), nullptr, nullptr);
}

int posi_initialize_physical_values(posi_handle* h) {
    if (!h) return POSI_ERR_ARG;
    if (h->sf[POSI_SF_TIME] != 0.) {
        g_last_error = "physical values cannot be initialized on a resumed simulation";
        return POSI_ERR_STATE;
    }
    return posi_batch_initialize_physical_values(h->b) == POSI_OK ? refresh_mirror(h) : POSI_ERR_CUDA;
}

namespace {
// The reference's panic text for a frozen system (src/particles/universe.rs:224-237,
// src/particles/common.rs:5-7, src/integrator/whfast.rs:792-805).
std::string fatal_message(const int64_t* si) {
    const int64_t pair = si[POSI_SI_FAIL_PAIR], i = pair / 1024, j = pair % 1024;
    switch (si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK) {
        case POSI_SYS_ROCHE:
            return "Particle " + std::to_string(i) + " was destroyed by particle " + std::to_string(j) +
                   " due to close encounter!";
        case POSI_SYS_COLLISION:
            return "Collision between particle " + std::to_string(i) + " and " + std::to_string(j) + "!";
        case POSI_SYS_EJECTED: return "Particle " + std::to_string(j) + " has been ejected!";
        case POSI_SYS_ZERO_INERTIA: return "Moment of inertia is zero";
        case POSI_SYS_BISECTION_LIMIT: return "Kepler solver bisection did not converge";
        default: return "fatal system status " + std::to_string(si[POSI_SI_STATUS]);
    }
}
}  // namespace

namespace {
// src/integrator/ias15.rs:420-463, n_steps times: the adaptive step makes the
// triggers unpredictable on the host, so every step is one launch followed by
// a read of its trigger flags, its historic record and the system status.
int iterate_ias15(posi_handle* h, int64_t n_steps, int64_t* steps_done, int* recovery_trigger) {
    posi_batch* b = h->b;
    const int64_t n = h->si[POSI_SI_N];
    std::vector<double> record;
    std::vector<unsigned char> bytes;
    if (h->hist) record.resize((size_t)n * posi::kHistoryFields);
    LaunchArgs a{};
    a.op = posi::OP_STEPS;
    a.n_steps = 1;
    const int64_t it0 = h->si[POSI_SI_ITERATION];
    bool rec = false;
    for (int64_t k = 0; k < n_steps && !rec; ++k) {
        if (h->hist) CK(cudaMemsetAsync(b->d_hist, 0xff, record.size() * sizeof(double), b->stream));
        CK(cudaMemsetAsync(b->d_flags, 0, sizeof(int32_t), b->stream));
        for (const Bucket& bk : b->buckets) CK(b->launch(bk, a));
        int32_t flags = 0;
        CK(cudaMemcpyAsync(&flags, b->d_flags, sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream));
        if (h->hist)
            CK(cudaMemcpyAsync(record.data(), b->d_hist, record.size() * sizeof(double), cudaMemcpyDeviceToHost,
                               b->stream));
        CK(cudaStreamSynchronize(b->stream));
        if (h->hist && !std::isnan(record[0])) {
            bytes.clear();
            posi::encode_history_record(record.data(), n, bytes);
            if (std::fwrite(bytes.data(), 1, bytes.size(), h->hist) != bytes.size()) {
                g_last_error = "cannot write the history file";
                return POSI_ERR_IO;
            }
        }
        int rc = refresh_mirror(h);
        if (rc != POSI_OK) return rc;
        if (steps_done) *steps_done = h->si[POSI_SI_ITERATION] - it0;
        const int64_t fatal = h->si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK;
        if (fatal == POSI_SYS_COMPLETED) return POSI_COMPLETED;
        if (fatal) {
            g_last_error = fatal_message(h->si.data());
            return POSI_ERR_PHYSICS;
        }
        rec = (flags & 1) != 0;
    }
    if (recovery_trigger) *recovery_trigger = rec ? 1 : 0;
    return POSI_OK;
}
}  // namespace

int posi_iterate(posi_handle* h, int64_t n_steps, int64_t* steps_done, int* recovery_trigger) {
    if (!h || n_steps < 0) return POSI_ERR_ARG;
    if (steps_done) *steps_done = 0;
    if (recovery_trigger) *recovery_trigger = 0;
    if (h->si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK) {
        if ((h->si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK) == POSI_SYS_COMPLETED) return POSI_COMPLETED;
        g_last_error = fatal_message(h->si.data());
        return POSI_ERR_PHYSICS;
    }
    if (h->b->ias15) return iterate_ias15(h, n_steps, steps_done, recovery_trigger);
    // Predict, with the kernel's own time arithmetic, how many steps run before
    // a step reports a recovery trigger or completes the simulation; the plain
    // path then runs exactly that many steps.
    double t = h->sf[POSI_SF_TIME], last_hist = h->sf[POSI_SF_LAST_HIST];
    const double dt = h->sf[POSI_SF_DT], limit = h->sf[POSI_SF_TIME_LIMIT];
    const double hp = h->sf[POSI_SF_HIST_PERIOD], lr = h->sf[POSI_SF_LAST_REC], rp = h->sf[POSI_SF_REC_PERIOD];
    int64_t k = 0;
    bool rec = false;
    while (k < n_steps) {
        const bool first = last_hist < 0.;
        const bool ht = last_hist + hp <= t;
        const bool rt = lr + rp <= t;
        if (first || ht) last_hist = first ? 0. : last_hist + hp;
        t += dt;
        ++k;
        if (t + dt > limit) break;
        if (first || rt) { rec = true; break; }
    }
    // The k steps run as few multi-step launches: one when no history file is
    // attached, else one per historic record (a launch opens with the
    // trigger step, whose record the kernel leaves in the device buffer; the
    // buffer is filled with NaN first, so a system that stopped earlier
    // leaves it untouched and nothing is appended).
    LaunchArgs a{};
    a.op = posi::OP_STEPS;
    posi_batch* b = h->b;
    const int64_t n = h->si[POSI_SI_N];
    std::vector<double> record;
    std::vector<unsigned char> bytes;
    if (h->hist) record.resize((size_t)n * posi::kHistoryFields);
    auto run_segment = [&](int64_t len, bool with_record) -> int {
        if (len == 0) return POSI_OK;
        if (with_record) CK(cudaMemsetAsync(b->d_hist, 0xff, record.size() * sizeof(double), b->stream));
        a.n_steps = len;
        for (const Bucket& bk : b->buckets) CK(b->launch(bk, a));
        if (!with_record) return POSI_OK;
        CK(cudaMemcpyAsync(record.data(), b->d_hist, record.size() * sizeof(double), cudaMemcpyDeviceToHost,
                           b->stream));
        CK(cudaStreamSynchronize(b->stream));
        if (std::isnan(record[0])) return POSI_OK;
        bytes.clear();
        posi::encode_history_record(record.data(), n, bytes);
        if (std::fwrite(bytes.data(), 1, bytes.size(), h->hist) != bytes.size()) {
            g_last_error = "cannot write the history file";
            return POSI_ERR_IO;
        }
        return POSI_OK;
    };
    if (!h->hist) {
        int rc = run_segment(k, false);
        if (rc != POSI_OK) return rc;
    } else {
        double lh = h->sf[POSI_SF_LAST_HIST], tt = h->sf[POSI_SF_TIME];
        int64_t seg = 0;
        bool seg_record = false;
        for (int64_t i = 0; i < k; ++i) {
            const bool trig = lh < 0. || lh + hp <= tt;
            if (trig) {
                lh = lh < 0. ? 0. : lh + hp;
                int rc = run_segment(seg, seg_record);
                if (rc != POSI_OK) return rc;
                seg = 0;
                seg_record = true;
            }
            tt += dt;
            ++seg;
        }
        int rc = run_segment(seg, seg_record);
        if (rc != POSI_OK) return rc;
    }
    CK(cudaStreamSynchronize(b->stream));
    const int64_t it0 = h->si[POSI_SI_ITERATION];
    int rc = refresh_mirror(h);
    if (rc != POSI_OK) return rc;
    if (steps_done) *steps_done = h->si[POSI_SI_ITERATION] - it0;
    const int64_t fatal = h->si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK;
    if (fatal == POSI_SYS_COMPLETED) return POSI_COMPLETED;
    if (fatal) {
        g_last_error = fatal_message(h->si.data());
        return POSI_ERR_PHYSICS;
    }
    if (recovery_trigger) *recovery_trigger = rec ? 1 : 0;
    return POSI_OK;
}

int posi_gravity_calculate_acceleration(posi_handle* h, int ignore_terms) {
    if (!h || ignore_terms < 0 || ignore_terms > 2) return POSI_ERR_ARG;
    LaunchArgs a{};
    a.op = posi::OP_GRAVITY;
    a.ignore_terms = ignore_terms;
    int rc = run_op(h->b, a);
    if (rc != POSI_OK) return rc;
    rc = refresh_mirror(h);
    if (rc != POSI_OK) return rc;
    return (h->si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK) && (h->si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK) != POSI_SYS_COMPLETED
               ? POSI_ERR_PHYSICS : POSI_OK;
}

int posi_calculate_additional_effects(posi_handle* h, double current_time, int evolution, int dangular_momentum_dt,
                                      int accelerations) {
    if (!h) return POSI_ERR_ARG;
    if (!accelerations) {
        g_last_error = "the WHFast path always evaluates accelerations";
        return POSI_ERR_UNSUPPORTED;
    }
    LaunchArgs a{};
    a.op = posi::OP_EFFECTS;
    a.t_eval = current_time;
    a.evolution = evolution;
    a.dl = dangular_momentum_dt;
    a.acc = accelerations;
    int rc = run_op(h->b, a);
    if (rc != POSI_OK) return rc;
    return refresh_mirror(h);
}

int posi_get_state(const posi_handle* h, int64_t* sys_i64, double* sys_f64, int64_t* body_i64, double* body_f64,
                   double* roche) {
    if (!h) return POSI_ERR_ARG;
    return batch_get(h->b, sys_i64, sys_f64, body_i64, body_f64, roche);
}

int posi_set_state(posi_handle* h, const int64_t* sys_i64, const double* sys_f64, const int64_t* body_i64,
                   const double* body_f64) {
    if (!h) return POSI_ERR_ARG;
    if (sys_i64 && sys_i64[POSI_SI_N] != h->si[POSI_SI_N]) return POSI_ERR_ARG;
    int rc = batch_set(h->b, sys_i64, sys_f64, body_i64, body_f64);
    if (rc != POSI_OK) return rc;
    return refresh_mirror(h);
}

// src/integrator/output.rs:63-89 get_universe_history_writer: open (create or
// append), refuse a file shorter than the history the snapshot accounts for,
// and drop anything beyond it.
int posi_open_history(posi_handle* h, const char* path, int64_t expected_bytes) {
    if (!h || !path || expected_bytes < 0) return POSI_ERR_ARG;
    if (h->hist) { std::fclose(h->hist); h->hist = nullptr; }
    std::FILE* f = std::fopen(path, "ab");
    if (!f) { g_last_error = std::string("cannot open ") + path; return POSI_ERR_IO; }
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fclose(f);
    if (size < expected_bytes) {
        g_last_error = "historic snapshots do not contain all the expected history (" + std::to_string(size) +
                       " bytes) as indicated by the recovery snapshot (" + std::to_string(expected_bytes) + " bytes)";
        return POSI_ERR_STATE;
    }
    if (truncate(path, (off_t)expected_bytes) != 0) { g_last_error = "cannot truncate the history file"; return POSI_ERR_IO; }
    h->hist = std::fopen(path, "ab");
    if (!h->hist) { g_last_error = std::string("cannot open ") + path; return POSI_ERR_IO; }
    posi_batch* b = h->b;
    if (!b->d_hist) CK(cudaMalloc(&b->d_hist, (size_t)b->stride * posi::kHistoryFields * sizeof(double)));
    return POSI_OK;
}

int posi_close_history(posi_handle* h) {
    if (!h) return POSI_ERR_ARG;
    if (h->hist) {
        std::fclose(h->hist);
        h->hist = nullptr;
    }
    return POSI_OK;
}

// src/integrator/whfast.rs:307-316 + src/integrator/output.rs:28-54
int posi_write_recovery_snapshot(posi_handle* h, const char* path) {
    if (!h || !path) return POSI_ERR_ARG;
    if (!h->doc) {
        g_last_error = "recovery snapshots need a handle opened from a JSON case";
        return POSI_ERR_UNSUPPORTED;
    }
    std::string p(path);
    const size_t dot = p.find_last_of('.');
    const size_t slash = p.find_last_of('/');
    const bool has_ext = dot != std::string::npos && (slash == std::string::npos || dot > slash);
    const bool binary = posi::is_bincode_path(p);
    h->sf[POSI_SF_LAST_REC] = h->sf[POSI_SF_TIME];
    int rc = batch_set(h->b, nullptr, h->sf.data(), nullptr, nullptr);
    if (rc != POSI_OK) return rc;
    if (h->hist) std::fflush(h->hist);
    const int64_t n = h->si[POSI_SI_N];
    std::vector<int64_t> si(POSI_SI_COUNT), bi((size_t)n * POSI_BI_COUNT);
    std::vector<double> sf(POSI_SF_COUNT), bf((size_t)n * POSI_BF_COUNT), roche((size_t)n * n);
    rc = batch_get(h->b, si.data(), sf.data(), bi.data(), bf.data(), roche.data());
    if (rc != POSI_OK) return rc;
    std::vector<double> ias;
    if (h->b->ias15) {
        ias.resize((size_t)n * POSI_IAS_COUNT);
        if ((rc = posi_batch_get_ias15(h->b, ias.data())) != POSI_OK) return rc;
    }
    std::string err;
    if (!posi::update_case_document(*h->doc, n, si.data(), sf.data(), bi.data(), bf.data(), roche.data(),
                                    ias.empty() ? nullptr : ias.data(), err)) {
        g_last_error = err;
        return POSI_ERR_PARSE;
    }
    // keep one backup every 12 hours (the file name collides within a period)
    std::FILE* probe = std::fopen(path, "rb");
    if (probe) {
        std::fclose(probe);
        std::time_t now = std::time(nullptr);
        std::tm g;
        gmtime_r(&now, &g);
        char stamp[32];
        std::strftime(stamp, sizeof stamp, "%Y%m%dT", &g);
        const std::string backup = (has_ext ? p.substr(0, dot) : p) + "." + stamp + (g.tm_hour < 12 ? "AM" : "PM") + ".bin";
        std::rename(path, backup.c_str());
    }
    // src/integrator/output.rs:43-51: pretty JSON for a ".json" path,
    // bincode otherwise
    std::string text;
    if (binary) {
        if (!posi::json_to_bincode(*h->doc, text, err)) {
            g_last_error = err;
            return POSI_ERR_PARSE;
        }
    } else {
        posi::write_json(*h->doc, text);
    }
    std::FILE* f = std::fopen(path, "wb");
    if (!f) { g_last_error = std::string("cannot write ") + path; return POSI_ERR_IO; }
    const size_t w = std::fwrite(text.data(), 1, text.size(), f);
    std::fclose(f);
    return w == text.size() ? POSI_OK : POSI_ERR_IO;
}

// Recovery snapshot conversion between the JSON and bincode forms (each
// path's form by its extension, as the reference picks it).
int posi_convert_snapshot(const char* src, const char* dst) {
    if (!src || !dst) return POSI_ERR_ARG;
    std::ifstream f(src, std::ios::binary);
    if (!f) {
        g_last_error = std::string("cannot open ") + src;
        return POSI_ERR_IO;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    posi::json::Value doc;
    std::string err;
    if (posi::is_bincode_path(src)) {
        if (!posi::bincode_to_json(text, doc, err)) { g_last_error = err; return POSI_ERR_PARSE; }
    } else {
        posi::json::Parser parser(text.data(), text.size());
        if (!parser.parse(doc, err)) { g_last_error = "JSON: " + err; return POSI_ERR_PARSE; }
    }
    std::string out;
    if (posi::is_bincode_path(dst)) {
        if (!posi::json_to_bincode(doc, out, err)) { g_last_error = err; return POSI_ERR_PARSE; }
    } else {
        posi::write_json(doc, out);
    }
    std::FILE* o = std::fopen(dst, "wb");
    if (!o) { g_last_error = std::string("cannot write ") + dst; return POSI_ERR_IO; }
    const size_t w = std::fwrite(out.data(), 1, out.size(), o);
    std::fclose(o);
    return w == out.size() ? POSI_OK : POSI_ERR_IO;
}

// ---- batched --------------------------------------------------------------

posi_batch* posi_batch_create(int64_t n_systems, int64_t nmax, const int64_t* sys_i64, const double* sys_f64,
                              const int64_t* body_i64, const double* body_f64, const double* tables,
                              int64_t n_tables, const double* roche, int mode, int mapping, int* status) {
    return create_batch(n_systems, nmax, sys_i64, sys_f64, body_i64, body_f64, tables, n_tables, roche, mode,
                        mapping, status);
}

void posi_batch_destroy(posi_batch* b) { free_batch(b); }

int posi_batch_size(const posi_batch* b, int64_t* n_systems, int64_t* nmax) {
    if (!b) return POSI_ERR_ARG;
    if (n_systems) *n_systems = b->n_sys;
    if (nmax) *nmax = b->nmax;
    return POSI_OK;
}

int posi_batch_initialize_physical_values(posi_batch* b) {
    if (!b) return POSI_ERR_ARG;
    LaunchArgs a{};
    a.op = posi::OP_INIT;
    int rc = run_op(b, a);
    if (rc != POSI_OK) return rc;
    return compute_roche(b);
}

int posi_batch_iterate(posi_batch* b, int64_t n_steps, int64_t steps_per_launch) {
    if (!b || n_steps < 0) return POSI_ERR_ARG;
    if (n_steps == 0) return POSI_OK;
    if (steps_per_launch <= 0 || steps_per_launch > n_steps) steps_per_launch = n_steps;
    const int64_t chunks = (n_steps + steps_per_launch - 1) / steps_per_launch;
    if (!b->graph || b->graph_steps != n_steps || b->graph_spl != steps_per_launch) {
        if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
        // balanced schedules of every (chunk length, bucket), made before the
        // capture and kept with the graph; a schedule assumes its bucket has
        // the GPU to itself, so buckets launched side by side run plain
        // (measured on the uneven ensemble: 594.7 us per step with schedules
        // against 586.2 us without)
        const int slots = b->sms * (posi::kSchedBlockThreads / 32);
        std::vector<int32_t> tables;
        std::map<std::pair<int64_t, size_t>, std::pair<size_t, int>> plan;  // -> (offset, sub-launches)
        for (int64_t c = 0; c < chunks; ++c) {
            const int64_t len = std::min(steps_per_launch, n_steps - c * steps_per_launch);
            for (size_t k = 0; k < b->buckets.size(); ++k) {
                const Bucket& bk = b->buckets[k];
                if (!b->balanced || b->ias15 || bk.G < 4 || b->buckets.size() > 1 || plan.count({len, k})) continue;
                const int jobs = (int)((bk.count + (32 / bk.G) - 1) / (32 / bk.G));
                std::vector<int32_t> t;
                int launches = 0;
                if (build_schedule(b->sms, jobs, len, t, launches)) {
                    plan[{len, k}] = {tables.size(), launches};
                    tables.insert(tables.end(), t.begin(), t.end());
                }
            }
        }
        cudaFree(b->d_sched);
        b->d_sched = nullptr;
        if (!tables.empty()) {
            CK(cudaMalloc(&b->d_sched, tables.size() * sizeof(int32_t)));
            CK(cudaMemcpy(b->d_sched, tables.data(), tables.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        }
        b->last_launches = 0;
        const size_t nbk = b->buckets.size();
        const bool fan = nbk > 1;
        if (fan) {
            if (!b->fork) CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
            while (b->side.size() < nbk) {
                cudaStream_t st;
                cudaEvent_t e;
                CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
                CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                b->side.push_back(st);
                b->side_done.push_back(e);
            }
        }
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        LaunchArgs a{};
        a.op = posi::OP_STEPS;
        cudaError_t err = cudaSuccess;
        for (int64_t c = 0; c < chunks && err == cudaSuccess; ++c) {
            a.n_steps = std::min(steps_per_launch, n_steps - c * steps_per_launch);
            if (fan) err = cudaEventRecord(b->fork, b->stream);
            for (size_t k = 0; k < nbk && err == cudaSuccess; ++k) {
                const Bucket& bk = b->buckets[k];
                cudaStream_t on = fan ? b->side[k] : b->stream;
                if (fan && (err = cudaStreamWaitEvent(on, b->fork, 0)) != cudaSuccess) break;
                auto it = plan.find({a.n_steps, k});
                if (it == plan.end()) {
                    err = b->launch(bk, a, on);
                    ++b->last_launches;
                } else {
                    LaunchArgs s = a;
                    s.op = posi::OP_STEPS_SCHED;
                    s.sched_blocks = b->sms;
                    for (int l = 0; l < it->second.second && err == cudaSuccess; ++l) {
                        const int32_t* row = b->d_sched + it->second.first + (size_t)l * 2 * slots;
                        s.slot_job = row;
                        s.slot_steps = row + slots;
                        err = b->launch(bk, s, on);
                        ++b->last_launches;
                    }
                }
                if (fan && err == cudaSuccess) err = cudaEventRecord(b->side_done[k], on);
            }
            for (size_t k = 0; fan && k < nbk && err == cudaSuccess; ++k)
                err = cudaStreamWaitEvent(b->stream, b->side_done[k], 0);
        }
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        CK(err);
        CK(e2);
        err = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        CK(err);
        b->graph_steps = n_steps;
        b->graph_spl = steps_per_launch;
    }
    CK(cudaEventRecord(b->ev0, b->stream));
    CK(cudaGraphLaunch(b->graph, b->stream));
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    return POSI_OK;
}

int posi_batch_set_balanced(posi_batch* b, int on) {
    if (!b) return POSI_ERR_ARG;
    if (b->balanced != (on != 0) && b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        b->graph_steps = -1;
    }
    b->balanced = on != 0;
    return POSI_OK;
}

int posi_batch_get_state(const posi_batch* b, int64_t* sys_i64, double* sys_f64, int64_t* body_i64, double* body_f64,
                         double* roche) {
    if (!b) return POSI_ERR_ARG;
    return batch_get(b, sys_i64, sys_f64, body_i64, body_f64, roche);
}

int posi_batch_set_state(posi_batch* b, const int64_t* sys_i64, const double* sys_f64, const int64_t* body_i64,
                         const double* body_f64) {
    if (!b) return POSI_ERR_ARG;
    return batch_set(b, sys_i64, sys_f64, body_i64, body_f64);
}

int posi_batch_get_ias15(const posi_batch* b, double* body_ias) {
    if (!b || !body_ias) return POSI_ERR_ARG;
    if (!b->ias15) {
        g_last_error = "not an IAS15 batch";
        return POSI_ERR_STATE;
    }
    int rc = download_aos<double>(b, body_ias, b->d_ias, b->stride, POSI_IAS_COUNT);
    if (rc != POSI_OK) return rc;
    CK(cudaStreamSynchronize(b->stream));
    return POSI_OK;
}

int posi_batch_set_ias15(posi_batch* b, const double* body_ias) {
    if (!b || !body_ias) return POSI_ERR_ARG;
    if (!b->ias15) {
        g_last_error = "not an IAS15 batch";
        return POSI_ERR_STATE;
    }
    int rc = upload_aos<double>(b, body_ias, b->d_ias, b->stride, POSI_IAS_COUNT);
    if (rc != POSI_OK) return rc;
    CK(cudaStreamSynchronize(b->stream));
    return POSI_OK;
}

int posi_get_ias15(const posi_handle* h, double* body_ias) {
    if (!h) return POSI_ERR_ARG;
    return posi_batch_get_ias15(h->b, body_ias);
}

int posi_set_ias15(posi_handle* h, const double* body_ias) {
    if (!h) return POSI_ERR_ARG;
    return posi_batch_set_ias15(h->b, body_ias);
}

// Autotuner: for every body count present, run each admissible lane mapping
// (2..32 lanes per system, at least one lane per body) on the systems of that
// count for probe_steps steps -- once to warm up, once timed with CUDA events
// -- restoring their state after every trial, and keep the cheapest (below).
// The buckets are then rebuilt with the chosen mappings.
int posi_batch_autotune(posi_batch* b, int64_t probe_steps, int32_t* lanes_by_n) {
    if (!b || probe_steps < 1) return POSI_ERR_ARG;
    if (b->ias15) {
        // the IAS15 kernel takes the smallest lane group that holds a system
        if (lanes_by_n)
            for (int k = 0; k <= POSI_MAX_BODIES; ++k)
                lanes_by_n[k] = b->mapping_of_n.count(k) ? b->mapping_of_n.at(k) : 0;
        return POSI_OK;
    }
    const size_t nb = (size_t)b->stride;
    const size_t bytes_bf = nb * POSI_BF_COUNT * sizeof(double), bytes_bi = nb * POSI_BI_COUNT * sizeof(int64_t);
    const size_t bytes_sf = (size_t)b->n_sys * POSI_SF_COUNT * sizeof(double);
    const size_t bytes_si = (size_t)b->n_sys * POSI_SI_COUNT * sizeof(int64_t);
    const size_t bytes_fl = (size_t)b->n_sys * sizeof(int32_t);
    char* save = nullptr;
    CK(cudaMalloc(&save, bytes_bf + bytes_bi + bytes_sf + bytes_si + bytes_fl));
    struct Saved {
        char* p;
        ~Saved() { cudaFree(p); }
    } guard{save};
    char* p_bf = save;
    char* p_bi = p_bf + bytes_bf;
    char* p_sf = p_bi + bytes_bi;
    char* p_si = p_sf + bytes_sf;
    char* p_fl = p_si + bytes_si;
    auto copy_all = [&](bool to_save) -> int {
        auto cp = [&](void* dst, const void* src, size_t n) {
            return cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToDevice, b->stream);
        };
        if (to_save) {
            CK(cp(p_bf, b->d_bf, bytes_bf)); CK(cp(p_bi, b->d_bi, bytes_bi)); CK(cp(p_sf, b->d_sf, bytes_sf));
            CK(cp(p_si, b->d_si, bytes_si)); CK(cp(p_fl, b->d_flags, bytes_fl));
        } else {
            CK(cp(b->d_bf, p_bf, bytes_bf)); CK(cp(b->d_bi, p_bi, bytes_bi)); CK(cp(b->d_sf, p_sf, bytes_sf));
            CK(cp(b->d_si, p_si, bytes_si)); CK(cp(b->d_flags, p_fl, bytes_fl));
        }
        return POSI_OK;
    };
    int rc = copy_all(true);
    if (rc != POSI_OK) return rc;
    // systems of each body count, in bucket order
    std::map<int64_t, std::vector<int32_t>> by_n;
    for (int32_t s : b->host_list) by_n[b->n_of[s]].push_back(s);
    int32_t* d_probe = nullptr;
    CK(cudaMalloc(&d_probe, (size_t)b->n_sys * sizeof(int32_t)));
    struct ListGuard {
        int32_t* p;
        ~ListGuard() { cudaFree(p); }
    } lguard{d_probe};
    std::map<int64_t, int> chosen;
    b->tuned_ms_of_n.clear();
    b->probe_ms_of_n.clear();
    LaunchArgs a{};
    a.op = posi::OP_STEPS;
    a.n_steps = probe_steps;
    // A bucket probed alone with fewer warps than the GPU has SMSPs times
    // its longest lane's chain, whatever its lane group.  When the buckets
    // run side by side and together fill the SMSPs, what a bucket costs the
    // others is the SMSP time it holds: its probe time x min(warps, SMSPs) /
    // SMSPs.  So with several buckets that together hold at least one warp
    // per SMSP at their smallest groups, the mapping minimises that share;
    // otherwise (one bucket, or a GPU the buckets do not fill) its time.
    const int64_t smsps = 4 * (int64_t)b->sms;
    int64_t min_warps = 0;
    for (auto& kv : by_n) {
        const int64_t per_warp = 32 / posi::group_size_for(kv.first);
        min_warps += ((int64_t)kv.second.size() + per_warp - 1) / per_warp;
    }
    const bool shared_gpu = by_n.size() > 1 && min_warps >= smsps;
    for (auto& kv : by_n) {
        const int64_t n = kv.first;
        const std::vector<int32_t>& sys = kv.second;
        CK(cudaMemcpyAsync(d_probe, sys.data(), sys.size() * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream));
        double best = 1e300, best_ms = 0.;
        int best_g = posi::group_size_for(n);
        std::array<double, 6> probes;
        probes.fill(-1.);
        for (int G = posi::group_size_for(n); G <= 32; G *= 2) {
            a.G = G;
            DevView v = b->view(0, (int32_t)sys.size());
            v.list = d_probe;
            float ms = 0.f;
            for (int trial = 0; trial < 2; ++trial) {
                CK(cudaEventRecord(b->ev0, b->stream));
                CK(b->mode == POSI_MODE_EXACT ? posi::launch_exact(v, a, b->stream) : posi::launch_fast(v, a, b->stream));
                CK(cudaEventRecord(b->ev1, b->stream));
                CK(cudaEventSynchronize(b->ev1));
                CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
                if ((rc = copy_all(false)) != POSI_OK) return rc;
            }
            const int64_t warps = ((int64_t)sys.size() + (32 / G) - 1) / (32 / G);
            const double cost = shared_gpu ? ms * (double)std::min(warps, smsps) / (double)smsps : ms;
            if (cost < best) { best = cost; best_ms = ms; best_g = G; }
            int k = 0;
            while ((1 << k) < G) ++k;
            probes[(size_t)k] = ms;
        }
        chosen[n] = best_g;
        b->tuned_ms_of_n[n] = best_ms;
        b->probe_ms_of_n[n] = probes;
    }
    CK(cudaStreamSynchronize(b->stream));
    std::vector<int64_t> si((size_t)b->n_sys * POSI_SI_COUNT);
    if ((rc = batch_get(b, si.data(), nullptr, nullptr, nullptr, nullptr)) != POSI_OK) return rc;
    if ((rc = build_buckets(b, si.data(), &chosen)) != POSI_OK) return rc;
    if (lanes_by_n) {
        for (int k = 0; k <= POSI_MAX_BODIES; ++k) lanes_by_n[k] = chosen.count(k) ? chosen[k] : 0;
    }
    return POSI_OK;
}

int posi_batch_autotune_report(const posi_batch* b, int64_t n, double* ms_by_lanes) {
    if (!b || !ms_by_lanes) return POSI_ERR_ARG;
    auto it = b->probe_ms_of_n.find(n);
    if (it == b->probe_ms_of_n.end()) {
        g_last_error = "no autotuned systems of " + std::to_string(n) + " bodies";
        return POSI_ERR_STATE;
    }
    for (size_t k = 0; k < 6; ++k) ms_by_lanes[k] = it->second[k];
    return POSI_OK;
}

int posi_batch_mapping_for(const posi_batch* b, int64_t n) {
    if (!b) return -1;
    auto it = b->mapping_of_n.find(n);
    return it == b->mapping_of_n.end() ? -1 : it->second;
}

int posi_batch_last_timing(const posi_batch* b, double* ms, int64_t* launches) {
    if (!b) return POSI_ERR_ARG;
    if (ms) *ms = b->last_ms;
    if (launches) *launches = b->last_launches;
    return POSI_OK;
}

}  // extern "C"

namespace posi {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace posi

// ---- adjoint ----------------------------------------------------------------
// Checkpointed reverse mode over a batch (no reference counterpart: the
// reference has no derivatives; its users take finite differences).
struct posi_adjoint {
    posi_batch* b = nullptr;
    int64_t n_steps = 0, every = 0, n_chunks = 0;
    bool have_forward = false;
    size_t bytes_bf = 0, bytes_sf = 0, bytes_si = 0, bytes_ck = 0;
    char* d_ckpt = nullptr;   // n_chunks states: the chunks' starts
    // Backward pass: chunk c is re-integrated from a copy of its checkpoint in
    // work slot c % n_buf, writing tape c % n_buf on rec_stream, while the
    // reverse sweep of chunk c + 1 runs on the batch stream (two buffers; one
    // when the second tape does not fit, and then the two alternate).
    int n_buf = 0;
    char* d_work = nullptr;    // n_buf states
    double* d_tape[2] = {nullptr, nullptr};
    cudaStream_t rec_stream = nullptr;
    cudaEvent_t rec_done[2] = {nullptr, nullptr}, rev_done[2] = {nullptr, nullptr}, ready = nullptr;
    double* d_lam = nullptr;
    double* d_grad = nullptr;
    int32_t* d_err = nullptr;
    int32_t* d_list = nullptr;
    std::vector<Bucket> buckets;  // by adjoint lane group
    double fwd_ms = 0., bwd_ms = 0., record_ms = 0., reverse_ms = 0.;
};

namespace {
void free_adjoint(posi_adjoint* a) {
    if (!a) return;
    cudaFree(a->d_ckpt); cudaFree(a->d_work); cudaFree(a->d_tape[0]); cudaFree(a->d_tape[1]);
    cudaFree(a->d_lam); cudaFree(a->d_grad); cudaFree(a->d_err); cudaFree(a->d_list);
    for (int k = 0; k < 2; ++k) {
        if (a->rec_done[k]) cudaEventDestroy(a->rec_done[k]);
        if (a->rev_done[k]) cudaEventDestroy(a->rev_done[k]);
    }
    if (a->ready) cudaEventDestroy(a->ready);
    if (a->rec_stream) cudaStreamDestroy(a->rec_stream);
    delete a;
}

// Saves the batch state into checkpoint slot `slot`.
int adj_save_state(posi_adjoint* a, int64_t slot) {
    posi_batch* b = a->b;
    char* base = a->d_ckpt + (size_t)slot * a->bytes_ck;
    auto cp = [&](void* dst, const void* src, size_t n) { return cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToDevice, b->stream); };
    CK(cp(base, b->d_bf, a->bytes_bf));
    CK(cp(base + a->bytes_bf, b->d_sf, a->bytes_sf));
    CK(cp(base + a->bytes_bf + a->bytes_sf, b->d_si, a->bytes_si));
    return POSI_OK;
}

// A state (body fields, system scalars and integers) laid out as a checkpoint.
struct StateRef {
    double* bf;
    double* sf;
    int64_t* si;
};

StateRef state_at(const posi_adjoint* a, char* base) {
    return {(double*)base, (double*)(base + a->bytes_bf), (int64_t*)(base + a->bytes_bf + a->bytes_sf)};
}

posi::AdjView adj_view(const posi_adjoint* a, const Bucket& bk, const StateRef& x, double* tape) {
    const posi_batch* b = a->b;
    posi::AdjView v;
    v.n_sys = b->n_sys; v.nmax = b->nmax; v.stride = b->stride;
    v.bf = x.bf; v.bi = b->d_bi; v.sf = x.sf; v.si = x.si;
    v.list = a->d_list + bk.offset; v.n_list = bk.count;
    v.tape = tape; v.lam = a->d_lam; v.grad = a->d_grad; v.err = a->d_err;
    return v;
}
}  // namespace

posi_adjoint* posi_adjoint_create(posi_batch* b, int64_t n_steps, int64_t checkpoint_every, int* status) {
    auto fail = [&](int code, const std::string& msg, posi_adjoint* a) -> posi_adjoint* {
        g_last_error = msg;
        free_adjoint(a);
        if (status) *status = code;
        return nullptr;
    };
    if (!b || n_steps < 1 || checkpoint_every < 1) return fail(POSI_ERR_ARG, "bad arguments", nullptr);
    std::vector<int64_t> si((size_t)b->n_sys * POSI_SI_COUNT);
    if (batch_get(b, si.data(), nullptr, nullptr, nullptr, nullptr) != POSI_OK) return fail(POSI_ERR_CUDA, g_last_error, nullptr);
    std::map<int, std::vector<int32_t>> by_g;
    for (int64_t s = 0; s < b->n_sys; ++s) {
        const int64_t* x = si.data() + s * POSI_SI_COUNT;
        if (x[POSI_SI_COORDS] != POSI_JACOBI)
            return fail(POSI_ERR_UNSUPPORTED, "the adjoint supports Jacobi coordinates only", nullptr);
        if (x[POSI_SI_EVOLUTION] != 0)
            return fail(POSI_ERR_UNSUPPORTED, "the adjoint supports non-evolving bodies only", nullptr);
        if (x[POSI_SI_GR] != 0 && x[POSI_SI_GR_IMPL] != POSI_GR_KIDDER1995)
            return fail(POSI_ERR_UNSUPPORTED, "the adjoint supports Kidder1995 general relativity only", nullptr);
        if (x[POSI_SI_WIND] != 0 || x[POSI_SI_DISK] != 0)
            return fail(POSI_ERR_UNSUPPORTED, "the adjoint does not support wind or disk", nullptr);
        if (x[POSI_SI_INTEGRATOR] != POSI_INTEGRATOR_WHFAST)
            return fail(POSI_ERR_UNSUPPORTED, "the adjoint differentiates the WHFast step only", nullptr);
        const int G = posi::adjoint_group_size(x[POSI_SI_N]);
        if (G == 0) return fail(POSI_ERR_UNSUPPORTED, "the adjoint supports systems of up to 8 bodies", nullptr);
        by_g[G].push_back((int32_t)s);
    }
    posi_adjoint* a = new posi_adjoint();
    a->b = b;
    a->n_steps = n_steps;
    a->every = checkpoint_every;
    a->n_chunks = (n_steps + checkpoint_every - 1) / checkpoint_every;
    const size_t nb = (size_t)b->stride;
    a->bytes_bf = nb * POSI_BF_COUNT * sizeof(double);
    a->bytes_sf = (size_t)b->n_sys * POSI_SF_COUNT * sizeof(double);
    a->bytes_si = (size_t)b->n_sys * POSI_SI_COUNT * sizeof(int64_t);
    a->bytes_ck = (a->bytes_bf + a->bytes_sf + a->bytes_si + 255) / 256 * 256;
    std::vector<int32_t> list;
    for (auto& kv : by_g) {
        Bucket bk;
        bk.G = kv.first;
        bk.offset = (int32_t)list.size();
        bk.count = (int32_t)kv.second.size();
        list.insert(list.end(), kv.second.begin(), kv.second.end());
        a->buckets.push_back(bk);
    }
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess) { g_last_error = cudaGetErrorString(e); return false; }
        return true;
    };
    const size_t bytes_tape = (size_t)checkpoint_every * posi::kAdjTapeFields * nb * sizeof(double);
    if (!ok(posi::prepare_adjoint()) ||
        !ok(cudaMalloc(&a->d_ckpt, a->bytes_ck * (size_t)a->n_chunks)) ||
        !ok(cudaMalloc(&a->d_tape[0], bytes_tape)) ||
        !ok(cudaMalloc(&a->d_lam, nb * 12 * sizeof(double))) || !ok(cudaMalloc(&a->d_grad, nb * 2 * sizeof(double))) ||
        !ok(cudaMalloc(&a->d_err, (size_t)b->n_sys * sizeof(int32_t))) ||
        !ok(cudaMalloc(&a->d_list, list.size() * sizeof(int32_t))) ||
        !ok(cudaMemcpyAsync(a->d_list, list.data(), list.size() * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream)) ||
        !ok(cudaStreamSynchronize(b->stream)))
        return fail(POSI_ERR_CUDA, g_last_error, a);
    // the second tape and work slot are optional
    a->n_buf = 1;
    if (a->n_chunks > 1 && cudaMalloc(&a->d_tape[1], bytes_tape) == cudaSuccess) a->n_buf = 2;
    cudaGetLastError();
    if (!ok(cudaMalloc(&a->d_work, a->bytes_ck * (size_t)a->n_buf)) ||
        !ok(cudaStreamCreateWithFlags(&a->rec_stream, cudaStreamNonBlocking)) ||
        !ok(cudaEventCreateWithFlags(&a->ready, cudaEventDisableTiming)))
        return fail(POSI_ERR_CUDA, g_last_error, a);
    for (int k = 0; k < 2; ++k)
        if (!ok(cudaEventCreateWithFlags(&a->rec_done[k], cudaEventDisableTiming)) ||
            !ok(cudaEventCreateWithFlags(&a->rev_done[k], cudaEventDisableTiming)))
            return fail(POSI_ERR_CUDA, g_last_error, a);
    if (status) *status = POSI_OK;
    return a;
}

void posi_adjoint_destroy(posi_adjoint* a) { free_adjoint(a); }

int posi_adjoint_forward(posi_adjoint* a) {
    if (!a) return POSI_ERR_ARG;
    posi_batch* b = a->b;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, b->stream));
    int rc = POSI_OK;
    for (int64_t c = 0; c < a->n_chunks && rc == POSI_OK; ++c) {
        if ((rc = adj_save_state(a, c)) != POSI_OK) break;
        const int64_t len = std::min(a->every, a->n_steps - c * a->every);
        rc = posi_batch_iterate(b, len, len);
    }
    CK(cudaEventRecord(e1, b->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    a->fwd_ms = ms;
    a->have_forward = rc == POSI_OK;
    return rc;
}

int posi_adjoint_backward(posi_adjoint* a, const double* lam_final, double* lam_initial, double* grad,
                          int32_t* system_flags) {
    if (!a || !lam_final) return POSI_ERR_ARG;
    if (!a->have_forward) {
        g_last_error = "posi_adjoint_forward must run first";
        return POSI_ERR_STATE;
    }
    posi_batch* b = a->b;
    const int64_t nb = b->stride;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, b->stream));
    // adjoint of the final state, [system][body][12] -> field-major
    CK(cudaMemcpyAsync(b->d_stage, lam_final, (size_t)nb * 12 * sizeof(double), cudaMemcpyDefault, b->stream));
    aos_to_soa<double><<<grid_for(nb * 12), 256, 0, b->stream>>>((const double*)b->d_stage, a->d_lam, nb, 12);
    CK(cudaGetLastError());
    CK(cudaMemsetAsync(a->d_grad, 0, (size_t)nb * 2 * sizeof(double), b->stream));
    CK(cudaMemsetAsync(a->d_err, 0, (size_t)b->n_sys * sizeof(int32_t), b->stream));
    // The chunks' re-integrations are independent (each starts from its
    // checkpoint), so chunk c - 1 is re-integrated on rec_stream while the
    // reverse sweep of chunk c runs; the batch's own state is not touched.
    CK(cudaEventRecord(a->ready, b->stream));
    CK(cudaStreamWaitEvent(a->rec_stream, a->ready, 0));
    // per chunk: record start / end (rec_stream), reverse start / end
    std::vector<cudaEvent_t> marks((size_t)a->n_chunks * 4);
    for (auto& e : marks) CK(cudaEventCreate(&e));
    for (int64_t c = a->n_chunks - 1; c >= 0; --c) {
        const int buf = (int)(c % a->n_buf);
        const int64_t len = std::min(a->every, a->n_steps - c * a->every);
        char* work = a->d_work + (size_t)buf * a->bytes_ck;
        const StateRef x = state_at(a, work);
        double* tape = a->d_tape[buf];
        cudaEvent_t* mk = marks.data() + (size_t)c * 4;
        // the buffers' previous reader is the reverse sweep of chunk c + n_buf
        if (c + a->n_buf < a->n_chunks) CK(cudaStreamWaitEvent(a->rec_stream, a->rev_done[buf], 0));
        CK(cudaEventRecord(mk[0], a->rec_stream));
        CK(cudaMemcpyAsync(work, a->d_ckpt + (size_t)c * a->bytes_ck, a->bytes_ck, cudaMemcpyDeviceToDevice,
                           a->rec_stream));
        if (b->mode == POSI_MODE_FAST) {
            // re-integrate the chunk with the forward kernel itself, writing
            // the step records as it goes
            LaunchArgs la{};
            la.op = posi::OP_STEPS_REC;
            la.n_steps = len;
            for (const Bucket& bk : b->buckets) {
                la.G = bk.G;
                DevView v = b->view(bk.offset, bk.count);
                v.bf = x.bf; v.sf = x.sf; v.si = x.si;
                v.rec = tape;
                CK(posi::launch_fast(v, la, a->rec_stream));
            }
        } else {
            for (const Bucket& bk : a->buckets)
                CK(posi::launch_adjoint(adj_view(a, bk, x, tape), 0, len, bk.G, a->rec_stream));
        }
        CK(cudaEventRecord(mk[1], a->rec_stream));
        CK(cudaEventRecord(a->rec_done[buf], a->rec_stream));
        CK(cudaStreamWaitEvent(b->stream, a->rec_done[buf], 0));
        CK(cudaEventRecord(mk[2], b->stream));
        for (const Bucket& bk : a->buckets)
            CK(posi::launch_adjoint(adj_view(a, bk, x, tape), 1, len, bk.G, b->stream));
        CK(cudaEventRecord(mk[3], b->stream));
        CK(cudaEventRecord(a->rev_done[buf], b->stream));
    }
    CK(cudaStreamSynchronize(b->stream));
    a->record_ms = a->reverse_ms = 0.;
    for (int64_t c = 0; c < a->n_chunks; ++c) {
        float m1 = 0.f, m2 = 0.f;
        cudaEventElapsedTime(&m1, marks[(size_t)c * 4], marks[(size_t)c * 4 + 1]);
        cudaEventElapsedTime(&m2, marks[(size_t)c * 4 + 2], marks[(size_t)c * 4 + 3]);
        a->record_ms += m1;
        a->reverse_ms += m2;
    }
    for (auto& e : marks) cudaEventDestroy(e);
    CK(cudaEventRecord(e1, b->stream));
    // results, [system][body][12] and [system][body][2]
    if (lam_initial) {
        soa_to_aos<double><<<grid_for(nb * 12), 256, 0, b->stream>>>(a->d_lam, (double*)b->d_stage, nb, 12);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(lam_initial, b->d_stage, (size_t)nb * 12 * sizeof(double), cudaMemcpyDefault, b->stream));
        CK(cudaStreamSynchronize(b->stream));
    }
    if (grad) {
        soa_to_aos<double><<<grid_for(nb * 2), 256, 0, b->stream>>>(a->d_grad, (double*)b->d_stage, nb, 2);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(grad, b->d_stage, (size_t)nb * 2 * sizeof(double), cudaMemcpyDefault, b->stream));
        CK(cudaStreamSynchronize(b->stream));
    }
    std::vector<int32_t> err((size_t)b->n_sys);
    CK(cudaMemcpyAsync(err.data(), a->d_err, err.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    a->bwd_ms = ms;
    if (system_flags) {
        // systems the forward run froze (collision, Roche limit, ejection...)
        std::vector<int64_t> si((size_t)b->n_sys * POSI_SI_COUNT);
        int rc;
        if ((rc = batch_get(b, si.data(), nullptr, nullptr, nullptr, nullptr)) != POSI_OK) return rc;
        for (int64_t s = 0; s < b->n_sys; ++s) {
            const int64_t st = si[(size_t)s * POSI_SI_COUNT + POSI_SI_STATUS] & POSI_SYS_FATAL_MASK;
            system_flags[s] = err[(size_t)s] | ((st != 0 && st != POSI_SYS_COMPLETED) ? POSI_ADJ_FROZEN : 0);
        }
    }
    return POSI_OK;
}

int posi_adjoint_last_timing(const posi_adjoint* a, double* forward_ms, double* backward_ms, double* record_ms,
                             double* reverse_ms) {
    if (!a) return POSI_ERR_ARG;
    if (forward_ms) *forward_ms = a->fwd_ms;
    if (backward_ms) *backward_ms = a->bwd_ms;
    if (record_ms) *record_ms = a->record_ms;
    if (reverse_ms) *reverse_ms = a->reverse_ms;
    return POSI_OK;
}
