// large.cu -- host side of the many-body engine (large_device.cuh).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/posidonius_gb300.h"
#include "kernels.h"
#include "large_device.cuh"

struct posi_large {
    int64_t n = 0;
    int coords = POSI_DEMOCRATIC_HELIOCENTRIC;
    int grid = 0, ntile = 0, per_block = 0, per_block_tan = 32;
    double *d_bf = nullptr, *d_sf = nullptr, *d_roche = nullptr, *d_near2 = nullptr, *d_pos = nullptr,
           *d_gpart = nullptr,
           *d_bpart = nullptr, *d_tot = nullptr, *d_tan = nullptr, *d_dpos = nullptr;
    int64_t *d_bi = nullptr, *d_si = nullptr;
    unsigned* d_bar = nullptr;   // [0] arrival count of the grid's barriers, [2] of the body blocks'; zeroed per launch
    int* d_ctl = nullptr;
    int* d_err = nullptr;
    unsigned long long* d_bad = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double last_ms = 0.;
};

namespace {

void free_large(posi_large* L) {
    if (!L) return;
    cudaFree(L->d_bf); cudaFree(L->d_sf); cudaFree(L->d_roche); cudaFree(L->d_near2); cudaFree(L->d_pos);
    cudaFree(L->d_gpart);
    cudaFree(L->d_bpart); cudaFree(L->d_tot); cudaFree(L->d_bi); cudaFree(L->d_si); cudaFree(L->d_bar); cudaFree(L->d_ctl); cudaFree(L->d_err);
    cudaFree(L->d_bad); cudaFree(L->d_tan); cudaFree(L->d_dpos);
    if (L->e0) cudaEventDestroy(L->e0);
    if (L->e1) cudaEventDestroy(L->e1);
    if (L->stream) cudaStreamDestroy(L->stream);
    delete L;
}

#define LCK(call)                                                                         \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            posi::set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));    \
            return POSI_ERR_CUDA;                                                         \
        }                                                                                 \
    } while (0)

// host row-major [rows][fields] <-> device field-major [fields][rows]
template <typename T>
std::vector<T> to_field_major(const T* a, int64_t rows, int fields) {
    std::vector<T> o((size_t)rows * fields);
    for (int64_t r = 0; r < rows; ++r)
        for (int f = 0; f < fields; ++f) o[(size_t)f * rows + r] = a[(size_t)r * fields + f];
    return o;
}
template <typename T>
void from_field_major(const std::vector<T>& o, T* a, int64_t rows, int fields) {
    for (int64_t r = 0; r < rows; ++r)
        for (int f = 0; f < fields; ++f) a[(size_t)r * fields + f] = o[(size_t)f * rows + r];
}

}  // namespace

extern "C" {

posi_large* posi_large_create(int64_t n, const int64_t* sys_i64, const double* sys_f64, const int64_t* body_i64,
                              const double* body_f64, int* status) {
    auto fail = [&](int code, const std::string& msg, posi_large* L) -> posi_large* {
        posi::set_last_error(msg);
        free_large(L);
        if (status) *status = code;
        return nullptr;
    };
    if (n < 2 || !sys_i64 || !sys_f64 || !body_i64 || !body_f64) return fail(POSI_ERR_ARG, "bad arguments", nullptr);
    if (sys_i64[POSI_SI_N] != n) return fail(POSI_ERR_ARG, "sys_i64[POSI_SI_N] differs from n", nullptr);
    if (sys_i64[POSI_SI_COORDS] < POSI_JACOBI || sys_i64[POSI_SI_COORDS] > POSI_WHDS)
        return fail(POSI_ERR_ARG, "unknown coordinates type", nullptr);
    if (sys_i64[POSI_SI_EVOLUTION] != 0)
        return fail(POSI_ERR_UNSUPPORTED, "the many-body engine supports non-evolving bodies only", nullptr);
    if (sys_i64[POSI_SI_GR] != 0 && sys_i64[POSI_SI_GR_IMPL] != POSI_GR_KIDDER1995)
        return fail(POSI_ERR_UNSUPPORTED, "the many-body engine supports Kidder1995 general relativity only", nullptr);
    if (sys_i64[POSI_SI_WIND] != 0 || sys_i64[POSI_SI_DISK] != 0)
        return fail(POSI_ERR_UNSUPPORTED, "the many-body engine does not support wind or disk", nullptr);
    if (sys_i64[POSI_SI_INTEGRATOR] != POSI_INTEGRATOR_WHFAST)
        return fail(POSI_ERR_UNSUPPORTED, "the many-body engine integrates with WHFast only", nullptr);
    const int64_t host = sys_i64[POSI_SI_HOST];
    if (host < 0 || host >= n) return fail(POSI_ERR_ARG, "host index out of range", nullptr);
    for (int64_t i = 0; i < n; ++i)
        if (body_f64[i * POSI_BF_COUNT + POSI_BF_MASS] > body_f64[host * POSI_BF_COUNT + POSI_BF_MASS])
            return fail(POSI_ERR_ARG, "the host must be the most massive body", nullptr);
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(POSI_ERR_CUDA, "no CUDA device", nullptr);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, posi_many::large_steps_kernel<0>, posi_many::kBlock, 0) !=
            cudaSuccess || per_sm < 1)
        return fail(POSI_ERR_CUDA, "occupancy query failed", nullptr);
    posi_large* L = new posi_large();
    L->n = n;
    L->coords = (int)sys_i64[POSI_SI_COORDS];
    L->grid = sms;  // one block per SM: every block resident
    if ((int64_t)L->grid * posi_many::kBlock < n)
        return fail(POSI_ERR_UNSUPPORTED, "too many bodies for one resident grid (" +
                                              std::to_string((int64_t)L->grid * posi_many::kBlock) + " at most)", L);
    // tiles of 32 bodies for the pair loop; bodies in the first blocks, 32
    // per block (more only when the grid's blocks would not hold them): the
    // tangent kernels need that layout (a warp per direction beside the
    // primal warp), and the same one keeps the primal state of a tangent run
    // the plain run's bit for bit (the reductions add block rows in order)
    L->ntile = (int)((n + 31) / 32);
    {
        const int64_t need = (n + L->grid - 1) / L->grid;
        L->per_block = (int)std::min<int64_t>(posi_many::kBlock, std::max<int64_t>(32, (need + 31) / 32 * 32));
    }
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess) { posi::set_last_error(cudaGetErrorString(e)); return false; }
        return true;
    };
    if (!ok(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking)) || !ok(cudaEventCreate(&L->e0)) ||
        !ok(cudaEventCreate(&L->e1)) ||
        !ok(cudaMalloc(&L->d_bf, (size_t)n * POSI_BF_COUNT * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_bi, (size_t)n * POSI_BI_COUNT * sizeof(int64_t))) ||
        !ok(cudaMalloc(&L->d_sf, POSI_SF_COUNT * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_si, POSI_SI_COUNT * sizeof(int64_t))) ||
        !ok(cudaMalloc(&L->d_roche, (size_t)n * n * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_near2, (size_t)n * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_pos, (size_t)3 * n * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_gpart, (size_t)posi_many::kPairSplit * L->ntile * 3 * (1 + posi_many::kMaxTangents) * n *
                                        sizeof(double))) ||
        !ok(cudaMalloc(&L->d_bpart, (size_t)2 * L->grid * posi_many::BP_ROW * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_tot, posi_many::BP_ROW * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_tan, (size_t)posi_many::kMaxTangents * 12 * n * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_dpos, (size_t)posi_many::kMaxTangents * 3 * n * sizeof(double))) ||
        !ok(cudaMalloc(&L->d_bar, 4 * sizeof(unsigned))) || !ok(cudaMalloc(&L->d_err, sizeof(int))) ||
        !ok(cudaMalloc(&L->d_ctl, sizeof(int))) || !ok(cudaMalloc(&L->d_bad, sizeof(unsigned long long))) ||
        !ok(cudaMemset(L->d_bar, 0, 4 * sizeof(unsigned))) || !ok(cudaMemset(L->d_err, 0, sizeof(int))))
        return fail(POSI_ERR_CUDA, std::string("allocation failed"), L);
    int rc = posi_large_set_state(L, sys_i64, sys_f64, body_i64, body_f64);
    if (rc != POSI_OK) return fail(rc, "upload failed", L);
    if (status) *status = POSI_OK;
    return L;
}

void posi_large_destroy(posi_large* L) { free_large(L); }

int posi_large_set_state(posi_large* L, const int64_t* sys_i64, const double* sys_f64, const int64_t* body_i64,
                         const double* body_f64) {
    if (!L) return POSI_ERR_ARG;
    const int64_t n = L->n;
    if (body_f64) {
        auto bf = to_field_major(body_f64, n, POSI_BF_COUNT);
        LCK(cudaMemcpy(L->d_bf, bf.data(), bf.size() * sizeof(double), cudaMemcpyHostToDevice));
        // src/particles/universe.rs:177-196, libm pow like Rust's powf
        // near2[i]: the largest squared threshold of body i's checks (Roche
        // radius of row i, sum of radii), so that the kernel reads the table
        // only for pairs that are that close
        std::vector<double> roche((size_t)n * n, 0.), near2((size_t)n, 0.);
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = 0; j < n; ++j) {
                if (i == j) continue;
                const double mi = body_f64[i * POSI_BF_COUNT + POSI_BF_MASS], mj = body_f64[j * POSI_BF_COUNT + POSI_BF_MASS];
                const double ri = body_f64[i * POSI_BF_COUNT + POSI_BF_RADIUS], rj = body_f64[j * POSI_BF_COUNT + POSI_BF_RADIUS];
                const double rr = mi > mj ? (rj / 0.462) * std::pow(mi / mj, 1. / 3.)
                                          : (ri / 0.462) * std::pow(mj / mi, 1. / 3.);
                roche[(size_t)i * n + j] = rr;
                near2[i] = std::max(near2[i], std::max(rr * rr, (ri + rj) * (ri + rj)));
            }
        // a margin of 1e-12 relative covers the rounding of the kernel's own
        // products against the host's
        for (auto& x : near2) x *= 1. + 1e-12;
        LCK(cudaMemcpy(L->d_roche, roche.data(), roche.size() * sizeof(double), cudaMemcpyHostToDevice));
        LCK(cudaMemcpy(L->d_near2, near2.data(), near2.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (body_i64) {
        auto bi = to_field_major(body_i64, n, POSI_BI_COUNT);
        LCK(cudaMemcpy(L->d_bi, bi.data(), bi.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
    }
    if (sys_f64) LCK(cudaMemcpy(L->d_sf, sys_f64, POSI_SF_COUNT * sizeof(double), cudaMemcpyHostToDevice));
    if (sys_i64) LCK(cudaMemcpy(L->d_si, sys_i64, POSI_SI_COUNT * sizeof(int64_t), cudaMemcpyHostToDevice));
    return POSI_OK;
}

int posi_large_get_state(const posi_large* L, int64_t* sys_i64, double* sys_f64, int64_t* body_i64,
                         double* body_f64) {
    if (!L) return POSI_ERR_ARG;
    const int64_t n = L->n;
    LCK(cudaStreamSynchronize(L->stream));
    if (body_f64) {
        std::vector<double> bf((size_t)n * POSI_BF_COUNT);
        LCK(cudaMemcpy(bf.data(), L->d_bf, bf.size() * sizeof(double), cudaMemcpyDeviceToHost));
        from_field_major(bf, body_f64, n, POSI_BF_COUNT);
    }
    if (body_i64) {
        std::vector<int64_t> bi((size_t)n * POSI_BI_COUNT);
        LCK(cudaMemcpy(bi.data(), L->d_bi, bi.size() * sizeof(int64_t), cudaMemcpyDeviceToHost));
        from_field_major(bi, body_i64, n, POSI_BI_COUNT);
    }
    if (sys_f64) LCK(cudaMemcpy(sys_f64, L->d_sf, POSI_SF_COUNT * sizeof(double), cudaMemcpyDeviceToHost));
    if (sys_i64) LCK(cudaMemcpy(sys_i64, L->d_si, POSI_SI_COUNT * sizeof(int64_t), cudaMemcpyDeviceToHost));
    return POSI_OK;
}

// src/integrator/whfast.rs:226-233 (spins; the Roche radii are set with the state)
int posi_large_initialize_physical_values(posi_large* L) {
    if (!L) return POSI_ERR_ARG;
    const int64_t n = L->n;
    std::vector<double> bf((size_t)n * POSI_BF_COUNT);
    int rc = posi_large_get_state(L, nullptr, nullptr, nullptr, bf.data());
    if (rc != POSI_OK) return rc;
    for (int64_t i = 0; i < n; ++i) {
        double* F = bf.data() + (size_t)i * POSI_BF_COUNT;
        if (F[POSI_BF_MOI] == 0.) {
            posi::set_last_error("moment of inertia is zero");
            return POSI_ERR_PHYSICS;
        }
        for (int q = 0; q < 3; ++q) F[POSI_BF_SX + q] = F[POSI_BF_LX + q] / F[POSI_BF_MOI];
        F[POSI_BF_NSV2] = F[POSI_BF_SX] * F[POSI_BF_SX] + F[POSI_BF_SY] * F[POSI_BF_SY] + F[POSI_BF_SZ] * F[POSI_BF_SZ];
    }
    auto f = to_field_major(bf.data(), n, POSI_BF_COUNT);
    LCK(cudaMemcpy(L->d_bf, f.data(), f.size() * sizeof(double), cudaMemcpyHostToDevice));
    return POSI_OK;
}

}  // extern "C"

namespace {

// One cooperative launch of the engine (NT tangent directions) and its
// error report.
template <int NT, int CO = POSI_DEMOCRATIC_HELIOCENTRIC>
int run_large(posi_large* L, int64_t n_steps, const int32_t* seed_body, const int32_t* seed_param) {
    int per_sm = 0;
    LCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, posi_many::large_steps_kernel<NT, CO>,
                                                      posi_many::kBlock, 0));
    if (per_sm < 1) {
        posi::set_last_error("the engine's blocks do not fit one per SM");
        return POSI_ERR_CUDA;
    }
    posi_many::LDev d{};
    d.n = L->n;
    d.bf = L->d_bf; d.bi = L->d_bi; d.sf = L->d_sf; d.si = L->d_si; d.roche = L->d_roche;
    d.near2 = L->d_near2;
    d.pos = L->d_pos; d.gpart = L->d_gpart; d.bpart = L->d_bpart; d.tot = L->d_tot; d.bar = L->d_bar;
    d.bbar = L->d_bar + 2;
    d.ctl = L->d_ctl;
    d.err = L->d_err;
    d.bad = L->d_bad;
    d.ntile = L->ntile;
    d.per_block = NT > 0 ? L->per_block_tan : L->per_block;
    d.nbb = (int)((L->n + d.per_block - 1) / d.per_block);
    if (d.nbb > L->grid) {
        posi::set_last_error("too many bodies for the resident grid");
        return POSI_ERR_UNSUPPORTED;
    }
    d.tan = L->d_tan;
    d.dpos = L->d_dpos;
    for (int k = 0; k < posi_many::kMaxTangents; ++k) {
        d.seed_body[k] = seed_body ? seed_body[k] : -1;
        d.seed_param[k] = seed_param ? seed_param[k] : 0;
    }
    LCK(cudaMemsetAsync(L->d_bad, 0xff, sizeof(unsigned long long), L->stream));
    LCK(cudaMemsetAsync(L->d_ctl, 0, sizeof(int), L->stream));
    LCK(cudaMemsetAsync(L->d_bar, 0, 4 * sizeof(unsigned), L->stream));  // the barriers' arrival counts
    void* args[] = {&d, &n_steps};
    LCK(cudaEventRecord(L->e0, L->stream));
    LCK(cudaLaunchCooperativeKernel((const void*)posi_many::large_steps_kernel<NT, CO>, dim3(L->grid),
                                    dim3(posi_many::kBlock), args, 0, L->stream));
    LCK(cudaEventRecord(L->e1, L->stream));
    LCK(cudaEventSynchronize(L->e1));
    float ms = 0.f;
    LCK(cudaEventElapsedTime(&ms, L->e0, L->e1));
    L->last_ms = ms;
    int err = 0;
    LCK(cudaMemcpy(&err, L->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err & posi_many::LE_BARRIER) {
        posi::set_last_error("grid barrier wait ran out (the launch was abandoned; state unchanged)");
        cudaMemset(L->d_err, 0, sizeof(int));
        cudaMemset(L->d_bar, 0, 4 * sizeof(unsigned));
        return POSI_ERR_CUDA;
    }
    if (err & posi_many::LE_KEPLER) {
        posi::set_last_error("a Kepler solve did not converge");
        cudaMemset(L->d_err, 0, sizeof(int));
        return POSI_ERR_PHYSICS;
    }
    int64_t si[POSI_SI_COUNT];
    LCK(cudaMemcpy(si, L->d_si, sizeof(si), cudaMemcpyDeviceToHost));
    const int64_t fatal = si[POSI_SI_STATUS] & POSI_SYS_FATAL_MASK;
    if (fatal == POSI_SYS_COMPLETED) return POSI_COMPLETED;
    if (fatal) {
        posi::set_last_error("system frozen by a physical event (status " + std::to_string(fatal) + ", pair " +
                             std::to_string(si[POSI_SI_FAIL_PAIR]) + " = i * n + j)");
        return POSI_ERR_PHYSICS;
    }
    return POSI_OK;
}

}  // namespace

extern "C" {

int posi_large_iterate(posi_large* L, int64_t n_steps) {
    if (!L || n_steps < 0) return POSI_ERR_ARG;
    if (n_steps == 0) return POSI_OK;
    if (L->coords == POSI_JACOBI) return run_large<0, POSI_JACOBI>(L, n_steps, nullptr, nullptr);
    if (L->coords == POSI_WHDS) return run_large<0, POSI_WHDS>(L, n_steps, nullptr, nullptr);
    return run_large<0>(L, n_steps, nullptr, nullptr);
}

int posi_large_iterate_tangent(posi_large* L, int64_t n_steps, int32_t n_dirs, const int32_t* seed_body,
                               const int32_t* seed_param, double* tangents) {
    if (!L || n_steps < 0 || n_dirs < 1 || n_dirs > posi_many::kMaxTangents || !seed_body || !seed_param || !tangents) {
        posi::set_last_error("bad arguments (1 to 4 directions, seeds and tangents required)");
        return POSI_ERR_ARG;
    }
    if (L->coords != POSI_DEMOCRATIC_HELIOCENTRIC) {
        posi::set_last_error("the tangent runs integrate in democratic-heliocentric coordinates");
        return POSI_ERR_UNSUPPORTED;
    }
    const int64_t n = L->n;
    for (int d = 0; d < n_dirs; ++d) {
        if (seed_body[d] < -1 || seed_body[d] >= n || (seed_param[d] != posi_many::SEED_SIGMA &&
                                                        seed_param[d] != posi_many::SEED_K2)) {
            posi::set_last_error("seed " + std::to_string(d) + " out of range");
            return POSI_ERR_ARG;
        }
    }
    // the kernels carry 1, 2 or 4 directions; padding directions are zero
    const int nt = n_dirs == 1 ? 1 : n_dirs == 2 ? 2 : 4;
    // one warp per direction next to the primal warp of every 32 bodies
    if ((n + L->per_block_tan - 1) / L->per_block_tan > L->grid) {
        posi::set_last_error("tangents need at most 32 bodies per block (" +
                             std::to_string((int64_t)L->grid * 32) + " bodies on this device)");
        return POSI_ERR_UNSUPPORTED;
    }
    int32_t sb[posi_many::kMaxTangents], sp[posi_many::kMaxTangents];
    for (int d = 0; d < posi_many::kMaxTangents; ++d) {
        sb[d] = d < n_dirs ? seed_body[d] : -1;
        sp[d] = d < n_dirs ? seed_param[d] : 0;
    }
    // host [dir][body][12] <-> device [dir][12][body]
    std::vector<double> dev((size_t)nt * 12 * n, 0.);
    for (int d = 0; d < n_dirs; ++d)
        for (int64_t i = 0; i < n; ++i)
            for (int f = 0; f < 12; ++f) dev[((size_t)d * 12 + f) * n + i] = tangents[((size_t)d * n + i) * 12 + f];
    LCK(cudaMemcpy(L->d_tan, dev.data(), dev.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (n_steps == 0) return POSI_OK;
    int rc;
    switch (nt) {
        case 1: rc = run_large<1>(L, n_steps, sb, sp); break;
        case 2: rc = run_large<2>(L, n_steps, sb, sp); break;
        default: rc = run_large<4>(L, n_steps, sb, sp); break;
    }
    if (rc == POSI_ERR_CUDA) return rc;  // barrier failure: the launch wrote nothing back
    LCK(cudaMemcpy(dev.data(), L->d_tan, dev.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int d = 0; d < n_dirs; ++d)
        for (int64_t i = 0; i < n; ++i)
            for (int f = 0; f < 12; ++f) tangents[((size_t)d * n + i) * 12 + f] = dev[((size_t)d * 12 + f) * n + i];
    return rc;
}

int posi_large_last_timing(const posi_large* L, double* ms) {
    if (!L) return POSI_ERR_ARG;
    if (ms) *ms = L->last_ms;
    return POSI_OK;
}

}  // extern "C"
