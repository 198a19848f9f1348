// adjoint.cu -- launchers of the adjoint kernels (adjoint_device.cuh).
#include <climits>
#include <mutex>
#include <string>

#include "adjoint_device.cuh"
#include "kernels.h"

namespace posi {

static_assert(posi_adj::SV_COUNT == kAdjTapeFields, "record layout");
static_assert(posi_adj::LM_COUNT == 12 && posi_adj::GD_COUNT == 2, "adjoint layout");

namespace {
template <int G>
cudaError_t launch_adj_g(const AdjView& v, int which, int64_t k_steps, cudaStream_t stream) {
    posi_adj::AdjDev d;
    d.n_sys = v.n_sys; d.nmax = v.nmax; d.stride = v.stride;
    d.bf = v.bf; d.bi = v.bi; d.sf = v.sf; d.si = v.si;
    d.list = v.list; d.n_list = v.n_list;
    d.tape = v.tape; d.lam = v.lam; d.grad = v.grad; d.err = v.err;
    const int threads = kBlockThreads;
    const int groups_per_block = threads / G;
    const int blocks = (int)((v.n_list + groups_per_block - 1) / groups_per_block);
    if (blocks <= 0) return cudaSuccess;
    const size_t smem = (size_t)groups_per_block * posi_adj::AdjSmem<G>::bytes;
    if (which == 0)
        posi_adj::adj_record_kernel<G><<<blocks, threads, smem, stream>>>(d, k_steps);
    else
        posi_adj::adj_reverse_kernel<G><<<blocks, threads, smem, stream>>>(d, k_steps);
    return cudaGetLastError();
}

template <int G>
cudaError_t prepare_adj_g() {
    const int smem = (kBlockThreads / G) * posi_adj::AdjSmem<G>::bytes;
    cudaError_t e = cudaFuncSetAttribute(posi_adj::adj_record_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(posi_adj::adj_reverse_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}
}  // namespace

int adjoint_group_size(int64_t n) {
    if (n < 1) return 0;
    if (n <= 2) return 2;
    if (n <= 4) return 4;
    if (n <= 8) return 8;
    return 0;
}

cudaError_t launch_adjoint(const AdjView& v, int which, int64_t k_steps, int G, cudaStream_t stream) {
    switch (G) {
        case 2: return launch_adj_g<2>(v, which, k_steps, stream);
        case 4: return launch_adj_g<4>(v, which, k_steps, stream);
        case 8: return launch_adj_g<8>(v, which, k_steps, stream);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t prepare_adjoint() {
    cudaError_t e;
    if ((e = prepare_adj_g<2>()) != cudaSuccess) return e;
    if ((e = prepare_adj_g<4>()) != cudaSuccess) return e;
    return prepare_adj_g<8>();
}

}  // namespace posi

// ---------------------------------------------------------------------------
// Allocation-free adjoint of a short run (posi_adjoint_vjp_static).
//
// For callers that may not allocate device memory: applications whose device
// memory is owned by their own pool or arena (a framework's caching
// allocator that has reserved the GPU, an embedded solver given a fixed
// budget), and latency-sensitive loops in which a cudaMalloc -- which can
// synchronise the device -- is not acceptable.  The step records live in one
// file-scope device array instead; its address is taken once per device.
// ---------------------------------------------------------------------------
namespace posi {
namespace {

constexpr size_t kStaticScratchBytes = size_t(48) << 20;  // 48 MiB
__device__ __align__(256) unsigned char g_adj_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_setup;  // guards the once-per-device set-up below

__global__ void static_list_and_check(int32_t* list, int32_t n_sys, int64_t nmax, const int64_t* si,
                                      int32_t* flags) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_sys) return;
    const int64_t n = si[(int64_t)POSI_SI_N * n_sys + s];
    const bool ok = si[(int64_t)POSI_SI_COORDS * n_sys + s] == POSI_JACOBI &&
                    si[(int64_t)POSI_SI_EVOLUTION * n_sys + s] == 0 && n >= 1 && n <= nmax &&
                    (si[(int64_t)POSI_SI_GR * n_sys + s] == 0 ||
                     si[(int64_t)POSI_SI_GR_IMPL * n_sys + s] == POSI_GR_KIDDER1995) &&
                    si[(int64_t)POSI_SI_WIND * n_sys + s] == 0 && si[(int64_t)POSI_SI_DISK * n_sys + s] == 0 &&
                    si[(int64_t)POSI_SI_INTEGRATOR * n_sys + s] == POSI_INTEGRATOR_WHFAST;
    flags[s] = ok ? 0 : POSI_ADJ_UNSUPPORTED;
    // a refused system stays out of the record and reverse kernels: its body
    // count may exceed nmax, and its lanes would then index the next system
    list[s] = ok ? s : -1;
}

}  // namespace
}  // namespace posi

extern "C" int posi_adjoint_vjp_static(int64_t n_systems, int64_t nmax, const int64_t* d_sys_i64,
                                       const double* d_sys_f64, const int64_t* d_body_i64, const double* d_body_f64,
                                       int64_t n_steps, double* d_lam, double* d_grad, int32_t* d_flags,
                                       void* stream) {
    using namespace posi;
    if (n_systems < 1 || n_systems > INT32_MAX || nmax < 1 || n_steps < 1 || !d_sys_i64 || !d_sys_f64 ||
        !d_body_i64 || !d_body_f64 || !d_lam || !d_grad || !d_flags) {
        set_last_error("posi_adjoint_vjp_static: bad arguments");
        return POSI_ERR_ARG;
    }
    const int G = adjoint_group_size(nmax);
    if (G == 0) {
        set_last_error("posi_adjoint_vjp_static: systems of up to 8 bodies only");
        return POSI_ERR_UNSUPPORTED;
    }
    const int64_t stride = n_systems * nmax;
    const size_t list_bytes = ((size_t)n_systems * sizeof(int32_t) + 255) / 256 * 256;
    const size_t step_bytes = (size_t)posi_adj::SV_COUNT * sizeof(double) * (size_t)stride;
    // bounded by division first, so that no product below can wrap
    if ((uint64_t)nmax > kStaticScratchBytes || (uint64_t)stride > kStaticScratchBytes / sizeof(double) ||
        list_bytes > kStaticScratchBytes || (uint64_t)n_steps > (kStaticScratchBytes - list_bytes) / step_bytes) {
        set_last_error("posi_adjoint_vjp_static: " + std::to_string(n_steps) + " steps x " +
                       std::to_string(n_systems) + " systems x " + std::to_string(nmax) +
                       " bodies of step records do not fit the " + std::to_string(kStaticScratchBytes) +
                       "-byte static scratch (at most " +
                       std::to_string(kStaticScratchBytes / (posi_adj::SV_COUNT * sizeof(double))) +
                       " body-steps)");
        return POSI_ERR_ARG;
    }
    const size_t tape_bytes = (size_t)n_steps * step_bytes;  // a multiple of 8; the list follows it
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_last_error("posi_adjoint_vjp_static: no usable current device");
        return POSI_ERR_CUDA;
    }
    // set-up, once per device (the first call on a device must come before
    // any stream capture); host threads making their first calls together
    // wait for one another
    char* base = nullptr;
    {
        std::lock_guard<std::mutex> setup_lock(g_scratch_setup);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_adj_scratch);
            if (e != cudaSuccess || !p) {
                set_last_error(std::string("posi_adjoint_vjp_static: cudaGetSymbolAddress: ") +
                               cudaGetErrorString(e));
                return POSI_ERR_CUDA;
            }
            e = prepare_adjoint();
            if (e != cudaSuccess) {
                set_last_error(std::string("posi_adjoint_vjp_static: ") + cudaGetErrorString(e));
                return POSI_ERR_CUDA;
            }
            g_scratch_ptr[dev] = p;
        }
        base = (char*)g_scratch_ptr[dev];
    }
    AdjView v;
    v.n_sys = n_systems;
    v.nmax = nmax;
    v.stride = stride;
    v.bf = d_body_f64;
    v.bi = d_body_i64;
    v.sf = d_sys_f64;
    v.si = d_sys_i64;
    v.tape = (double*)base;
    int32_t* list = (int32_t*)(base + tape_bytes);
    v.list = list;
    v.n_list = (int32_t)n_systems;
    v.lam = d_lam;
    v.grad = d_grad;
    v.err = d_flags;
    cudaStream_t st = (cudaStream_t)stream;
    static_list_and_check<<<(int)((n_systems + 255) / 256), 256, 0, st>>>(list, (int32_t)n_systems, nmax, d_sys_i64,
                                                                       d_flags);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_adjoint(v, 0, n_steps, G, st);
    if (e == cudaSuccess) e = launch_adjoint(v, 1, n_steps, G, st);
    if (e != cudaSuccess) {
        set_last_error(std::string("posi_adjoint_vjp_static: ") + cudaGetErrorString(e));
        return POSI_ERR_CUDA;
    }
    return POSI_OK;
}
