// kernels_impl.cuh -- launch wrappers, included once per arithmetic mode.
#pragma once
#include "kernels.h"
#include "whfast_device.cuh"

namespace POSI_NS {

static_assert(sizeof(Dev) == sizeof(posi::DevView), "device view layout");

template <int G>
static cudaError_t launch_g(const posi::DevView& v, const posi::LaunchArgs& a, cudaStream_t stream) {
    Dev d;
    d.n_sys = v.n_sys; d.nmax = v.nmax; d.stride = v.stride;
    d.bf = v.bf; d.bi = v.bi; d.sf = v.sf; d.si = v.si;
    d.roche = v.roche; d.tables = v.tables; d.list = v.list; d.n_list = v.n_list;
    d.step_flags = v.step_flags;
    d.hist = v.hist;
    d.rec = v.rec;
    d.ias = v.ias;
    const int threads = posi::kBlockThreads;
    const int groups_per_block = threads / G;
    const int blocks = (int)((v.n_list + groups_per_block - 1) / groups_per_block);
    if (blocks <= 0) return cudaSuccess;
    const size_t smem = (size_t)groups_per_block * GroupSmem<G>::bytes;
    switch (a.op) {
        case posi::OP_STEPS:
            whfast_steps_kernel<G><<<blocks, threads, smem, stream>>>(d, a.n_steps);
            break;
#if !POSI_EXACT
        case posi::OP_STEPS_REC:
            if (!d.rec) return cudaErrorInvalidValue;
            whfast_steps_kernel<G, true><<<blocks, threads, smem, stream>>>(d, a.n_steps);
            break;
#endif
        case posi::OP_STEPS_SCHED:
            if constexpr (G >= 4) {
                if (!a.slot_job || !a.slot_steps || a.sched_blocks <= 0) return cudaErrorInvalidValue;
                const size_t ssmem = (size_t)(posi::kSchedBlockThreads / G) * GroupSmem<G>::bytes;
                whfast_sched_kernel<G><<<a.sched_blocks, posi::kSchedBlockThreads, ssmem, stream>>>(d, a.slot_job,
                                                                                                   a.slot_steps);
                break;
            } else {
                return cudaErrorInvalidValue;
            }
        case posi::OP_INIT:
            init_physical_kernel<G><<<blocks, threads, smem, stream>>>(d);
            break;
        case posi::OP_GRAVITY:
            gravity_kernel<G><<<blocks, threads, smem, stream>>>(d, a.ignore_terms);
            break;
        case posi::OP_EFFECTS:
            additional_effects_kernel<G><<<blocks, threads, smem, stream>>>(d, a.t_eval, a.evolution, a.dl, a.acc);
            break;
        default:
            return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int G>
static cudaError_t prepare_g() {
    const int smem = (posi::kBlockThreads / G) * GroupSmem<G>::bytes;
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(whfast_steps_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess) return e;
#if !POSI_EXACT
    if ((e = cudaFuncSetAttribute(whfast_steps_kernel<G, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess) return e;
#endif
    if constexpr (G >= 4) {
        const int ssmem = (posi::kSchedBlockThreads / G) * GroupSmem<G>::bytes;
        if ((e = cudaFuncSetAttribute(whfast_sched_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, ssmem)) !=
            cudaSuccess)
            return e;
    }
    if ((e = cudaFuncSetAttribute(init_physical_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(gravity_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess) return e;
    return cudaFuncSetAttribute(additional_effects_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

// Dynamic shared memory above 48 KB must be allowed per kernel, outside any
// stream capture.
static cudaError_t prepare_all() {
    cudaError_t e;
    if ((e = prepare_g<2>()) != cudaSuccess) return e;
    if ((e = prepare_g<4>()) != cudaSuccess) return e;
    if ((e = prepare_g<8>()) != cudaSuccess) return e;
    if ((e = prepare_g<16>()) != cudaSuccess) return e;
    return prepare_g<32>();
}

static cudaError_t launch_any(const posi::DevView& v, const posi::LaunchArgs& a, cudaStream_t stream) {
    switch (a.G) {
        case 2: return launch_g<2>(v, a, stream);
        case 4: return launch_g<4>(v, a, stream);
        case 8: return launch_g<8>(v, a, stream);
        case 16: return launch_g<16>(v, a, stream);
        case 32: return launch_g<32>(v, a, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace POSI_NS
