// ias15_impl.cuh -- launch wrappers of the IAS15 kernels, included once per
// arithmetic mode (a translation unit of their own, compiled next to the
// WHFast kernels).
#pragma once
#include "kernels.h"
#include "whfast_device.cuh"

namespace POSI_NS {

#include "ias15_device.cuh"

template <int G>
static cudaError_t launch_ias15_g(const posi::DevView& v, const posi::LaunchArgs& a, cudaStream_t stream) {
    if (!v.ias) return cudaErrorInvalidValue;
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
    ias15_steps_kernel<G><<<blocks, threads, smem, stream>>>(d, a.n_steps);
    return cudaGetLastError();
}

template <int G>
static cudaError_t prepare_ias15_g() {
    const int smem = (posi::kBlockThreads / G) * GroupSmem<G>::bytes;
    return cudaFuncSetAttribute(ias15_steps_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

static cudaError_t prepare_ias15_all() {
    cudaError_t e;
    if ((e = prepare_ias15_g<2>()) != cudaSuccess) return e;
    if ((e = prepare_ias15_g<4>()) != cudaSuccess) return e;
    if ((e = prepare_ias15_g<8>()) != cudaSuccess) return e;
    if ((e = prepare_ias15_g<16>()) != cudaSuccess) return e;
    return prepare_ias15_g<32>();
}

static cudaError_t launch_ias15_any(const posi::DevView& v, const posi::LaunchArgs& a, cudaStream_t stream) {
    switch (a.G) {
        case 2: return launch_ias15_g<2>(v, a, stream);
        case 4: return launch_ias15_g<4>(v, a, stream);
        case 8: return launch_ias15_g<8>(v, a, stream);
        case 16: return launch_ias15_g<16>(v, a, stream);
        case 32: return launch_ias15_g<32>(v, a, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace POSI_NS
