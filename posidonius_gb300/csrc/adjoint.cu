// adjoint.cu -- launchers of the adjoint kernels (adjoint_device.cuh).
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
