// Reference-order FP64 kernels: compiled with -fmad=false (no contraction).
#define POSI_EXACT 1
#include "kernels_impl.cuh"

namespace posi {
cudaError_t launch_exact(const DevView& d, const LaunchArgs& a, cudaStream_t stream) {
    if (a.op == OP_IAS15_STEPS) return launch_ias15_exact(d, a, stream);
    return posi_exact::launch_any(d, a, stream);
}
cudaError_t prepare_exact() {
    cudaError_t e = posi_exact::prepare_all();
    return e != cudaSuccess ? e : prepare_ias15_exact();
}
}  // namespace posi
