// Fast FP64 kernels: compiled with -fmad=true (multiply-add contraction).
#define POSI_EXACT 0
#include "kernels_impl.cuh"

namespace posi {
cudaError_t launch_fast(const DevView& d, const LaunchArgs& a, cudaStream_t stream) {
    if (a.op == OP_IAS15_STEPS) return launch_ias15_fast(d, a, stream);
    return posi_fast::launch_any(d, a, stream);
}
cudaError_t prepare_fast() {
    cudaError_t e = posi_fast::prepare_all();
    return e != cudaSuccess ? e : prepare_ias15_fast();
}
}  // namespace posi
