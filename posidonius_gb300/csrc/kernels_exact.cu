// Reference-order FP64 kernels: compiled with -fmad=false (no contraction).
#define POSI_EXACT 1
#include "kernels_impl.cuh"

namespace posi {
cudaError_t launch_exact(const DevView& d, const LaunchArgs& a, cudaStream_t stream) {
    return posi_exact::launch_any(d, a, stream);
}
cudaError_t prepare_exact() { return posi_exact::prepare_all(); }
}  // namespace posi
