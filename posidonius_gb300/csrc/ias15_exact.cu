// IAS15 kernels, reference operation order (-fmad=false).
#define POSI_EXACT 1
#include "ias15_impl.cuh"

namespace posi {
cudaError_t launch_ias15_exact(const DevView& d, const LaunchArgs& a, cudaStream_t stream) {
    return posi_exact::launch_ias15_any(d, a, stream);
}
cudaError_t prepare_ias15_exact() { return posi_exact::prepare_ias15_all(); }
}  // namespace posi
