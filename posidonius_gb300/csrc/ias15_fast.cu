// IAS15 kernels, FMA contraction (-fmad=true).
#define POSI_EXACT 0
#include "ias15_impl.cuh"

namespace posi {
cudaError_t launch_ias15_fast(const DevView& d, const LaunchArgs& a, cudaStream_t stream) {
    return posi_fast::launch_ias15_any(d, a, stream);
}
cudaError_t prepare_ias15_fast() { return posi_fast::prepare_ias15_all(); }
}  // namespace posi
