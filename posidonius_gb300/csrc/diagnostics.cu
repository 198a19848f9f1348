// diagnostics.cu -- FP64 rate probe of the device (roofline denominator).
//
// Each thread runs eight independent DFMA chains; the rate is
// 2 * threads * 8 * iters / time.  Launching it with 1..32 warps per SM shows
// how many resident warps the FP64 pipe needs to reach its peak.
#include <cuda_runtime.h>

#include "../../include/posidonius_gb300.h"

namespace {
__global__ void dfma_chains(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-7, x1 = x0 + 1e-9, x2 = x0 + 2e-9, x3 = x0 + 3e-9;
    double x4 = x0 + 4e-9, x5 = x0 + 5e-9, x6 = x0 + 6e-9, x7 = x0 + 7e-9;
    for (int k = 0; k < iters; ++k) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    const double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 1234.5) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains alive
}
}  // namespace

extern "C" int posi_fp64_probe(int blocks, int threads, int iters, double* ms, double* tflops) {
    if (blocks < 1 || threads < 1 || threads > 1024 || iters < 1) return POSI_ERR_ARG;
    double* out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return POSI_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dfma_chains<<<blocks, threads>>>(out, iters / 10 + 1, 0.9999999, 1e-9);  // warm-up
    cudaEventRecord(e0);
    dfma_chains<<<blocks, threads>>>(out, iters, 0.9999999, 1e-9);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return POSI_ERR_CUDA;
    if (ms) *ms = t;
    if (tflops) *tflops = 2.0 * 8.0 * (double)blocks * threads * iters / (t * 1e-3) / 1e12;
    return POSI_OK;
}
