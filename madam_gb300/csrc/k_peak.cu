// k_peak.cu -- FP64 throughput microbenchmark (the roofline denominator for the
// FP64 kernels of the plain form: the driver's measured peaks cover HBM copy and
// BF16 GEMM only).  Each thread runs 8 independent DFMA chains; the grid fills
// every SM several times over.
#include <cuda_runtime.h>

#include "../../include/mcbound.h"

namespace {
__global__ void __launch_bounds__(256) k_dfma(double *out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
           x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1.2345) out[blockIdx.x] = s;  // keep the chains alive
}
}  // namespace

extern "C" double mcb_measure_fp64_peak(void) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double *out = nullptr;
    if (cudaMalloc(&out, 65536 * sizeof(double)) != cudaSuccess) return -1.0;
    const int blocks = sms * 8, iters = 4096;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_dfma<<<blocks, 256>>>(out, 64, 0.999999, 1e-7);
    cudaEventRecord(a);
    for (int r = 0; r < 3; ++r) k_dfma<<<blocks, 256>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    double flops = 3.0 * blocks * 256.0 * iters * 8 * 2;
    return ms > 0 ? flops / (ms * 1e-3) / 1e9 : -1.0;
}
