// Measurement helpers that have no counterpart in the reference: the FP64 issue-rate
// probe used as the roofline ceiling of the FP64-bound stage kernels.
#include <cuda_runtime.h>

#include "../../include/maestro_adv.h"

namespace madv {

// Eight independent FMA chains per thread, kept live through the store.
__global__ void k_fp64_fma_chain(double* out, int iters, double a, double b) {
    double x[8];
    for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3 + c;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = __fma_rn(x[c], a, b);
    }
    double s = 0.0;
    for (int c = 0; c < 8; ++c) s += x[c];
    if (s == 12345.678) out[0] = s;  // never true; keeps the chains alive
}

}  // namespace madv

extern "C" int madv_probe_fp64_peak(double* tflops, void* stream) {
    if (!tflops) return MADV_ERR_PARAM;
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    double* out = nullptr;
    if (cudaMallocAsync(&out, sizeof(double), s) != cudaSuccess) return MADV_ERR_CUDA;
    const int threads = 256, blocks = nsm * 8, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    madv::k_fp64_fma_chain<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-9);  // warm-up
    cudaEventRecord(e0, s);
    madv::k_fp64_fma_chain<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-9);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, s);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return MADV_ERR_CUDA;
    const double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return MADV_OK;
}
