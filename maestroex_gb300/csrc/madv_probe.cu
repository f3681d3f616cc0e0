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

#include "madv_exact.cuh"

namespace madv {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

// Random doubles with exponents spread over [2^-1000, 2^1000], both signs, plus
// zeros, subnormals and values next to powers of two; each checked bit for bit.
__global__ void k_selftest(unsigned long long n, unsigned long long seed, RecipC r, double thr,
                           unsigned long long* fails) {
    const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const long long tb = dbits(thr);
    unsigned long long local = 0;
    for (unsigned long long idx = t; idx < n; idx += stride) {
        unsigned long long h = mix64(idx * 0x9e3779b97f4a7c15ULL + seed);
        double a;
        const int kind = (int)(h & 15);
        if (kind == 0) {
            a = (h & 16) ? -0.0 : 0.0;
        } else if (kind == 1) {
            a = __longlong_as_double((long long)((h >> 8) & 0x000fffffffffffffULL));  // subnormal
        } else {
            const unsigned long long mant = (h >> 12) & 0x000fffffffffffffULL;
            const unsigned long long ex = 23 + (mix64(h) % 2001);  // 2^-1000 .. 2^1000
            unsigned long long bits = (ex << 52) | (kind == 2 ? 0ULL : (kind == 3 ? 0x000fffffffffffffULL : mant));
            if (h & 32) bits |= 0x8000000000000000ULL;
            a = __longlong_as_double((long long)bits);
        }
        const double q = div_c(a, r);
        const double qi = a / r.y;
        if (dbits(q) != dbits(qi)) ++local;
        // integer comparisons against IEEE comparisons
        if (gt_t(a, tb) != (a > thr)) ++local;
        if (lt_negt(a, tb) != (a < -thr)) ++local;
        if (abs_gt_t(a, tb) != (fabs(a) > thr)) ++local;
        if (gt0(a) != (a > 0.0)) ++local;
        if (lt0(a) != (a < 0.0)) ++local;
        if (nz(a) != (fabs(a) > 0.0)) ++local;
        // bit-pattern scaling and product signs against the FP instructions, with operands
        // pushed to the ends of the exponent range every few draws
        const unsigned long long h2 = mix64(h ^ 0x5851f42d4c957f2dULL);
        double e = a;
        if ((h2 & 7) == 0) {  // near overflow / near the smallest normals
            const long long eb = (h2 & 8) ? (2040 + (long long)((h2 >> 4) % 7)) : (long long)((h2 >> 4) % 4);
            e = __longlong_as_double((dbits(a) & ~(0x7ffLL << 52)) | (eb << 52));
        }
        if (dbits(twice(e)) != dbits(2.0 * e)) ++local;
        if (dbits(half(e)) != dbits(0.5 * e)) ++local;
        // y with an exponent that puts Ex + Ey around the underflow limit of the product
        const long long ex = (dbits(e) >> 52) & 0x7ff;
        long long ey = (long long)((h2 >> 8) % 2047);
        if (h2 & 16) ey = 960 - ex + (long long)((h2 >> 20) % 24);
        if (ey < 0) ey = 0;
        if (ey > 2046) ey = 2046;
        const double yv = __longlong_as_double((long long)((h2 & 0x800fffffffffffffULL) | ((unsigned long long)ey << 52)));
        if (prod_gt0(e, yv) != (e * yv > 0.0)) ++local;
    }
    if (local) atomicAdd(fails, local);
}

}  // namespace madv

extern "C" int madv_selftest_exact(double y, double threshold, long long n, long long* failures, void* stream) {
    if (!failures || !(y > 0.0) || !(threshold >= 0.0) || n <= 0) return MADV_ERR_PARAM;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long* d = nullptr;
    if (cudaMallocAsync(&d, sizeof(*d), s) != cudaSuccess) return MADV_ERR_CUDA;
    cudaMemsetAsync(d, 0, sizeof(*d), s);
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    madv::k_selftest<<<nsm * 8, 256, 0, s>>>((unsigned long long)n, 0x1234567ULL, madv::make_recip(y), threshold, d);
    unsigned long long h = 0;
    cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    cudaFreeAsync(d, s);
    if (cudaGetLastError() != cudaSuccess) return MADV_ERR_CUDA;
    *failures = (long long)h;
    return MADV_OK;
}
