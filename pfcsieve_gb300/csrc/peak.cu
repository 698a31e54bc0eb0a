// peak.cu -- integer-pipe throughput probe (measurement helper for the
// roofline of the sieve kernels; no counterpart in the reference).
//
// Each thread runs 8 independent multiply-add chains so that latency is
// hidden; the multiplier comes from a kernel argument so the compiler cannot
// strength-reduce it.  Grid = 8 CTAs of 1024 threads per SM.  Variants:
//   0: 32-bit IMAD (x = x*m + c)
//   1: 32-bit multiply-high (x = umulhi(x, m) + c)
//   2: 32x32->64 wide multiply-add (x = (u64)x*m + c, both halves kept)
//   3: 32-bit add (x = x + m), the ALU reference
#include <cuda_runtime.h>

#include <cstdint>

#include "pfcsieve.h"

namespace {

template <int V>
__global__ void __launch_bounds__(1024) peak_kernel(uint32_t *out, uint32_t iters, uint32_t m) {
    uint32_t x0 = threadIdx.x, x1 = x0 ^ 0x1234u, x2 = x0 + 77u, x3 = x0 * 3u, x4 = x0 ^ 0xbeefu,
             x5 = x0 + 1234567u, x6 = x0 * 7u, x7 = ~x0;
    uint32_t y0 = 0, y1 = 0, y2 = 0, y3 = 0, y4 = 0, y5 = 0, y6 = 0, y7 = 0;
    for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            if (V == 0) {
                x0 = x0 * m + 1u; x1 = x1 * m + 3u; x2 = x2 * m + 5u; x3 = x3 * m + 7u;
                x4 = x4 * m + 9u; x5 = x5 * m + 11u; x6 = x6 * m + 13u; x7 = x7 * m + 15u;
            } else if (V == 1) {
                x0 = __umulhi(x0, m) + 1u; x1 = __umulhi(x1, m) + 3u; x2 = __umulhi(x2, m) + 5u;
                x3 = __umulhi(x3, m) + 7u; x4 = __umulhi(x4, m) + 9u; x5 = __umulhi(x5, m) + 11u;
                x6 = __umulhi(x6, m) + 13u; x7 = __umulhi(x7, m) + 15u;
            } else if (V == 2) {
                uint64_t t;
                t = (uint64_t)x0 * m + y0; x0 = (uint32_t)t; y0 = (uint32_t)(t >> 32);
                t = (uint64_t)x1 * m + y1; x1 = (uint32_t)t; y1 = (uint32_t)(t >> 32);
                t = (uint64_t)x2 * m + y2; x2 = (uint32_t)t; y2 = (uint32_t)(t >> 32);
                t = (uint64_t)x3 * m + y3; x3 = (uint32_t)t; y3 = (uint32_t)(t >> 32);
                t = (uint64_t)x4 * m + y4; x4 = (uint32_t)t; y4 = (uint32_t)(t >> 32);
                t = (uint64_t)x5 * m + y5; x5 = (uint32_t)t; y5 = (uint32_t)(t >> 32);
                t = (uint64_t)x6 * m + y6; x6 = (uint32_t)t; y6 = (uint32_t)(t >> 32);
                t = (uint64_t)x7 * m + y7; x7 = (uint32_t)t; y7 = (uint32_t)(t >> 32);
            } else {
                x0 += m; x1 ^= x0; x2 += m; x3 ^= x2; x4 += m; x5 ^= x4; x6 += m; x7 ^= x6;
            }
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 ^ x1 ^ x2 ^ x3 ^ x4 ^ x5 ^ x6 ^ x7 ^ y0 ^ y1 ^ y2 ^
                                                 y3 ^ y4 ^ y5 ^ y6 ^ y7;
}

}  // namespace

// Measured throughput of `variant` in operations per second (one IMAD, one
// mul.hi, one wide multiply-add (counted as one) or one add = one op).
extern "C" int pfc_bench_int_peak(int device, int variant, double *ops_per_s) {
    if (!ops_per_s || variant < 0 || variant > 3) return PFC_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return PFC_ERR_NO_DEVICE;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = sms * 2, threads = 1024;
    uint32_t *out = nullptr;
    if (cudaMalloc(&out, (size_t)blocks * threads * 4) != cudaSuccess) return PFC_ERR_NOMEM;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const uint32_t iters = 4096, m = 0x9e3779b1u;
    auto launch = [&](void) {
        switch (variant) {
            case 0: peak_kernel<0><<<blocks, threads>>>(out, iters, m); break;
            case 1: peak_kernel<1><<<blocks, threads>>>(out, iters, m); break;
            case 2: peak_kernel<2><<<blocks, threads>>>(out, iters, m); break;
            default: peak_kernel<3><<<blocks, threads>>>(out, iters, m); break;
        }
    };
    launch();  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(a);
        launch();
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return PFC_ERR_CUDA;
    const double ops = (double)blocks * threads * iters * 16.0 * 8.0;
    *ops_per_s = ops / (best * 1e-3);
    return PFC_OK;
}
