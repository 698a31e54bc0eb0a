// verify.cu -- device self-check of a job's tables against slow products.
//
// The reference checks its power and product tables once per run by
// computing each product a second, slow way on the GPU modulo 2^64 - 59 and
// comparing (kernels/verifyslow.cl, kernels/verify.cl, cl_sieve.cpp:917-970,
// 1100-1140, 1270-1310); a mismatch ends the run.  Here the fast side is the
// job's own setup program run by the production setup kernel on a test prime
// its arithmetic accepts (2^31 - 1 for class-32 words, 2^62 - 57 for 896-bit
// words, 2^64 - 59 for 64-bit words), and the slow side is a grid-stride
// product over k in [2, n0 - 1] split into primes and composites by a
// deterministic Miller-Rabin test (bases 2, 7, 61, exact below 4.76e9), which
// does not use the host sieve that built the tables.  The primorial walk's
// prime list and the compositorial prime flags of [nmin, nmax) are checked the
// same way (product and count).
#include <cuda_runtime.h>

#include <vector>

#include "devmem.hpp"
#include "walk.cuh"

namespace pfc {

constexpr int kTestPrimes = kVerifyPrimes;

__device__ __forceinline__ uint64_t test_prime(int i) {
    return i == 0 ? 2147483647ull : (i == 1 ? 4611686018427387847ull : 18446744073709551557ull);
}

// deterministic Miller-Rabin for 32-bit k (bases 2, 7, 61)
__device__ bool is_prime32(uint32_t k) {
    if (k < 2) return false;
    if (k < 4) return true;
    if (!(k & 1u)) return false;
    Mont32 m;
    m.init(k);
    const uint32_t nm1 = k - 1, mone = k - m.one;
    const int t = __ffs(nm1) - 1;
    const uint32_t d = nm1 >> t;
    const uint32_t bases[3] = {2u, 7u, 61u};
    for (int i = 0; i < 3; ++i) {
        const uint32_t a = bases[i] % k;
        if (a == 0) continue;
        uint32_t x = m.to_mont(a), r = m.one;
        for (uint32_t e = d; e; e >>= 1) {  // r = a^d
            if (e & 1u) r = m.mul(r, x);
            x = m.mul(x, x);
        }
        if (r == m.one || r == mone) continue;
        bool ok = false;
        for (int s = 1; s < t && !ok; ++s) {
            r = m.mul(r, r);
            ok = r == mone;
        }
        if (!ok) return false;
    }
    return true;
}

// Over k in [lo, hi): products of the primes and of the composites modulo each
// test prime, and the prime count.  One record of 2*kTestPrimes plain residues
// and a count per block.
__global__ void __launch_bounds__(256) slow_products_kernel(uint64_t lo, uint64_t hi, uint64_t *out) {
    Mont64 m[kTestPrimes];
    uint64_t P[kTestPrimes], C[kTestPrimes];
#pragma unroll
    for (int i = 0; i < kTestPrimes; ++i) {
        m[i].init(test_prime(i));
        P[i] = C[i] = m[i].one;
    }
    uint64_t count = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = lo + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < hi; k += stride) {
        const bool prime = is_prime32((uint32_t)k);
        count += prime;
#pragma unroll
        for (int i = 0; i < kTestPrimes; ++i) {
            const uint64_t km = m[i].to_mont(k);
            if (prime) P[i] = m[i].mul(P[i], km);
            else C[i] = m[i].mul(C[i], km);
        }
    }
    __shared__ uint64_t sh[256];
    for (int v = 0; v < 2 * kTestPrimes + 1; ++v) {
        const int i = v % kTestPrimes;
        uint64_t x = v < kTestPrimes ? P[i] : (v < 2 * kTestPrimes ? C[i] : count);
        sh[threadIdx.x] = x;
        __syncthreads();
        for (int s = 128; s > 0; s >>= 1) {
            if (threadIdx.x < s) {
                sh[threadIdx.x] = v < 2 * kTestPrimes ? m[i].mul(sh[threadIdx.x], sh[threadIdx.x + s])
                                                      : sh[threadIdx.x] + sh[threadIdx.x + s];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            x = sh[0];
            out[(uint64_t)blockIdx.x * (2 * kTestPrimes + 1) + v] = v < 2 * kTestPrimes ? m[i].mul(x, 1) : x;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ host side

static uint64_t mulmod(uint64_t a, uint64_t b, uint64_t p) {
    return (uint64_t)((unsigned __int128)a * b % p);
}

// slow products over [lo, hi) (plain residues mod each test prime)
int slow_products(pfc_ctx *c, uint64_t lo, uint64_t hi, SlowProducts &out) {
    for (int i = 0; i < kTestPrimes; ++i) out.P[i] = out.C[i] = 1;
    out.count = 0;
    if (hi <= lo) return PFC_OK;
    const unsigned blocks = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((hi - lo + 255) / 256, 8u * c->sms));
    DArr<uint64_t> d;
    CK(d.alloc(c, (size_t)blocks * (2 * kTestPrimes + 1)));
    slow_products_kernel<<<blocks, 256, 0, c->st>>>(lo, hi, d.p);
    c->launches++;
    std::vector<uint64_t> h((size_t)blocks * (2 * kTestPrimes + 1));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), d.p, h.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    d.release(c);
    CK(e);
    for (unsigned b = 0; b < blocks; ++b) {
        const uint64_t *r = &h[(size_t)b * (2 * kTestPrimes + 1)];
        for (int i = 0; i < kTestPrimes; ++i) {
            out.P[i] = mulmod(out.P[i], r[i], kVerifyPrime[i]);
            out.C[i] = mulmod(out.C[i], r[kTestPrimes + i], kVerifyPrime[i]);
        }
        out.count += r[2 * kTestPrimes];
    }
    return PFC_OK;
}

}  // namespace pfc
