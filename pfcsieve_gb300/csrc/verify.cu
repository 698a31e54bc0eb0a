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

#include <algorithm>
#include <climits>
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

// ------------------------------------------------------- hit re-verification
//
// The CPU check of every hit (cl_sieve.cpp:509-540, verifyprime.cpp:199-268)
// on the device, all hits at once: the hit's verification product -- the
// type's start value (34!, 101#, 44!/44#) times every k in [35, n] (type 0),
// times the primes in [103, n] or the composites in [45, n] (the list of the
// search's mode, as the CPU check builds it) -- must be +1 or -1 modulo p with
// the hit's sign.  One CTA of 256 threads per hit: each thread multiplies a
// contiguous sub-range of k as plain multipliers in four chains (one
// reduction each, the power of R fixed once at the end), and the threads'
// products are combined by shuffles and through shared memory.
// Nothing here uses the sieve's tables or its walk, so the check is
// independent of the arithmetic it checks.

namespace pfc {

struct VerifyRec {
    uint64_t p, start;
    uint32_t lo, hi;     // k in [lo, hi]
    uint32_t what;       // 0 every k, 1 primes, 2 composites, 3 none
    int32_t sign;
};

__global__ void __launch_bounds__(256) verify_hits_kernel(const VerifyRec *r, uint32_t cnt, const uint32_t *primebits,
                                                          uint8_t *bad) {
    __shared__ uint64_t part[8];
    if (blockIdx.x >= cnt) return;   // whole blocks
    const VerifyRec h = r[blockIdx.x];
    const uint32_t t = threadIdx.x;
    Mont64 m;
    m.init(h.p);
    uint64_t a0 = m.one, a1 = m.one, a2 = m.one, a3 = m.one;
    uint32_t taken = 0;
    if (h.what != 3 && h.hi >= h.lo) {
        const uint32_t per = (h.hi - h.lo) / blockDim.x + 1;
        const uint32_t s = h.lo + t * per;   // <= hi + blockDim.x: no wrap below 2^31 + 256
        const uint32_t e = s <= h.hi ? min(s + per, h.hi + 1) : s;
        uint32_t k = s;
        if (h.what == 0) {
            for (; k + 3 < e; k += 4) {
                a0 = redc64(a0, k, m.p, m.pinv);
                a1 = redc64(a1, k + 1, m.p, m.pinv);
                a2 = redc64(a2, k + 2, m.p, m.pinv);
                a3 = redc64(a3, k + 3, m.p, m.pinv);
            }
            for (; k < e; ++k) a0 = redc64(a0, k, m.p, m.pinv);
            taken = e - s;
        } else {
            const uint32_t want = h.what == 1 ? 1u : 0u;
            for (; k < e; ++k)
                if (((__ldg(primebits + (k >> 5)) >> (k & 31)) & 1u) == want) {
                    if (taken & 1) a1 = redc64(a1, k, m.p, m.pinv);
                    else a0 = redc64(a0, k, m.p, m.pinv);
                    ++taken;
                }
        }
    }
    // each reduction by a plain k lowered the power of R by one
    uint64_t acc = m.mul(m.mul(m.mul(a0, a1), m.mul(a2, a3)), m.mont_R_pow(taken));
#pragma unroll
    for (int o = 16; o; o >>= 1) acc = m.mul(acc, __shfl_down_sync(0xffffffffu, acc, o));
    if ((t & 31) == 0) part[t >> 5] = acc;
    __syncthreads();
    if (t == 0) {
        for (uint32_t i = 1; i < (blockDim.x >> 5); ++i) acc = m.mul(acc, part[i]);
        const uint64_t v = m.mul(acc, m.to_mont(h.start));
        bad[blockIdx.x] = h.sign < 0 ? v != m.one : v != m.p - m.one;
    }
}

}  // namespace pfc

extern "C" int pfc_verify_factors_device(pfc_ctx *c, unsigned mode, uint32_t nmax, const pfc_factor *f, size_t n,
                                         uint8_t *bad, size_t *failed) {
    using namespace pfc;
    if (!c || (!f && n) || !failed) return PFC_ERR_ARG;
    *failed = 0;
    if (n == 0) return PFC_OK;
    if (n > (1u << 26)) return PFC_ERR_ARG;
    CK(cudaSetDevice(c->device));
    std::vector<VerifyRec> rec(n);
    uint32_t top = 0;
    bool lists = false;
    for (size_t i = 0; i < n; ++i) {
        const pfc_factor &x = f[i];
        if (x.p < 3 || !(x.p & 1) || x.type < 0 || x.type > 2 || x.nc == 0 || x.nc == INT32_MIN) return PFC_ERR_ARG;
        const uint32_t an = (uint32_t)(x.nc < 0 ? -x.nc : x.nc);
        VerifyRec &v = rec[i];
        v.p = x.p;
        v.start = verify_start(x.type, x.p);
        v.sign = x.nc < 0 ? -1 : 1;
        if (x.type == 0) {
            v.what = 0;
            v.lo = 35;
            v.hi = an;
        } else if (mode & PFC_PRIMORIAL) {   // primes in [103, nmax] (cl_sieve.cpp:1468-1476)
            v.what = 1;
            v.lo = 103;
            v.hi = std::min(an, nmax);
        } else if (mode & PFC_COMPOSITORIAL) {   // composites in [45, nmax) (cl_sieve.cpp:1478-1492)
            v.what = 2;
            v.lo = 45;
            v.hi = std::min(an, nmax ? nmax - 1 : 0u);
        } else {
            v.what = 3;
            v.lo = 1;
            v.hi = 0;
        }
        if (v.what == 1 || v.what == 2) {
            lists = true;
            top = std::max(top, v.hi);
        }
    }
    if (lists && (!c->vbits || top > c->vbits_top)) {
        // prime flags up to at least twice the range asked for, kept in the
        // context for later calls
        const uint32_t want = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(2ull * top, 1u << 20), 0x7FFFFFFFull);
        std::vector<uint32_t> bits(want / 32 + 1, 0u);
        for (uint32_t q : primes_between(2, want)) bits[q >> 5] |= 1u << (q & 31);
        if (c->vbits) {
            dfree_bytes(c, c->vbits, c->vbits_bytes);
            c->vbits = nullptr;
            c->vbits_top = 0;
            c->vbits_bytes = 0;
        }
        void *vb = nullptr;
        CK(dalloc_bytes(c, &vb, bits.size() * 4));
        cudaError_t e = cudaMemcpyAsync(vb, bits.data(), bits.size() * 4, cudaMemcpyHostToDevice, c->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);   // `bits` is freed on return
        if (e != cudaSuccess) {
            dfree_bytes(c, vb, bits.size() * 4);
            CK(e);
        }
        c->h2d += bits.size() * 4;
        c->vbits = static_cast<uint32_t *>(vb);
        c->vbits_top = want;
        c->vbits_bytes = bits.size() * 4;
    }
    DArr<VerifyRec> d_rec;
    DArr<uint8_t> d_bad;
    std::vector<uint8_t> hb(n);
    cudaError_t e = d_rec.upload(c, rec);
    if (e == cudaSuccess) e = d_bad.alloc(c, n);
    if (e == cudaSuccess) {
        verify_hits_kernel<<<(unsigned)n, 256, 0, c->st>>>(d_rec.p, (uint32_t)n, c->vbits, d_bad.p);
        c->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hb.data(), d_bad.p, n, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    c->d2h += n;
    d_rec.release(c);
    d_bad.release(c);
    CK(e);
    size_t nb = 0;
    for (size_t i = 0; i < n; ++i) nb += hb[i] != 0;
    if (bad) std::copy(hb.begin(), hb.end(), bad);
    *failed = nb;
    return nb ? PFC_ERR_VERIFY : PFC_OK;
}
