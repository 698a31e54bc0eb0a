// gen.cu -- candidate-prime generator (replaces kernels/getsegprimes.cl and
// kernels/addsmallprimes.cl).
//
// A candidate is a prime 3..113, or an odd x >= 114 with no prime factor
// <= 113 that is a base-2 strong probable prime (getsegprimes.cl:110-223).
// The sieve bound must stay exactly 113: base-2 pseudoprimes with no factor
// <= 113 are candidates in the reference and enter its checksum.
//
// Layout: each thread owns one 64-bit word of the segment's odd numbers
// (128 integers).  The 29 small-prime patterns (one 64-bit mask per residue,
// 1591 masks, 12.4 KB) sit in shared memory; a word's composite mask is the OR
// of 29 pattern lookups indexed by x0 mod s (32-bit arithmetic from a per-tile
// base residue).  Survivors are popped bit by bit, tested with SPRP-2 in
// 32-bit (x < 2^32) or 64-bit Montgomery arithmetic, and appended to the
// class-32 (x < 2^31) or class-64 list with one atomic per warp (ballot + popc).
#include "arith.cuh"
#include "kernels.cuh"

namespace pfc {

#define PFC_SIEVE_LIST \
    PFC_SIEVE_STEP(0, 3, 0) \
    PFC_SIEVE_STEP(1, 5, 3) \
    PFC_SIEVE_STEP(2, 7, 8) \
    PFC_SIEVE_STEP(3, 11, 15) \
    PFC_SIEVE_STEP(4, 13, 26) \
    PFC_SIEVE_STEP(5, 17, 39) \
    PFC_SIEVE_STEP(6, 19, 56) \
    PFC_SIEVE_STEP(7, 23, 75) \
    PFC_SIEVE_STEP(8, 29, 98) \
    PFC_SIEVE_STEP(9, 31, 127) \
    PFC_SIEVE_STEP(10, 37, 158) \
    PFC_SIEVE_STEP(11, 41, 195) \
    PFC_SIEVE_STEP(12, 43, 236) \
    PFC_SIEVE_STEP(13, 47, 279) \
    PFC_SIEVE_STEP(14, 53, 326) \
    PFC_SIEVE_STEP(15, 59, 379) \
    PFC_SIEVE_STEP(16, 61, 438) \
    PFC_SIEVE_STEP(17, 67, 499) \
    PFC_SIEVE_STEP(18, 71, 566) \
    PFC_SIEVE_STEP(19, 73, 637) \
    PFC_SIEVE_STEP(20, 79, 710) \
    PFC_SIEVE_STEP(21, 83, 789) \
    PFC_SIEVE_STEP(22, 89, 872) \
    PFC_SIEVE_STEP(23, 97, 961) \
    PFC_SIEVE_STEP(24, 101, 1058) \
    PFC_SIEVE_STEP(25, 103, 1159) \
    PFC_SIEVE_STEP(26, 107, 1262) \
    PFC_SIEVE_STEP(27, 109, 1369) \
    PFC_SIEVE_STEP(28, 113, 1478)

static const uint32_t kPrimes29[kSmallPrimes] = {3,  5,  7,  11, 13, 17, 19, 23, 29, 31,
                                                 37, 41, 43, 47, 53, 59, 61, 67, 71, 73,
                                                 79, 83, 89, 97, 101, 103, 107, 109, 113};
__constant__ uint32_t c_primes29[kSmallPrimes] = {3,  5,  7,  11, 13, 17, 19, 23, 29, 31,
                                                  37, 41, 43, 47, 53, 59, 61, 67, 71, 73,
                                                  79, 83, 89, 97, 101, 103, 107, 109, 113};

// bit x set for the primes below 128 (x < 128)
__device__ __forceinline__ bool small_prime(uint32_t x) {
    const uint64_t lo = 0x28208a20a08a28acull;  // primes < 64
    const uint64_t hi = 0x800228a202088288ull;  // primes in [64, 128)
    return x < 64 ? ((lo >> x) & 1) : ((hi >> (x - 64)) & 1);
}

// warp-aggregated append of x to list (one atomicAdd per warp)
template <class W>
__device__ __forceinline__ void warp_append(bool take, W x, W *list, uint32_t cap, uint32_t *count) {
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    const unsigned lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) {
        const uint32_t idx = base + __popc(m & ((1u << lane) - 1u));
        if (idx < cap) list[idx] = x;
    }
}

__global__ void __launch_bounds__(256) gen_kernel(GenArgs a) {
    __shared__ uint64_t spat[kPatEntries];
    __shared__ uint32_t smod[kSmallPrimes];
    for (int i = threadIdx.x; i < kPatEntries; i += blockDim.x) spat[i] = a.pat[i];

    // a.share threads (1, 2 or 4) share one word, each testing the survivors
    // of its 64/share bits: small segments then have enough threads
    const uint32_t share = a.share, log_share = share == 4 ? 2 : share == 2 ? 1 : 0;
    const uint64_t nwords = (a.nodd + 63) >> 6;
    const uint64_t nunits = nwords << log_share;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t u0 = (uint64_t)blockIdx.x * blockDim.x; u0 < nunits; u0 += stride) {
        const uint64_t w0 = u0 >> log_share;   // first word of the tile (blockDim is a multiple of share)
        __syncthreads();
        if (threadIdx.x < kSmallPrimes) {
            // (base + 128*w0) mod s, without overflow
            const uint32_t s = c_primes29[threadIdx.x];
            const uint32_t wm = (uint32_t)(w0 % s);
            smod[threadIdx.x] = (a.bmod[threadIdx.x] + (128u * wm) % s) % s;
        }
        __syncthreads();

        const uint32_t tw = threadIdx.x >> log_share;   // word within the tile
        const uint64_t w = w0 + tw;
        uint64_t mask = ~0ull;  // set bit = not a candidate
        if (w < nwords) {
            mask = 0;
            const uint32_t t128 = 128u * tw;
#define PFC_SIEVE_STEP(k, s, off) mask |= spat[(off) + (smod[k] + t128) % (s)];
            PFC_SIEVE_LIST
#undef PFC_SIEVE_STEP
            const uint64_t left = a.nodd - 64 * w;
            if (left < 64) mask |= ~0ull << left;
            const uint64_t x0 = a.base + 128 * w;
            if (x0 < 128) {
                // below 114 the candidates are exactly the small primes
                // (addsmallprimes.cl:25-38); the sieve marked them composite
                for (int j = 0; j < 64; ++j) {
                    const uint64_t x = x0 + 2 * j;
                    if (x >= 114) break;
                    if (small_prime((uint32_t)x)) mask &= ~(1ull << j);
                    else mask |= 1ull << j;
                }
            }
            if (share > 1) {   // keep this thread's slice of the word
                const uint32_t bits = 64u >> log_share, q = threadIdx.x & (share - 1);
                const uint64_t mine = (bits == 64 ? ~0ull : ((1ull << bits) - 1)) << (q * bits);
                mask |= ~mine;
            }
        }
        while (__any_sync(0xffffffffu, mask != ~0ull)) {
            const bool have = mask != ~0ull;
            uint64_t x = 0;
            bool pass = false;
            if (have) {
                const int j = __ffsll((long long)~mask) - 1;
                mask |= 1ull << j;
                x = a.base + 128 * w + 2 * (uint64_t)j;
                if (x < 114) pass = true;
                else if (x < (1ull << 32)) pass = sprp2_32((uint32_t)x);
                else pass = sprp2_64(x);
            }
            const bool c32 = pass && x < kClassSplit;
            const bool c64 = pass && x >= kClassSplit;
            warp_append<uint32_t>(c32, (uint32_t)x, a.p32, a.cap32, a.count + 0);
            warp_append<uint64_t>(c64, x, a.p64, a.cap64, a.count + 1);
        }
    }
}

int launch_gen(const GenArgs &a, int sms, cudaStream_t st) {
    if (a.nodd == 0) return 0;
    const uint64_t nwords = (a.nodd + 63) >> 6;
    // segments of fewer words than four CTAs per SM share each word between
    // threads (measured: 10^6 integers near 10^7 took 44 us in 31 CTAs)
    GenArgs g = a;
    const uint64_t fill = (uint64_t)sms * 4 * 256;
    g.share = nwords * 2 > fill ? 1 : (nwords * 4 > fill ? 2 : 4);
    uint64_t blocks = (nwords * g.share + 255) / 256;
    const uint64_t maxb = (uint64_t)sms * 8;   // persistent-style: <= 8 resident CTAs per SM
    if (blocks > maxb) blocks = maxb;
    gen_kernel<<<(unsigned)blocks, 256, 0, st>>>(g);
    return 1;
}

void build_pattern_table(uint64_t *pat, uint32_t *primes29) {
    int off = 0;
    for (int k = 0; k < kSmallPrimes; ++k) {
        const uint32_t s = kPrimes29[k];
        primes29[k] = s;
        for (uint32_t r = 0; r < s; ++r) {
            uint64_t m = 0;
            for (uint32_t j = 0; j < 64; ++j)
                if ((r + 2 * j) % s == 0) m |= 1ull << j;
            pat[off + r] = m;
        }
        off += s;
    }
}

}  // namespace pfc
