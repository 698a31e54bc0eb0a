// setup_tc.cu -- the setup of class-64 candidates below 2^64/3 (the lazy
// class) with the table-word fold on the tensor cores (tcgen05).
//
// The setup evaluates a program of 896-bit table words Z (products of
// primes, kernels.cuh Prog) into each candidate's residue.  The costly part
// on the integer pipe is the fold of each word against the candidate's
// position residues, T = sum_b z_b w_b with w_b = 2^(8b+32) mod p: an exact
// integer contraction (words x bytes) x (bytes x candidates).  Here it runs
// on the tensor cores in bf16 with fp32 accumulation and stays exact:
//   * a word is its 112 bytes z_b (0..255, exact in bf16);
//   * a candidate's 64-bit residues w_b are split into 8 byte planes
//     W_a[b] = byte a of w_b (0..255);
//   * D_a[word, cand] = sum_b z_b W_a[b] < 112 * 255 * 255 < 2^23, exact in
//     the fp32 accumulator;
//   * T = sum_a D_a 2^(8a) < 2^79 is assembled on the CUDA cores.
// One CTA of 256 threads owns 64 candidates: their byte planes stay in
// shared memory (8 x 14 KB) as the MMA's B operand (N = 64, K-major), and
// the program's words stream through in tiles of 128 (A operand, M = 128,
// K = 112: seven MMAs of K = 16 per plane, 56 per tile, into 8 x 64 TMEM
// columns, word = TMEM lane).  Per tile:
//   1. the threads convert the words' limbs into 112 bf16 bytes (A tile);
//   2. one thread issues the 56 tcgen05.mma and a commit to an mbarrier;
//   3. each thread reads one word's 8 sums for a share of the candidates
//      (tcgen05.ld; the warps of a lane quadrant split the candidates),
//      assembles T and reduces it to u = T 2^-96 R (mod p, lazy), so that
//      u = Z (mod p) and multiplying it in lowers the power of R by one, as a
//      word on the integer pipe does;
//   4. per candidate the words' u are multiplied into the accumulator in
//      program order (Horner: a group's squarings come before its words):
//      four threads per candidate, each over a quarter of the tile, when no
//      group starts inside the tile, else one thread in order.
// The result equals setup_kernel<Cls64L>'s: same program, exact arithmetic,
// canonical residues at the end.  Every wait is bounded; after a timeout the
// kernel sets bit 1 of `flags`, frees its TMEM and stores nothing.
#include <cuda_runtime.h>

#include <cstdint>

#include "walk.cuh"

namespace pfc {
namespace {

constexpr int kTcThreads = 256;               // two warps per TMEM lane quadrant
constexpr int kTcGroups = kTcThreads / 128;   // warp groups (each covers the 128 lanes)
constexpr int kTcParts = kTcThreads / 64;     // threads per candidate
constexpr int kTcWords = 128;                 // words per tile: MMA M, TMEM lanes
constexpr int kTcCands = 64;                  // candidates per CTA: MMA N
constexpr int kTcBytes = 112;                 // bytes of a 896-bit word: MMA K
constexpr int kTcPlanes = 8;                  // byte planes of a 64-bit residue
constexpr uint32_t kRowGroup = (kTcBytes / 8) * 128;              // 1792 B between 8-row core groups
constexpr uint32_t kATile = (kTcWords / 8) * kRowGroup;           // 28,672 B
constexpr uint32_t kBPlane = (kTcCands / 8) * kRowGroup;          // 14,336 B
constexpr uint32_t kOffA = 0;
constexpr uint32_t kOffB = kOffA + kATile;                         // 8 planes
constexpr uint32_t kOffU = kOffB + kTcPlanes * kBPlane;            // u64 [64 cands][128 words]
constexpr uint32_t kOffPart = kOffU + kTcCands * kTcWords * 8;     // u64 [parts][64] partial products
constexpr uint32_t kOffCand = kOffPart + kTcParts * kTcCands * 8;  // p, one (u64) and q (u32) per candidate
constexpr uint32_t kOffMisc = kOffCand + kTcCands * 24;            // mbarrier, TMEM address, timeout flag
constexpr uint32_t kSmemBytes = kOffMisc + 64;
static_assert(kSmemBytes <= 227 * 1024, "setup_tc shared memory");
static_assert(kOffB % 1024 == 0 && kOffU % 16 == 0 && kOffMisc % 8 == 0, "setup_tc alignment");
constexpr uint32_t kTmemCols = 512;           // 8 planes x 64 candidates
constexpr long kWaitLimit = 1L << 26;         // mbarrier polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle; core matrices of
// 8 rows x 16 bytes, K-adjacent cores 128 B apart (leading byte offset),
// 8-row groups kRowGroup apart (stride byte offset), descriptor version 1
__device__ __forceinline__ uint64_t mdesc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(kRowGroup >> 4) << 32) |
           (1ull << 46);
}

// byte offset of the core-matrix row holding elements (r, 8 k8 .. 8 k8 + 7)
__device__ __forceinline__ uint32_t tile_off(uint32_t r, uint32_t k8) { return (r / 8) * kRowGroup + k8 * 128 + (r % 8) * 16; }

// bf16 bits of an integer 0..255 (exact): the float v, whose low 16 bits are 0
__device__ __forceinline__ uint32_t bf16_of_byte(uint32_t v) {
    return __float_as_uint(__uint_as_float(0x4B000000u | v) - 8388608.0f) >> 16;
}

// eight bytes -> eight bf16 (16 bytes, one core-matrix row)
__device__ __forceinline__ uint4 bf16x8(uint64_t bytes8) {
    uint32_t h[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) h[i] = bf16_of_byte((uint32_t)(bytes8 >> (8 * i)) & 0xFFu);
    return make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16), h[6] | (h[7] << 16));
}

// bytes 8 k8 .. 8 k8 + 7 of a 896-bit word given as 32 limbs of 28 bits
__device__ __forceinline__ uint64_t word_bytes8(const uint32_t (&limb)[kWideLimbs], int k8) {
    const int bit = 64 * k8, i = bit / 28, o = bit % 28;
    // bits [bit, bit + 64) lie in limbs i .. i + 3 (o + 64 <= 91 < 112)
    unsigned __int128 acc = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (i + j < kWideLimbs) acc |= (unsigned __int128)limb[i + j] << (28 * j);
    return (uint64_t)(acc >> o);
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (long it = 0; it < kWaitLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// the 8 plane sums of this thread's word (TMEM lane) for candidates c0..c0+7
__device__ __forceinline__ void load_sums(uint32_t taddr, uint32_t c0, uint32_t (&v)[kTcPlanes][8]) {
#pragma unroll
    for (int a = 0; a < kTcPlanes; ++a) {
        const uint32_t addr = taddr + a * kTcCands + c0;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                     : "=r"(v[a][0]), "=r"(v[a][1]), "=r"(v[a][2]), "=r"(v[a][3]), "=r"(v[a][4]), "=r"(v[a][5]),
                       "=r"(v[a][6]), "=r"(v[a][7])
                     : "r"(addr)
                     : "memory");
    }
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// an exact fp32 integer 0 <= x < 2^23 (given as its bits) as uint32
__device__ __forceinline__ uint32_t f2u23(uint32_t bits) {
    return __float_as_uint(__uint_as_float(bits) + 8388608.0f) & 0x7FFFFFu;
}

__device__ __forceinline__ void sync_tc() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ uint64_t mulw2(uint64_t s, uint64_t u, uint64_t p, uint32_t q) {
    const uint32_t w[2] = {(uint32_t)u, (uint32_t)(u >> 32)};
    return mul_wide_word<2>(s, w, p, q);
}

}  // namespace

__global__ void __launch_bounds__(kTcThreads, 1) setup_tc_kernel(ClassBuf<uint64_t> c, SetupArgs<WideWord> a,
                                                                 uint32_t *flags) {
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t tid = threadIdx.x, warp = tid / 32;
    const uint32_t cnt = min(*c.count, c.cap);
    const uint32_t c0 = blockIdx.x * kTcCands;
    if (c0 >= cnt) return;   // whole CTA idle

    uint64_t *U = reinterpret_cast<uint64_t *>(sm + kOffU);
    uint64_t *part = reinterpret_cast<uint64_t *>(sm + kOffPart);
    uint64_t *cand_p = reinterpret_cast<uint64_t *>(sm + kOffCand);
    uint64_t *cand_one = cand_p + kTcCands;
    uint32_t *cand_q = reinterpret_cast<uint32_t *>(cand_one + kTcCands);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + kOffMisc);
    uint32_t *taddr_slot = reinterpret_cast<uint32_t *>(sm + kOffMisc + 8);
    uint32_t *timeout = reinterpret_cast<uint32_t *>(sm + kOffMisc + 12);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(taddr_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)) : "memory");
        *timeout = 0;
    }

    // this thread's candidate and part: kTcParts threads per candidate (part 0
    // holds the accumulator)
    const uint32_t cl = tid % kTcCands, prt = tid / kTcCands;
    const uint32_t ci = c0 + cl;
    const bool act = ci < cnt;
    Mont64 m;
    m.init(act ? c.p[ci] : 0x1FFFFFFFFFFFFFFFull);   // an idle slot works on 2^61 - 1
    if (prt == 0) {
        cand_p[cl] = m.p;
        cand_one[cl] = m.one;
        cand_q[cl] = m.q32;
    }

    // B operand: the candidate's residues w_b = 2^(8b+32) mod p as 8 byte
    // planes (each part writes its share of the 14 groups of 8 bytes)
    {
        constexpr uint32_t kChunk = (kTcBytes / 8 + kTcParts - 1) / kTcParts;
        const uint32_t k8a = min(prt * kChunk, (uint32_t)(kTcBytes / 8)),
                       k8b = min(k8a + kChunk, (uint32_t)(kTcBytes / 8));
        const uint64_t c256 = m.to_mont(256);
        uint64_t x = m.p > (1ull << 32) ? (1ull << 32) : (1ull << 32) - m.p;   // 2^32 mod p
        for (uint32_t b = 0; b < 8 * k8a; ++b) x = m.mul(x, c256);
        for (uint32_t k8 = k8a; k8 < k8b; ++k8) {
            uint64_t w[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                w[j] = x;
                x = m.mul(x, c256);
            }
#pragma unroll
            for (int pl = 0; pl < kTcPlanes; ++pl) {
                uint64_t bytes = 0;
#pragma unroll
                for (int j = 0; j < 8; ++j) bytes |= ((w[j] >> (8 * pl)) & 0xFFull) << (8 * j);
                *reinterpret_cast<uint4 *>(sm + kOffB + pl * kBPlane + tile_off(cl, k8)) = bf16x8(bytes);
            }
        }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    sync_tc();
    const uint32_t tbase = *taddr_slot;
    const uint32_t quad = warp % 4, wgroup = warp / 4;      // TMEM lane quadrant, warp group
    const uint32_t taddr = tbase + ((quad * 32u) << 16);    // this warp's TMEM lanes
    const uint32_t word = quad * 32 + (tid % 32);           // this thread's word of a tile
    // f32 <- bf16 x bf16, both K-major, N = 64, M = 128
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcCands >> 3) << 17) |
                           ((uint32_t)(kTcWords >> 4) << 24);

    uint32_t parity = 0;
    bool failed = false;
    uint64_t s0 = 0, s1 = 0;
    const int nprog = a.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL) ? 2 : 1;
    uint64_t acc = m.one;   // the candidate's accumulator (part 0)
    for (int pi = 0; pi < nprog && !failed; ++pi) {
        const Prog<WideWord> &pg = pi == 0 ? a.a : a.b;
        uint32_t w_first = 0, w_end = 0;
        if (pg.ngroups) {
            w_first = __ldg(pg.groups);
            w_end = __ldg(pg.groups + 3 * (pg.ngroups - 1) + 1);
        }
        uint32_t g = 0;   // first group whose squarings are still due
        for (uint32_t t0 = w_first; t0 < w_end; t0 += kTcWords) {
            const uint32_t t1 = min(t0 + kTcWords, w_end);
            // 1. A tile: word t0 + word as 112 bf16 bytes (zeros past the end);
            //    the warp groups take alternate groups of 8 bytes
            {
                uint32_t limb[kWideLimbs];
                const bool have = t0 + word < t1;
                const uint4 *src = reinterpret_cast<const uint4 *>(pg.words + (have ? t0 + word : t0));
#pragma unroll
                for (int k = 0; k < kWideLimbs / 4; ++k) {
                    const uint4 z = have ? __ldg(src + k) : make_uint4(0, 0, 0, 0);
                    limb[4 * k] = z.x;
                    limb[4 * k + 1] = z.y;
                    limb[4 * k + 2] = z.z;
                    limb[4 * k + 3] = z.w;
                }
#pragma unroll
                for (int k8 = 0; k8 < kTcBytes / 8; ++k8)
                    if (k8 % kTcGroups == (int)wgroup)
                        *reinterpret_cast<uint4 *>(sm + kOffA + tile_off(word, k8)) = bf16x8(word_bytes8(limb, k8));
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            sync_tc();
            // 2. the tile's products, plane after plane
            if (tid == 0) {
                const uint32_t aaddr = smem_u32(sm + kOffA);
#pragma unroll 1
                for (int pl = 0; pl < kTcPlanes; ++pl) {
                    const uint32_t baddr = smem_u32(sm + kOffB + pl * kBPlane);
#pragma unroll
                    for (int s = 0; s < kTcBytes / 16; ++s) {
                        const uint64_t da = mdesc(aaddr + s * 256), db = mdesc(baddr + s * 256);
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tbase + pl * kTcCands),
                            "l"(da), "l"(db), "r"(idesc), "r"((uint32_t)s)
                            : "memory");
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(mbar))
                             : "memory");
            }
            if (!mbar_wait(smem_u32(mbar), parity)) atomicOr(timeout, 1u);
            parity ^= 1;
            sync_tc();
            if (*timeout) {
                failed = true;
                break;
            }
            // 3. u = T 2^-96 R for this thread's word and its warp group's candidates
            for (uint32_t cc = wgroup * (kTcCands / kTcGroups); cc < (wgroup + 1) * (kTcCands / kTcGroups); cc += 8) {
                uint32_t v[kTcPlanes][8];
                load_sums(taddr, cc, v);
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    uint32_t e[kTcPlanes];
#pragma unroll
                    for (int pl = 0; pl < kTcPlanes; ++pl) e[pl] = f2u23(v[pl][j]);
                    const uint64_t L = (uint64_t)e[0] + ((uint64_t)e[1] << 8) + ((uint64_t)e[2] << 16) +
                                       ((uint64_t)e[3] << 24);
                    const uint64_t H = (uint64_t)e[4] + ((uint64_t)e[5] << 8) + ((uint64_t)e[6] << 16) +
                                       ((uint64_t)e[7] << 24);
                    const uint64_t M = (L >> 32) + H;
                    const uint32_t tw[3] = {(uint32_t)L, (uint32_t)M, (uint32_t)(M >> 32)};
                    const uint32_t cj = cc + j;
                    U[cj * kTcWords + word] = mul_wide_word<3>(cand_one[cj], tw, cand_p[cj], cand_q[cj]);
                }
            }
            // 4. the words into each candidate's accumulator, in program order
            bool inside = false;   // a group starts strictly inside the tile
            for (uint32_t gg = g; gg < pg.ngroups; ++gg) {
                const uint32_t b = __ldg(pg.groups + 3 * gg);
                if (b >= t1) break;
                if (b > t0) {
                    inside = true;
                    break;
                }
            }
            __syncthreads();   // U complete
            if (prt == 0) {
                for (; g < pg.ngroups && __ldg(pg.groups + 3 * g) <= t0; ++g)
                    for (uint32_t k = __ldg(pg.groups + 3 * g + 2); k > 0; --k) acc = Cls64L::sq(m, acc);
            }
            if (!inside) {
                constexpr uint32_t kSpan = kTcWords / kTcParts;
                const uint32_t lo = t0 + kSpan * prt, hi = min(lo + kSpan, t1);
                uint64_t P = m.one;
                for (uint32_t w = lo; w < hi; ++w) P = mulw2(P, U[cl * kTcWords + (w - t0)], m.p, m.q32);
                if (prt > 0) part[prt * kTcCands + cl] = P;
                __syncthreads();
                if (prt == 0) {
                    acc = mulw2(acc, P, m.p, m.q32);
#pragma unroll
                    for (int h = 1; h < kTcParts; ++h) acc = mulw2(acc, part[h * kTcCands + cl], m.p, m.q32);
                }
            } else if (prt == 0) {
                for (uint32_t w = t0; w < t1; ++w) {
                    for (; g < pg.ngroups && __ldg(pg.groups + 3 * g) <= w; ++g)
                        for (uint32_t k = __ldg(pg.groups + 3 * g + 2); k > 0; --k) acc = Cls64L::sq(m, acc);
                    acc = mulw2(acc, U[cl * kTcWords + (w - t0)], m.p, m.q32);
                }
            }
        }
        if (failed) break;
        if (prt == 0) {
            for (; g < pg.ngroups; ++g)   // groups after the last word: squarings only
                for (uint32_t k = __ldg(pg.groups + 3 * g + 2); k > 0; --k) acc = Cls64L::sq(m, acc);
            for (uint32_t k = 0; k < pg.final_sq; ++k) acc = Cls64L::sq(m, acc);
            acc = m.mul(acc, m.mont_R_pow(pg.corr));
            if (nprog == 2 && pi == 0) s1 = acc;
            else s0 = acc;
        }
    }

    sync_tc();
    if (failed) {
        if (tid == 0) atomicOr(flags, 2u);
    } else if (prt == 0 && act) {
        c.s0[ci] = s0;
        c.s1[ci] = s1;
        c.nnext[ci] = a.nnext0;
    }
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTmemCols) : "memory");
}

// One CTA of 256 threads per 64 candidates, one CTA per SM (shared memory).
int launch_setup64w_tc(const ClassBuf<uint64_t> &c, const SetupArgs<WideWord> &a, uint32_t *flags, cudaStream_t st) {
    if (!c.cap) return 0;
    static bool configured[64] = {false};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (!configured[dev]) {
        if (cudaFuncSetAttribute(setup_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes) !=
            cudaSuccess)
            return 0;
        configured[dev] = true;
    }
    setup_tc_kernel<<<(c.cap + kTcCands - 1) / kTcCands, kTcThreads, kSmemBytes, st>>>(c, a, flags);
    return 1;
}

}  // namespace pfc
