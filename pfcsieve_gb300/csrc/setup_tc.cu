// setup_tc.cu -- the setup of class-32 candidates and of class-64 candidates
// below 2^64/3 (the lazy class) with the table-word fold on the tensor cores
// (tcgen05), for programs of at least kTcMinWords32 / kTcMinWords64 words
// (kernels.cuh).  The description below is of class 64; class 32 follows it.
//
// The setup evaluates a program of table words Z (products of primes,
// kernels.cuh Prog) into each candidate's residue.  The costly part on the
// integer pipe is the fold of each word against the candidate's position
// residues, T = sum_b z_b w_b with w_b = 2^(8b+32) mod p: an exact integer
// contraction (words x bytes) x (bytes x candidates).  Here it runs on the
// tensor cores in fp16 with fp32 accumulation and stays exact:
//   * the words are 1792-bit: each is the product of a pair of the program's
//     896-bit words (host.hpp TcProg), so half as many words reach the
//     CUDA cores; a word is its 224 bytes z_b (0..255, exact in fp16);
//   * a candidate's 64-bit residues w_b are split into 8 byte planes
//     W_a[b] = byte a of w_b (0..255);
//   * the bytes are summed in two halves of 112, each into its own fp32
//     accumulator: D_{a,h}[word, cand] = 2^23 + sum_{b in half h} z_b W_a[b].
//     The first MMA of each half writes 2048 * 4096 = 2^23 into every sum, and
//     a half's sum is at most 112 * 255 * 255 < 2^23, so every partial sum is
//     an integer in [2^23, 2^24), exact in fp32, and the fp32 bits of D are
//     0x4B000000 + the integer sum;
//   * T = sum_a (D_{a,0} + D_{a,1} - 2^24) 2^(8a) < 2^79 is assembled on the
//     CUDA cores.
// The programs are first laid out as fp16 byte tiles of 128 words (A operand,
// M = 128, K = 224, the shared-memory image; tc_pack_kernel multiplies the
// word pairs, once per job).  One CTA of 512 threads owns 32 candidates:
// their byte planes stay in shared memory as the MMA's B operand, K-major,
// one 8-row core group per candidate (row = plane), so that one MMA with
// N = 256 covers the 32 candidates x 8 planes and a candidate's 8 sums of a
// half are adjacent TMEM columns (two halves x 256 columns, word = TMEM lane;
// per half a bias MMA and seven MMAs of K = 16, 16 per tile).  Per tile t:
//   1. each thread reads one word's sums for a share of the candidates
//      (tcgen05.ld, 4 candidates x 8 planes per load and half; the four warps
//      of a lane quadrant split the candidates), assembles T and reduces it
//      by one Montgomery round, u = (T + m p) / 2^32 with m = -T p^-1 mod 2^32,
//      so u = T 2^-32 = Z (mod p) and u < 2^48 + p, stored in shared memory;
//      meanwhile tile t+1 arrives by one bulk copy (cp.async.bulk);
//   2. the products of tile t+1 are issued; they run while
//   3. fifteen threads of each candidate (one per warp but the first, whose
//      thread 0 issued the products) multiply a fifteenth of the tile's u
//      into their running products, two independent chains per thread (two
//      lazy rounds per product; a product lowers the power of R by one, as a
//      word on the integer pipe does).  At a group start that carries
//      squarings (Horner over exponent bits) every thread squares each of its
//      running products (squaring distributes over their Montgomery product);
//      at the end of a program they are combined into the accumulator (a tree
//      over the threads of the candidate).
// Class 32 (p < 2^31) runs the same kernel with 4 byte planes, 64 candidates
// per CTA (N = 64 x 4 = 256 again), T < 2^47 reduced by one 32-bit round and
// one Montgomery product (R = 2^32) per word.  The result equals
// setup_kernel<Cls64L>'s or setup_kernel<Cls32>'s: the same product of the
// same words in the same Horner order, exact arithmetic, canonical residues
// at the end.  Every wait is bounded; after a timeout the kernel sets bit 1 of
// `flags`, frees its TMEM and stores nothing.
#include <cuda_runtime.h>

#include <cstdint>

#include "walk.cuh"

namespace pfc {
namespace {

constexpr int kTcThreads = 512;
constexpr int kTcGroups = kTcThreads / 128;   // warp groups (each covers the 128 TMEM lanes)
constexpr int kTcWords = 128;                 // words per tile: MMA M, TMEM lanes
constexpr int kTcN = 256;                     // MMA N: candidates x byte planes
constexpr int kTcBytes = 224;                 // bytes of a 1792-bit word: MMA K
constexpr int kTcHalfBytes = kTcBytes / 2;    // bytes summed into one accumulator
constexpr int kTcChains = 2;                  // independent product chains per thread
constexpr uint32_t kRowGroup = (kTcBytes / 8) * 128;              // 3584 B between 8-row core groups
constexpr uint32_t kBiasRowGroup = 2 * 128;                       // bias tiles: K = 16
constexpr uint32_t kATile = (kTcWords / 8) * kRowGroup;           // 57,344 B
constexpr uint32_t kBTile = (kTcN / 8) * kRowGroup;               // 114,688 B: rows = candidate x plane
constexpr uint32_t kUStride = kTcWords + 1;   // words per candidate row; odd: column reads hit distinct banks
constexpr uint32_t kOffA = 0;
constexpr uint32_t kOffB = kOffA + kATile;
constexpr uint32_t kOffABias = kOffB + kBTile;                                // 128 x 16, column 0 = 2048
constexpr uint32_t kOffBBias = kOffABias + (kTcWords / 8) * kBiasRowGroup;    // 256 x 16, column 0 = 4096
constexpr uint32_t kOffU = kOffBBias + (kTcN / 8) * kBiasRowGroup;            // reduced words [cands][kUStride]
static_assert(kOffB % 16 == 0 && kOffABias % 16 == 0 && kOffBBias % 16 == 0 && kOffU % 16 == 0,
              "setup_tc alignment");
static_assert(kATile % 16 == 0, "bulk copies move multiples of 16 bytes");
static_assert(kTcHalfBytes % 16 == 0, "setup_tc shape");
constexpr uint32_t kTmemCols = 2 * kTcN;      // 2 halves x 256 (column = 256 h + planes c + plane)
constexpr long kWaitLimit = 1L << 26;         // mbarrier polls before giving up
constexpr uint32_t kBiasBits = 0x4B000000u;   // fp32 bits of 2^23

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle; core matrices of
// 8 rows x 16 bytes, K-adjacent cores 128 B apart (leading byte offset),
// 8-row groups `sbo` apart (stride byte offset), descriptor version 1
__device__ __forceinline__ uint64_t mdesc(uint32_t addr, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// byte offset of the core-matrix row holding elements (r, 8 k8 .. 8 k8 + 7)
__device__ __forceinline__ uint32_t tile_off(uint32_t r, uint32_t k8, uint32_t rowgroup = kRowGroup) {
    return (r / 8) * rowgroup + k8 * 128 + (r % 8) * 16;
}

// two bytes (bits 0-7 and 8-15 of x, or 16-23 and 24-31 with hi) -> two
// fp16 0..255: the fp16 of 1024 + v is 0x6400 | v (v < 1024), less 1024
template <bool HI>
__device__ __forceinline__ uint32_t f16x2_of_bytes(uint32_t x) {
    const uint32_t y = __byte_perm(x, 0x64u, HI ? 0x4342u : 0x4140u);
    uint32_t r;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(y), "r"(0x64006400u));
    return r;
}

// eight bytes -> eight fp16 (16 bytes, one core-matrix row)
__device__ __forceinline__ uint4 f16x8(uint64_t bytes8) {
    const uint32_t lo = (uint32_t)bytes8, hi = (uint32_t)(bytes8 >> 32);
    return make_uint4(f16x2_of_bytes<false>(lo), f16x2_of_bytes<true>(lo), f16x2_of_bytes<false>(hi),
                      f16x2_of_bytes<true>(hi));
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

// 32 columns of this thread's TMEM lane from column `col`
__device__ __forceinline__ void ld32(uint32_t taddr, uint32_t col, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr + col)
        : "memory");
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

// the program's word range [first, end)
__device__ __forceinline__ void prog_range(const Prog<WideWord> &pg, uint32_t &first, uint32_t &end) {
    first = end = 0;
    if (pg.ngroups) {
        first = __ldg(pg.groups);
        end = __ldg(pg.groups + 3 * (pg.ngroups - 1) + 1);
    }
}

// What differs between the size classes: the residue type, its byte planes,
// the reduction of T and the product of a reduced word into a running value.
template <class T>
struct TcClass;

// class 64 below 2^64/3: residues in [0, 2p) between squarings, lazy rounds
template <>
struct TcClass<Cls64L> {
    using W = uint64_t;
    using M = Mont64;
    static constexpr int kPlanes = 8;
    static constexpr uint64_t kIdle = 0x1FFFFFFFFFFFFFFFull;   // an idle slot works on 2^61 - 1
    __device__ static __forceinline__ uint32_t qv(const M &m) { return m.q32; }   // -p^-1 mod 2^32
    __device__ static __forceinline__ W two32(const M &m) {   // 2^32 mod p
        return m.p > (1ull << 32) ? (1ull << 32) : (1ull << 32) - m.p;
    }
    // T = L + 2^32 H < 2^79: u = (T + m p) / 2^32 with m = -T p^-1 mod 2^32,
    // so u = T 2^-32 (mod p) and u < 2^48 + p; tw0 + lo(m p0) = 2^32 [tw0 != 0]
    __device__ static __forceinline__ W reduce(uint64_t L, uint64_t H, W p, uint32_t q) {
        const uint32_t tw0 = (uint32_t)L;
        const uint64_t Mh = (L >> 32) + H;
        const uint32_t mm = tw0 * q;
        const uint64_t lo = (uint64_t)mm * (uint32_t)p;
        return Mh + (uint64_t)mm * (uint32_t)(p >> 32) + (lo >> 32) + (tw0 != 0 ? 1u : 0u);
    }
    __device__ static __forceinline__ W prod(const M &m, W s, W u) { return mulw2(s, u, m.p, m.q32); }
    __device__ static __forceinline__ W sq(const M &m, W s) { return Cls64L::sq(m, s); }
};

// class 32: canonical residues, R = 2^32
template <>
struct TcClass<Cls32> {
    using W = uint32_t;
    using M = Mont32;
    static constexpr int kPlanes = 4;
    static constexpr uint32_t kIdle = 0x7FFFFFFFu;   // an idle slot works on 2^31 - 1
    __device__ static __forceinline__ uint32_t qv(const M &m) { return m.pinv; }   // p^-1 mod 2^32
    __device__ static __forceinline__ W two32(const M &m) { return m.one; }
    // T = L < 2^48: with m = lo(T) p^-1 mod 2^32, T - m p = 0 (mod 2^32), so
    // u = hi(T) - hi(m p) exactly, in (-p, 2^17), plus p when negative:
    // u = T 2^-32 (mod p), u < 2^31
    __device__ static __forceinline__ W reduce(uint64_t L, uint64_t, W p, uint32_t pinv) {
        const uint32_t m1 = (uint32_t)L * pinv;
        const int64_t u = (int64_t)(L >> 32) - (int64_t)(((uint64_t)m1 * p) >> 32);
        return (W)(u < 0 ? u + p : u);
    }
    // s < p and u < 2^31: s u < p 2^32, one canonical round
    __device__ static __forceinline__ W prod(const M &m, W s, W u) { return m.mul(s, u); }
    __device__ static __forceinline__ W sq(const M &m, W s) { return m.mul(s, s); }
};

template <class T>
struct TcLayout {
    using W = typename TcClass<T>::W;
    static constexpr int kPlanes = TcClass<T>::kPlanes;
    static constexpr int kCands = kTcN / kPlanes;              // candidates per CTA
    static constexpr int kParts = kTcThreads / kCands;         // threads per candidate in the products
    static constexpr uint32_t kOffPart = kOffU + kCands * kUStride * sizeof(W);   // running products [parts][cands]
    static constexpr uint32_t kOffCand = kOffPart + kParts * kCands * sizeof(W);  // p (W) and q (u32) per candidate
    static constexpr uint32_t kOffCorr = (kOffCand + kCands * 12 + 7) & ~7u;      // Mont(R^corr) [2 programs][cands]
    static constexpr uint32_t kOffMisc = (kOffCorr + 2 * kCands * sizeof(W) + 15) & ~15u;   // 2 mbarriers, TMEM address, flag
    // parts that build byte planes; the first one after them computes the
    // programs' power-of-R corrections meanwhile
    static constexpr uint32_t kChunk = (kTcBytes / 8 + kParts - 1) / kParts;
    static constexpr uint32_t kBusy = (kTcBytes / 8 + kChunk - 1) / kChunk;
    static_assert(kBusy < (uint32_t)kParts, "a part left for the corrections");
    static constexpr uint32_t kSmemBytes = kOffMisc + 64;
    static_assert(kSmemBytes <= 227 * 1024, "setup_tc shared memory");
    static_assert(kCands % 32 == 0 && (kParts & (kParts - 1)) == 0,
                  "a part of the products is whole warps: part 0 holds the warp that issues the MMAs");
};

}  // namespace

// One thread per word slot of a tile: the 1792-bit word (the product of a
// pair of 896-bit words, or one alone; zero past the end) as 224 fp16 bytes
// in the tile's shared-memory image.  The product is formed column by column
// in radix 2^28 (a column sums at most 32 products of 28-bit limbs, below
// 2^61 with its carry) and written eight bytes at a time.
__global__ void tc_pack_kernel(const WideWord *words, const uint32_t *src, uint32_t nw, uint32_t ntiles, uint4 *out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntiles * kTcWords) return;
    const uint32_t tile = i / kTcWords, slot = i % kTcWords;
    uint32_t x[kWideLimbs], y[kWideLimbs];
    const bool have = i < nw;
    const uint32_t s = have ? __ldg(src + i) : 0u;
    const bool pair = have && (s >> 31);
    const uint32_t w = s & 0x7FFFFFFFu;
#pragma unroll
    for (int k = 0; k < kWideLimbs; ++k) {
        x[k] = have ? words[w].limb[k] : 0u;
        y[k] = pair ? words[w + 1].limb[k] : (k == 0 ? 1u : 0u);
    }
    unsigned char *tb = reinterpret_cast<unsigned char *>(out) + (size_t)tile * kATile;
    uint64_t carry = 0, bits = 0;
    int nbits = 0;
    uint32_t k8 = 0;
    for (int c = 0; c < 2 * kWideLimbs; ++c) {
        uint64_t col = carry;
        for (int a = c < kWideLimbs ? 0 : c - kWideLimbs + 1; a <= c && a < kWideLimbs; ++a)
            col += (uint64_t)x[a] * y[c - a];
        const uint64_t limb = col & ((1ull << kWideRadixBits) - 1u);
        carry = col >> kWideRadixBits;
        // 28 new bits above the nbits (< 64) already gathered
        bits |= limb << nbits;
        if (nbits + kWideRadixBits >= 64) {   // 64 bits complete
            *reinterpret_cast<uint4 *>(tb + tile_off(slot, k8++)) = f16x8(bits);
            const int used = 64 - nbits;      // bits of this limb in the completed group
            bits = used < kWideRadixBits ? limb >> used : 0;
            nbits = kWideRadixBits - used;
        } else {
            nbits += kWideRadixBits;
        }
    }
}

template <class T>
__global__ void __launch_bounds__(kTcThreads, 1)
    setup_tc_kernel(ClassBuf<typename TcClass<T>::W> c, SetupArgs<WideWord> a, TcTiles ta, TcTiles tb,
                    uint32_t *flags, uint32_t block0) {
    using C = TcClass<T>;
    using Lay = TcLayout<T>;
    using W = typename C::W;
    constexpr int kCands = Lay::kCands, kParts = Lay::kParts, kPlanes = Lay::kPlanes;
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t tid = threadIdx.x, warp = tid / 32;
    const uint32_t cnt = min(*c.count, c.cap);
    const uint32_t c0 = (blockIdx.x + block0) * kCands;
    if (c0 >= cnt) return;   // whole CTA idle

    W *U = reinterpret_cast<W *>(sm + kOffU);
    W *part = reinterpret_cast<W *>(sm + Lay::kOffPart);
    W *cand_p = reinterpret_cast<W *>(sm + Lay::kOffCand);
    uint32_t *cand_q = reinterpret_cast<uint32_t *>(sm + Lay::kOffCand + kCands * 8);
    uint64_t *mbar_mma = reinterpret_cast<uint64_t *>(sm + Lay::kOffMisc);
    uint64_t *mbar_load = reinterpret_cast<uint64_t *>(sm + Lay::kOffMisc + 8);
    uint32_t *taddr_slot = reinterpret_cast<uint32_t *>(sm + Lay::kOffMisc + 16);
    uint32_t *timeout = reinterpret_cast<uint32_t *>(sm + Lay::kOffMisc + 20);
    W *corr_pow = reinterpret_cast<W *>(sm + Lay::kOffCorr);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(taddr_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar_mma)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar_load)) : "memory");
        *timeout = 0;
    }

    // this thread's candidate and part: kParts threads per candidate (part 0
    // holds the accumulator)
    const uint32_t cl = tid % kCands, prt = tid / kCands;
    const uint32_t ci = c0 + cl;
    const bool act = ci < cnt;
    typename C::M m;
    m.init(act ? c.p[ci] : (W)C::kIdle);
    if (prt == 0) {
        cand_p[cl] = m.p;
        cand_q[cl] = C::qv(m);
    }

    // bias tiles: A column 0 = 2048, B column 0 = 4096 (fp16), the rest 0
    for (uint32_t r = tid; r < kTcWords + kTcN; r += kTcThreads) {
        const bool isa = r < kTcWords;
        const uint32_t row = isa ? r : r - kTcWords;
        unsigned char *base = sm + (isa ? kOffABias : kOffBBias);
        *reinterpret_cast<uint4 *>(base + tile_off(row, 0, kBiasRowGroup)) =
            make_uint4(isa ? 0x6800u : 0x6C00u, 0, 0, 0);
        *reinterpret_cast<uint4 *>(base + tile_off(row, 1, kBiasRowGroup)) = make_uint4(0, 0, 0, 0);
    }

    // B operand: the candidate's residues w_b = 2^(8b+32) mod p as byte
    // planes, rows kPlanes c .. kPlanes c + kPlanes - 1 (each part writes its
    // share of the 28 groups of 8 bytes, starting from 2^32 256^b0 mod p by
    // square-and-multiply; the plane order is rotated by the candidate so
    // that a warp's stores spread over the banks)
    {
        constexpr uint32_t kChunk = Lay::kChunk;
        const uint32_t k8a = min(prt * kChunk, (uint32_t)(kTcBytes / 8)),
                       k8b = min(k8a + kChunk, (uint32_t)(kTcBytes / 8));
        const W c256 = m.to_mont(256);
        W x = C::two32(m);
        {
            W pw = m.one, base = c256;
            for (uint32_t e = 8 * k8a; e; e >>= 1) {
                if (e & 1) pw = m.mul(pw, base);
                base = m.mul(base, base);
            }
            x = m.mul(x, pw);
        }
        for (uint32_t k8 = k8a; k8 < k8b; ++k8) {
            W w[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                w[j] = x;
                x = m.mul(x, c256);
            }
#pragma unroll
            for (int r = 0; r < kPlanes; ++r) {
                const int pl = (r + (int)cl) % kPlanes;
                uint64_t bytes = 0;
#pragma unroll
                for (int j = 0; j < 8; ++j) bytes |= (uint64_t)((w[j] >> (8 * pl)) & 0xFFu) << (8 * j);
                *reinterpret_cast<uint4 *>(sm + kOffB + tile_off(kPlanes * cl + pl, k8)) = f16x8(bytes);
            }
        }
    }

    // the power-of-R corrections Mont(R^corr) of the programs, on the part(s)
    // that build no byte planes (read by part 0 at the end of each program)
    const int nprog0 = a.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL) ? 2 : 1;
    for (int pi = 0; pi < nprog0; ++pi)
        if (prt == Lay::kBusy + ((uint32_t)pi % (kParts - Lay::kBusy)))
            corr_pow[pi * kCands + cl] = m.mont_R_pow((pi == 0 ? a.a : a.b).corr);

    const uint32_t quad = warp % 4, wgroup = warp / 4;      // TMEM lane quadrant, warp group
    const uint32_t word = quad * 32 + (tid % 32);           // this thread's word of a tile
    // f32 <- f16 x f16, both K-major, N = 256, M = 128
    const uint32_t idesc = (1u << 4) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcWords >> 4) << 24);
    const int nprog = a.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL) ? 2 : 1;

    // tile i of program pi into the A region (one thread), completing on mbar_load
    auto load_tile = [&](int pi, uint32_t i) {
        const TcTiles &tt = pi == 0 ? ta : tb;
        const unsigned char *src = reinterpret_cast<const unsigned char *>(tt.tiles) + (size_t)i * kATile;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar_load)),
                     "r"(kATile)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                smem_u32(sm + kOffA)),
            "l"(src), "r"(kATile), "r"(smem_u32(mbar_load))
            : "memory");
    };
    // the tile's products: per half of the bytes, a bias product and seven
    // K-steps into that half's 256 columns
    auto issue_mma = [&](uint32_t tbase) {
        const uint32_t aaddr = smem_u32(sm + kOffA), baddr = smem_u32(sm + kOffB),
                       abias = smem_u32(sm + kOffABias), bbias = smem_u32(sm + kOffBBias);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint32_t d = tbase + h * kTcN;
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, 0, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                "l"(mdesc(abias, kBiasRowGroup)), "l"(mdesc(bbias, kBiasRowGroup)), "r"(idesc)
                : "memory");
#pragma unroll
            for (int s = 0; s < kTcHalfBytes / 16; ++s) {
                const uint32_t off = (uint32_t)(h * (kTcHalfBytes / 16) + s) * 256;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, 1, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
                    "l"(mdesc(aaddr + off, kRowGroup)), "l"(mdesc(baddr + off, kRowGroup)), "r"(idesc)
                    : "memory");
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(mbar_mma))
                     : "memory");
    };
    // the tile after tile i of program pi, across programs; false at the end
    auto next_tile = [&](int &pi, uint32_t &i, bool started) -> bool {
        for (;;) {
            if (pi >= nprog) return false;
            const uint32_t t = started ? i + 1 : 0;
            if (t < (pi == 0 ? ta : tb).ntiles) {
                i = t;
                return true;
            }
            ++pi;
            started = false;
        }
    };

    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    sync_tc();
    const uint32_t tbase = *taddr_slot;
    const uint32_t taddr = tbase + ((quad * 32u) << 16);    // this warp's TMEM lanes

    uint32_t par_mma = 0, par_load = 0;
    bool failed = false;
    W s0 = 0, s1 = 0;
    W P[kTcChains];          // this part's running products (part 0, chain 0: the accumulator)
#pragma unroll
    for (int k = 0; k < kTcChains; ++k) P[k] = m.one;
    uint32_t g = 0;          // first group of the current program whose squarings are still due
    int fin = 0;             // programs finished

    // the threads' products into part 0's accumulator, a tree over the parts
    // (uniform: every thread calls it)
    auto combine = [&]() {
#pragma unroll
        for (int k = 1; k < kTcChains; ++k) {
            P[0] = C::prod(m, P[0], P[k]);
            P[k] = m.one;
        }
#pragma unroll
        for (uint32_t stride = 1; stride < (uint32_t)kParts; stride <<= 1) {
            part[prt * kCands + cl] = P[0];
            __syncthreads();
            if ((prt & (2 * stride - 1)) == 0) P[0] = C::prod(m, P[0], part[(prt + stride) * kCands + cl]);
            __syncthreads();
        }
        if (prt != 0) P[0] = m.one;
    };
    // end of program pi: remaining squarings, the power-of-R correction,
    // result; the combined search's second program (primorial words)
    // continues from the first's result, so part 0 keeps it
    auto finish = [&](int pi) {
        const Prog<WideWord> &pg = pi == 0 ? a.a : a.b;
        combine();
        if (prt == 0) {
            W acc = P[0];
            for (; g < pg.ngroups; ++g)
                for (uint32_t k = __ldg(pg.groups + 3 * g + 2); k > 0; --k) acc = C::sq(m, acc);
            for (uint32_t k = 0; k < pg.final_sq; ++k) acc = C::sq(m, acc);
            acc = m.mul(acc, corr_pow[pi * kCands + cl]);
            if (nprog == 2 && pi == 0) s1 = acc;
            else s0 = acc;
            P[0] = acc;
        }
        g = 0;
    };

    int cpi = 0;
    uint32_t ci_t = 0;
    bool have = next_tile(cpi, ci_t, false);
    if (have && tid == 0) {
        load_tile(cpi, ci_t);
        if (!mbar_wait(smem_u32(mbar_load), par_load)) *timeout = 1;
        else issue_mma(tbase);
    }
    par_load ^= 1;
    while (have) {
        if (!mbar_wait(smem_u32(mbar_mma), par_mma)) atomicOr(timeout, 1u);
        par_mma ^= 1;
        sync_tc();
        if (*timeout) {
            failed = true;
            break;
        }
        int npi = cpi;
        uint32_t ni_t = ci_t;
        const bool nhave = next_tile(npi, ni_t, true);
        if (nhave && tid == 0) load_tile(npi, ni_t);   // the A region is free: the products are done
        // 1. u = T 2^-32 (mod p) for this thread's word and its warp group's candidates
        constexpr int kPerLoad = 32 / kPlanes;   // candidates per 32-column load
        for (uint32_t cc = wgroup * (kCands / kTcGroups); cc < (wgroup + 1) * (kCands / kTcGroups); cc += kPerLoad) {
            uint32_t v0[32], v1[32];
            ld32(taddr, kPlanes * cc, v0);
            ld32(taddr, kTcN + kPlanes * cc, v1);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < kPerLoad; ++j) {
                // plane sums e_a = D_{a,0} + D_{a,1} - 2^24 < 2^24 (the two bias
                // patterns add to 2 x 0x4B000000 < 2^32)
                uint32_t e[8];
#pragma unroll
                for (int pl = 0; pl < 8; ++pl)
                    e[pl] = pl < kPlanes ? v0[kPlanes * j + pl] + v1[kPlanes * j + pl] - 2u * kBiasBits : 0u;
                // T = L + 2^32 H
                const uint64_t L = (uint64_t)e[0] + ((uint64_t)e[1] << 8) + ((uint64_t)e[2] << 16) +
                                   ((uint64_t)e[3] << 24);
                const uint64_t H = (uint64_t)e[4] + ((uint64_t)e[5] << 8) + ((uint64_t)e[6] << 16) +
                                   ((uint64_t)e[7] << 24);
                const uint32_t cj = cc + j;
                U[cj * kUStride + word] = C::reduce(L, H, cand_p[cj], cand_q[cj]);
            }
        }
        // 2. the next tile's products (TMEM is free once every thread's loads
        //    above are complete; the bulk copy has had step 1 to land)
        sync_tc();
        if (nhave && tid == 0) {
            if (!mbar_wait(smem_u32(mbar_load), par_load)) *timeout = 1;   // seen after the next wait
            else issue_mma(tbase);
        }
        if (nhave) par_load ^= 1;
        while (fin < cpi) finish(fin++);   // programs without words
        // 3. the tile's u into the running products, in segments between the
        //    group starts inside the tile
        {
            const Prog<WideWord> &pg = cpi == 0 ? a.a : a.b;
            uint32_t first, end;
            prog_range(pg, first, end);
            const uint32_t t0 = first + ci_t * kTcWords, t1 = min(t0 + kTcWords, end);
            uint32_t s = t0;
            for (;;) {
                uint32_t k = 0;
                for (; g < pg.ngroups && __ldg(pg.groups + 3 * g) <= s; ++g) k += __ldg(pg.groups + 3 * g + 2);
                // a group start's squarings, applied by every thread to each of
                // its running products: the accumulator is their Montgomery
                // product A = P_0 (x) ... (x) P_{n-1} = (prod P) R^-(n-1), and
                // squaring each, P (x) P = P^2 R^-1, gives (prod P)^2 R^-(2n-1)
                // = A (x) A, so no combining is needed until the program ends
                for (; k > 0; --k) {
#pragma unroll
                    for (int c2 = 0; c2 < kTcChains; ++c2) P[c2] = C::sq(m, P[c2]);
                }
                // the words go to parts 1.. : part 0 is warp 0, whose first
                // thread has just issued the next tile's products (it waits
                // while the tensor pipe takes them) and holds the accumulator
                const uint32_t e = g < pg.ngroups ? min(t1, __ldg(pg.groups + 3 * g)) : t1;
                const uint32_t span = (e - s + kParts - 2) / (kParts - 1);
                const uint32_t lo = prt ? min(s + span * (prt - 1), e) : e, hi = prt ? min(lo + span, e) : e;
                const W *row = U + cl * kUStride + (lo - t0);
                const uint32_t n = hi - lo;
                uint32_t i = 0;
                for (; i + kTcChains <= n; i += kTcChains) {
#pragma unroll
                    for (int k = 0; k < kTcChains; ++k) P[k] = C::prod(m, P[k], row[i + k]);
                }
                for (; i < n; ++i) P[0] = C::prod(m, P[0], row[i]);
                s = e;
                if (s >= t1) break;
            }
        }
        if (!nhave || npi != cpi) finish(fin++);
        cpi = npi;
        ci_t = ni_t;
        have = nhave;
    }
    if (!failed)
        while (fin < nprog) finish(fin++);

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

size_t tc_tile_bytes() { return kATile; }
uint32_t tc_tile_words() { return kTcWords; }

int launch_tc_pack(const WideWord *words, const uint32_t *src, uint32_t nw, uint32_t ntiles, void *out,
                   cudaStream_t st) {
    if (!ntiles) return 0;
    const uint32_t n = ntiles * kTcWords;
    tc_pack_kernel<<<(n + 127) / 128, 128, 0, st>>>(words, src, nw, ntiles, reinterpret_cast<uint4 *>(out));
    return 1;
}

// One CTA of 512 threads per 32 (class 64) or 64 (class 32) candidates, one
// CTA per SM (shared memory); blocks [block0, block0 + nblocks) of the class
// buffer (nblocks 0: to the end).
uint32_t tc_setup_blocks(uint32_t cands) { return (cands + TcLayout<Cls64L>::kCands - 1) / TcLayout<Cls64L>::kCands; }
uint32_t tc_setup_blocks32(uint32_t cands) { return (cands + TcLayout<Cls32>::kCands - 1) / TcLayout<Cls32>::kCands; }

template <class T>
static int launch_tc(const ClassBuf<typename TcClass<T>::W> &c, const SetupArgs<WideWord> &a, const TcTiles &ta,
                     const TcTiles &tb, uint32_t *flags, cudaStream_t st, uint32_t block0, uint32_t nblocks) {
    if (!c.cap) return 0;
    constexpr int kCands = TcLayout<T>::kCands;
    const uint32_t all = (c.cap + kCands - 1) / kCands;
    if (block0 >= all) return 0;
    if (nblocks == 0 || nblocks > all - block0) nblocks = all - block0;
    static bool configured[64] = {false};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (!configured[dev]) {
        if (cudaFuncSetAttribute(setup_tc_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)TcLayout<T>::kSmemBytes) != cudaSuccess)
            return 0;
        configured[dev] = true;
    }
    setup_tc_kernel<T><<<nblocks, kTcThreads, TcLayout<T>::kSmemBytes, st>>>(c, a, ta, tb, flags, block0);
    return 1;
}

int launch_setup64w_tc(const ClassBuf<uint64_t> &c, const SetupArgs<WideWord> &a, const TcTiles &ta,
                       const TcTiles &tb, uint32_t *flags, cudaStream_t st, uint32_t block0, uint32_t nblocks) {
    return launch_tc<Cls64L>(c, a, ta, tb, flags, st, block0, nblocks);
}

int launch_setup32_tc(const ClassBuf<uint32_t> &c, const SetupArgs<WideWord> &a, const TcTiles &ta,
                      const TcTiles &tb, uint32_t *flags, cudaStream_t st, uint32_t block0, uint32_t nblocks) {
    return launch_tc<Cls32>(c, a, ta, tb, flags, st, block0, nblocks);
}

}  // namespace pfc
