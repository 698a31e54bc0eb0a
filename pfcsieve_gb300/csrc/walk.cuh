// walk.cuh -- the walk machinery shared by the per-job kernels (sieve.cu)
// and the batch kernel (batch.cu): size-class traits, hit appends,
// multiplier loads, the per-block walk and its replay.
//
// Drift walk.  The reference keeps r and n both in Montgomery form and spends
// an add-mod per n to advance Mont(n) (iterate.cl:73-74).  Here the
// multiplier is the plain integer n (or the prime q for n#), and each step is
// one reduction s <- s*n*R^-1.  Starting a block of B steps from s = r*R, after
// j+1 steps s = r_{j+1} * R^-j, so r_{j+1} = +-1 exactly when s equals
// T[j] = R^-j mod p or p - T[j].  The B targets are per-thread registers
// computed once per launch; one multiplication by K = R^(B+1) returns s to
// Montgomery form at the end of the block.  Hits are rare, so a block only
// ORs its comparisons into one predicate; if any lane of the warp saw a hit
// the warp replays that block from its saved start with per-step recording.
//
// Single-chain searches walk NC candidates per thread.  The combined search
// (-! -c) walks the factorial and the compositorial chain of one candidate
// together (fused: shared targets, counter and loop); both take their
// multipliers from a per-chunk table, n for the factorial and, for the
// compositorial, n at composite n and 1 at prime n (the reference skips prime
// n, iterate.cl:137-140, 181-184): multiplying by 1 keeps the drift at one
// power of R per step, and the replay skips the test where the multiplier is
// 1.  The fast path tests every step: at a prime n the compositorial value is
// the previous step's, so an unmasked match there only repeats a hit already
// seen and costs one replay, never a wrong record.  The per-step work of a
// class-32 chain is three integer multiplies (two 32x32->64, one low), one
// subtract, and an absolute value and two compares for the hit test.
#pragma once
#include <type_traits>
#include "arith.cuh"
#include "kernels.cuh"

namespace pfc {

constexpr unsigned kFull = 0xffffffffu;

// Size-class traits.  Each class supplies: the fast step and its hit filter
// (a superset test: every true hit passes, rare false alarms are dropped by
// the exact replay), the targets of the drift walk, the restore constant for
// r fast steps, the exact canonical step used by the replay, and the setup
// and checksum helpers.

struct Cls32 {
    using W = uint32_t;
    using M = Mont32;
    static constexpr int B = 16;          // block length with two candidates per thread
    static constexpr int B_FUSED = 16;    // block length of the fused -! -c walk
    static constexpr int NC = 2;          // candidates per thread in single-chain walks
    // targets: one register per step (p - T formed in the test) for the
    // two-candidate walks, which are register-bound; two for the fused walk,
    // which is issue-bound and saves the add
    struct TgtA {
        W t;
    };
    struct TgtB {
        W t, nt;
    };
    template <bool FUSED>
    using Tgt = typename std::conditional<FUSED, TgtB, TgtA>::type;
    // walk residues signed in (-p, p), p < 2^31; after j+1 steps from r*R,
    // x = r' * R^-j, so the targets are T_j = R^-j
    __device__ static __forceinline__ W target0(const M &) { return 1; }
    __device__ static __forceinline__ W next_target(const M &m, W t) { return m.mul(t, 1); }
    __device__ static __forceinline__ void mk(const M &, W t, TgtA &g) { g.t = t; }
    __device__ static __forceinline__ void mk(const M &m, W t, TgtB &g) {
        g.t = t;
        g.nt = m.p - t;
    }
    __device__ static __forceinline__ W fstep(const M &m, W x, uint32_t n) {
        return (W)redc31s((int32_t)x, n, (int32_t)m.p, m.pinv);
    }
    // x = +-T (mod p) <=> |x| in {T, p - T} <=> |x| == T or |x| + T == p
    __device__ static __forceinline__ bool fhit(const M &m, W x, const TgtA &g) {
        const uint32_t ax = (uint32_t)abs((int32_t)x);
        return (ax == g.t) | (ax + g.t == m.p);
    }
    __device__ static __forceinline__ bool fhit(const M &, W x, const TgtB &g) {
        const uint32_t ax = (uint32_t)abs((int32_t)x);
        return (ax == g.t) | (ax == g.nt);
    }
    // r fast steps leave r' * R^(1-r): multiply by K = R^(r+1) (and R^-1)
    __device__ static __forceinline__ W K(const M &m, int r) { return m.mont_R_pow((uint64_t)r); }
    __device__ static __forceinline__ W restore(const M &m, W x, W K) { return fstep(m, x, K); }
    __device__ static __forceinline__ W canon(const M &m, W x) { return (int32_t)x < 0 ? x + m.p : x; }
    __device__ static __forceinline__ W step(const M &m, W s, uint32_t n) { return redc32(s, n, m.p, m.pinv); }
    // setup: 896-bit table words Z = sum z_i 2^(28 i) (limbs z_i < 2^28) and
    // squarings, canonical residues.  Per candidate the residues
    // w_i = 2^(28 i + 32) mod p < 2^31 are kept in registers; a word is folded
    // as T = sum z_i w_i = Z 2^32 (mod p), one wide multiply-add per limb
    // (each term < 2^59: all 32 in one 64-bit accumulator), then
    // s <- s T 2^-64 = s Z R^-1 by two Montgomery rounds on the 32-bit halves
    // of T.  Each word lowers the power of R = 2^32 by one.
    using SW = WideWord;
    struct SC {
        uint32_t w[kWideLimbs];
    };
    __device__ static __forceinline__ SC sctx(const M &m) {
        SC c;
        const uint32_t k60 = m.mul(m.r2, 1u << kWideRadixBits);   // 2^60 mod p
        uint32_t x = m.one;                                         // 2^32 mod p
#pragma unroll
        for (int i = 0; i < kWideLimbs; ++i) {
            c.w[i] = x;
            x = m.mul(x, k60);                                      // x 2^28
        }
        return c;
    }
    // s < p: both rounds stay below 2^64 (s t < 2^63, m p < 2^63) and the
    // result is below 2p before the conditional subtraction
    // SMEM: the word is read from shared memory (a staged copy) instead of
    // through the read-only global path
    template <bool SMEM = false>
    __device__ static __forceinline__ W word(const M &m, const SC &c, W s, const SW *wp) {
        const uint4 *v = reinterpret_cast<const uint4 *>(wp);
        uint64_t t = 0;
#pragma unroll
        for (int k = 0; k < kWideLimbs / 4; ++k) {
            const uint4 z = SMEM ? v[k] : __ldg(v + k);
            t += (uint64_t)z.x * c.w[4 * k];
            t += (uint64_t)z.y * c.w[4 * k + 1];
            t += (uint64_t)z.z * c.w[4 * k + 2];
            t += (uint64_t)z.w * c.w[4 * k + 3];
        }
        const uint32_t q = 0u - m.pinv;
        const uint64_t a = (uint64_t)s * (uint32_t)t;
        const uint64_t b = (a + (uint64_t)((uint32_t)a * q) * m.p) >> 32;
        const uint64_t d = b + (uint64_t)s * (uint32_t)(t >> 32);
        const uint32_t r = (uint32_t)((d + (uint64_t)((uint32_t)d * q) * m.p) >> 32);
        return r >= m.p ? r - m.p : r;
    }
    __device__ static __forceinline__ W sq(const M &m, W s) { return m.mul(s, s); }
    // checksum form: residue * 2^64 mod p from its class-32 Montgomery form
    __device__ static __forceinline__ uint64_t term(const M &m, W s) { return m.mul(s, m.r2); }
    __device__ static __forceinline__ uint64_t mont64_of(const M &m, uint32_t v) { return m.mul(m.mul(v, m.r2), m.r2); }
};

// p >= 2^31, canonical residues, R = 2^64 (any p < 2^64)
struct Cls64 {
    using W = uint64_t;
    using M = Mont64;
    static constexpr int B = 8;
    static constexpr int B_FUSED = 8;
    static constexpr int NC = 1;
    struct TgtB {
        W t, nt;
    };
    template <bool FUSED>
    using Tgt = TgtB;
    __device__ static __forceinline__ W target0(const M &) { return 1; }
    __device__ static __forceinline__ W next_target(const M &m, W t) { return m.mul(t, 1); }
    __device__ static __forceinline__ void mk(const M &m, W t, TgtB &g) {
        g.t = t;
        g.nt = m.p - t;
    }
    __device__ static __forceinline__ W fstep(const M &m, W x, uint32_t n) { return redc64_u32(x, n, m.p, m.pinv); }
    __device__ static __forceinline__ bool fhit(const M &, W x, const TgtB &g) { return (x == g.t) | (x == g.nt); }
    __device__ static __forceinline__ W K(const M &m, int r) { return m.mont_R_pow((uint64_t)r); }
    __device__ static __forceinline__ W restore(const M &m, W x, W K) { return m.mul(x, K); }
    __device__ static __forceinline__ W canon(const M &, W x) { return x; }
    __device__ static __forceinline__ W step(const M &m, W s, uint32_t n) { return redc64_u32(s, n, m.p, m.pinv); }
    using SW = uint64_t;
    struct SC {};
    __device__ static __forceinline__ SC sctx(const M &) { return {}; }
    __device__ static __forceinline__ W word(const M &m, const SC &, W s, SW w) { return redc64(s, w, m.p, m.pinv); }
    __device__ static __forceinline__ W sq(const M &m, W s) { return m.mul(s, s); }
    __device__ static __forceinline__ uint64_t term(const M &, W s) { return s; }
    __device__ static __forceinline__ uint64_t mont64_of(const M &m, uint32_t v) { return m.to_mont(v); }
};

// 2^31 < p < 2^64/3: the walk takes lazy one-word steps (R' = 2^32, residues in
// [0, 2p), redc64l) from the R = 2^64 setup values.  After j+1 steps from
// r*2^64, x = r' * 2^64 * 2^(-32(j+1)) (mod p), so the targets are
// U_j = 2^(32-32j) mod p; x = +-U (mod p) with x in [0, 2p) means x is one of
// U, U + p, p - U, 2p - U, and the fast filter compares the low 32 bits of x
// with those four (a false alarm costs one replay).
struct Cls64L {
    using W = uint64_t;
    using M = Mont64;
    static constexpr int B = 16;
    static constexpr int B_FUSED = 16;
    static constexpr int NC = 1;
    struct TgtA {
        uint32_t u;  // low 32 bits of U; the four lifts are formed in the test
    };
    template <bool FUSED>
    using Tgt = TgtA;
    __device__ static __forceinline__ W canon(const M &m, W x) { return x >= m.p ? x - m.p : x; }
    __device__ static __forceinline__ W target0(const M &m) { return canon(m, redc64l(m.one, 1u, m.p, m.q32)); }
    __device__ static __forceinline__ W next_target(const M &m, W t) { return canon(m, redc64l(t, 1u, m.p, m.q32)); }
    __device__ static __forceinline__ void mk(const M &, W t, TgtA &g) { g.u = (uint32_t)t; }
    __device__ static __forceinline__ W fstep(const M &m, W x, uint32_t n) { return redc64l(x, n, m.p, m.q32); }
    // low words: x in {U, U + p} <=> lo(x) - lo(U) in {0, lo(p)};
    //            x in {p - U, 2p - U} <=> lo(x) + lo(U) in {lo(p), lo(2p)}
    __device__ static __forceinline__ bool fhit(const M &m, W x, const TgtA &g) {
        const uint32_t lo = (uint32_t)x, pl = (uint32_t)m.p;
        const uint32_t d = lo - g.u, e = lo + g.u;
        return (d == 0u) | (d == pl) | (e == pl) | (e == 2u * pl);
    }
    // r lazy steps leave r' * 2^64 * 2^(-32r): K = 2^(32r) * 2^64 mod p, the
    // Montgomery form of 2^(32r), from Mont(2^(64k)) = mont_R_pow(k)
    __device__ static __forceinline__ W K(const M &m, int r) {
        const W k = m.mont_R_pow((uint64_t)((r + 1) >> 1));
        return (r & 1) ? canon(m, redc64l(k, 1u, m.p, m.q32)) : k;
    }
    // x*K*2^-64 by two lazy one-limb rounds (x < 2p, any K < 2^64, 3p < 2^64),
    // back to [0, 2p) by one conditional subtraction
    __device__ static __forceinline__ W restore(const M &m, W x, W K) {
        uint64_t c = redc64l(x, (uint32_t)K, m.p, m.q32);
        c = cios_round(c, x, (uint32_t)(K >> 32), m.p, m.q32);
        return c >= 2 * m.p ? c - m.p : c;
    }
    __device__ static __forceinline__ W step(const M &m, W s, uint32_t n) { return canon(m, redc64l(s, n, m.p, m.q32)); }
    // setup (p < 2^64/3): 896-bit table words Z = sum z_i 2^(28 i) (limbs
    // z_i < 2^28).  Per candidate the residues w_i = 2^(28 i + 32) mod p
    // (canonical) are kept in registers; a word is folded into 96 bits as
    // T = sum z_i w_i = Z 2^32 (mod p) with one wide multiply-add per limb and
    // 32-bit half (z_i lo(w_i) < 2^60: sixteen terms per 64-bit accumulator;
    // z_i hi(w_i) < 2^58.5: all 32 in one), then s <- s T 2^-96 = s Z R^-1 by
    // three lazy rounds.  Each word lowers the power of R = 2^64 by one;
    // values stay in [0, 2p), canonical before a squaring.
    using SW = WideWord;
    struct SC {
        uint64_t w[kWideLimbs];
    };
    // from the top: w_31 = 2^900 = Mont(2^(64*14)) 2^-32 2^-28, then
    // w_i = w_(i+1) 2^-28 = redc(w_(i+1) * 16), one lazy round each
    static_assert(kWideRadixBits == 28 && kWideLimbs % 16 == 0, "2^(28(L-1)+92) must be a power of R");
    __device__ static __forceinline__ SC sctx(const M &m) {
        SC c;
        constexpr uint64_t kTop = (28ull * (kWideLimbs - 1) + 92) / 64 - 1;
        uint64_t x = redc64l(m.mont_R_pow(kTop), 1u, m.p, m.q32);
#pragma unroll
        for (int i = kWideLimbs - 1; i >= 0; --i) {
            x = canon(m, redc64l(x, 16u, m.p, m.q32));
            c.w[i] = x;
        }
        return c;
    }
    template <bool SMEM = false>
    __device__ static __forceinline__ W word(const M &m, const SC &c, W s, const SW *wp) {
        const uint4 *v = reinterpret_cast<const uint4 *>(wp);
        uint64_t u0 = 0, u1 = 0, hv = 0;
#pragma unroll
        for (int k = 0; k < kWideLimbs / 4; ++k) {
            const uint4 z4 = SMEM ? v[k] : __ldg(v + k);
            const uint32_t z[4] = {z4.x, z4.y, z4.z, z4.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int i = 4 * k + j;
                const uint64_t lo = (uint64_t)z[j] * (uint32_t)c.w[i];
                if (i < kWideLimbs / 2) u0 += lo;
                else u1 += lo;
                hv += (uint64_t)z[j] * (uint32_t)(c.w[i] >> 32);
            }
        }
        // T = u0 + u1 + hv 2^32 < 2^96 as three 32-bit limbs
        const uint64_t u = u0 + u1;
        const uint64_t mid = (u >> 32) + ((uint64_t)(u < u0) << 32) + hv;
        const uint32_t t[3] = {(uint32_t)u, (uint32_t)mid, (uint32_t)(mid >> 32)};
        return mul_wide_word<3>(s, t, m.p, m.q32);
    }
    __device__ static __forceinline__ W sq(const M &m, W s) {
        s = canon(m, s);
        return m.mul(s, s);
    }
    __device__ static __forceinline__ uint64_t term(const M &, W s) { return s; }
    __device__ static __forceinline__ uint64_t mont64_of(const M &m, uint32_t v) { return m.to_mont(v); }
};

template <class W>
__device__ __forceinline__ W ldg(const W *p) { return __ldg(p); }

// Evaluate a setup program from Montgomery-form `acc` (see kernels.cuh Prog).
// Wide words are staged through shared memory by the whole CTA (every thread
// of the CTA must call this with the same program); narrow ones are loaded
// four at a time.
template <class T>
__device__ typename T::W run_prog(const typename T::M &m, const typename T::SC &sc, const Prog<typename T::SW> &pg,
                                  typename T::W acc) {
    for (uint32_t g = 0; g < pg.ngroups; ++g) {
        const uint32_t b = __ldg(pg.groups + 3 * g), e = __ldg(pg.groups + 3 * g + 1);
        const uint32_t sq = __ldg(pg.groups + 3 * g + 2);
        for (uint32_t k = 0; k < sq; ++k) acc = T::sq(m, acc);
        uint32_t i = b;
        if constexpr (std::is_same<typename T::SW, WideWord>::value) {
            // every thread of the CTA runs the same program: the CTA copies
            // kStageWords words at a time into shared memory with one coalesced
            // load and the threads read the limbs there (all threads of the
            // CTA must call run_prog; trip counts are uniform)
            constexpr uint32_t kStageWords = 16, kVec = sizeof(WideWord) / 16;
            __shared__ uint4 stage[kStageWords * kVec];
            const uint4 *src = reinterpret_cast<const uint4 *>(pg.words);
            for (; i < e; i += kStageWords) {
                const uint32_t nw = min(kStageWords, e - i);
                __syncthreads();
                for (uint32_t j = threadIdx.x; j < nw * kVec; j += blockDim.x)
                    stage[j] = __ldg(src + (size_t)i * kVec + j);
                __syncthreads();
                for (uint32_t u = 0; u < nw; ++u)
                    acc = T::template word<true>(m, sc, acc, reinterpret_cast<const WideWord *>(stage + u * kVec));
            }
        } else {
            for (; i + 4 <= e; i += 4) {
                acc = T::word(m, sc, acc, ldg(pg.words + i));
                acc = T::word(m, sc, acc, ldg(pg.words + i + 1));
                acc = T::word(m, sc, acc, ldg(pg.words + i + 2));
                acc = T::word(m, sc, acc, ldg(pg.words + i + 3));
            }
            for (; i < e; ++i) acc = T::word(m, sc, acc, ldg(pg.words + i));
        }
    }
    for (uint32_t k = 0; k < pg.final_sq; ++k) acc = T::sq(m, acc);
    return m.mul(acc, m.mont_R_pow(pg.corr));
}

// warp-aggregated bounded append of one hit per lane (all 32 lanes call it);
// batches also record the job of each hit in h.tag
__device__ __forceinline__ void append_hit(bool hit, uint64_t p, int32_t nc, int32_t type, const HitBuf &h) {
    const unsigned msk = __ballot_sync(kFull, hit);
    if (!msk) return;
    const unsigned lane = threadIdx.x & 31;
    const int leader = __ffs(msk) - 1;
    unsigned long long base = 0;
    if ((int)lane == leader) base = atomicAdd(h.count, (unsigned long long)__popc(msk));
    base = __shfl_sync(kFull, base, leader);
    if (hit) {
        const unsigned long long idx = base + __popc(msk & ((1u << lane) - 1u));
        if (idx < h.cap) {
            pfc_factor f;
            f.p = p;
            f.nc = nc;
            f.type = type;
            h.buf[idx] = f;
            if (h.tag) h.tag[idx] = h.tagval;
        }
    }
}

// Multipliers of steps k .. k+B-1 (uniform across the warp): k itself when
// `mult` is null, else mult[k - base ...] (vector loads when aligned).
template <int B>
__device__ __forceinline__ void load_mult(const uint32_t *mult, uint32_t base, uint32_t k, bool vec, uint32_t (&mv)[B]) {
    if (!mult) {
#pragma unroll
        for (int j = 0; j < B; ++j) mv[j] = k + j;
    } else if (vec) {
        const uint4 *src = reinterpret_cast<const uint4 *>(mult + (k - base));
#pragma unroll
        for (int j = 0; j < B / 4; ++j) {
            const uint4 v = __ldg(src + j);
            mv[4 * j] = v.x;
            mv[4 * j + 1] = v.y;
            mv[4 * j + 2] = v.z;
            mv[4 * j + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < B; ++j) mv[j] = __ldg(mult + (k - base) + j);
    }
}

// Replay `len` steps of one chain from the block start x with the exact
// per-step test and record the hits.  A multiplier of 1 marks a prime n of
// the compositorial walk: nothing was multiplied there, so nothing is tested.
template <class T>
__device__ __noinline__ void replay_chain(const typename T::M m, typename T::W x, const uint32_t *mult,
                                          uint32_t base, uint32_t k, int len, int32_t type, bool active,
                                          const HitBuf h) {
    using W = typename T::W;
    x = T::canon(m, x);
    W t = T::target0(m);
    for (int j = 0; j < len; ++j) {
        if (j) t = T::next_target(m, t);
        const uint32_t mul = mult ? __ldg(mult + (k - base) + j) : k + j;
        x = T::step(m, x, mul);
        const bool hit = active && mul != 1u && (x == t || x == m.p - t);
        append_hit(hit, m.p, x == t ? -(int32_t)mul : (int32_t)mul, type, h);
    }
}

// Walk steps [a.lo, a.hi) of the streams of one thread.  Each thread runs
// two independent streams of steps so that the scheduler always has a second
// dependent chain to interleave:
//   FUSED (-! -c): the factorial chain (multiplier n) and the compositorial
//     chain (multiplier table a.mult2) of one candidate, sharing its targets;
//   otherwise NC candidates (1 or 2) on the same multiplier sequence.
// x holds canonical Montgomery-form residues on entry and on exit.  Inactive
// streams hold 0, which never matches a target (targets are nonzero mod p),
// so they never trigger a replay.
template <class T, int NC, bool FUSED, int B = (FUSED ? T::B_FUSED : T::B)>
__device__ __forceinline__ void walk_streams(const typename T::M (&m)[NC], typename T::W (&x)[FUSED ? 2 : NC],
                                             const bool (&act)[NC], const WalkArgs &a, const HitBuf &h) {
    using W = typename T::W;
    constexpr int NS = FUSED ? 2 : NC;
    typename T::template Tgt<FUSED> tg[NC][B];
    W K[NC];
#pragma unroll
    for (int s = 0; s < NC; ++s) {
        W t = T::target0(m[s]);
#pragma unroll
        for (int j = 0; j < B; ++j) {
            T::mk(m[s], t, tg[s][j]);
            if (j + 1 < B) t = T::next_target(m[s], t);
        }
        K[s] = T::K(m[s], B);
    }

    const uint32_t *mult0 = a.mult;   // fused: the factorial's n from a table, or computed when null
    const uint32_t *mult1 = a.mult2;
    const bool vec = ((a.lo - a.base) & 3u) == 0;
    uint32_t k = a.lo;
    const uint32_t nblk = (a.hi - a.lo) / B;
    for (uint32_t b = 0; b < nblk; ++b, k += B) {
        uint32_t mv[B], cv[B];
        load_mult<B>(mult0, a.base, k, vec, mv);
        if (FUSED) load_mult<B>(mult1, a.base, k, vec, cv);
        W xs[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) xs[s] = x[s];
        bool any = false;
#pragma unroll
        for (int j = 0; j < B; ++j) {
            if (FUSED) {
                x[0] = T::fstep(m[0], x[0], mv[j]);
                x[NS - 1] = T::fstep(m[0], x[NS - 1], cv[j]);
                any |= T::fhit(m[0], x[0], tg[0][j]) | T::fhit(m[0], x[NS - 1], tg[0][j]);
            } else {
#pragma unroll
                for (int s = 0; s < NC; ++s) {
                    x[s] = T::fstep(m[s], x[s], mv[j]);
                    any |= T::fhit(m[s], x[s], tg[s][j]);
                }
            }
        }
        if (__any_sync(kFull, any)) {
            if (FUSED) {
                replay_chain<T>(m[0], xs[0], mult0, a.base, k, B, a.type, act[0], h);
                replay_chain<T>(m[0], xs[NS - 1], mult1, a.base, k, B, a.type2, act[0], h);
            } else {
#pragma unroll
                for (int s = 0; s < NC; ++s) replay_chain<T>(m[s], xs[s], mult0, a.base, k, B, a.type, act[s], h);
            }
        }
        // back to Montgomery form
        if (FUSED) {
            x[0] = T::restore(m[0], x[0], K[0]);
            x[NS - 1] = T::restore(m[0], x[NS - 1], K[0]);
        } else {
#pragma unroll
            for (int s = 0; s < NC; ++s) x[s] = T::restore(m[s], x[s], K[s]);
        }
    }

    const int r = (int)(a.hi - k);
    if (r > 0) {  // tail of fewer than B steps, same filter and replay
        W xs[NS];
#pragma unroll
        for (int s = 0; s < NS; ++s) xs[s] = x[s];
        bool any = false;
#pragma unroll
        for (int j = 0; j < B; ++j) {
            if (j < r) {
                const uint32_t mul0 = mult0 ? __ldg(mult0 + (k - a.base) + j) : k + j;
                if (FUSED) {
                    const uint32_t mul1 = __ldg(mult1 + (k - a.base) + j);
                    x[0] = T::fstep(m[0], x[0], mul0);
                    x[NS - 1] = T::fstep(m[0], x[NS - 1], mul1);
                    any |= T::fhit(m[0], x[0], tg[0][j]) | T::fhit(m[0], x[NS - 1], tg[0][j]);
                } else {
#pragma unroll
                    for (int s = 0; s < NC; ++s) {
                        x[s] = T::fstep(m[s], x[s], mul0);
                        any |= T::fhit(m[s], x[s], tg[s][j]);
                    }
                }
            }
        }
        if (__any_sync(kFull, any)) {
            if (FUSED) {
                replay_chain<T>(m[0], xs[0], mult0, a.base, k, r, a.type, act[0], h);
                replay_chain<T>(m[0], xs[NS - 1], mult1, a.base, k, r, a.type2, act[0], h);
            } else {
#pragma unroll
                for (int s = 0; s < NC; ++s) replay_chain<T>(m[s], xs[s], mult0, a.base, k, r, a.type, act[s], h);
            }
        }
#pragma unroll
        for (int s = 0; s < NC; ++s) {
            const W Kr = T::K(m[s], r);
            if (FUSED) {
                x[0] = T::restore(m[0], x[0], Kr);
                x[NS - 1] = T::restore(m[0], x[NS - 1], Kr);
            } else {
                x[s] = T::restore(m[s], x[s], Kr);
            }
        }
    }

    // canonical form for the state store and the check
    if (FUSED) {
        x[0] = T::canon(m[0], x[0]);
        x[NS - 1] = T::canon(m[0], x[NS - 1]);
    } else {
#pragma unroll
        for (int s = 0; s < NC; ++s) x[s] = T::canon(m[s], x[s]);
    }
}

}  // namespace pfc
