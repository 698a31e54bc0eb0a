// sieve.cu -- setup, iterate and check kernels (replace kernels/setup.cl,
// kernels/iterate.cl and kernels/check.cl).
//
// One thread owns one candidate prime p for the whole n range; its residues
// live in registers between the loads at launch start and the stores at
// launch end.  Two size classes (arith.cuh): class 32 (p < 2^32, R = 2^32)
// and class 64 (R = 2^64).
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
// Each launch walks one residue chain.  The combined search (-! -c) walks the
// factorial chain over n and then the compositorial chain over a multiplier
// table holding n at composite n and 1 at prime n (the reference skips prime
// n, iterate.cl:137-140, 181-184): multiplying by 1 keeps the drift at one
// power of R per step, and the replay skips the test where the multiplier is
// 1.  The fast path tests every step: at a prime n the compositorial value is
// the previous step's, so an unmasked match there only repeats a hit already
// seen and costs one replay, never a wrong record.  The per-step work is three
// integer multiplies (IMAD.WIDE, IMAD, IMAD.HI), one compare and conditional
// add for the reduction, and two compares for the hit test.
#include "arith.cuh"
#include "kernels.cuh"

namespace pfc {

constexpr unsigned kFull = 0xffffffffu;

struct Cls32 {
    using W = uint32_t;
    using M = Mont32;
    static constexpr int B = 8;           // block length with two candidates per thread
    static constexpr int B_FUSED = 16;    // block length of the fused -! -c walk
    static constexpr int NC = 2;          // candidates per thread in single-chain walks
    static constexpr bool kSigned = true; // walk residues signed in (-p, p), p < 2^31
    // fast walk step and its hit test: x = +-T (mod p) <=> |x| in {T, p - T}
    __device__ static __forceinline__ W fstep(const M &m, W x, uint32_t n) {
        return (W)redc31s((int32_t)x, n, (int32_t)m.p, m.pinv);
    }
    __device__ static __forceinline__ bool fhit(W x, W t, W nt) {
        const uint32_t ax = (uint32_t)abs((int32_t)x);
        return (ax == t) | (ax == nt);
    }
    __device__ static __forceinline__ W canon(const M &m, W x) { return (int32_t)x < 0 ? x + m.p : x; }
    // x*K*R^-1 for the block restore (K < p < 2^31)
    __device__ static __forceinline__ W restore(const M &m, W x, W K) { return fstep(m, x, K); }
    __device__ static __forceinline__ W step(const M &m, W s, uint32_t n) { return redc32(s, n, m.p, m.pinv); }
    __device__ static __forceinline__ W word(const M &m, W s, W w) { return redc32(s, w, m.p, m.pinv); }
    // checksum form: residue * 2^64 mod p from its class-32 Montgomery form
    __device__ static __forceinline__ uint64_t term(const M &m, W s) { return m.mul(s, m.r2); }
    __device__ static __forceinline__ uint64_t mont64_of(const M &m, uint32_t v) { return m.mul(m.mul(v, m.r2), m.r2); }
};

struct Cls64 {
    using W = uint64_t;
    using M = Mont64;
    static constexpr int B = 8;
    static constexpr int B_FUSED = 8;
    static constexpr int NC = 1;
    static constexpr bool kSigned = false;
    __device__ static __forceinline__ W fstep(const M &m, W x, uint32_t n) { return redc64_u32(x, n, m.p, m.pinv); }
    __device__ static __forceinline__ bool fhit(W x, W t, W nt) { return (x == t) | (x == nt); }
    __device__ static __forceinline__ W canon(const M &, W x) { return x; }
    __device__ static __forceinline__ W restore(const M &m, W x, W K) { return m.mul(x, K); }
    __device__ static __forceinline__ W step(const M &m, W s, uint32_t n) { return redc64_u32(s, n, m.p, m.pinv); }
    __device__ static __forceinline__ W word(const M &m, W s, W w) { return redc64(s, w, m.p, m.pinv); }
    __device__ static __forceinline__ uint64_t term(const M &, W s) { return s; }
    __device__ static __forceinline__ uint64_t mont64_of(const M &m, uint32_t v) { return m.to_mont(v); }
};

template <class W>
__device__ __forceinline__ W ldg(const W *p) { return __ldg(p); }

// --------------------------------------------------------------------- setup

// Evaluate a setup program from Montgomery-form `acc` (see kernels.cuh Prog).
template <class T>
__device__ typename T::W run_prog(const typename T::M &m, const Prog<typename T::W> &pg, typename T::W acc) {
    for (uint32_t g = 0; g < pg.ngroups; ++g) {
        const uint32_t b = __ldg(pg.groups + 3 * g), e = __ldg(pg.groups + 3 * g + 1);
        const uint32_t sq = __ldg(pg.groups + 3 * g + 2);
        for (uint32_t k = 0; k < sq; ++k) acc = m.mul(acc, acc);
        uint32_t i = b;
        for (; i + 4 <= e; i += 4) {
            acc = T::word(m, acc, ldg(pg.words + i));
            acc = T::word(m, acc, ldg(pg.words + i + 1));
            acc = T::word(m, acc, ldg(pg.words + i + 2));
            acc = T::word(m, acc, ldg(pg.words + i + 3));
        }
        for (; i < e; ++i) acc = T::word(m, acc, ldg(pg.words + i));
    }
    for (uint32_t k = 0; k < pg.final_sq; ++k) acc = m.mul(acc, acc);
    return m.mul(acc, m.mont_R_pow(pg.corr));
}

template <class T>
__global__ void __launch_bounds__(256) setup_kernel(ClassBuf<typename T::W> c, SetupArgs<typename T::W> a) {
    using W = typename T::W;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t cnt = min(*c.count, c.cap);
    if (i >= cnt) return;
    typename T::M m;
    m.init(c.p[i]);
    W s0, s1 = 0;
    if (a.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL)) {
        s1 = run_prog<T>(m, a.a, m.one);      // (n-1)!/(n-1)#
        s0 = run_prog<T>(m, a.b, s1);         // (n-1)! = that * (n-1)#
    } else {
        s0 = run_prog<T>(m, a.a, m.one);
    }
    c.s0[i] = s0;
    c.s1[i] = s1;
    c.nnext[i] = a.nnext0;
}

// ------------------------------------------------------------------- iterate

// warp-aggregated bounded append of one hit per lane (all 32 lanes call it)
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
    W t = 1;
    for (int j = 0; j < len; ++j) {
        if (j) t = m.mul(t, 1);
        const uint32_t mul = mult ? __ldg(mult + (k - base) + j) : k + j;
        x = T::step(m, x, mul);
        const bool hit = active && mul != 1u && (x == t || x == m.p - t);
        append_hit(hit, m.p, x == t ? -(int32_t)mul : (int32_t)mul, type, h);
    }
}

// One walk launch.  Each thread runs two independent streams of steps so
// that the scheduler always has a second dependent chain to interleave:
//   FUSED (-! -c): the factorial chain (multiplier n) and the compositorial
//     chain (multiplier table) of one candidate, sharing its targets;
//   otherwise NC candidates (1 or 2) on the same multiplier sequence.
// Inactive streams hold 0, which never matches a target (targets are in
// [1, p-1]), so they never trigger a replay.
template <class T, int NC, bool FUSED>
__global__ void __launch_bounds__(256) walk_kernel(ClassBuf<typename T::W> c, WalkArgs a, HitBuf h) {
    using W = typename T::W;
    constexpr int B = FUSED ? T::B_FUSED : T::B;
    constexpr int NS = FUSED ? 2 : NC;   // streams per thread
    const uint32_t cnt = min(*c.count, c.cap);
    const uint32_t blk0 = blockIdx.x * blockDim.x * NC;
    if (blk0 >= cnt) return;  // whole block idle

    uint32_t idx[NC];
    bool act[NC];
    typename T::M m[NC];
    W x[NS];
#pragma unroll
    for (int s = 0; s < NC; ++s) {
        idx[s] = blk0 + s * blockDim.x + threadIdx.x;
        act[s] = idx[s] < cnt;
        m[s].init(act[s] ? c.p[idx[s]] : (W)3);
    }
    if (FUSED) {
        x[0] = act[0] ? c.s0[idx[0]] : 0;
        x[NS - 1] = act[0] ? c.s1[idx[0]] : 0;
    } else {
        W *st = a.chain ? c.s1 : c.s0;
#pragma unroll
        for (int s = 0; s < NC; ++s) x[s] = act[s] ? st[idx[s]] : 0;
    }

    W tg[NC][B], ntg[NC][B], K[NC];
#pragma unroll
    for (int s = 0; s < NC; ++s) {
        tg[s][0] = 1;
#pragma unroll
        for (int j = 1; j < B; ++j) tg[s][j] = m[s].mul(tg[s][j - 1], 1);
#pragma unroll
        for (int j = 0; j < B; ++j) ntg[s][j] = m[s].p - tg[s][j];
        K[s] = m[s].mont_R_pow(B);
    }

    const uint32_t *mult0 = FUSED ? nullptr : a.mult;
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
                any |= T::fhit(x[0], tg[0][j], ntg[0][j]) | T::fhit(x[NS - 1], tg[0][j], ntg[0][j]);
            } else {
#pragma unroll
                for (int s = 0; s < NC; ++s) {
                    x[s] = T::fstep(m[s], x[s], mv[j]);
                    any |= T::fhit(x[s], tg[s][j], ntg[s][j]);
                }
            }
        }
        if (__any_sync(kFull, any)) {
            if (FUSED) {
                replay_chain<T>(m[0], xs[0], nullptr, a.base, k, B, a.type, act[0], h);
                replay_chain<T>(m[0], xs[NS - 1], mult1, a.base, k, B, a.type2, act[0], h);
            } else {
#pragma unroll
                for (int s = 0; s < NC; ++s) replay_chain<T>(m[s], xs[s], mult0, a.base, k, B, a.type, act[s], h);
            }
        }
        // back to Montgomery form (class 32: |x*K| < p^2 < p*2^31)
        if (FUSED) {
            x[0] = T::restore(m[0], x[0], K[0]);
            x[NS - 1] = T::restore(m[0], x[NS - 1], K[0]);
        } else {
#pragma unroll
            for (int s = 0; s < NC; ++s) x[s] = T::restore(m[s], x[s], K[s]);
        }
    }

    // canonical form for the tail, the state store and the check kernel
    if (FUSED) {
        x[0] = T::canon(m[0], x[0]);
        x[NS - 1] = T::canon(m[0], x[NS - 1]);
    } else {
#pragma unroll
        for (int s = 0; s < NC; ++s) x[s] = T::canon(m[s], x[s]);
    }
    const int r = (int)(a.hi - k);
    if (r > 0) {  // tail of fewer than B steps
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
                    x[0] = T::step(m[0], x[0], mul0);
                    x[NS - 1] = T::step(m[0], x[NS - 1], mul1);
                    any |= (x[0] == tg[0][j]) | (x[0] == ntg[0][j]) | (x[NS - 1] == tg[0][j]) |
                           (x[NS - 1] == ntg[0][j]);
                } else {
#pragma unroll
                    for (int s = 0; s < NC; ++s) {
                        x[s] = T::step(m[s], x[s], mul0);
                        any |= (x[s] == tg[s][j]) | (x[s] == ntg[s][j]);
                    }
                }
            }
        }
        if (__any_sync(kFull, any)) {
            if (FUSED) {
                replay_chain<T>(m[0], xs[0], nullptr, a.base, k, r, a.type, act[0], h);
                replay_chain<T>(m[0], xs[NS - 1], mult1, a.base, k, r, a.type2, act[0], h);
            } else {
#pragma unroll
                for (int s = 0; s < NC; ++s) replay_chain<T>(m[s], xs[s], mult0, a.base, k, r, a.type, act[s], h);
            }
        }
#pragma unroll
        for (int s = 0; s < NC; ++s) {
            const W Kr = m[s].mont_R_pow((uint64_t)r);
            if (FUSED) {
                x[0] = m[0].mul(x[0], Kr);
                x[NS - 1] = m[0].mul(x[NS - 1], Kr);
            } else {
                x[s] = m[s].mul(x[s], Kr);
            }
        }
    }

    const uint32_t walked = (a.hi - a.lo) * (FUSED ? 2u : 1u);
    if (FUSED) {
        if (act[0]) {
            c.s0[idx[0]] = x[0];
            c.s1[idx[0]] = x[NS - 1];
            c.nnext[idx[0]] += walked;
        }
    } else {
        W *st = a.chain ? c.s1 : c.s0;
#pragma unroll
        for (int s = 0; s < NC; ++s)
            if (act[s]) {
                st[idx[s]] = x[s];
                c.nnext[idx[s]] += walked;
            }
    }
}

__global__ void cmult_kernel(uint32_t *out, const uint32_t *primebits, uint32_t nmin, uint32_t lo, uint32_t len,
                             uint32_t padded) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < padded; k += gridDim.x * blockDim.x) {
        uint32_t v = 1u;
        if (k < len) {
            const uint32_t n = lo + k, off = n - nmin;
            const bool prime = (__ldg(primebits + (off >> 5)) >> (off & 31)) & 1u;
            v = prime ? 1u : n;
        }
        out[k] = v;
    }
}

// --------------------------------------------------------------------- check

template <class T>
__global__ void __launch_bounds__(256) check_kernel(ClassBuf<typename T::W> c, CheckArgs a) {
    const uint32_t cnt = min(*c.count, c.cap);
    if (blockIdx.x * blockDim.x >= cnt) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < cnt;
    unsigned long long term = 0;
    bool bad = false;
    if (active) {
        typename T::M m;
        m.init(c.p[i]);
        typename T::W s0 = c.s0[i], s1 = c.s1[i];
        if (s0 >= m.p) s0 -= m.p;                           // walks leave [0, 2p)
        if (s1 >= m.p) s1 -= m.p;
        term = T::term(m, s0);                              // check.cl:59,115,161
        if (a.mode != PFC_PRIMORIAL) term += T::mont64_of(m, a.nlast);
        if (a.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL)) term += T::term(m, s1);
        bad = c.nnext[i] != a.nend;                         // check.cl:61-73
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) term += __shfl_down_sync(kFull, term, o);
    if ((threadIdx.x & 31) == 0 && term) atomicAdd(a.termsum, term);
    if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0) atomicOr(a.flags, 1u);
}

// ------------------------------------------------------------------ launches

static inline unsigned grid_for(uint32_t cap) { return (cap + 255) / 256; }

int launch_setup32(const ClassBuf<uint32_t> &c, const SetupArgs<uint32_t> &a, cudaStream_t st) {
    if (!c.cap) return 0;
    setup_kernel<Cls32><<<grid_for(c.cap), 256, 0, st>>>(c, a);
    return 1;
}
int launch_setup64(const ClassBuf<uint64_t> &c, const SetupArgs<uint64_t> &a, cudaStream_t st) {
    if (!c.cap) return 0;
    setup_kernel<Cls64><<<grid_for(c.cap), 256, 0, st>>>(c, a);
    return 1;
}

template <class T>
static int launch_walk(const ClassBuf<typename T::W> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st) {
    if (!c.cap || a.hi <= a.lo) return 0;
    if (a.mult2) {
        walk_kernel<T, 1, true><<<grid_for(c.cap), 256, 0, st>>>(c, a, h);
    } else {
        const uint32_t per_block = 256u * T::NC;
        walk_kernel<T, T::NC, false><<<(c.cap + per_block - 1) / per_block, 256, 0, st>>>(c, a, h);
    }
    return 1;
}
int launch_walk32(const ClassBuf<uint32_t> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st) {
    return launch_walk<Cls32>(c, a, h, st);
}
int launch_walk64(const ClassBuf<uint64_t> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st) {
    return launch_walk<Cls64>(c, a, h, st);
}

int launch_cmult(uint32_t *out, const uint32_t *primebits, uint32_t nmin, uint32_t lo, uint32_t hi,
                 cudaStream_t st) {
    const uint32_t len = hi - lo, padded = (len + 15u) & ~15u;
    unsigned blocks = (padded + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (!padded) return 0;
    cmult_kernel<<<blocks, 256, 0, st>>>(out, primebits, nmin, lo, len, padded);
    return 1;
}

int launch_check32(const ClassBuf<uint32_t> &c, const CheckArgs &a, cudaStream_t st) {
    if (!c.cap) return 0;
    check_kernel<Cls32><<<grid_for(c.cap), 256, 0, st>>>(c, a);
    return 1;
}
int launch_check64(const ClassBuf<uint64_t> &c, const CheckArgs &a, cudaStream_t st) {
    if (!c.cap) return 0;
    check_kernel<Cls64><<<grid_for(c.cap), 256, 0, st>>>(c, a);
    return 1;
}

}  // namespace pfc
