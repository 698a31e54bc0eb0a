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
// Compositorial steps at prime n multiply by 1 instead of n (the reference
// skips them, iterate.cl:137-140): the drift stays one power of R per step and
// the hit test at that step is masked off.
#include "arith.cuh"
#include "kernels.cuh"

namespace pfc {

constexpr unsigned kFull = 0xffffffffu;

struct Cls32 {
    using W = uint32_t;
    using M = Mont32;
    static constexpr int B = 16;
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

// composite flags for n .. n+B-1 (bit j set <=> n+j composite); uniform loads
template <int B>
__device__ __forceinline__ uint32_t comp_bits(const IterArgs &a, uint32_t n) {
    const uint32_t off = n - a.nmin;
    const uint32_t k = off >> 5, sh = off & 31;
    const uint64_t v = ((uint64_t)__ldg(a.primebits + k + 1) << 32) | __ldg(a.primebits + k);
    return ~(uint32_t)(v >> sh) & (uint32_t)((1ull << B) - 1);
}

// Replay `len` steps from the block start with explicit per-step recording.
// X: factorial (or primorial / compositorial-only) residue, Y: compositorial
// residue of the combined search.
template <class T, unsigned MODE>
__device__ __noinline__ void replay_block(const typename T::M &m, typename T::W x, typename T::W y,
                                          uint32_t n, int len, uint32_t cbits, const uint32_t *q,
                                          bool active, const HitBuf &h) {
    using W = typename T::W;
    W t = 1;
    for (int j = 0; j < len; ++j) {
        if (j) t = m.mul(t, 1);
        const W nt = m.p - t;
        if (MODE == PFC_PRIMORIAL) {
            const uint32_t qq = __ldg(q + j);
            x = T::step(m, x, qq);
            const bool hit = active && (x == t || x == nt);
            append_hit(hit, m.p, x == t ? -(int32_t)qq : (int32_t)qq, PFC_TYPE_PRIMORIAL, h);
        } else {
            const uint32_t nn = n + j;
            if (MODE & PFC_FACTORIAL) {
                x = T::step(m, x, nn);
                const bool hit = active && (x == t || x == nt);
                append_hit(hit, m.p, x == t ? -(int32_t)nn : (int32_t)nn, PFC_TYPE_FACTORIAL, h);
            }
            if (MODE & PFC_COMPOSITORIAL) {
                const bool comp = (cbits >> j) & 1;
                W &z = (MODE & PFC_FACTORIAL) ? y : x;
                z = T::step(m, z, comp ? nn : 1u);
                const bool hit = active && comp && (z == t || z == nt);
                append_hit(hit, m.p, z == t ? -(int32_t)nn : (int32_t)nn, PFC_TYPE_COMPOSITORIAL, h);
            }
        }
    }
}

template <class T, unsigned MODE>
__global__ void __launch_bounds__(256) iterate_kernel(ClassBuf<typename T::W> c, IterArgs a, HitBuf h) {
    using W = typename T::W;
    constexpr int B = T::B;
    constexpr bool kF = (MODE & PFC_FACTORIAL) != 0;
    constexpr bool kC = (MODE & PFC_COMPOSITORIAL) != 0;
    constexpr bool kP = MODE == PFC_PRIMORIAL;
    constexpr bool kFC = kF && kC;

    const uint32_t cnt = min(*c.count, c.cap);
    if (blockIdx.x * blockDim.x >= cnt) return;  // whole block idle
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < cnt;

    typename T::M m;
    m.init(active ? c.p[i] : (W)3);
    W x = active ? c.s0[i] : 0;
    W y = (kFC && active) ? c.s1[i] : 0;

    W tg[B], ntg[B];
    tg[0] = 1;
#pragma unroll
    for (int j = 1; j < B; ++j) tg[j] = m.mul(tg[j - 1], 1);
#pragma unroll
    for (int j = 0; j < B; ++j) ntg[j] = m.p - tg[j];
    const W K = m.mont_R_pow(B);

    uint32_t n = a.lo;
    const uint32_t nblk = (a.hi - a.lo) / B;
    for (uint32_t b = 0; b < nblk; ++b, n += B) {
        const W x0 = x, y0 = y;
        const uint32_t cb = kC ? comp_bits<B>(a, n) : 0u;
        bool any = false;
        if (kP) {
            const uint32_t *q = a.qlist + n;
#pragma unroll
            for (int j = 0; j < B; ++j) {
                x = T::step(m, x, __ldg(q + j));
                any |= (x == tg[j]) | (x == ntg[j]);
            }
        } else {
#pragma unroll
            for (int j = 0; j < B; ++j) {
                if (kF) {
                    x = T::step(m, x, n + j);
                    any |= (x == tg[j]) | (x == ntg[j]);
                }
                if (kC) {
                    const bool comp = (cb >> j) & 1;
                    W &z = kFC ? y : x;
                    z = T::step(m, z, comp ? n + j : 1u);
                    any |= comp & ((z == tg[j]) | (z == ntg[j]));
                }
            }
        }
        if (__any_sync(kFull, any && active))
            replay_block<T, MODE>(m, x0, y0, n, B, cb, kP ? a.qlist + n : nullptr, active, h);
        x = m.mul(x, K);
        if (kFC) y = m.mul(y, K);
    }

    // tail of fewer than B steps
    const int r = (int)(a.hi - n);
    if (r > 0) {
        const W x0 = x, y0 = y;
        const uint32_t cb = kC ? comp_bits<B>(a, n) : 0u;
        bool any = false;
#pragma unroll
        for (int j = 0; j < B; ++j) {
            if (j < r) {
                if (kP) {
                    x = T::step(m, x, __ldg(a.qlist + n + j));
                    any |= (x == tg[j]) | (x == ntg[j]);
                } else {
                    if (kF) {
                        x = T::step(m, x, n + j);
                        any |= (x == tg[j]) | (x == ntg[j]);
                    }
                    if (kC) {
                        const bool comp = (cb >> j) & 1;
                        W &z = kFC ? y : x;
                        z = T::step(m, z, comp ? n + j : 1u);
                        any |= comp & ((z == tg[j]) | (z == ntg[j]));
                    }
                }
            }
        }
        if (__any_sync(kFull, any && active))
            replay_block<T, MODE>(m, x0, y0, n, r, cb, kP ? a.qlist + n : nullptr, active, h);
        const W Kr = m.mont_R_pow((uint64_t)r);
        x = m.mul(x, Kr);
        if (kFC) y = m.mul(y, Kr);
    }

    if (active) {
        c.s0[i] = x;
        if (kFC) c.s1[i] = y;
        if (c.nnext[i] == a.lo) c.nnext[i] = a.hi;
        else c.nnext[i] = 0xffffffffu;   // out-of-order chunk: fails the check
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
        term = T::term(m, c.s0[i]);                         // check.cl:59,115,161
        if (a.mode != PFC_PRIMORIAL) term += T::mont64_of(m, a.nlast);
        if (a.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL)) term += T::term(m, c.s1[i]);
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
static int launch_iter(const ClassBuf<typename T::W> &c, const IterArgs &a, const HitBuf &h, cudaStream_t st) {
    if (!c.cap || a.hi <= a.lo) return 0;
    const unsigned g = grid_for(c.cap);
    switch (a.mode) {
        case PFC_FACTORIAL: iterate_kernel<T, PFC_FACTORIAL><<<g, 256, 0, st>>>(c, a, h); break;
        case PFC_PRIMORIAL: iterate_kernel<T, PFC_PRIMORIAL><<<g, 256, 0, st>>>(c, a, h); break;
        case PFC_COMPOSITORIAL: iterate_kernel<T, PFC_COMPOSITORIAL><<<g, 256, 0, st>>>(c, a, h); break;
        case PFC_FACTORIAL | PFC_COMPOSITORIAL:
            iterate_kernel<T, PFC_FACTORIAL | PFC_COMPOSITORIAL><<<g, 256, 0, st>>>(c, a, h);
            break;
        default: return 0;
    }
    return 1;
}
int launch_iterate32(const ClassBuf<uint32_t> &c, const IterArgs &a, const HitBuf &h, cudaStream_t st) {
    return launch_iter<Cls32>(c, a, h, st);
}
int launch_iterate64(const ClassBuf<uint64_t> &c, const IterArgs &a, const HitBuf &h, cudaStream_t st) {
    return launch_iter<Cls64>(c, a, h, st);
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
