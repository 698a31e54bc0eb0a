// sieve.cu -- setup, walk and check kernels of one job (replace
// kernels/setup.cl, kernels/iterate.cl and kernels/check.cl); the walk itself
// is in walk.cuh.
//
// One thread owns one candidate prime p (two in class-32 single-chain walks)
// for a launch; its residues live in registers between the loads at launch
// start and the stores at launch end.
#include <type_traits>

#include "walk.cuh"

namespace pfc {

// --------------------------------------------------------------------- setup

template <class T>
__global__ void __launch_bounds__(256) setup_kernel(ClassBuf<typename T::W> c, SetupArgs<typename T::SW> a) {
    using W = typename T::W;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t cnt = min(*c.count, c.cap);
    if (blockIdx.x * blockDim.x >= cnt) return;   // whole CTAs only: run_prog stages words per CTA
    const bool act = i < cnt;
    typename T::M m;
    m.init(act ? c.p[i] : (W)3);
    const typename T::SC sc = T::sctx(m);
    W s0, s1 = 0;
    if (a.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL)) {
        s1 = run_prog<T>(m, sc, a.a, m.one);      // (n-1)!/(n-1)#
        s0 = run_prog<T>(m, sc, a.b, s1);         // (n-1)! = that * (n-1)#
    } else {
        s0 = run_prog<T>(m, sc, a.a, m.one);
    }
    if (act) {
        c.s0[i] = s0;
        c.s1[i] = s1;
        c.nnext[i] = a.nnext0;
    }
}

// The start residues of a split walk's boundaries, all in one launch: CTA
// row blockIdx.y evaluates boundary y + 1's programs for every candidate
// (the rows run side by side instead of one launch after another).
template <class T>
__global__ void __launch_bounds__(256) split_setup_kernel(ClassBuf<typename T::W> c, SplitSetup<typename T::SW> ss,
                                                          typename T::W *out0, typename T::W *out1) {
    using W = typename T::W;
    const uint32_t k = blockIdx.y;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t cnt = min(*c.count, c.cap);
    if (blockIdx.x * blockDim.x >= cnt || k + 1 >= ss.n) return;   // whole CTAs only (staged words)
    const bool act = i < cnt;
    typename T::M m;
    m.init(act ? c.p[i] : (W)3);
    const typename T::SC sc = T::sctx(m);
    W s0, s1 = 0;
    if (ss.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL)) {
        s1 = run_prog<T>(m, sc, ss.a[k], m.one);
        s0 = run_prog<T>(m, sc, ss.b[k], s1);
    } else {
        s0 = run_prog<T>(m, sc, ss.a[k], m.one);
    }
    if (act) {
        out0[(size_t)k * c.cap + i] = s0;
        out1[(size_t)k * c.cap + i] = s1;
    }
}

// ------------------------------------------------------------------- walk

// One walk launch over all candidates of a class (see walk_streams): NC
// candidates per thread (or the two chains of one, FUSED), blocks of B steps.
// SPLIT: sub-range blockIdx.y of a split walk (kernels.cuh SplitArgs).
template <class T, int NC, bool FUSED, int B, bool SPLIT>
__device__ __forceinline__ void walk_body(ClassBuf<typename T::W> c, WalkArgs a, HitBuf h,
                                          SplitArgs<typename T::W> sp) {
    using W = typename T::W;
    constexpr int NS = FUSED ? 2 : NC;   // streams per thread
    const uint32_t cnt = min(*c.count, c.cap);
    const uint32_t blk0 = blockIdx.x * blockDim.x * NC;
    if (blk0 >= cnt) return;  // whole block idle
    const uint32_t sub = SPLIT ? blockIdx.y : 0;
    const bool last = !SPLIT || sub + 1 == sp.n;
    if (SPLIT) {   // unrolled selects keep the boundary array in the parameter bank
#pragma unroll
        for (int k = 0; k < kMaxSplit; ++k)
            if ((uint32_t)k == sub) {
                a.lo = sp.start[k];
                a.hi = sp.start[k + 1];
            }
    }

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
    // start residues: the candidate's state, or the sub-range's start
    W *in0 = c.s0, *in1 = c.s1;
    if (SPLIT && sub > 0) {
        in0 = sp.s0 + (size_t)(sub - 1) * sp.pitch;
        in1 = sp.s1 + (size_t)(sub - 1) * sp.pitch;
    }
    if (FUSED) {
        x[0] = act[0] ? in0[idx[0]] : 0;
        x[NS - 1] = act[0] ? in1[idx[0]] : 0;
    } else {
        const W *st = a.chain ? in1 : in0;
#pragma unroll
        for (int s = 0; s < NC; ++s) x[s] = act[s] ? st[idx[s]] : 0;
    }
    walk_streams<T, NC, FUSED, B>(m, x, act, a, h);
    const uint32_t walked = (a.hi - a.lo) * (FUSED ? 2u : 1u);
    if (FUSED) {
        if (act[0]) {
            if (last) {
                c.s0[idx[0]] = x[0];
                c.s1[idx[0]] = x[NS - 1];
            }
            if (SPLIT) atomicAdd(c.nnext + idx[0], walked);
            else c.nnext[idx[0]] += walked;
        }
    } else {
        W *st = a.chain ? c.s1 : c.s0;
#pragma unroll
        for (int s = 0; s < NC; ++s)
            if (act[s]) {
                if (last) st[idx[s]] = x[s];
                if (SPLIT) atomicAdd(c.nnext + idx[s], walked);
                else c.nnext[idx[s]] += walked;
            }
    }
}

// Two kernels over the same body.  walk_kernel carries only the CTA size:
// with it ptxas settles the fused class-32 walk at 80 registers, three CTAs
// per SM (stating a minimum of one CTA per SM instead let it take 96, two
// CTAs: 843 against 793 ms on the combined search).  walk_kernel3 asks for
// three CTAs per SM: the lazy class-64 walk in blocks of 32 (80 registers
// instead of 92, a 20-byte spill: 75.4 against 76.9 ms on the primorial
// search near 2^62) and split walks (99 registers, two CTAs, unbounded).
template <class T, int NC, bool FUSED, int B, bool SPLIT = false>
__global__ void __launch_bounds__(256) walk_kernel(ClassBuf<typename T::W> c, WalkArgs a, HitBuf h,
                                                   SplitArgs<typename T::W> sp) {
    walk_body<T, NC, FUSED, B, SPLIT>(c, a, h, sp);
}
template <class T, int NC, bool FUSED, int B, bool SPLIT = false>
__global__ void __launch_bounds__(256, 3) walk_kernel3(ClassBuf<typename T::W> c, WalkArgs a, HitBuf h,
                                                       SplitArgs<typename T::W> sp) {
    walk_body<T, NC, FUSED, B, SPLIT>(c, a, h, sp);
}
template <class T, int B, bool SPLIT>
constexpr bool walk_bounded() { return (std::is_same<T, Cls64L>::value && B == 32) || SPLIT; }

// Multiplier tables of one chunk [lo, lo + len): the compositorial's (n at
// composite n, 1 at prime n) when `out` is set and the factorial's (n) when
// `ramp` is set; the walks load them four at a time, which costs fewer
// instructions than forming n in every step.
__global__ void cmult_kernel(uint32_t *out, uint32_t *ramp, const uint32_t *primebits, uint32_t nmin, uint32_t lo,
                             uint32_t len, uint32_t padded) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < padded; k += gridDim.x * blockDim.x) {
        if (out) {
            uint32_t v = 1u;
            if (k < len) {
                const uint32_t n = lo + k, off = n - nmin;
                const bool prime = (__ldg(primebits + (off >> 5)) >> (off & 31)) & 1u;
                v = prime ? 1u : n;
            }
            out[k] = v;
        }
        if (ramp) ramp[k] = lo + k;
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

int launch_setup32(const ClassBuf<uint32_t> &c, const SetupArgs<WideWord> &a, cudaStream_t st) {
    if (!c.cap) return 0;
    setup_kernel<Cls32><<<grid_for(c.cap), 256, 0, st>>>(c, a);
    return 1;
}
int launch_setup64(const ClassBuf<uint64_t> &c, const SetupArgs<uint64_t> &a, cudaStream_t st) {
    if (!c.cap) return 0;
    setup_kernel<Cls64><<<grid_for(c.cap), 256, 0, st>>>(c, a);
    return 1;
}
int launch_setup64w(const ClassBuf<uint64_t> &c, const SetupArgs<WideWord> &a, cudaStream_t st) {
    if (!c.cap) return 0;
    setup_kernel<Cls64L><<<grid_for(c.cap), 256, 0, st>>>(c, a);
    return 1;
}

template <class T>
static int launch_split_setup(const ClassBuf<typename T::W> &c, const SplitSetup<typename T::SW> &ss,
                              typename T::W *s0, typename T::W *s1, cudaStream_t st) {
    if (!c.cap || ss.n < 2 || ss.n > (uint32_t)kMaxSplit) return 0;
    split_setup_kernel<T><<<dim3(grid_for(c.cap), ss.n - 1), 256, 0, st>>>(c, ss, s0, s1);
    return 1;
}
int launch_split_setup32(const ClassBuf<uint32_t> &c, const SplitSetup<WideWord> &ss, uint32_t *s0, uint32_t *s1,
                         cudaStream_t st) {
    return launch_split_setup<Cls32>(c, ss, s0, s1, st);
}
int launch_split_setup64(const ClassBuf<uint64_t> &c, const SplitSetup<uint64_t> &ss, uint64_t *s0, uint64_t *s1,
                         cudaStream_t st) {
    return launch_split_setup<Cls64>(c, ss, s0, s1, st);
}
int launch_split_setup64w(const ClassBuf<uint64_t> &c, const SplitSetup<WideWord> &ss, uint64_t *s0, uint64_t *s1,
                          cudaStream_t st) {
    return launch_split_setup<Cls64L>(c, ss, s0, s1, st);
}

// Walk variants (candidates per thread, block length) per size class and walk
// kind; entry 0 is the default, pfc_autotune measures the others.  Register
// bounds for four CTAs of 256 per SM (64 registers) were measured and dropped:
// the fused class-32 walk ran 1.3% slower, the two-candidate one 23% slower.
// Blocks of 32 are the lazy class-64 default: 77.0 ms against 80.0 ms for
// blocks of 16 on the primorial search near 2^62 (1.16e6 candidates x 78,473
// prime n); two candidates per thread there took 81.5 ms.
struct WalkVariant {
    int nc, b;
};
static const WalkVariant kVar32[] = {{2, 16}, {2, 8}, {1, 16}};
static const WalkVariant kVar32F[] = {{1, 16}, {1, 8}};
static const WalkVariant kVar64L[] = {{1, 32}, {1, 16}, {1, 8}, {2, 16}};
static const WalkVariant kVar64LF[] = {{1, 16}, {1, 8}};
static const WalkVariant kVar64[] = {{1, 8}};
static const WalkVariant kVar64F[] = {{1, 8}};

template <size_t N>
static const WalkVariant *table(const WalkVariant (&v)[N], int *n) {
    *n = (int)N;
    return v;
}

static const WalkVariant *variants(int cls, bool fused, int *n) {
    if (cls == 0) return fused ? table(kVar32F, n) : table(kVar32, n);
    if (cls == 1) return fused ? table(kVar64LF, n) : table(kVar64L, n);
    return fused ? table(kVar64F, n) : table(kVar64, n);
}

int walk_variant_count(int cls, bool fused) {
    int n = 0;
    variants(cls, fused, &n);
    return n;
}

int walk_variant_shape(int cls, bool fused, int variant, int *nc, int *b) {
    int n = 0;
    const WalkVariant *v = variants(cls, fused, &n);
    if (variant < 0 || variant >= n) return -1;
    *nc = v[variant].nc;
    *b = v[variant].b;
    return 0;
}

// SM count of the current device (cached per device)
static int device_sms() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

// Candidate sets too small to give every SM several CTAs of 256 threads
// (about three are resident per SM at the walks' register counts) leave SMs
// idle or unevenly loaded; their walks run in CTAs of 128 threads, sized from
// the class capacity (an upper estimate of the count).  Measured on GB300 for
// 61,945 candidates x 19,899 n, two candidates per thread: 0.745 ms in CTAs of
// 128 (64 and 32 the same), 0.772 ms in CTAs of 256; one candidate per thread
// was slower at every CTA size (0.82-0.87 ms): with so few chains per SM the
// walk is latency-bound and two chains per thread hide more of it than more
// warps do.
constexpr uint32_t kWalkFullCtas = 3;

static bool walk_small(uint32_t cap, int nc, int sms) {
    return (uint64_t)cap < (uint64_t)sms * kWalkFullCtas * 256u * (uint32_t)nc;
}

static unsigned walk_cta_threads(uint32_t cap, int nc, int sms) { return walk_small(cap, nc, sms) ? 128 : 256; }

template <class T, int NC, bool FUSED, int B>
static int launch_one(const ClassBuf<typename T::W> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st) {
    const unsigned threads = walk_cta_threads(c.cap, NC, device_sms());
    const uint32_t per_block = threads * NC;
    SplitArgs<typename T::W> none{};
    none.n = 1;
    if constexpr (walk_bounded<T, B, false>())
        walk_kernel3<T, NC, FUSED, B><<<(c.cap + per_block - 1) / per_block, threads, 0, st>>>(c, a, h, none);
    else
        walk_kernel<T, NC, FUSED, B><<<(c.cap + per_block - 1) / per_block, threads, 0, st>>>(c, a, h, none);
    return 1;
}

// a split walk: grid y runs over the sub-ranges
template <class T, int NC, bool FUSED, int B>
static int launch_split(const ClassBuf<typename T::W> &c, const WalkArgs &a, const HitBuf &h,
                        const SplitArgs<typename T::W> &sp, cudaStream_t st) {
    const unsigned threads = walk_cta_threads(c.cap * sp.n, NC, device_sms());
    const uint32_t per_block = threads * NC;
    const dim3 grid((c.cap + per_block - 1) / per_block, sp.n);
    walk_kernel3<T, NC, FUSED, B, true><<<grid, threads, 0, st>>>(c, a, h, sp);
    return 1;
}

// the default shape of each class for split walks
template <class T>
static int launch_walk_split(const ClassBuf<typename T::W> &c, const WalkArgs &a, const HitBuf &h,
                             const SplitArgs<typename T::W> &sp, cudaStream_t st) {
    if (!c.cap || sp.n < 1 || sp.n > (uint32_t)kMaxSplit) return 0;
    if (a.mult2) {
        if constexpr (std::is_same<T, Cls64>::value) return launch_split<T, 1, true, 8>(c, a, h, sp, st);
        else return launch_split<T, 1, true, 16>(c, a, h, sp, st);
    }
    if constexpr (std::is_same<T, Cls32>::value) return launch_split<T, 2, false, 16>(c, a, h, sp, st);
    else if constexpr (std::is_same<T, Cls64L>::value) return launch_split<T, 1, false, 32>(c, a, h, sp, st);
    else return launch_split<T, 1, false, 8>(c, a, h, sp, st);
}

// the compiled shapes of each class (others fall back to the default)
template <class T>
static int launch_walk(const ClassBuf<typename T::W> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st,
                       int cls, int variant, const SplitArgs<typename T::W> *sp) {
    if (!c.cap || a.hi <= a.lo) return 0;
    if (sp && sp->n > 1) return launch_walk_split<T>(c, a, h, *sp, st);
    int n = 0;
    const WalkVariant *vs = variants(cls, a.mult2 != nullptr, &n);
    const WalkVariant v = vs[(variant >= 0 && variant < n) ? variant : 0];
    if (a.mult2) {
        if (v.b == 8) return launch_one<T, 1, true, 8>(c, a, h, st);
        return launch_one<T, 1, true, 16>(c, a, h, st);
    }
    const bool two = v.nc == 2;
    if constexpr (std::is_same<T, Cls32>::value) {
        if (two && v.b == 8) return launch_one<T, 2, false, 8>(c, a, h, st);
        if (two) return launch_one<T, 2, false, 16>(c, a, h, st);
        return launch_one<T, 1, false, 16>(c, a, h, st);
    } else if constexpr (std::is_same<T, Cls64L>::value) {
        if (two) return launch_one<T, 2, false, 16>(c, a, h, st);
        if (v.b == 32) return launch_one<T, 1, false, 32>(c, a, h, st);
        if (v.b == 8) return launch_one<T, 1, false, 8>(c, a, h, st);
        return launch_one<T, 1, false, 16>(c, a, h, st);
    } else {
        return launch_one<T, 1, false, 8>(c, a, h, st);
    }
}
int launch_walk32(const ClassBuf<uint32_t> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st, int variant,
                  const SplitArgs<uint32_t> *sp) {
    return launch_walk<Cls32>(c, a, h, st, 0, variant, sp);
}
int launch_walk64(const ClassBuf<uint64_t> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st, bool lazy,
                  int variant, const SplitArgs<uint64_t> *sp) {
    return lazy ? launch_walk<Cls64L>(c, a, h, st, 1, variant, sp) : launch_walk<Cls64>(c, a, h, st, 2, variant, sp);
}

int launch_cmult(uint32_t *out, uint32_t *ramp, const uint32_t *primebits, uint32_t nmin, uint32_t lo, uint32_t hi,
                 cudaStream_t st) {
    const uint32_t len = hi - lo, padded = (len + 15u) & ~15u;
    unsigned blocks = (padded + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    if (!padded) return 0;
    cmult_kernel<<<blocks, 256, 0, st>>>(out, ramp, primebits, nmin, lo, len, padded);
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
