// noalloc.cu -- pfc_segment_noalloc: one p-segment of a search with no device
// allocation at all.
//
// Who needs it: callers that cannot call cudaMalloc/cudaFree while they run
// this path -- a serving process that has already reserved the whole device
// under its own memory budget and admits work against it, or a host that keeps
// other streams busy and must not issue those calls (cudaFree synchronises the
// device).  They pass their own device buffers for the outputs; every
// intermediate (candidate lists and residues, setup tables, prime flags,
// compositorial multipliers, counters) lives in the one file-scope array
// below, which each GPU that loads the library holds until the process exits.
//
// The kernels are the ones pfc_segment launches (gen.cu, sieve.cu); only the
// memory they are given differs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "host.hpp"
#include "kernels.cuh"
#include "pfcsieve.h"

using namespace pfc;

namespace {

// ----- limits of one call (the scratch layout below is sized for them)
constexpr uint32_t kCands = 1u << 18;        // candidates per size class
constexpr uint32_t kWords32 = 1u << 12;      // setup program words, class 32 (896-bit)
constexpr uint32_t kWords64 = 1u << 16;      // setup program words, class 64
constexpr uint32_t kGroups = 256;            // setup program groups (x3 u32) in all
constexpr uint32_t kNRange = 1u << 22;       // nmax - nmin
constexpr uint32_t kPrimesN = 1u << 18;      // primes in [nmin, nmax) for n#
constexpr uint32_t kChunk = 1u << 16;        // n per walk launch (compositorial table)

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets in the scratch array
constexpr size_t kOffStats = 0;                                            // Stats
constexpr size_t kOffPat = align256(kOffStats + 64);                      // sieve patterns
constexpr size_t kOffC32 = align256(kOffPat + kPatEntries * 8);           // p,s0,s1,nnext u32
constexpr size_t kOffC64 = align256(kOffC32 + (size_t)kCands * 16);       // p,s0,s1 u64 + nnext
constexpr size_t kOffW32 = align256(kOffC64 + (size_t)kCands * 28);
constexpr size_t kOffW64 = align256(kOffW32 + (size_t)kWords32 * sizeof(WideWord));
constexpr size_t kOffGrp = align256(kOffW64 + (size_t)kWords64 * 8);
constexpr size_t kOffBits = align256(kOffGrp + (size_t)kGroups * 12);
constexpr size_t kOffQ = align256(kOffBits + ((size_t)kNRange / 32 + 2) * 4);
constexpr size_t kOffCm = align256(kOffQ + ((size_t)kPrimesN + 32) * 4);
constexpr size_t kEnd = align256(kOffCm + (size_t)kChunk * 4);
static_assert(kEnd <= PFC_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds PFC_NOALLOC_SCRATCH_BYTES");

struct Stats {
    uint32_t counts[2];
    uint32_t flags;
    uint32_t pad;
    unsigned long long termsum;
    unsigned long long hits;
};

}  // namespace

// The scratch of every pfc_segment_noalloc call on this device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[PFC_NOALLOC_SCRATCH_BYTES];

namespace {

// d_totals = {checksum terms, candidates, hits, flags}; flag bit 0: candidate
// overflow, bit 1: n-counter validation failure
__global__ void noalloc_finish_kernel(uint64_t *totals, uint32_t cap) {
    const Stats *s = reinterpret_cast<const Stats *>(g_noalloc_scratch + kOffStats);
    uint64_t flags = 0;
    if (s->counts[0] > cap || s->counts[1] > cap) flags |= 1;
    if (s->flags & 1u) flags |= 2;
    totals[0] = s->termsum;
    totals[1] = (uint64_t)s->counts[0] + s->counts[1];
    totals[2] = s->hits;
    totals[3] = flags;
}

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_base[kMaxDevices] = {nullptr};

// Once per device, with that device current: resolve the device address of
// the scratch array (host code cannot use the symbol itself) and store the
// sieve pattern table in it.
int device_scratch(int dev, unsigned char **base) {
    if (dev < 0 || dev >= kMaxDevices) return PFC_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_base[dev]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return PFC_ERR_CUDA;
        std::vector<uint64_t> pat(kPatEntries);
        uint32_t pr[kSmallPrimes];
        build_pattern_table(pat.data(), pr);
        if (cudaMemcpy((unsigned char *)ptr + kOffPat, pat.data(), pat.size() * 8, cudaMemcpyHostToDevice) !=
            cudaSuccess)
            return PFC_ERR_CUDA;
        g_base[dev] = (unsigned char *)ptr;
    }
    *base = g_base[dev];
    return PFC_OK;
}

// Candidates per size class that one call holds: kCands, or less when the
// environment sets PFCSIEVE_NOALLOC_CAND_CAP (tests use it to exercise the
// candidate-overflow flag; values above kCands are ignored).
uint32_t cand_capacity() {
    const char *v = getenv("PFCSIEVE_NOALLOC_CAND_CAP");
    if (!v || !*v) return kCands;
    const unsigned long long c = strtoull(v, nullptr, 10);
    return c >= 1 && c < kCands ? (uint32_t)c : kCands;
}

// Lower bound on the bits of any setup program for (nmin - 1): every program
// multiplies at least the primes q <= (nmin - 1) / 2 (the compositorial's
// exponents e_q - 1 are non-zero exactly there), and their product has
// theta(x) / ln 2 bits, theta(x) > x (1 - 1 / ln x) for x >= 41 (Rosser and
// Schoenfeld, 1962).  Lets a call whose tables cannot fit the scratch be
// rejected before the host sieves primes up to nmax.
double setup_bits_lower_bound(uint32_t startN) {
    const double x = startN / 2;
    if (x < 41) return 0;
    return x * (1.0 - 1.0 / std::log(x)) / std::log(2.0);
}

double est_cands(uint64_t lo, uint64_t hi) {
    if (hi <= lo) return 0;
    const double a = (double)std::max<uint64_t>(lo, 114);
    return (double)(hi - lo) / std::log(a) * 1.25 + 30.0;
}

}  // namespace

extern "C" int pfc_segment_noalloc(unsigned mode, uint32_t nmin, uint32_t nmax, uint64_t p_lo, uint64_t p_hi,
                                   pfc_factor *d_hits, uint64_t hit_cap, uint64_t *d_totals, void *stream) {
    // ----- arguments and limits (checked before any device work)
    const bool valid_mode = mode == PFC_FACTORIAL || mode == PFC_PRIMORIAL || mode == PFC_COMPOSITORIAL ||
                            mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL);
    if (!valid_mode || !d_totals || (!d_hits && hit_cap)) return PFC_ERR_ARG;
    if (p_lo < 3 || p_hi <= p_lo || nmin < 101 || nmax < nmin || nmax > 0x7FFFFFFFu) return PFC_ERR_ARG;
    if (nmax - nmin > kNRange) return PFC_ERR_ARG;
    const uint64_t split = kClassSplit;
    const double e32 = est_cands(p_lo, std::min(p_hi, split));
    const double e64 = est_cands(std::max(p_lo, split), p_hi);
    if (e32 > kCands || e64 > kCands) return PFC_ERR_ARG;
    const uint32_t startN = nmin - 1;
    if (setup_bits_lower_bound(startN) > std::max<double>(kWords32 * 896.0, kWords64 * 64.0)) return PFC_ERR_ARG;

    // The call enqueues copies from host memory that lives only for the call
    // and waits for the stream at the end; on a stream that is being captured
    // either would end the caller's capture with an error, so refuse first.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing((cudaStream_t)stream, &capture) != cudaSuccess ||
        capture != cudaStreamCaptureStatusNone)
        return PFC_ERR_STATE;

    // size classes present, and which setup program forms they need: 896-bit
    // words below 2^64/3 (class 32 and the lazy class 64), 64-bit words above
    const bool use32 = p_lo < split, use64 = p_hi > split;
    const bool wide64 = use64 && p_hi <= kLazyEnd;
    const bool need_wide = use32 || wide64, need_narrow = use64 && !wide64;

    const uint32_t plim = (mode & PFC_COMPOSITORIAL) ? nmax : std::max(startN, nmax ? nmax - 1 : 0);
    const std::vector<uint32_t> primes = primes_between(2, plim);
    const std::vector<uint32_t> below(primes.begin(), std::upper_bound(primes.begin(), primes.end(), startN));
    HostProg<WideWord> a32, b32;
    HostProg<uint64_t> a64, b64;
    auto build = [&](auto &a, auto &b) {
        if (mode == PFC_FACTORIAL) return build_power_prog(startN, 0, primes, a);
        if (mode == PFC_COMPOSITORIAL) return build_power_prog(startN, 1, primes, a);
        if (mode == PFC_PRIMORIAL) return build_product_prog(below, a);
        return build_power_prog(startN, 1, primes, a) && build_product_prog(below, b);
    };
    if ((need_wide && !build(a32, b32)) || (need_narrow && !build(a64, b64))) return PFC_ERR_ARG;
    if (a32.words.size() + b32.words.size() > kWords32 || a64.words.size() + b64.words.size() > kWords64 ||
        a32.groups.size() + b32.groups.size() + a64.groups.size() + b64.groups.size() > 3 * kGroups)
        return PFC_ERR_ARG;
    std::vector<uint32_t> qlist;
    if (mode == PFC_PRIMORIAL) {
        qlist.assign(std::lower_bound(primes.begin(), primes.end(), nmin),
                     std::lower_bound(primes.begin(), primes.end(), nmax));
        if (qlist.size() > kPrimesN) return PFC_ERR_ARG;
        qlist.resize(qlist.size() + 32, 1u);
    }

    // ----- device and scratch
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PFC_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major != 10 || prop.minor != 3)
        return PFC_ERR_NO_DEVICE;
    unsigned char *base = nullptr;
    int rc = device_scratch(dev, &base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;

    Stats *stats = reinterpret_cast<Stats *>(base + kOffStats);
    uint32_t *counts = &stats->counts[0];
    WideWord *w32 = reinterpret_cast<WideWord *>(base + kOffW32);
    uint64_t *w64 = reinterpret_cast<uint64_t *>(base + kOffW64);
    uint32_t *grp = reinterpret_cast<uint32_t *>(base + kOffGrp);
    uint32_t *bits = reinterpret_cast<uint32_t *>(base + kOffBits);
    uint32_t *q = reinterpret_cast<uint32_t *>(base + kOffQ);
    uint32_t *cm = reinterpret_cast<uint32_t *>(base + kOffCm);

    std::vector<cudaError_t> errs;
    // counters start at zero on every call (the array keeps the last call's contents)
    errs.push_back(cudaMemsetAsync(stats, 0, sizeof(Stats), st));

    // setup programs: words and groups of a32, b32, a64, b64 packed in order
    auto place = [&](const auto &h, auto *words, size_t &woff, size_t &goff) {
        using W = typename std::decay_t<decltype(h.words)>::value_type;
        Prog<W> p;
        p.words = words + woff;
        p.groups = grp + goff;
        p.ngroups = (uint32_t)(h.groups.size() / 3);
        p.final_sq = h.final_sq;
        p.corr = h.corr;
        if (!h.words.empty())
            errs.push_back(cudaMemcpyAsync(words + woff, h.words.data(), h.words.size() * sizeof(W),
                                           cudaMemcpyHostToDevice, st));
        if (!h.groups.empty())
            errs.push_back(cudaMemcpyAsync(grp + goff, h.groups.data(), h.groups.size() * 4,
                                           cudaMemcpyHostToDevice, st));
        woff += h.words.size();
        goff += h.groups.size();
        return p;
    };
    size_t wo32 = 0, wo64 = 0, go = 0;
    SetupArgs<WideWord> s32;
    SetupArgs<uint64_t> s64;
    s32.mode = s64.mode = mode;
    s32.nnext0 = s64.nnext0 = 0;
    s32.a = place(a32, w32, wo32, go);
    s32.b = place(b32, w32, wo32, go);
    s64.a = place(a64, w64, wo64, go);
    s64.b = place(b64, w64, wo64, go);
    if (mode & PFC_COMPOSITORIAL) {
        const std::vector<uint32_t> pb = prime_bitmap(nmin, nmax, primes);
        errs.push_back(cudaMemcpyAsync(bits, pb.data(), pb.size() * 4, cudaMemcpyHostToDevice, st));
    }
    if (!qlist.empty())
        errs.push_back(cudaMemcpyAsync(q, qlist.data(), qlist.size() * 4, cudaMemcpyHostToDevice, st));

    // candidate classes inside the scratch
    const uint32_t cap = cand_capacity();
    ClassBuf<uint32_t> c32;
    c32.p = reinterpret_cast<uint32_t *>(base + kOffC32);
    c32.s0 = c32.p + kCands;
    c32.s1 = c32.s0 + kCands;
    c32.nnext = c32.s1 + kCands;
    c32.cap = cap;
    c32.count = counts;
    ClassBuf<uint64_t> c64;
    c64.p = reinterpret_cast<uint64_t *>(base + kOffC64);
    c64.s0 = c64.p + kCands;
    c64.s1 = c64.s0 + kCands;
    c64.nnext = reinterpret_cast<uint32_t *>(c64.s1 + kCands);
    c64.cap = cap;
    c64.count = counts + 1;

    // generate
    GenArgs g;
    memset(&g, 0, sizeof(g));
    const uint64_t gbase = p_lo | 1;
    g.base = gbase;
    g.nodd = p_hi > gbase ? (p_hi - gbase + 1) / 2 : 0;
    g.p32 = c32.p;
    g.p64 = c64.p;
    g.cap32 = use32 ? cap : 0;
    g.cap64 = use64 ? cap : 0;
    g.count = counts;
    g.pat = reinterpret_cast<const uint64_t *>(base + kOffPat);
    static const uint32_t sp[kSmallPrimes] = {3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37,  41,  43,  47,  53,
                                              59, 61, 67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113};
    for (int k = 0; k < kSmallPrimes; ++k) g.bmod[k] = (uint32_t)(gbase % sp[k]);
    launch_gen(g, prop.multiProcessorCount, st);

    // setup
    if (use32) launch_setup32(c32, s32, st);
    if (wide64) launch_setup64w(c64, s32, st);
    else if (use64) launch_setup64(c64, s64, st);

    // walks over [nmin, nmax) (prime indices for n#), in chunks of kChunk
    HitBuf h{};
    h.buf = d_hits;
    h.count = &stats->hits;
    h.cap = hit_cap;
    const uint32_t lo = mode == PFC_PRIMORIAL ? 0u : nmin;
    const uint32_t hi = mode == PFC_PRIMORIAL ? (uint32_t)(qlist.empty() ? 0 : qlist.size() - 32) : nmax;
    for (uint32_t a = lo; a < hi;) {
        const uint32_t b = (uint32_t)std::min<uint64_t>((uint64_t)a + kChunk, hi);
        WalkArgs w;
        w.lo = a;
        w.hi = b;
        w.mult = nullptr;
        w.mult2 = nullptr;
        w.base = 0;
        w.type = w.type2 = 0;
        w.chain = 0;
        if (mode == PFC_PRIMORIAL) {
            w.mult = q;
            w.type = PFC_TYPE_PRIMORIAL;
        } else {
            if (mode & PFC_COMPOSITORIAL) {
                launch_cmult(cm, nullptr, bits, nmin, a, b, st);
                w.base = a;
            }
            if (mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL)) {
                w.mult2 = cm;
                w.type = PFC_TYPE_FACTORIAL;
                w.type2 = PFC_TYPE_COMPOSITORIAL;
            } else if (mode == PFC_FACTORIAL) {
                w.type = PFC_TYPE_FACTORIAL;
            } else {
                w.mult = cm;
                w.type = PFC_TYPE_COMPOSITORIAL;
            }
        }
        if (use32) launch_walk32(c32, w, h, st, 0);
        if (use64) launch_walk64(c64, w, h, st, p_hi <= kLazyWalkEnd, 0);
        a = b;
    }

    // check, then the totals into the caller's buffer
    CheckArgs ck;
    ck.mode = mode;
    ck.nlast = nmax - 1;
    const uint32_t len = hi - lo;
    ck.nend = mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL) ? 2 * len : len;
    ck.termsum = &stats->termsum;
    ck.flags = &stats->flags;
    if (use32) launch_check32(c32, ck, st);
    if (use64) launch_check64(c64, ck, st);
    noalloc_finish_kernel<<<1, 1, 0, st>>>(d_totals, cap);

    errs.push_back(cudaGetLastError());
    // the host tables above must outlive their copies: wait for the stream
    errs.push_back(cudaStreamSynchronize(st));
    for (cudaError_t e : errs)
        if (e != cudaSuccess) return PFC_ERR_CUDA;
    return PFC_OK;
}
