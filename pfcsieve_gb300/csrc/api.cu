// api.cu -- C ABI implementation (include/pfcsieve.h): context, job tables,
// stage calls and the segment driver.
//
// Device memory of a job (all owned by the context budget):
//   class-32 candidates: p, s0, s1 (u32) and nnext (u32)   16 B / candidate
//   class-64 candidates: p, s0, s1 (u64) and nnext (u32)   28 B / candidate
//   hit list pfc_factor[hitcap] + 64-bit counter
//   setup programs (896-bit words for class 32 and for class 64 below 2^64/3,
//   u64 words above), prime flags of [nmin, nmax) (1 bit per n)
//   or the prime list of [nmin, nmax) for the primorial walk
//   per-segment accumulators: counts[2], termsum, flags
//
// Per segment (pfc_segment): candidate generation and a count read-back, then
// the segment body (setup, walk launches, check, stats read-back) replayed as
// the job's CUDA graph.  Also here: the table self-check and the autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "devmem.hpp"
#include "host.hpp"
#include "kernels.cuh"
#include "pfcsieve.h"

using namespace pfc;

struct pfc_job {
    pfc_ctx *ctx = nullptr;
    unsigned mode = 0;
    uint32_t nmin = 0, nmax = 0;
    uint64_t pmin = 0, pmax = 0;

    DevProg<WideWord> a32, b32;   // class 32 (896-bit words)
    DevProg<uint64_t> a64, b64;   // class 64 at or above 2^64/3 (64-bit words)
    DevProg<WideWord> aw, bw;     // class 64 below 2^64/3 (896-bit words)
    // the tensor-core setup: aw, bw in their paired form (TcProg), packed into
    // fp16 tiles on first use
    TcProg tcp[2];
    uint64_t tc_words = 0;        // 896-bit words of the search's programs (both)
    DArr<uint8_t> tct;
    DArr<uint32_t> tc_src, tc_groups;
    Prog<WideWord> tc_view[2] = {};
    uint32_t tc_ntiles[2] = {0, 0};
    bool tc_packed = false;
    uint64_t setup_mulmods32 = 0, setup_mulmods64 = 0;
    DArr<uint32_t> primebits;
    DArr<uint32_t> qlist;
    DArr<uint32_t> cmult;       // compositorial multipliers of the current chunk
    DArr<uint32_t> ramp;        // the combined search's factorial multipliers (n) of the chunk
    std::vector<uint32_t> h_qlist;

    DevClass<uint32_t> c32;
    DevClass<uint64_t> c64;
    DArr<pfc_factor> hits;
    DArr<SegStats> stats;       // device copy of SegStats
    SegStats *h_stats = nullptr;  // pinned

    uint64_t termsum = 0, primecount = 0;
    int stage = 0;              // 0 idle, 1 generated, 2 set up, 3 checked
    bool stats_fresh = true;    // h_stats mirrors the device stats (no work enqueued since the last read)
    uint32_t next_it = 0;       // next n (or prime index) for pfc_iterate
    uint64_t seg_lo = 0, seg_hi = 0;
    bool use32 = false, use64 = false;   // size classes the segment can hold
    uint64_t pairs = 0;

    // split walk of the current segment (kernels.cuh SplitArgs): sub-ranges,
    // their boundaries, the setup programs of the starts (boundaries 1..n-1;
    // 896-bit words for class 32 and the lazy class 64, 64-bit words above
    // 2^64/3) and the start residues per class ((n-1) blocks of s0, then
    // (n-1) of s1, one class capacity each)
    uint32_t split_n = 1;
    uint32_t split_start[kMaxSplit + 1] = {0};
    bool split_wide = false, split_narrow = false;
    std::vector<DevProg<WideWord>> split_wa, split_wb;
    std::vector<DevProg<uint64_t>> split_na, split_nb;
    DArr<uint32_t> split32;
    DArr<uint64_t> split64;

    // the post-generation part of a segment captured as a CUDA graph, replayed
    // while the key (buffers, launch shapes, kernel choices) is unchanged
    struct GraphKey {
        const void *p32, *p64, *hits, *cmult, *ramp, *split32, *split64;
        uint64_t cap32, cap64, hitcap;
        int lazy, use32, use64, var[3][2], setup_tc;
        uint32_t split_n, split_start[kMaxSplit + 1];
    };
    cudaGraphExec_t graph = nullptr;
    GraphKey gkey{};
    uint64_t graph_kernels = 0;
    uint64_t segments = 0;   // segments committed (the first one runs without a graph)
};

// ------------------------------------------------------------------ helpers

static uint32_t* counts_ptr(pfc_job *j) { return &j->stats.p->counts[0]; }

static unsigned long long *hitcount_ptr(pfc_job *j) { return &j->stats.p->hits; }

static uint32_t iter_end(const pfc_job *j) {
    return j->mode == PFC_PRIMORIAL ? (uint32_t)j->h_qlist.size() : j->nmax;
}
static uint32_t iter_begin(const pfc_job *j) { return j->mode == PFC_PRIMORIAL ? 0u : j->nmin; }

// steps every candidate walks over the whole search (all its chains)
static uint32_t steps_needed(const pfc_job *j) {
    const uint32_t len = iter_end(j) - iter_begin(j);
    return j->mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL) ? 2 * len : len;
}

// longest n chunk of one launch (bounds the compositorial multiplier table)
constexpr uint32_t kMaxChunk = 1u << 22;

// expected candidates in [lo, hi) (an over-estimate: density 1/ln x falls)
static double est_cands(uint64_t lo, uint64_t hi) {
    if (hi <= lo) return 0;
    const double a = (double)std::max<uint64_t>(lo, 114);
    return (double)(hi - lo) / std::log(a) * 1.25 + 30.0;
}

// ----------------------------------------------------------------- context

extern "C" int pfc_ctx_create(int device, uint64_t mem_budget, pfc_ctx **out) {
    if (!out) return PFC_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return PFC_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3) return PFC_ERR_NO_DEVICE;  // kernels are built for sm_103a only
    CK(cudaSetDevice(device));
    pfc_ctx *c = new (std::nothrow) pfc_ctx();
    if (!c) return PFC_ERR_NOMEM;
    c->device = device;
    c->sms = prop.multiProcessorCount;
    snprintf(c->name, sizeof(c->name), "%s", prop.name);
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    c->budget = mem_budget ? mem_budget : (uint64_t)(0.9 * (double)fr);
    const char *g = getenv("PFCSIEVE_CUDA_GRAPHS");
    c->graphs = !(g && g[0] == '0');
    const char *sp = getenv("PFCSIEVE_SPLIT");
    c->split = !(sp && sp[0] == '0');
    const char *tc = getenv("PFCSIEVE_SETUP_TC");
    c->setup_tc = !(tc && tc[0] == '0');
    cudaError_t e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        e = cudaMemPoolCreate(&c->pool, &props);
    }
    if (e == cudaSuccess) {
        uint64_t keep = ~0ull;   // keep freed blocks between jobs
        e = cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = dalloc_bytes(c, (void **)&c->d_pat, kPatEntries * sizeof(uint64_t));
    if (e == cudaSuccess) {
        std::vector<uint64_t> pat(kPatEntries);
        uint32_t pr[kSmallPrimes];
        build_pattern_table(pat.data(), pr);
        e = cudaMemcpyAsync(c->d_pat, pat.data(), pat.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, c->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    }
    if (e != cudaSuccess) {
        pfc_ctx_destroy(c);
        return cuda_fail(e);
    }
    *out = c;
    return PFC_OK;
}

extern "C" int pfc_ctx_destroy(pfc_ctx *c) {
    if (!c) return PFC_ERR_ARG;
    cudaSetDevice(c->device);
    if (c->st) {
        dfree_bytes(c, c->d_pat, kPatEntries * sizeof(uint64_t));
        dfree_bytes(c, c->vbits, c->vbits_bytes);
        cudaStreamSynchronize(c->st);
    }
    if (c->pool) cudaMemPoolDestroy(c->pool);
    for (void *h : c->pinned_stats) cudaFreeHost(h);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return PFC_OK;
}

extern "C" void *pfc_ctx_stream(pfc_ctx *c) { return c ? (void *)c->st : nullptr; }

extern "C" uint64_t pfc_ctx_launch_count(pfc_ctx *c) { return c ? c->launches : 0; }

extern "C" int pfc_ctx_transfer_bytes(pfc_ctx *c, uint64_t *h2d, uint64_t *d2h) {
    if (!c) return PFC_ERR_ARG;
    if (h2d) *h2d = c->h2d;
    if (d2h) *d2h = c->d2h;
    return PFC_OK;
}

extern "C" int pfc_ctx_device_info(pfc_ctx *c, char *name, size_t cap, int *sms) {
    if (!c) return PFC_ERR_ARG;
    if (name && cap) snprintf(name, cap, "%s", c->name);
    if (sms) *sms = c->sms;
    return PFC_OK;
}

// --------------------------------------------------------------------- job

static int job_release(pfc_job *j) {
    pfc_ctx *c = j->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->st);
    if (j->graph) cudaGraphExecDestroy(j->graph);
    j->graph = nullptr;
    j->a32.release(c);
    j->b32.release(c);
    j->a64.release(c);
    j->b64.release(c);
    j->aw.release(c);
    j->bw.release(c);
    j->tct.release(c);
    j->tc_src.release(c);
    j->tc_groups.release(c);
    j->primebits.release(c);
    j->qlist.release(c);
    j->cmult.release(c);
    j->ramp.release(c);
    j->c32.release(c);
    j->c64.release(c);
    j->hits.release(c);
    j->stats.release(c);
    for (auto &pg : j->split_wa) pg.release(c);
    for (auto &pg : j->split_wb) pg.release(c);
    for (auto &pg : j->split_na) pg.release(c);
    for (auto &pg : j->split_nb) pg.release(c);
    j->split32.release(c);
    j->split64.release(c);
    if (j->h_stats) c->pinned_stats.push_back(j->h_stats);   // kept for the next job
    j->h_stats = nullptr;
    return PFC_OK;
}

// the setup programs of a search for one word type: F, C, P one program (a);
// the combined search a = (n-1)!/(n-1)#, b = the primorial words after it
template <class W>
static bool build_progs(unsigned mode, uint32_t startN, const std::vector<uint32_t> &primes,
                        const std::vector<uint32_t> &below, HostProg<W> &a, HostProg<W> &b) {
    if (mode == PFC_FACTORIAL) return build_power_prog(startN, 0, primes, a);
    if (mode == PFC_COMPOSITORIAL) return build_power_prog(startN, 1, primes, a);
    if (mode == PFC_PRIMORIAL) return build_product_prog(below, a);
    return build_power_prog(startN, 1, primes, a) && build_product_prog(below, b);
}

// the context's prime list, covering at least [2, lim] (replaced by a longer
// one when a larger limit is asked for; callers bound every use by value and
// hold the pointer while they use the list)
static std::shared_ptr<const std::vector<uint32_t>> ctx_primes(pfc_ctx *c, uint32_t lim) {
    if (!c->primes || lim > c->primes_lim) {
        c->primes = std::make_shared<const std::vector<uint32_t>>(primes_between(2, lim));
        c->primes_lim = lim;
    }
    return c->primes;
}

// the setup programs of (mode, startN) in the word types asked for, from the
// context's cache or built into it; nullptr if a program cannot be built
static std::shared_ptr<const ProgSet> ctx_progs(pfc_ctx *c, unsigned mode, uint32_t startN, bool wide, bool narrow) {
    const std::pair<unsigned, uint32_t> key(mode, startN);
    auto it = c->progs.find(key);
    std::shared_ptr<ProgSet> ps = it != c->progs.end() ? it->second : nullptr;
    if (ps && (!wide || ps->has_wide) && (!narrow || ps->has_narrow)) return ps;
    auto fresh = std::make_shared<ProgSet>(ps ? *ps : ProgSet());
    if ((wide && !fresh->has_wide) || (narrow && !fresh->has_narrow)) {
        const std::shared_ptr<const std::vector<uint32_t>> plist = ctx_primes(c, std::max<uint32_t>(startN, 2));
        const std::vector<uint32_t> &primes = *plist;
        const std::vector<uint32_t> below(primes.begin(), std::upper_bound(primes.begin(), primes.end(), startN));
        if (wide && !fresh->has_wide) {
            if (!build_progs(mode, startN, primes, below, fresh->wa, fresh->wb)) return nullptr;
            fresh->has_wide = true;
        }
        if (narrow && !fresh->has_narrow) {
            if (!build_progs(mode, startN, primes, below, fresh->na, fresh->nb)) return nullptr;
            fresh->has_narrow = true;
        }
    }
    if (ps) c->prog_bytes -= ps->bytes();
    else c->prog_order.push_back(key);
    c->progs[key] = fresh;
    c->prog_bytes += fresh->bytes();
    while (c->prog_bytes > pfc_ctx::kProgCacheBytes && c->prog_order.size() > 1) {   // drop the oldest
        auto old = c->progs.find(c->prog_order.front());
        if (old->first == key) break;
        c->prog_bytes -= old->second->bytes();
        c->progs.erase(old);
        c->prog_order.pop_front();
    }
    return fresh;
}

extern "C" int pfc_setup_program_size(unsigned mode, uint32_t nmin, int wide, uint64_t *words,
                                      uint64_t *squarings) {
    if (!words || !squarings) return PFC_ERR_ARG;
    const bool valid_mode = mode == PFC_FACTORIAL || mode == PFC_PRIMORIAL || mode == PFC_COMPOSITORIAL ||
                            mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL);
    if (!valid_mode || nmin < 101 || nmin > 0x7FFFFFFFu) return PFC_ERR_ARG;
    const uint32_t startN = nmin - 1;
    const std::vector<uint32_t> primes = primes_between(2, startN);
    bool ok;
    uint64_t w = 0, m = 0;
    if (wide) {
        HostProg<WideWord> a, b;
        ok = build_progs(mode, startN, primes, primes, a, b);
        w = a.words.size() + b.words.size();
        m = a.mulmods() + b.mulmods();
    } else {
        HostProg<uint64_t> a, b;
        ok = build_progs(mode, startN, primes, primes, a, b);
        w = a.words.size() + b.words.size();
        m = a.mulmods() + b.mulmods();
    }
    if (!ok) return PFC_ERR_ARG;
    *words = w;
    *squarings = m - w;
    return PFC_OK;
}

namespace {
// host replay of a setup program, the way the device runs it: the
// accumulator holds x R^d, a squaring and a product with a table word each
// lower d by one (a*b*R^-1), and the end multiplies by Mont(R^corr); exact
// 128-bit modular arithmetic, R = 2^64 mod p
typedef unsigned __int128 u128e;
struct HostMont {
    uint64_t p, rinv;
    uint64_t mul(uint64_t a, uint64_t b) const { return (uint64_t)((u128e)a * b % p); }
    uint64_t redc(uint64_t a, uint64_t b) const { return mul(mul(a, b), rinv); }
};
uint64_t host_word(const HostMont &m, uint64_t w) { return w % m.p; }
uint64_t host_word(const HostMont &m, const WideWord &w) {
    uint64_t z = 0;   // sum of limb_k 2^(28 k), from the top limb
    for (int k = kWideLimbs - 1; k >= 0; --k)
        z = (uint64_t)((((u128e)z << kWideRadixBits) + w.limb[k]) % m.p);
    return z;
}
// a^-1 mod p for gcd(a, p) = 1 (extended Euclid)
uint64_t host_inv(uint64_t a, uint64_t p) {
    __int128 r0 = p, r1 = a % p, t0 = 0, t1 = 1;
    while (r1) {
        const __int128 q = r0 / r1, r2 = r0 - q * r1, t2 = t0 - q * t1;
        r0 = r1, r1 = r2, t0 = t1, t1 = t2;
    }
    if (r0 != 1) return 0;
    return (uint64_t)(t0 < 0 ? t0 + p : t0);
}
uint64_t host_pow(const HostMont &m, uint64_t b, uint64_t e) {
    uint64_t r = 1 % m.p;
    for (; e; e >>= 1, b = m.mul(b, b))
        if (e & 1) r = m.mul(r, b);
    return r;
}
// groups of (first word, end word, squarings before the group) over words
// given by value(i)
template <class F>
uint64_t host_run(const HostMont &m, const std::vector<uint32_t> &groups, uint32_t final_sq, uint64_t corr,
                  uint64_t acc, F value) {
    for (size_t g = 0; g + 2 < groups.size(); g += 3) {
        for (uint32_t k = 0; k < groups[g + 2]; ++k) acc = m.redc(acc, acc);
        for (uint32_t i = groups[g]; i < groups[g + 1]; ++i) acc = m.redc(acc, value(i));
    }
    for (uint32_t k = 0; k < final_sq; ++k) acc = m.redc(acc, acc);
    const uint64_t R = (uint64_t)(((u128e)1 << 64) % m.p);
    return m.redc(acc, host_pow(m, R, corr + 1));   // Mont(R^corr) = R^(corr+1)
}
template <class W>
uint64_t host_prog(const HostMont &m, const HostProg<W> &pg, uint64_t acc) {
    return host_run(m, pg.groups, pg.final_sq, pg.corr, acc, [&](uint32_t i) { return host_word(m, pg.words[i]); });
}
uint64_t host_tc_prog(const HostMont &m, const HostProg<WideWord> &pg, uint64_t acc) {
    TcProg tp;
    if (!build_tc_prog(pg, tp)) return ~0ull;
    return host_run(m, tp.groups, tp.final_sq, tp.corr, acc, [&](uint32_t i) {
        const uint32_t s = tp.src[i] & 0x7FFFFFFFu;
        const uint64_t z = host_word(m, pg.words[s]);
        return (tp.src[i] & 0x80000000u) ? m.mul(z, host_word(m, pg.words[s + 1])) : z;
    });
}
}  // namespace

extern "C" int pfc_setup_program_eval(unsigned mode, uint32_t nmin, int form, uint64_t p, uint64_t *s0,
                                      uint64_t *s1) {
    if (!s0 || !s1 || p < 3 || !(p & 1) || form < 0 || form > 2) return PFC_ERR_ARG;
    const bool valid_mode = mode == PFC_FACTORIAL || mode == PFC_PRIMORIAL || mode == PFC_COMPOSITORIAL ||
                            mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL);
    if (!valid_mode || nmin < 101 || nmin > 0x7FFFFFFFu) return PFC_ERR_ARG;
    const uint32_t startN = nmin - 1;
    const std::vector<uint32_t> primes = primes_between(2, startN);
    HostMont m;
    m.p = p;
    const uint64_t R = (uint64_t)(((u128e)1 << 64) % p);
    m.rinv = host_inv(R, p);   // p odd: 2^64 is invertible
    uint64_t a = 0, b = 0;
    bool ok;
    if (form == 0) {
        HostProg<uint64_t> pa, pb;
        ok = build_progs(mode, startN, primes, primes, pa, pb);
        if (ok) {
            a = host_prog(m, pa, R);   // Mont(1) = R
            b = host_prog(m, pb, a);   // the combined search continues from the first result
        }
    } else {
        HostProg<WideWord> pa, pb;
        ok = build_progs(mode, startN, primes, primes, pa, pb);
        if (ok) {
            a = form == 1 ? host_prog(m, pa, R) : host_tc_prog(m, pa, R);
            b = form == 1 ? host_prog(m, pb, a) : host_tc_prog(m, pb, a);
            ok = a != ~0ull && b != ~0ull;
        }
    }
    if (!ok) return PFC_ERR_ARG;
    const bool two = mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL);
    *s0 = m.mul(two ? b : a, m.rinv);   // plain residues
    *s1 = two ? m.mul(a, m.rinv) : 0;
    return PFC_OK;
}

extern "C" int pfc_job_create(pfc_ctx *c, unsigned mode, uint32_t nmin, uint32_t nmax, uint64_t pmin,
                              uint64_t pmax, pfc_job **out) {
    if (!c || !out) return PFC_ERR_ARG;
    *out = nullptr;
    // setupSearch (cl_sieve.cpp:600-641) and the CLI ranges (main.cpp:58-72)
    const bool valid_mode = mode == PFC_FACTORIAL || mode == PFC_PRIMORIAL || mode == PFC_COMPOSITORIAL ||
                            mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL);
    if (!valid_mode) return PFC_ERR_ARG;
    if (pmin < 3 || pmax <= pmin) return PFC_ERR_ARG;
    if (nmin < 101 || nmax < nmin || nmax > 0x7FFFFFFFu) return PFC_ERR_ARG;
    CK(cudaSetDevice(c->device));
    pfc_job *j = new (std::nothrow) pfc_job();
    if (!j) return PFC_ERR_NOMEM;
    j->ctx = c;
    j->mode = mode;
    j->nmin = nmin;
    j->nmax = nmax;
    j->pmin = pmin;
    j->pmax = pmax;

    const uint32_t startN = nmin - 1;
    const uint32_t plim = (mode & PFC_COMPOSITORIAL) ? nmax : std::max(startN, nmax - 1);
    const std::shared_ptr<const std::vector<uint32_t>> plist = ctx_primes(c, plim);
    const std::vector<uint32_t> &primes = *plist;
    const bool need32 = pmin < kClassSplit;
    const bool needw = pmax > kClassSplit && pmin < kLazyEnd;
    const bool need64 = pmax > kLazyEnd;
    // class 32 and class 64 below 2^64/3 share the 896-bit programs
    const std::shared_ptr<const ProgSet> ps = ctx_progs(c, mode, startN, need32 || needw, need64);
    if (!ps) {
        delete j;
        return PFC_ERR_ARG;
    }
    const HostProg<WideWord> empty_w;
    const HostProg<uint64_t> empty_n;
    const HostProg<WideWord> &a32 = need32 ? ps->wa : empty_w, &b32 = need32 ? ps->wb : empty_w;
    const HostProg<WideWord> &aw = needw ? ps->wa : empty_w, &bw = needw ? ps->wb : empty_w;
    const HostProg<uint64_t> &a64 = need64 ? ps->na : empty_n, &b64 = need64 ? ps->nb : empty_n;
    j->setup_mulmods32 = a32.mulmods() + b32.mulmods();
    j->setup_mulmods64 = need64 ? a64.mulmods() + b64.mulmods() : aw.mulmods() + bw.mulmods();

    j->tc_words = ps->wa.words.size() + ps->wb.words.size();
    if ((needw && j->tc_words >= kTcMinWords64) || (need32 && j->tc_words >= kTcMinWords32)) {
        // the tensor-core setups of both classes use the paired form
        const HostProg<WideWord> *wide[2] = {needw ? &aw : &a32, needw ? &bw : &b32};
        for (int k = 0; k < 2; ++k) {
            if (!build_tc_prog(*wide[k], j->tcp[k])) {
                delete j;
                return PFC_ERR_ARG;
            }
            j->tc_ntiles[k] = ((uint32_t)j->tcp[k].src.size() + tc_tile_words() - 1) / tc_tile_words();
        }
    }

    cudaError_t e = j->a32.upload(c, a32);
    if (e == cudaSuccess) e = j->a64.upload(c, a64);
    if (e == cudaSuccess) e = j->aw.upload(c, aw);
    if (e == cudaSuccess) e = j->bw.upload(c, bw);
    if (e == cudaSuccess) e = j->b32.upload(c, b32);
    if (e == cudaSuccess) e = j->b64.upload(c, b64);
    if (e == cudaSuccess && (mode & PFC_COMPOSITORIAL)) e = j->primebits.upload(c, prime_bitmap(nmin, nmax, primes));
    if (e == cudaSuccess && mode == PFC_PRIMORIAL) {
        auto lo = std::lower_bound(primes.begin(), primes.end(), nmin);
        auto hi = std::lower_bound(primes.begin(), primes.end(), nmax);
        j->h_qlist.assign(lo, hi);
        std::vector<uint32_t> padded = j->h_qlist;
        padded.resize(padded.size() + 32, 1u);
        e = j->qlist.upload(c, padded);
    }
    if (e == cudaSuccess) e = j->stats.alloc(c, 1);
    if (e == cudaSuccess) e = cudaMemsetAsync(j->stats.p, 0, sizeof(SegStats), c->st);
    if (e == cudaSuccess) {
        if (!c->pinned_stats.empty()) {
            j->h_stats = static_cast<SegStats *>(c->pinned_stats.back());
            c->pinned_stats.pop_back();
        } else {
            e = cudaMallocHost((void **)&j->h_stats, sizeof(SegStats));
        }
        if (e == cudaSuccess) memset(j->h_stats, 0, sizeof(SegStats));   // mirrors the zeroed device stats
    }
    if (e == cudaSuccess) e = j->hits.alloc(c, 1u << 20);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
        job_release(j);
        delete j;
        return cuda_fail(e);
    }
    *out = j;
    return PFC_OK;
}

extern "C" int pfc_job_submit(pfc_ctx *c, unsigned mode, uint32_t nmin, uint32_t nmax, uint64_t pmin,
                              uint64_t pmax, pfc_job **out) {
    return pfc_job_create(c, mode, nmin, nmax, pmin, pmax, out);
}

extern "C" int pfc_job_destroy(pfc_job *j) {
    if (!j) return PFC_ERR_ARG;
    job_release(j);
    delete j;
    return PFC_OK;
}

extern "C" int pfc_job_segment_end(pfc_job *j, uint64_t p_lo, uint64_t *p_hi) {
    if (!j || !p_hi || p_lo < j->pmin || p_lo >= j->pmax) return PFC_ERR_ARG;
    // candidates per segment: bounded by a quarter of the budget at 28 B each
    // and by 2^26
    const double maxc = std::min<double>((double)(1u << 26), (double)j->ctx->budget / 4.0 / 28.0);
    const double ln = std::log((double)std::max<uint64_t>(p_lo, 114));
    const double span = maxc * ln * 0.75;
    uint64_t hi = (span >= (double)(j->pmax - p_lo)) ? j->pmax : p_lo + (uint64_t)span;
    if (hi <= p_lo) hi = std::min(j->pmax, p_lo + 1);
    *p_hi = hi;
    return PFC_OK;
}

// ------------------------------------------------------------- stage calls

static int ensure_class_caps(pfc_job *j, uint64_t lo, uint64_t hi) {
    const uint64_t split = kClassSplit;
    const double e32 = est_cands(lo, std::min(hi, split));
    const double e64 = est_cands(std::max(lo, split), hi);
    const double lim = 4.0e9;
    if (e32 > lim || e64 > lim) return PFC_ERR_NOMEM;
    CK(j->c32.ensure(j->ctx, lo < split ? (uint32_t)e32 : 0u));
    CK(j->c64.ensure(j->ctx, hi > split ? (uint32_t)e64 : 0u));
    j->use32 = lo < split;
    j->use64 = hi > split;
    return PFC_OK;
}

static int enqueue_gen(pfc_job *j, uint64_t lo, uint64_t hi) {
    pfc_ctx *c = j->ctx;
    CK(cudaMemsetAsync(counts_ptr(j), 0, 2 * sizeof(uint32_t), c->st));
    GenArgs g;
    memset(&g, 0, sizeof(g));
    const uint64_t base = lo | 1;
    g.base = base;
    g.nodd = hi > base ? (hi - base + 1) / 2 : 0;
    g.p32 = j->c32.p.p;
    g.p64 = j->c64.p.p;
    g.cap32 = j->use32 ? j->c32.cap : 0;
    g.cap64 = j->use64 ? j->c64.cap : 0;
    g.count = counts_ptr(j);
    g.pat = c->d_pat;
    static const uint32_t sp[kSmallPrimes] = {3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37,  41,  43,  47,  53,
                                              59, 61, 67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113};
    for (int k = 0; k < kSmallPrimes; ++k) g.bmod[k] = (uint32_t)(base % sp[k]);
    c->launches += launch_gen(g, c->sms, c->st);
    CK(cudaGetLastError());
    j->seg_lo = lo;
    j->seg_hi = hi;
    j->stage = 1;
    return PFC_OK;
}

extern "C" int pfc_gen_candidates(pfc_job *j, uint64_t p_lo, uint64_t p_hi) {
    if (!j || p_lo < j->pmin || p_hi > j->pmax || p_hi <= p_lo) return PFC_ERR_ARG;
    CK(cudaSetDevice(j->ctx->device));
    j->stats_fresh = false;
    int rc = ensure_class_caps(j, p_lo, p_hi);
    if (rc) return rc;
    return enqueue_gen(j, p_lo, p_hi);
}

// The wide programs as fp16 tiles for the tensor-core setup, packed once per
// job on the context stream (before any capture of a segment graph).
static int tc_prepare(pfc_job *j) {
    if (j->tc_packed) return PFC_OK;
    pfc_ctx *c = j->ctx;
    const size_t tb = tc_tile_bytes(), na = j->tc_ntiles[0], nb = j->tc_ntiles[1];
    const TcProg &pa = j->tcp[0], &pb = j->tcp[1];
    std::vector<uint32_t> src(pa.src), groups(pa.groups);
    src.insert(src.end(), pb.src.begin(), pb.src.end());
    groups.insert(groups.end(), pb.groups.begin(), pb.groups.end());
    CK(j->tct.alloc(c, std::max<size_t>((na + nb) * tb, 16)));
    CK(j->tc_src.upload(c, src));
    CK(j->tc_groups.upload(c, groups));
    // the words: the lazy class-64 copy of the programs, or the class-32 one (the same programs)
    const bool w64 = j->aw.view.ngroups || j->bw.view.ngroups;
    const WideWord *wa = w64 ? j->aw.words.p : j->a32.words.p, *wb = w64 ? j->bw.words.p : j->b32.words.p;
    c->launches += launch_tc_pack(wa, j->tc_src.p, (uint32_t)pa.src.size(), (uint32_t)na, j->tct.p, c->st);
    c->launches += launch_tc_pack(wb, j->tc_src.p + pa.src.size(), (uint32_t)pb.src.size(), (uint32_t)nb,
                                  j->tct.p + na * tb, c->st);
    CK(cudaGetLastError());
    for (int k = 0; k < 2; ++k) {
        const TcProg &tp = j->tcp[k];
        Prog<WideWord> &v = j->tc_view[k];
        v.words = nullptr;
        v.groups = j->tc_groups.p + (k ? pa.groups.size() : 0);
        v.ngroups = (uint32_t)(tp.groups.size() / 3);
        v.final_sq = tp.final_sq;
        v.corr = tp.corr;
    }
    j->tc_packed = true;   // (pageable uploads are staged before the calls return)
    return PFC_OK;
}

static bool tc_setup_applies(const pfc_job *j) {
    return j->use64 && j->seg_hi <= kLazyEnd && j->ctx->setup_tc && j->tc_words >= kTcMinWords64;
}
static bool tc_setup32_applies(const pfc_job *j) {
    return j->use32 && j->ctx->setup_tc && j->tc_words >= kTcMinWords32;
}

static int enqueue_setup(pfc_job *j) {
    pfc_ctx *c = j->ctx;
    SetupArgs<WideWord> s32;
    s32.mode = j->mode;
    s32.a = j->a32.view;
    s32.b = j->b32.view;
    s32.nnext0 = 0;
    SetupArgs<uint64_t> s64;
    s64.mode = j->mode;
    s64.a = j->a64.view;
    s64.b = j->b64.view;
    s64.nnext0 = 0;
    SetupArgs<WideWord> sw;
    sw.mode = j->mode;
    sw.a = j->aw.view;
    sw.b = j->bw.view;
    sw.nnext0 = 0;
    if (j->use32) {
        if (tc_setup32_applies(j)) {
            const int rc = tc_prepare(j);
            if (rc) return rc;
            const TcTiles ta{j->tct.p, j->tc_ntiles[0]},
                tb{j->tct.p + (size_t)j->tc_ntiles[0] * tc_tile_bytes(), j->tc_ntiles[1]};
            SetupArgs<WideWord> stc = s32;
            stc.a = j->tc_view[0];
            stc.b = j->tc_view[1];
            CK(cudaMemsetAsync(&j->stats.p->tc_err, 0, sizeof(uint32_t), c->st));
            c->launches += launch_setup32_tc(j->c32.view(counts_ptr(j)), stc, ta, tb, &j->stats.p->tc_err, c->st);
        } else {
            c->launches += launch_setup32(j->c32.view(counts_ptr(j)), s32, c->st);
        }
    }
    if (j->use64) {
        if (tc_setup_applies(j)) {
            const int rc = tc_prepare(j);
            if (rc) return rc;
            const TcTiles ta{j->tct.p, j->tc_ntiles[0]},
                tb{j->tct.p + (size_t)j->tc_ntiles[0] * tc_tile_bytes(), j->tc_ntiles[1]};
            SetupArgs<WideWord> stc = sw;
            stc.a = j->tc_view[0];
            stc.b = j->tc_view[1];
            if (!tc_setup32_applies(j)) CK(cudaMemsetAsync(&j->stats.p->tc_err, 0, sizeof(uint32_t), c->st));
            c->launches += launch_setup64w_tc(j->c64.view(counts_ptr(j) + 1), stc, ta, tb, &j->stats.p->tc_err, c->st);
        } else if (j->seg_hi <= kLazyEnd) {
            c->launches += launch_setup64w(j->c64.view(counts_ptr(j) + 1), sw, c->st);
        } else {
            c->launches += launch_setup64(j->c64.view(counts_ptr(j) + 1), s64, c->st);
        }
    }
    CK(cudaGetLastError());
    j->stage = 2;
    j->next_it = iter_begin(j);
    return PFC_OK;
}

extern "C" int pfc_setup(pfc_job *j) {
    if (!j) return PFC_ERR_ARG;
    if (j->stage < 1) return PFC_ERR_STATE;
    CK(cudaSetDevice(j->ctx->device));
    j->stats_fresh = false;
    return enqueue_setup(j);
}

static HitBuf hitbuf(pfc_job *j) {
    HitBuf h{};
    h.buf = j->hits.p;
    h.count = hitcount_ptr(j);
    h.cap = j->hits.n;
    return h;
}

// the walks of one chunk [lo, hi) (n values, or prime indices for n#):
// factorial over n, compositorial over its multiplier table, primorial over
// the prime list; each for both size classes
static int enqueue_iter_range(pfc_job *j, uint32_t lo, uint32_t hi, bool split = false) {
    pfc_ctx *c = j->ctx;
    const HitBuf h = hitbuf(j);
    SplitArgs<uint32_t> sp32{};
    SplitArgs<uint64_t> sp64{};
    if (split) {
        sp32.n = sp64.n = j->split_n;
        for (uint32_t k = 0; k <= j->split_n; ++k) sp32.start[k] = sp64.start[k] = j->split_start[k];
        sp32.pitch = j->c32.cap;
        sp32.s0 = j->split32.p;
        sp32.s1 = j->split32.p ? j->split32.p + (size_t)(j->split_n - 1) * j->c32.cap : nullptr;
        sp64.pitch = j->c64.cap;
        sp64.s0 = j->split64.p;
        sp64.s1 = j->split64.p ? j->split64.p + (size_t)(j->split_n - 1) * j->c64.cap : nullptr;
    }
    auto walk = [&](const WalkArgs &w) {
        const int fused = w.mult2 != nullptr;
        const bool lazy = j->seg_hi <= kLazyWalkEnd;
        if (j->use32)
            c->launches += launch_walk32(j->c32.view(counts_ptr(j)), w, h, c->st, c->walk_var[0][fused],
                                         split ? &sp32 : nullptr);
        if (j->use64)
            c->launches += launch_walk64(j->c64.view(counts_ptr(j) + 1), w, h, c->st, lazy,
                                         c->walk_var[lazy ? 1 : 2][fused], split ? &sp64 : nullptr);
    };
    WalkArgs w;
    w.lo = lo;
    w.hi = hi;
    w.mult = nullptr;
    w.mult2 = nullptr;
    w.base = 0;
    w.type = w.type2 = 0;
    w.chain = 0;
    if (j->mode == PFC_PRIMORIAL) {
        w.mult = j->qlist.p;
        w.type = PFC_TYPE_PRIMORIAL;
        walk(w);
        CK(cudaGetLastError());
        return PFC_OK;
    }
    if (j->mode & PFC_COMPOSITORIAL) {
        // multiplier tables of the chunk: compositorial (n or 1) and, for the
        // fused walk, factorial (n; the plain factorial walk forms n itself,
        // shared by its two candidates, and gains nothing from a table)
        const size_t need = ((size_t)(hi - lo) + 15) & ~(size_t)15;
        const bool comp = true, fact = (j->mode & PFC_FACTORIAL) != 0;
        if (comp && j->cmult.n < need) CK(j->cmult.alloc(c, std::max<size_t>(need, 4096)));
        if (fact && j->ramp.n < need) CK(j->ramp.alloc(c, std::max<size_t>(need, 4096)));
        c->launches += launch_cmult(comp ? j->cmult.p : nullptr, fact ? j->ramp.p : nullptr, j->primebits.p,
                                    j->nmin, lo, hi, c->st);
        w.base = lo;
    }
    if (j->mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL)) {
        // one launch walks both chains of each candidate
        w.mult = j->ramp.p;
        w.mult2 = j->cmult.p;
        w.type = PFC_TYPE_FACTORIAL;
        w.type2 = PFC_TYPE_COMPOSITORIAL;
    } else if (j->mode == PFC_FACTORIAL) {
        w.type = PFC_TYPE_FACTORIAL;
    } else {
        w.mult = j->cmult.p;
        w.type = PFC_TYPE_COMPOSITORIAL;
    }
    walk(w);
    CK(cudaGetLastError());
    return PFC_OK;
}

// chunk length so one launch covers about `budget` candidate-steps
static uint32_t chunk_len(uint64_t count, double budget) {
    double L = budget / (double)std::max<uint64_t>(count, 1);
    L = std::max(16.0, std::min(L, 2147483648.0));
    return ((uint32_t)L + 15u) & ~15u;
}

// ------------------------------------------------------------ split walks
//
// A segment with few candidates leaves most of the GPU idle in its walk: each
// candidate's chain is a sequence of dependent multiplications, and a few
// chains per SM cannot hide their latency (61,945 candidates x 19,899 n ran at
// 10% warp occupancy, latency-bound).  When the whole walk fits one launch,
// the n range [lo, hi) is cut into S sub-ranges; the residue at each
// boundary b comes from a setup program for (b-1)! (or (b-1)!/(b-1)#, or the
// primorial of the primes below the boundary's prime), evaluated by the setup
// kernel, and one launch walks every (candidate, sub-range) pair.  S fills
// about two waves of resident CTAs; boundaries whose programs would cost more
// than a sixth of the walk (large nmin) disable the split.  Results are the
// same as the plain walk's: every n is tested once, hits carry their own n,
// the last sub-range leaves the final residue and nnext counts every step.

constexpr uint32_t kMinSplitLen = 2048;   // shortest sub-range worth a setup program

template <class W>
static uint64_t prog_cost(const HostProg<W> &a, const HostProg<W> &b) {
    // in walk steps: an 896-bit word costs about 15 class-32 steps of multiply
    // pipe, a 64-bit word about 2; squarings about one
    const uint64_t wc = sizeof(W) > 8 ? 15 : 2;
    const uint64_t words = a.words.size() + b.words.size();
    return words * wc + (a.mulmods() + b.mulmods() - words);
}

// Plan (and prepare) the split for a walk over the whole range of the current
// segment: j->split_n = 1 when the walk stays plain.  Host tables are built
// and uploaded here, before any graph capture.
static int split_prepare(pfc_job *j) {
    pfc_ctx *c = j->ctx;
    j->split_n = 1;
    const uint32_t lo = iter_begin(j), hi = iter_end(j), len = hi - lo;
    const uint64_t n32 = (j->use32 && j->c32.p.p) ? j->c32.cap : 0;
    const uint64_t n64 = (j->use64 && j->c64.p.p) ? j->c64.cap : 0;
    const uint32_t L = std::min(chunk_len(n32 + 3 * n64, 1.5e11), kMaxChunk);
    if (!c->split || len > L || n32 + n64 == 0) return PFC_OK;
    const bool fused = j->mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL);
    const uint64_t chains = (n32 + n64) * (fused ? 2 : 1);
    const uint64_t target = (uint64_t)c->sms * 3 * 256 * 2 * 2;   // two waves of CTAs, two chains a thread
    uint32_t S = (uint32_t)std::min<uint64_t>({(uint64_t)kMaxSplit, target / chains, len / kMinSplitLen});
    if (S < 2) return PFC_OK;
    const bool lazy = j->seg_hi <= kLazyEnd;
    const bool wide = n32 > 0 || (n64 > 0 && lazy), narrow = n64 > 0 && !lazy;
    const uint64_t walk = (uint64_t)len * (fused ? 2 : 1);

    // a lower bound on a boundary's program cost, before anything is built:
    // every program multiplies at least the primes up to (b-1)/2, whose
    // product has theta(x)/ln 2 > x (1 - 1/ln x)/ln 2 bits (x >= 41, Rosser
    // and Schoenfeld), 896 bits a word
    auto cost_floor = [](uint32_t b) {
        const double x = b / 2.0;
        return x < 41 ? 0.0 : x * (1.0 - 1.0 / std::log(x)) / std::log(2.0) / 896.0 * 15.0;
    };
    for (; S >= 2; --S) {
        uint32_t start[kMaxSplit + 1];
        const uint32_t step = ((len / S) + 15u) & ~15u;
        for (uint32_t k = 0; k < S; ++k) start[k] = lo + k * step;
        start[S] = hi;
        if (start[S - 1] >= hi) continue;
        double floor_cost = 0;
        for (uint32_t k = 1; k < S; ++k)
            floor_cost += cost_floor(j->mode == PFC_PRIMORIAL ? j->h_qlist[start[k]] : start[k]);
        if (floor_cost * 6 > (double)walk) continue;
        const bool same = j->split_wide == wide && j->split_narrow == narrow &&
                          j->split_wa.size() + j->split_na.size() > 0 &&
                          std::max(j->split_wa.size(), j->split_na.size()) == S - 1 &&
                          memcmp(start, j->split_start, sizeof(uint32_t) * (S + 1)) == 0;
        if (!same) {
            // the value before each boundary's first multiplier; the
            // boundaries' programs come from the context's cache
            std::vector<std::shared_ptr<const ProgSet>> ps(S);
            uint64_t cost = 0;
            for (uint32_t k = 1; k < S; ++k) {
                const uint32_t startN = (j->mode == PFC_PRIMORIAL ? j->h_qlist[start[k]] : start[k]) - 1;
                ps[k] = ctx_progs(c, j->mode, startN, wide, narrow);
                if (!ps[k]) return PFC_ERR_ARG;
                cost += wide ? prog_cost(ps[k]->wa, ps[k]->wb) : prog_cost(ps[k]->na, ps[k]->nb);
            }
            if (cost * 6 > walk) continue;   // boundaries too dear: fewer sub-ranges or none
            for (auto &pg : j->split_wa) pg.release(c);
            for (auto &pg : j->split_wb) pg.release(c);
            for (auto &pg : j->split_na) pg.release(c);
            for (auto &pg : j->split_nb) pg.release(c);
            j->split_wa.assign(wide ? S - 1 : 0, DevProg<WideWord>());
            j->split_wb.assign(wide ? S - 1 : 0, DevProg<WideWord>());
            j->split_na.assign(narrow ? S - 1 : 0, DevProg<uint64_t>());
            j->split_nb.assign(narrow ? S - 1 : 0, DevProg<uint64_t>());
            for (uint32_t k = 1; k < S; ++k) {
                if (wide) {
                    CK(j->split_wa[k - 1].upload(c, ps[k]->wa));
                    CK(j->split_wb[k - 1].upload(c, ps[k]->wb));
                }
                if (narrow) {
                    CK(j->split_na[k - 1].upload(c, ps[k]->na));
                    CK(j->split_nb[k - 1].upload(c, ps[k]->nb));
                }
            }
            j->split_wide = wide;
            j->split_narrow = narrow;
            memcpy(j->split_start, start, sizeof(uint32_t) * (S + 1));
        }
        // start residues of boundaries 1..S-1 for s0 and s1, per class
        const size_t need32 = (size_t)2 * (S - 1) * n32, need64 = (size_t)2 * (S - 1) * n64;
        if (n32 && j->split32.n < need32) CK(j->split32.alloc(c, need32));
        if (n64 && j->split64.n < need64) CK(j->split64.alloc(c, need64));
        j->split_n = S;
        return PFC_OK;
    }
    return PFC_OK;
}

// one setup launch per size class for the start residues of boundaries
// 1..split_n-1
static int enqueue_split_setup(pfc_job *j) {
    pfc_ctx *c = j->ctx;
    const uint32_t S = j->split_n;
    const bool lazy = j->seg_hi <= kLazyEnd;
    SplitSetup<WideWord> sw{};
    SplitSetup<uint64_t> sn{};
    sw.mode = sn.mode = j->mode;
    sw.n = sn.n = S;
    for (uint32_t k = 1; k < S; ++k) {
        if (j->split_wide) {
            sw.a[k - 1] = j->split_wa[k - 1].view;
            sw.b[k - 1] = j->split_wb[k - 1].view;
        }
        if (j->split_narrow) {
            sn.a[k - 1] = j->split_na[k - 1].view;
            sn.b[k - 1] = j->split_nb[k - 1].view;
        }
    }
    if (j->use32 && j->c32.p.p)
        c->launches += launch_split_setup32(j->c32.view(counts_ptr(j)), sw, j->split32.p,
                                            j->split32.p + (size_t)(S - 1) * j->c32.cap, c->st);
    if (j->use64 && j->c64.p.p) {
        uint64_t *s0 = j->split64.p, *s1 = j->split64.p + (size_t)(S - 1) * j->c64.cap;
        if (lazy) c->launches += launch_split_setup64w(j->c64.view(counts_ptr(j) + 1), sw, s0, s1, c->st);
        else c->launches += launch_split_setup64(j->c64.view(counts_ptr(j) + 1), sn, s0, s1, c->st);
    }
    CK(cudaGetLastError());
    return PFC_OK;
}

// [lo, hi) in launches of about 1.5e11 candidate-steps (class-64 steps
// weigh 3), so no launch runs for more than a fraction of a second; a walk
// over the whole range of a segment that split_prepare planned runs split.
static int enqueue_iter_chunked(pfc_job *j, uint32_t lo, uint32_t hi, uint64_t n32, uint64_t n64) {
    if (j->split_n > 1 && lo == iter_begin(j) && hi == iter_end(j)) {
        int rc = enqueue_split_setup(j);
        if (rc) return rc;
        return enqueue_iter_range(j, lo, hi, true);
    }
    const uint32_t L = std::min(chunk_len(n32 + 3 * n64, 1.5e11), kMaxChunk);
    while (lo < hi) {
        const uint32_t e = (uint32_t)std::min<uint64_t>((uint64_t)lo + L, hi);
        int rc = enqueue_iter_range(j, lo, e);
        if (rc) return rc;
        lo = e;
    }
    return PFC_OK;
}

extern "C" int pfc_iterate(pfc_job *j, uint32_t n_lo, uint32_t n_hi) {
    if (!j || n_hi < n_lo) return PFC_ERR_ARG;
    if (j->stage < 2) return PFC_ERR_STATE;
    CK(cudaSetDevice(j->ctx->device));
    j->stats_fresh = false;
    uint32_t lo = n_lo, hi = n_hi;
    if (j->mode == PFC_PRIMORIAL) {   // n range -> prime index range
        lo = (uint32_t)(std::lower_bound(j->h_qlist.begin(), j->h_qlist.end(), n_lo) - j->h_qlist.begin());
        hi = (uint32_t)(std::lower_bound(j->h_qlist.begin(), j->h_qlist.end(), n_hi) - j->h_qlist.begin());
        if (n_lo <= j->nmin) lo = 0;
        if (n_hi >= j->nmax) hi = (uint32_t)j->h_qlist.size();
    }
    if (lo != j->next_it || hi > iter_end(j)) return PFC_ERR_STATE;
    if (hi == lo) return PFC_OK;
    // one call over the whole range may walk split (split walks)
    j->split_n = 1;
    if (lo == iter_begin(j) && hi == iter_end(j)) {
        const int sr = split_prepare(j);
        if (sr) return sr;
    }
    int rc = enqueue_iter_chunked(j, lo, hi, j->c32.cap, j->c64.cap);
    if (rc) return rc;
    j->next_it = hi;
    return PFC_OK;
}

static int enqueue_check(pfc_job *j) {
    pfc_ctx *c = j->ctx;
    CheckArgs a;
    a.mode = j->mode;
    a.nlast = j->nmax - 1;
    a.nend = steps_needed(j);
    a.termsum = &j->stats.p->termsum;
    a.flags = &j->stats.p->flags;
    if (j->use32) c->launches += launch_check32(j->c32.view(counts_ptr(j)), a, c->st);
    if (j->use64) c->launches += launch_check64(j->c64.view(counts_ptr(j) + 1), a, c->st);
    CK(cudaGetLastError());
    return PFC_OK;
}

static int read_stats(pfc_job *j) {
    j->ctx->d2h += sizeof(SegStats);
    CK(cudaMemcpyAsync(j->h_stats, j->stats.p, sizeof(SegStats), cudaMemcpyDeviceToHost, j->ctx->st));
    CK(cudaStreamSynchronize(j->ctx->st));
    j->stats_fresh = true;
    return PFC_OK;
}

// fold the checked segment into the job totals
static int commit_segment(pfc_job *j) {
    const SegStats &s = *j->h_stats;
    if (s.counts[0] > j->c32.cap && j->c32.p.p) return PFC_ERR_CAND_OVERFLOW;
    if (s.counts[1] > j->c64.cap && j->c64.p.p) return PFC_ERR_CAND_OVERFLOW;
    if ((!j->c32.p.p && s.counts[0]) || (!j->c64.p.p && s.counts[1])) return PFC_ERR_CAND_OVERFLOW;
    if (s.tc_err) return PFC_ERR_CUDA;   // a tensor-core setup wait gave up
    if (s.flags & 1u) return PFC_ERR_VALIDATION;
    j->termsum += s.termsum;
    j->primecount += (uint64_t)s.counts[0] + s.counts[1];
    j->pairs += ((uint64_t)s.counts[0] + s.counts[1]) * (uint64_t)(j->nmax - j->nmin);
    j->stage = 3;
    ++j->segments;
    return PFC_OK;
}

extern "C" int pfc_check(pfc_job *j) {
    if (!j) return PFC_ERR_ARG;
    if (j->stage < 2 || j->next_it != iter_end(j)) return PFC_ERR_STATE;
    CK(cudaSetDevice(j->ctx->device));
    CK(cudaMemsetAsync(&j->stats.p->termsum, 0, sizeof(unsigned long long), j->ctx->st));
    CK(cudaMemsetAsync(&j->stats.p->flags, 0, sizeof(uint32_t), j->ctx->st));
    int rc = enqueue_check(j);
    if (rc) return rc;
    rc = read_stats(j);
    if (rc) return rc;
    return commit_segment(j);
}

// The part of a segment after candidate generation: clear the segment
// accumulators, setup, the walk in launches sized from the buffer capacities
// (so the sequence is the same for every segment of the job), the check and
// the read-back of the segment's stats into pinned host memory.
static int enqueue_segment_body(pfc_job *j) {
    pfc_ctx *c = j->ctx;
    CK(cudaMemsetAsync(&j->stats.p->termsum, 0, sizeof(unsigned long long), c->st));
    CK(cudaMemsetAsync(&j->stats.p->flags, 0, sizeof(uint32_t), c->st));
    int rc = enqueue_setup(j);
    if (rc) return rc;
    rc = enqueue_iter_chunked(j, iter_begin(j), iter_end(j), j->c32.p.p ? j->c32.cap : 0,
                              j->c64.p.p ? j->c64.cap : 0);
    if (rc) return rc;
    j->next_it = iter_end(j);
    rc = enqueue_check(j);
    if (rc) return rc;
    c->d2h += sizeof(SegStats);
    CK(cudaMemcpyAsync(j->h_stats, j->stats.p, sizeof(SegStats), cudaMemcpyDeviceToHost, c->st));
    return PFC_OK;
}

static int segment_body_stream(pfc_job *j) {
    const int rc = enqueue_segment_body(j);
    if (rc) return rc;
    CK(cudaStreamSynchronize(j->ctx->st));
    j->stats_fresh = true;
    return PFC_OK;
}

// The same body as one CUDA graph: captured at the first segment of the job
// and again when a buffer, a launch shape or a kernel choice changed, then
// replayed with one launch per segment.
static int segment_body_graph(pfc_job *j) {
    pfc_ctx *c = j->ctx;
    // a buffer the body would otherwise allocate while it is being captured
    if (j->mode & PFC_COMPOSITORIAL) {
        const uint64_t n32 = j->c32.p.p ? j->c32.cap : 0, n64 = j->c64.p.p ? j->c64.cap : 0;
        const size_t L = std::min(chunk_len(n32 + 3 * n64, 1.5e11), kMaxChunk);
        const size_t need = (((size_t)std::min<uint64_t>(L, iter_end(j) - iter_begin(j))) + 15) & ~(size_t)15;
        if ((j->mode & PFC_COMPOSITORIAL) && j->cmult.n < need) CK(j->cmult.alloc(c, std::max<size_t>(need, 4096)));
        if ((j->mode & PFC_FACTORIAL) && j->ramp.n < need) CK(j->ramp.alloc(c, std::max<size_t>(need, 4096)));
    }
    if (tc_setup_applies(j) || tc_setup32_applies(j)) {
        const int rc = tc_prepare(j);
        if (rc) return rc;
    }
    pfc_job::GraphKey k{};
    k.p32 = j->c32.p.p;
    k.p64 = j->c64.p.p;
    k.hits = j->hits.p;
    k.cmult = j->cmult.p;
    k.ramp = j->ramp.p;
    k.cap32 = j->c32.cap;
    k.cap64 = j->c64.cap;
    k.hitcap = j->hits.n;
    k.lazy = j->seg_hi <= kLazyWalkEnd;
    k.use32 = j->use32;
    k.use64 = j->use64;
    memcpy(k.var, c->walk_var, sizeof(k.var));
    k.split32 = j->split32.p;
    k.split64 = j->split64.p;
    k.split_n = j->split_n;
    k.setup_tc = c->setup_tc;
    if (j->split_n > 1) memcpy(k.split_start, j->split_start, sizeof(k.split_start));
    if (!j->graph || memcmp(&k, &j->gkey, sizeof(k)) != 0) {
        if (j->graph) cudaGraphExecDestroy(j->graph);
        j->graph = nullptr;
        const uint64_t l0 = c->launches, d0 = c->d2h;
        CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_segment_body(j);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(c->st, &g);
        j->graph_kernels = c->launches - l0;
        c->launches = l0;   // counted when the graph is launched
        c->d2h = d0;
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        CK(e);
        const cudaError_t ei = cudaGraphInstantiate(&j->graph, g, 0);
        cudaGraphDestroy(g);
        CK(ei);
        j->gkey = k;
    }
    CK(cudaGraphLaunch(j->graph, c->st));
    c->launches += j->graph_kernels;
    c->d2h += sizeof(SegStats);
    CK(cudaStreamSynchronize(c->st));
    j->stats_fresh = true;
    return PFC_OK;
}

extern "C" int pfc_segment(pfc_job *j, uint64_t p_lo, uint64_t p_hi) {
    if (!j || p_lo < j->pmin || p_hi > j->pmax || p_hi <= p_lo) return PFC_ERR_ARG;
    pfc_ctx *c = j->ctx;
    CK(cudaSetDevice(c->device));
    int rc = ensure_class_caps(j, p_lo, p_hi);
    if (rc) return rc;
    if (!j->stats_fresh) {   // stage calls left work or hits the host has not seen
        rc = read_stats(j);
        if (rc) return rc;
    }
    // generation and the segment body in one stream sequence (the grids are
    // sized from the buffer capacities, so no wait for the candidate counts);
    // a class or the hit list that overflowed is grown and the segment redone
    // from the hits of earlier segments
    const unsigned long long hit_base = j->h_stats->hits;
    for (int attempt = 0;; ++attempt) {
        rc = enqueue_gen(j, p_lo, p_hi);
        if (rc) return rc;
        rc = split_prepare(j);
        if (rc) return rc;
        // a graph pays off from the second segment of a job on: capturing and
        // instantiating it costs about as much as one small segment
        rc = (c->graphs && j->segments > 0) ? segment_body_graph(j) : segment_body_stream(j);
        if (rc) return rc;
        j->stage = 2;
        j->next_it = iter_end(j);
        const uint32_t n32 = j->h_stats->counts[0], n64 = j->h_stats->counts[1];
        const bool over32 = n32 > (j->c32.p.p ? j->c32.cap : 0);
        const bool over64 = n64 > (j->c64.p.p ? j->c64.cap : 0);
        const unsigned long long nh = j->h_stats->hits;
        const bool overhits = nh > j->hits.n;
        if (!over32 && !over64 && !overhits) break;
        if (attempt >= 3) return over32 || over64 ? PFC_ERR_CAND_OVERFLOW : PFC_ERR_HIT_OVERFLOW;
        if (over32) CK(j->c32.ensure(c, (uint32_t)std::min<uint64_t>(4000000000ull, n32 + n32 / 8 + 1024)));
        if (over64) CK(j->c64.ensure(c, (uint32_t)std::min<uint64_t>(4000000000ull, n64 + n64 / 8 + 1024)));
        if (overhits && !over32 && !over64) {
            // grow the hit list, keep the hits of earlier segments
            DArr<pfc_factor> bigger;
            CK(bigger.alloc(c, (size_t)(nh + nh / 4 + 4096)));
            if (hit_base)
                CK(cudaMemcpyAsync(bigger.p, j->hits.p, hit_base * sizeof(pfc_factor), cudaMemcpyDeviceToDevice, c->st));
            CK(cudaStreamSynchronize(c->st));
            j->hits.release(c);
            j->hits = bigger;
        }
        CK(cudaMemcpyAsync(hitcount_ptr(j), &hit_base, sizeof(hit_base), cudaMemcpyHostToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
        j->h_stats->hits = hit_base;
    }
    return commit_segment(j);
}

extern "C" int pfc_sync(pfc_job *j) {
    if (!j) return PFC_ERR_ARG;
    CK(cudaSetDevice(j->ctx->device));
    CK(cudaStreamSynchronize(j->ctx->st));
    return PFC_OK;
}

extern "C" int pfc_drain_hits(pfc_job *j, pfc_factor *buf, size_t cap, size_t *n) {
    if (!j || !n || (!buf && cap)) return PFC_ERR_ARG;
    pfc_ctx *c = j->ctx;
    CK(cudaSetDevice(c->device));
    if (!j->stats_fresh) {   // after a segment or a check the host copy is current
        const int rc = read_stats(j);
        if (rc) return rc;
    }
    const unsigned long long nh = j->h_stats->hits;
    *n = (size_t)nh;
    if (nh > j->hits.n) return PFC_ERR_HIT_OVERFLOW;   // device list incomplete
    const size_t copy = std::min<size_t>((size_t)nh, cap);
    if (copy) {
        c->d2h += copy * sizeof(pfc_factor);
        CK(cudaMemcpyAsync(buf, j->hits.p, copy * sizeof(pfc_factor), cudaMemcpyDeviceToHost, c->st));
    }
    if (nh > cap) {
        if (copy) CK(cudaStreamSynchronize(c->st));
        return PFC_ERR_HIT_OVERFLOW;
    }
    if (nh) CK(cudaMemsetAsync(hitcount_ptr(j), 0, sizeof(unsigned long long), c->st));
    if (copy) CK(cudaStreamSynchronize(c->st));   // buf is filled; the reset is ordered before later work
    j->h_stats->hits = 0;
    return PFC_OK;
}

extern "C" int pfc_job_totals(pfc_job *j, uint64_t *termsum, uint64_t *primecount) {
    if (!j) return PFC_ERR_ARG;
    if (termsum) *termsum = j->termsum;
    if (primecount) *primecount = j->primecount;
    return PFC_OK;
}

extern "C" int pfc_job_run(pfc_job *j, pfc_factor *buf, size_t cap, size_t *n) {
    if (!j || !n || (!buf && cap)) return PFC_ERR_ARG;
    size_t total = 0;
    bool overflow = false;
    std::vector<pfc_factor> tmp;
    for (uint64_t lo = j->pmin; lo < j->pmax;) {
        uint64_t hi;
        int rc = pfc_job_segment_end(j, lo, &hi);
        if (rc) return rc;
        rc = pfc_segment(j, lo, hi);
        if (rc) return rc;
        size_t got = 0;
        const size_t room = overflow ? 0 : cap - total;
        rc = pfc_drain_hits(j, overflow ? nullptr : buf + total, room, &got);
        if (rc == PFC_ERR_HIT_OVERFLOW) {
            overflow = true;
            // clear the device list so later segments keep counting
            CK(cudaMemsetAsync(hitcount_ptr(j), 0, sizeof(unsigned long long), j->ctx->st));
            CK(cudaStreamSynchronize(j->ctx->st));
            j->h_stats->hits = 0;
        } else if (rc) {
            return rc;
        }
        total += got;
        lo = hi;
    }
    *n = total;
    return overflow ? PFC_ERR_HIT_OVERFLOW : PFC_OK;
}

// ---------------------------------------------------------- introspection

extern "C" int pfc_segment_state(pfc_job *j, uint64_t *p, uint64_t *s0, uint64_t *s1, size_t cap, size_t *n) {
    if (!j || !n) return PFC_ERR_ARG;
    int rc = read_stats(j);
    if (rc) return rc;
    const uint32_t n32 = std::min(j->h_stats->counts[0], j->use32 ? j->c32.cap : 0u);
    const uint32_t n64 = std::min(j->h_stats->counts[1], j->use64 ? j->c64.cap : 0u);
    *n = (size_t)n32 + n64;
    if (*n > cap) return PFC_ERR_ARG;
    std::vector<uint32_t> a(n32), b(n32), d(n32);
    std::vector<uint64_t> e(n64), f(n64), g(n64);
    if (n32) {
        CK(cudaMemcpy(a.data(), j->c32.p.p, n32 * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(b.data(), j->c32.s0.p, n32 * 4, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(d.data(), j->c32.s1.p, n32 * 4, cudaMemcpyDeviceToHost));
    }
    if (n64) {
        CK(cudaMemcpy(e.data(), j->c64.p.p, n64 * 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(f.data(), j->c64.s0.p, n64 * 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(g.data(), j->c64.s1.p, n64 * 8, cudaMemcpyDeviceToHost));
    }
    typedef unsigned __int128 u128;
    for (uint32_t i = 0; i < n32; ++i) {
        // class 32 holds x*2^32 mod p (walks leave it in [0, 2p)): the
        // reference form is x*2^64 mod p
        p[i] = a[i];
        if (s0) s0[i] = (uint64_t)(((u128)b[i] << 32) % a[i]);
        if (s1) s1[i] = (uint64_t)(((u128)d[i] << 32) % a[i]);
    }
    for (uint32_t i = 0; i < n64; ++i) {
        p[n32 + i] = e[i];
        if (s0) s0[n32 + i] = f[i];
        if (s1) s1[n32 + i] = g[i];
    }
    return PFC_OK;
}

extern "C" uint64_t pfc_job_pairs(pfc_job *j) { return j ? j->pairs : 0; }

extern "C" uint64_t pfc_job_setup_mulmods(pfc_job *j, int cls64) {
    return j ? (cls64 ? j->setup_mulmods64 : j->setup_mulmods32) : 0;
}

// ------------------------------------------------------- table self-check

static uint64_t mulmod_h(uint64_t a, uint64_t b, uint64_t p) { return (uint64_t)((unsigned __int128)a * b % p); }
static uint64_t powmod_h(uint64_t a, uint64_t e, uint64_t p) {
    uint64_t r = 1 % p;
    a %= p;
    for (; e; e >>= 1) {
        if (e & 1) r = mulmod_h(r, a, p);
        a = mulmod_h(a, a, p);
    }
    return r;
}

// Run the job's setup programs of one word form on the single candidate p and
// return its residues in plain form (s1: the combined search's compositorial).
template <class W, class SW>
static int setup_on_prime(pfc_job *j, const DevProg<SW> &a, const DevProg<SW> &b, uint64_t p, uint64_t &s0,
                          uint64_t &s1) {
    pfc_ctx *c = j->ctx;
    DevClass<W> cls;
    DArr<uint32_t> cnt;
    CK(cls.ensure(c, 1));
    cudaError_t e = cnt.alloc(c, 1);
    const W pw = (W)p;
    const uint32_t one = 1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(cls.p.p, &pw, sizeof(W), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.p, &one, sizeof(one), cudaMemcpyHostToDevice, c->st);
    SetupArgs<SW> sa;
    sa.mode = j->mode;
    sa.a = a.view;
    sa.b = b.view;
    sa.nnext0 = 0;
    if (e == cudaSuccess) {
        const ClassBuf<W> view = cls.view(cnt.p);
        if constexpr (sizeof(W) == 4) c->launches += launch_setup32(view, sa, c->st);
        else if constexpr (std::is_same<SW, WideWord>::value) c->launches += launch_setup64w(view, sa, c->st);
        else c->launches += launch_setup64(view, sa, c->st);
        e = cudaGetLastError();
    }
    W h0 = 0, h1 = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h0, cls.s0.p, sizeof(W), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h1, cls.s1.p, sizeof(W), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    cls.release(c);
    cnt.release(c);
    CK(e);
    // Montgomery form with R = 2^32 (class 32) or 2^64 -> plain
    const uint64_t rinv = powmod_h(2, (p - 1) - (sizeof(W) == 4 ? 32 : 64), p);
    s0 = mulmod_h((uint64_t)h0, rinv, p);
    s1 = mulmod_h((uint64_t)h1, rinv, p);
    return PFC_OK;
}

extern "C" int pfc_job_verify_tables(pfc_job *j, uint64_t *table_bytes) {
    if (!j) return PFC_ERR_ARG;
    pfc_ctx *c = j->ctx;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->st));
    const uint32_t startN = j->nmin - 1;
    // slow side for the setup programs: k in [2, n0 - 1]
    SlowProducts sp;
    int rc = slow_products(c, 2, (uint64_t)startN + 1, sp);
    if (rc) return rc;
    uint64_t bytes = 0;
    struct Form {
        int form, t;   // setup form, test prime index
        bool built;
    } forms[3] = {{0, 0, j->a32.words.p != nullptr && j->pmin < kClassSplit},
                  {1, 1, j->aw.words.p != nullptr && j->pmax > kClassSplit && j->pmin < kLazyEnd},
                  {2, 2, j->a64.words.p != nullptr && j->pmax > kLazyEnd}};
    for (const Form &f : forms) {
        if (!f.built) continue;
        const uint64_t p = kVerifyPrime[f.t];
        uint64_t s0 = 0, s1 = 0;
        if (f.form == 0) {
            rc = setup_on_prime<uint32_t, WideWord>(j, j->a32, j->b32, p, s0, s1);
            bytes += (j->a32.words.n + j->b32.words.n) * sizeof(WideWord);
        } else if (f.form == 1) {
            rc = setup_on_prime<uint64_t, WideWord>(j, j->aw, j->bw, p, s0, s1);
            bytes += (j->aw.words.n + j->bw.words.n) * sizeof(WideWord);
        } else {
            rc = setup_on_prime<uint64_t, uint64_t>(j, j->a64, j->b64, p, s0, s1);
            bytes += (j->a64.words.n + j->b64.words.n) * 8;
        }
        if (rc) return rc;
        const uint64_t P = sp.P[f.t], C = sp.C[f.t], F = mulmod_h(P, C, p);
        bool ok;
        switch (j->mode) {
            case PFC_FACTORIAL: ok = s0 == F; break;
            case PFC_PRIMORIAL: ok = s0 == P; break;
            case PFC_COMPOSITORIAL: ok = s0 == C; break;
            default: ok = s0 == F && s1 == C; break;
        }
        if (!ok) return PFC_ERR_VALIDATION;
    }
    // walk tables of [nmin, nmax): the primorial's prime list, the
    // compositorial's prime flags, read back from the device
    if (j->mode != PFC_FACTORIAL && j->nmax > j->nmin) {
        SlowProducts rp;
        rc = slow_products(c, j->nmin, j->nmax, rp);
        if (rc) return rc;
        const uint64_t p = kVerifyPrime[2];
        uint64_t prod = 1, count = 0;
        if (j->mode == PFC_PRIMORIAL) {
            std::vector<uint32_t> q(j->h_qlist.size());
            if (!q.empty())
                CK(cudaMemcpy(q.data(), j->qlist.p, q.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            for (uint32_t v : q) prod = mulmod_h(prod, v, p);
            count = q.size();
            bytes += q.size() * 4;
        } else {
            std::vector<uint32_t> bits(j->primebits.n);
            CK(cudaMemcpy(bits.data(), j->primebits.p, bits.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            for (uint32_t k = 0; k < j->nmax - j->nmin; ++k)
                if ((bits[k >> 5] >> (k & 31)) & 1u) {
                    prod = mulmod_h(prod, j->nmin + k, p);
                    ++count;
                }
            bytes += bits.size() * 4;
        }
        if (count != rp.count || prod != rp.P[2]) return PFC_ERR_VALIDATION;
    }
    if (table_bytes) *table_bytes = bytes;
    return PFC_OK;
}

// ------------------------------------------------------------- autotuning

extern "C" int pfc_ctx_set_walk_variant(pfc_ctx *c, int cls, int fused, int variant) {
    if (!c || cls < 0 || cls > 2 || fused < 0 || fused > 1) return PFC_ERR_ARG;
    if (variant < 0 || variant >= walk_variant_count(cls, fused != 0)) return PFC_ERR_ARG;
    c->walk_var[cls][fused] = variant;
    return PFC_OK;
}

extern "C" int pfc_ctx_walk_variant(pfc_ctx *c, int cls, int fused, int *variant, int *nc, int *block) {
    if (!c || cls < 0 || cls > 2 || fused < 0 || fused > 1) return PFC_ERR_ARG;
    const int v = c->walk_var[cls][fused];
    int n = 0, b = 0;
    if (walk_variant_shape(cls, fused != 0, v, &n, &b)) return PFC_ERR_ARG;
    if (variant) *variant = v;
    if (nc) *nc = n;
    if (block) *block = b;
    return PFC_OK;
}

// Time every walk variant of one size class and walk kind on a synthetic
// search (the production kernels, one n-window per trial, best of three) and
// keep the fastest.
static int tune_one(pfc_ctx *c, int cls, int fused, char *report, size_t cap, size_t *used) {
    const int nv = walk_variant_count(cls, fused != 0);
    if (nv < 2) return PFC_OK;
    constexpr uint32_t kWin = 8192, kReps = 3;
    const uint32_t nmin = 101, nmax = nmin + kWin * (1 + nv * kReps);
    const uint64_t lo = cls == 0 ? 1000000000ull : (1ull << 40);
    const uint64_t hi = lo + (cls == 0 ? 5000000ull : 7000000ull);   // ~2.4e5 candidates
    pfc_job *j = nullptr;
    int rc = pfc_job_create(c, fused ? (PFC_FACTORIAL | PFC_COMPOSITORIAL) : PFC_FACTORIAL, nmin, nmax, lo, hi, &j);
    if (rc) return rc;
    rc = pfc_gen_candidates(j, lo, hi);
    if (!rc) rc = pfc_setup(j);
    const int saved = c->walk_var[cls][fused];
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (!rc && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) rc = PFC_ERR_CUDA;
    uint32_t n = nmin;
    if (!rc) rc = pfc_iterate(j, n, n + kWin);  // warm-up
    n += kWin;
    std::vector<float> best(nv, 1e30f);
    for (uint32_t r = 0; r < kReps && !rc; ++r)
        for (int v = 0; v < nv && !rc; ++v) {
            c->walk_var[cls][fused] = v;
            cudaEventRecord(e0, c->st);
            rc = pfc_iterate(j, n, n + kWin);
            cudaEventRecord(e1, c->st);
            n += kWin;
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = PFC_ERR_CUDA;
            float ms = 0;
            if (!rc) cudaEventElapsedTime(&ms, e0, e1);
            best[v] = std::min(best[v], ms);
        }
    int pick = saved;
    if (!rc) {
        pick = 0;
        for (int v = 1; v < nv; ++v)
            if (best[v] < best[pick]) pick = v;
        static const char *names[3] = {"class32", "class64-lazy", "class64"};
        for (int v = 0; v < nv; ++v) {
            int vn = 0, vb = 0;
            walk_variant_shape(cls, fused != 0, v, &vn, &vb);
            if (report && *used < cap)
                *used += snprintf(report + *used, cap - *used, "%s %s nc=%d b=%d %.3f ms%s\n", names[cls],
                                  fused ? "fused" : "single", vn, vb, best[v], v == pick ? " *" : "");
        }
    }
    c->walk_var[cls][fused] = pick;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    pfc_job_destroy(j);
    return rc;
}

extern "C" int pfc_autotune(pfc_ctx *c, char *report, size_t cap) {
    if (!c) return PFC_ERR_ARG;
    CK(cudaSetDevice(c->device));
    size_t used = 0;
    if (report && cap) report[0] = 0;
    for (int cls = 0; cls < 2; ++cls)
        for (int fused = 0; fused < 2; ++fused) {
            const int rc = tune_one(c, cls, fused, report, cap, &used);
            if (rc) return rc;
        }
    return PFC_OK;
}

extern "C" int pfc_ctx_set_graphs(pfc_ctx *c, int on) {
    if (!c) return PFC_ERR_ARG;
    c->graphs = on != 0;
    return PFC_OK;
}

extern "C" int pfc_ctx_set_split(pfc_ctx *c, int on) {
    if (!c) return PFC_ERR_ARG;
    c->split = on != 0;
    return PFC_OK;
}

extern "C" int pfc_ctx_set_setup_tc(pfc_ctx *c, int on) {
    if (!c) return PFC_ERR_ARG;
    c->setup_tc = on != 0;
    return PFC_OK;
}
