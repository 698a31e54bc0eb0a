// batch.cu -- many sieve jobs on the GPU at once: the batch kernel and the
// iteration-level scheduler behind pfc_batch_* (continuous batching).
//
// The reference runs one search per process and one kernel per stage
// (cl_sieve.cpp:1563-1726); a small search there leaves most of a large GPU
// idle.  Here every admitted job contributes blocks of candidates (256, or 512
// for two-candidate class-32 walks and for class-32 setup windows, which run
// one candidate per thread in CTAs of 512).  Each block has a timeline: its setup
// programs as a table of runs ([0, S): squarings, table words, the fork of
// the combined search), then its walk ([S, S+N): n steps, or prime steps for
// n#).  All blocks of a job share one position.  One iteration gives every
// running job (or, under the latency policy, every job the budget pays for)
// a window of its timeline; the iteration's windows, sorted by task cost, are
// one launch per class group (class 32, class 64 below 2^64/3, other class 64)
// and task kind (setup, walk, general) with one CTA per block, on six
// streams, dispatched by the hardware block scheduler, so jobs of every size
// and mode share the SMs.
// Between iterations the host admits new jobs as memory and slots allow,
// drains the hits (tagged with the job slot) and retires finished jobs:
// requests that arrive while others run join at the next iteration.
//
// Results equal the per-job path bit for bit: the same arithmetic (walk.cuh),
// the same setup programs evaluated in the same order, and the same check
// terms.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <thread>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "devmem.hpp"
#include "walk.cuh"

namespace pfc {

// ------------------------------------------------------------- device side

// One run of a setup program's timeline: `n` squarings (kind 0), `n` table
// words from words[a] (kind 1), or the fork of the combined search (kind 2:
// the compositorial residue is complete).  The runs of a search tile its
// setup positions [0, nsetup) in order; `start` is the first position.
struct SetupSeg {
    uint32_t start, kind, a, n;
};

template <class W>
struct JobDev {
    unsigned mode;
    uint32_t nmin, nlast;     // first n; nmax - 1
    uint32_t nsetup, nwalk;   // timeline: [0, nsetup) setup positions, then nwalk walk steps
    const SetupSeg *segs;     // runs of the setup timeline
    uint32_t nsegs;
    const void *words;        // table words of the setup programs (the class's setup word type)
    uint64_t corr_a, corr_b;  // drift corrections (first program; second of the combined search)
    const uint32_t *cmult;    // compositorial multipliers of [nmin, nmax)
    const uint32_t *qlist;    // primorial: primes in [nmin, nmax)
    ClassBuf<W> c;
    unsigned long long *termsum;
    uint32_t *flags;
};

struct BatchStats {  // one per job slot
    uint32_t counts[2];
    uint32_t flags;
    uint32_t pad;
    unsigned long long termsum;
};

struct Task {
    uint32_t slot, first, count, lo, hi;
};

// One iteration's window of one search in one size class: CTAs
// [first_cta, first_cta + nblocks) take the search's candidate blocks in
// order, each over timeline positions [lo, hi).  All blocks of a search
// share one position (they advance together), so an iteration is described
// by one window per search and class, not one record per block.
struct Window {
    uint32_t first_cta, nblocks, slot, ncand, lo, hi, pad0, pad1;
};

// Setup positions [lo, hi) of NC candidates: acc advances through the
// program, fork receives the compositorial residue at the fork.  Same
// operations as run_prog in the same order, resumable at any position.
template <class T, int NC, bool FUSED>
__device__ __forceinline__ void run_setup(const typename T::M (&m)[NC], typename T::W (&acc)[NC],
                                          typename T::W (&fork)[NC], const JobDev<typename T::W> &J, uint32_t lo,
                                          uint32_t hi) {
    using W = typename T::W;
    typename T::SC sc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) sc[c] = T::sctx(m[c]);
    uint32_t a = 0, b = J.nsegs;  // segs[a].start <= lo
    while (b - a > 1) {
        const uint32_t mid = (a + b) >> 1;
        if (__ldg(&J.segs[mid].start) <= lo) a = mid;
        else b = mid;
    }
    uint32_t pos = lo;
    for (uint32_t s = a; pos < hi && s < J.nsegs; ++s) {
        const uint4 g = __ldg(reinterpret_cast<const uint4 *>(J.segs + s));  // start, kind, a, n
        const uint32_t off = pos - g.x;
        const uint32_t len = g.y == 2 ? 1u : g.w;
        const uint32_t cnt = min(len - off, hi - pos);
        if (g.y == 0) {
            for (uint32_t k = 0; k < cnt; ++k) {
#pragma unroll
                for (int c = 0; c < NC; ++c) acc[c] = T::sq(m[c], acc[c]);
            }
        } else if (g.y == 1) {
            using SW = typename T::SW;
            const SW *wp = static_cast<const SW *>(J.words) + g.z + off;
            uint32_t k = 0;
            if constexpr (std::is_same<SW, WideWord>::value) {
                // Every thread of the CTA walks the same words: the CTA copies
                // kStageWords of them at a time into shared memory with one
                // coalesced load, and the threads read the limbs from there
                // (a table word read from global memory by every warp waited
                // on its loads: the pointer comes from the job record, so the
                // address is not known to be warp-uniform).  Trip counts are
                // uniform across the CTA, so every thread reaches the barriers.
                constexpr uint32_t kStageWords = 16, kVec = sizeof(WideWord) / 16;
                __shared__ uint4 stage[kStageWords * kVec];
                const uint4 *src = reinterpret_cast<const uint4 *>(wp);
                for (; k < cnt; k += kStageWords) {
                    const uint32_t nw = min(kStageWords, cnt - k);
                    __syncthreads();   // the previous chunk is consumed
                    for (uint32_t i = threadIdx.x; i < nw * kVec; i += blockDim.x)
                        stage[i] = __ldg(src + (size_t)k * kVec + i);
                    __syncthreads();
                    for (uint32_t u = 0; u < nw; ++u) {
                        const SW *sp = reinterpret_cast<const SW *>(stage + u * kVec);
#pragma unroll
                        for (int c = 0; c < NC; ++c) acc[c] = T::template word<true>(m[c], sc[c], acc[c], sp);
                    }
                }
            } else {
                constexpr uint32_t U = 4;
                for (; k + U <= cnt; k += U) {
                    SW wv[U];
#pragma unroll
                    for (uint32_t u = 0; u < U; ++u) wv[u] = ldg(wp + k + u);
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
#pragma unroll
                        for (uint32_t u = 0; u < U; ++u) acc[c] = T::word(m[c], sc[c], acc[c], wv[u]);
                    }
                }
                for (; k < cnt; ++k) {
                    const SW w = ldg(wp + k);
#pragma unroll
                    for (int c = 0; c < NC; ++c) acc[c] = T::word(m[c], sc[c], acc[c], w);
                }
            }
        } else {
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                acc[c] = m[c].mul(acc[c], m[c].mont_R_pow(J.corr_a));
                fork[c] = acc[c];
            }
        }
        pos += cnt;
    }
}

// Task kinds: a window inside a search's setup that does not end its
// timeline, a window inside its walk, or any other (the one that crosses from
// setup to walk, or that ends a timeline without walk steps).  The batch
// kernel is compiled per kind so that setup-only and walk-only launches carry
// only their own code and registers.
enum TaskKind { kAnyTask = 0, kSetupTask = 1, kWalkTask = 2 };

template <class T, int NC, bool FUSED, int KIND>
__device__ void run_task(const JobDev<typename T::W> &J, const Task &t, const HitBuf &h) {
    using W = typename T::W;
    constexpr int NS = FUSED ? 2 : NC;
    uint32_t idx[NC];
    bool act[NC];
    typename T::M m[NC];
    const uint32_t end = t.first + t.count;
#pragma unroll
    for (int s = 0; s < NC; ++s) {
        idx[s] = t.first + s * blockDim.x + threadIdx.x;
        act[s] = idx[s] < end;
        m[s].init(act[s] ? J.c.p[idx[s]] : (W)3);
    }
    const uint32_t S = J.nsetup, N = J.nwalk;
    W x[NS];
    uint32_t walked = 0;
    if (KIND != kWalkTask && t.lo < S) {
        // setup part: positions [lo, min(hi, S)) of the job's programs
        W acc[NC], fork[NC];
#pragma unroll
        for (int s = 0; s < NC; ++s) {
            acc[s] = t.lo == 0 ? m[s].one : (act[s] ? J.c.s0[idx[s]] : (W)0);
            fork[s] = (FUSED && t.lo > 0 && act[s]) ? J.c.s1[idx[s]] : (W)0;
        }
        const uint32_t e = min(t.hi, S);
        run_setup<T, NC, FUSED>(m, acc, fork, J, t.lo, e);
        if (e == S) {
#pragma unroll
            for (int s = 0; s < NC; ++s) acc[s] = m[s].mul(acc[s], m[s].mont_R_pow(FUSED ? J.corr_b : J.corr_a));
        }
        if (KIND == kSetupTask || e < S || (t.hi == S && N > 0)) {  // the walk starts in a later task
#pragma unroll
            for (int s = 0; s < NC; ++s)
                if (act[s]) {
                    J.c.s0[idx[s]] = acc[s];
                    if (FUSED) J.c.s1[idx[s]] = fork[s];
                    J.c.nnext[idx[s]] = 0;
                }
            return;
        }
        if (FUSED) {
            x[0] = acc[0];
            x[NS - 1] = fork[0];
        } else {
#pragma unroll
            for (int s = 0; s < NC; ++s) x[s] = acc[s];
        }
    } else {
        if (FUSED) {
            x[0] = act[0] ? J.c.s0[idx[0]] : 0;
            x[NS - 1] = act[0] ? J.c.s1[idx[0]] : 0;
        } else {
#pragma unroll
            for (int s = 0; s < NC; ++s) x[s] = act[s] ? J.c.s0[idx[s]] : 0;
        }
        walked = act[0] ? J.c.nnext[idx[0]] : 0;
    }

    // walk part: steps [max(lo, S) - S, hi - S) of the job's walk
    const uint32_t wlo = max(t.lo, S) - S, whi = t.hi - S;
    if (whi > wlo) {
        WalkArgs a;
        const bool prim = J.mode == PFC_PRIMORIAL;
        const uint32_t base = prim ? 0u : J.nmin;
        a.lo = base + wlo;
        a.hi = base + whi;
        a.base = base;
        a.mult = nullptr;
        a.mult2 = nullptr;
        a.chain = 0;
        a.type = a.type2 = 0;
        if (FUSED) {
            a.mult2 = J.cmult;
            a.type = PFC_TYPE_FACTORIAL;
            a.type2 = PFC_TYPE_COMPOSITORIAL;
        } else if (prim) {
            a.mult = J.qlist;
            a.type = PFC_TYPE_PRIMORIAL;
        } else if (J.mode == PFC_COMPOSITORIAL) {
            a.mult = J.cmult;
            a.type = PFC_TYPE_COMPOSITORIAL;
        } else {
            a.type = PFC_TYPE_FACTORIAL;
        }
        // the lazy class-64 walk kind in blocks of 32, as the per-job default
        // (fewer block restores; 75.4 against 76.9 ms per-job on the
        // primorial near 2^62); the others in the class's default blocks
        constexpr int WB = (KIND == kWalkTask && std::is_same<T, Cls64L>::value && !FUSED)
                               ? 32
                               : (FUSED ? T::B_FUSED : T::B);
        walk_streams<T, NC, FUSED, WB>(m, x, act, a, h);
        if (!FUSED && NC > 1) {
            // walked counts are equal for the candidates of one thread
        }
        walked += (whi - wlo) * (FUSED ? 2u : 1u);
    }

    if (t.hi < S + N) {
#pragma unroll
        for (int s = 0; s < NC; ++s)
            if (act[s]) {
                J.c.s0[idx[s]] = FUSED ? x[0] : x[s];
                if (FUSED) J.c.s1[idx[s]] = x[NS - 1];
                J.c.nnext[idx[s]] = walked;
            }
        return;
    }

    // last task of the block: checksum terms (check.cl:59,115,161) and the
    // step-count check of every candidate
    unsigned long long term = 0;
    bool bad = false;
#pragma unroll
    for (int s = 0; s < NC; ++s) {
        if (!act[s]) continue;
        const W x0 = FUSED ? x[0] : x[s];
        term += T::term(m[s], x0);
        if (J.mode != PFC_PRIMORIAL) term += T::mont64_of(m[s], J.nlast);
        if (FUSED) term += T::term(m[s], x[NS - 1]);
        bad |= walked != N * (FUSED ? 2u : 1u);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) term += __shfl_down_sync(kFull, term, o);
    if ((threadIdx.x & 31) == 0 && term) atomicAdd(J.termsum, term);
    if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0) atomicOr(J.flags, 1u);
}

// One CTA per task (a block of 256 candidates, 512 for two-candidate class-32
// walks, over one window).  The windows of an iteration are ordered by the
// cost of their tasks, longest first, and the hardware block scheduler hands
// CTAs to SMs as slots free up: a device-side work queue whose tail is spread
// over all SMs.  (A persistent grid taking tasks from an atomic counter let
// the last tasks of an iteration crowd onto a few SMs: 78% of the per-job
// path's throughput on a single large search, against 100% with hardware
// dispatch.)  Thread 0 finds its window by binary search over first_cta.
//
// CTAs per SM by kind (register budgets at 256 threads: 4 -> 64, 3 -> 85,
// 2 -> 128): setup with 64-bit words at four; setup with 896-bit words holds
// 32 position residues per candidate (two candidates per thread in class 32)
// and the general kind both setup and walk state; walks as measured per class.
template <class T, int KIND>
constexpr int batch_min_ctas() {
    if (KIND == kSetupTask) return std::is_same<typename T::SW, WideWord>::value ? 2 : 4;
    if (KIND == kAnyTask || sizeof(typename T::W) == 4) return 2;
    return T::B > 8 ? 3 : 2;
}

// Class-32 setup windows run one candidate per thread in CTAs of 512 (the
// shape of setup_kernel: 64 registers, 32 warps per SM); the two-candidate
// form at 256 threads ran a setup-bound search at half that speed.  Every
// other kind: 256 threads, T::NC candidates per thread (one in the fused walk).
template <class T, int KIND>
__host__ __device__ constexpr bool setup32_shape() { return KIND == kSetupTask && sizeof(typename T::W) == 4; }
template <class T, int KIND>
__host__ __device__ constexpr int task_threads() { return setup32_shape<T, KIND>() ? 512 : 256; }
template <class T, int KIND>
__host__ __device__ constexpr int task_nc() { return setup32_shape<T, KIND>() ? 1 : T::NC; }

template <class T, int KIND>
__global__ void __launch_bounds__(task_threads<T, KIND>(), setup32_shape<T, KIND>() ? 2 : batch_min_ctas<T, KIND>())
    batch_kernel(const Window *wins, uint32_t nwins, const JobDev<typename T::W> *jobs, HitBuf h) {
    // the task and its search record live in shared memory: every thread
    // reads the same fields, and registers stay free for the residues
    __shared__ Task st;
    __shared__ JobDev<typename T::W> sj;
    if (threadIdx.x == 0) {
        uint32_t a = 0, b = nwins;  // wins[a].first_cta <= blockIdx.x
        while (b - a > 1) {
            const uint32_t mid = (a + b) >> 1;
            if (wins[mid].first_cta <= blockIdx.x) a = mid;
            else b = mid;
        }
        const Window w = wins[a];
        sj = jobs[w.slot];
        const uint32_t per = (sj.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL) ? 1u : (uint32_t)task_nc<T, KIND>()) * blockDim.x;
        st.slot = w.slot;
        st.first = (blockIdx.x - w.first_cta) * per;
        st.count = min(per, w.ncand - st.first);
        st.lo = w.lo;
        st.hi = w.hi;
    }
    __syncthreads();
    HitBuf hh = h;
    hh.tagval = st.slot;
    if (sj.mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL)) run_task<T, 1, true, KIND>(sj, st, hh);
    else run_task<T, task_nc<T, KIND>(), false, KIND>(sj, st, hh);
}

// ------------------------------------------------------------------ host side

// queued -> prepared (host tables built) -> ready (on the device, candidates
// generated) -> running (blocks in the task list) -> done
enum JobState { kQueued = 0, kPrepared, kReady, kRunning, kDone };

struct BatchJob {
    uint64_t id = 0;
    unsigned mode = 0;
    uint32_t nmin = 0, nmax = 0;
    uint64_t pmin = 0, pmax = 0;
    int state = kQueued;
    uint32_t slot = 0;
    // host tables, built by prepare_job
    int prep_rc = PFC_OK;
    std::vector<WideWord> words32;     // class 32
    std::vector<uint32_t> cmult, qlist;
    std::vector<uint64_t> words64;   // class 64 at or above 2^64/3
    std::vector<WideWord> wordsw;      // class 64 below 2^64/3
    std::vector<SetupSeg> segs32, segs64;
    uint32_t nsetup32 = 0, nsetup64 = 0;
    // class 32 and class 64 below 2^64/3 on the tensor cores: the wide
    // programs' groups (first program's, then the second's) and their shapes
    bool tc = false;
    // per size class (0: class 32, 1: class 64 below 2^64/3)
    bool tc_wait[2] = {false, false};    // its setup is still running (no window of the class yet)
    cudaEvent_t tc_ev0[2] = {}, tc_ev1[2] = {};   // around that setup (throughput policy)
    uint32_t tc_block[2] = {0, 0}, tc_blocks[2] = {0, 0};   // latency policy: next candidate block, blocks
    uint64_t tc_iter[2] = {0, 0};    // iteration that launched the last blocks
    double tc_block_cost[2] = {0, 0};   // budget units (multiplies) per block
    SetupArgs<WideWord> tc_args{};   // the setup launch (programs, tiles), both classes
    TcTiles tc_ta{}, tc_tb{};
    // (the paired programs, host.hpp TcProg: word sources and groups of the
    // first program then the second's; tc_nw counts the 896-bit words of the
    // first program, tc_pw the paired words of each)
    std::vector<uint32_t> tcsrc, tcgroups;
    uint32_t tc_ng[2] = {0, 0}, tc_fsq[2] = {0, 0}, tc_nw[2] = {0, 0}, tc_pw[2] = {0, 0}, tc_ntiles[2] = {0, 0};
    uint64_t tc_corr[2] = {0, 0};
    uint64_t c32a = 0, c32b = 0, c64a = 0, c64b = 0;
    uint32_t nwalk = 0;
    bool use32 = false, use64 = false;
    uint32_t cap32 = 0, cap64 = 0;
    // device
    DArr<WideWord> d_words32;
    DArr<uint32_t> d_cmult, d_qlist;
    DArr<uint64_t> d_words64;
    DArr<WideWord> d_wordsw;
    DArr<uint32_t> d_tcgroups, d_tcsrc;
    DArr<uint8_t> d_tct;            // fp16 tiles of the wide programs
    DArr<SetupSeg> d_segs32, d_segs64;
    DevClass<uint32_t> c32;
    DevClass<uint64_t> c64;
    uint32_t n32 = 0, n64 = 0;      // candidates per class
    uint32_t pos32 = 0, pos64 = 0;  // timeline position of all blocks of a class
    uint32_t next32 = 0, next64 = 0;  // end of the window in flight
    uint32_t tot32 = 0, tot64 = 0;  // timeline lengths (setup positions + walk steps)
    uint32_t win = 0;               // this iteration's window (0: the common window L)
    bool wait = false;              // latency policy: no window this iteration
    uint32_t waited = 0;            // consecutive iterations without a window
    // results
    uint64_t termsum = 0, primecount = 0;
    uint32_t flags = 0;
    bool rerun = false;
    int status = PFC_OK;
    std::vector<pfc_factor> hits;
};

static double est_cands(uint64_t lo, uint64_t hi) {
    if (hi <= lo) return 0;
    const double a = (double)std::max<uint64_t>(lo, 114);
    return (double)(hi - lo) / std::log(a) * 1.25 + 30.0;
}

// append a setup program's runs (and words) to a search's timeline; returns
// the next position
template <class W>
static uint32_t append_prog(const HostProg<W> &h, uint32_t pos, std::vector<SetupSeg> &segs, std::vector<W> &words) {
    const uint32_t wbase = (uint32_t)words.size();
    words.insert(words.end(), h.words.begin(), h.words.end());
    for (size_t g = 0; g + 2 < h.groups.size(); g += 3) {
        const uint32_t b = h.groups[g], e = h.groups[g + 1], sq = h.groups[g + 2];
        if (sq) {
            segs.push_back({pos, 0u, 0u, sq});
            pos += sq;
        }
        if (e > b) {
            segs.push_back({pos, 1u, wbase + b, e - b});
            pos += e - b;
        }
    }
    if (h.final_sq) {
        segs.push_back({pos, 0u, 0u, h.final_sq});
        pos += h.final_sq;
    }
    return pos;
}

// the setup programs of a search for one word type (as pfc_job_create)
template <class W>
static bool build_progs(unsigned mode, uint32_t startN, const std::vector<uint32_t> &primes,
                        const std::vector<uint32_t> &below, HostProg<W> &a, HostProg<W> &b) {
    if (mode == PFC_FACTORIAL) return build_power_prog(startN, 0, primes, a);
    if (mode == PFC_COMPOSITORIAL) return build_power_prog(startN, 1, primes, a);
    if (mode == PFC_PRIMORIAL) return build_product_prog(below, a);
    return build_power_prog(startN, 1, primes, a) && build_product_prog(below, b);
}

static uint32_t prime_limit(const BatchJob *j) {
    const uint32_t startN = j->nmin - 1;
    return (j->mode & PFC_COMPOSITORIAL) ? j->nmax : std::max(startN, j->nmax - 1);
}

// Host tables of one search: the same programs, prime lists and multiplier
// table pfc_job_create builds (from the batch's shared prime list).
static void prepare_job(BatchJob *j, const std::vector<uint32_t> &cache) {
    const uint32_t startN = j->nmin - 1;
    const std::vector<uint32_t> primes(cache.begin(), std::upper_bound(cache.begin(), cache.end(), prime_limit(j)));
    const std::vector<uint32_t> below(primes.begin(), std::upper_bound(primes.begin(), primes.end(), startN));
    const unsigned mode = j->mode;
    const bool fc = mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL);
    const bool wide = j->pmax <= kLazyEnd;  // class 64 with 896-bit words
    HostProg<WideWord> a32, b32;
    HostProg<uint64_t> a64, b64;
    HostProg<WideWord> aw, bw;
    const bool ok = build_progs(mode, startN, primes, below, a32, b32) &&
                    (wide ? build_progs(mode, startN, primes, below, aw, bw)
                          : build_progs(mode, startN, primes, below, a64, b64));
    if (!ok) {
        j->prep_rc = PFC_ERR_ARG;
        return;
    }
    j->nsetup32 = append_prog(a32, 0, j->segs32, j->words32);
    j->nsetup64 = wide ? append_prog(aw, 0, j->segs64, j->wordsw) : append_prog(a64, 0, j->segs64, j->words64);
    j->c32a = a32.corr;
    j->c64a = wide ? aw.corr : a64.corr;
    if (wide) {
        const HostProg<WideWord> *pr[2] = {&aw, &bw};
        j->tc = true;
        for (int k = 0; k < (fc ? 2 : 1); ++k) {
            TcProg tp;
            if (!build_tc_prog(*pr[k], tp)) {
                j->tc = false;
                break;
            }
            j->tcsrc.insert(j->tcsrc.end(), tp.src.begin(), tp.src.end());
            j->tcgroups.insert(j->tcgroups.end(), tp.groups.begin(), tp.groups.end());
            j->tc_ng[k] = (uint32_t)(tp.groups.size() / 3);
            j->tc_fsq[k] = tp.final_sq;
            j->tc_corr[k] = tp.corr;
            j->tc_nw[k] = (uint32_t)pr[k]->words.size();
            j->tc_pw[k] = (uint32_t)tp.src.size();
            j->tc_ntiles[k] = (j->tc_pw[k] + tc_tile_words() - 1) / tc_tile_words();
        }
    }
    if (fc) {
        // fork: the compositorial residue is complete here
        j->segs32.push_back({j->nsetup32++, 2u, 0u, 1u});
        j->segs64.push_back({j->nsetup64++, 2u, 0u, 1u});
        j->nsetup32 = append_prog(b32, j->nsetup32, j->segs32, j->words32);
        j->nsetup64 = wide ? append_prog(bw, j->nsetup64, j->segs64, j->wordsw)
                           : append_prog(b64, j->nsetup64, j->segs64, j->words64);
        j->c32b = b32.corr;
        j->c64b = wide ? bw.corr : b64.corr;
    }
    if (mode & PFC_COMPOSITORIAL) {
        // n at composite n, 1 at prime n (iterate.cl:137-140, 181-184), padded for vector loads
        const std::vector<uint32_t> pb = prime_bitmap(j->nmin, j->nmax, primes);
        j->cmult.assign((size_t)(j->nmax - j->nmin) + 16, 1u);
        for (uint32_t k = 0; k < j->nmax - j->nmin; ++k)
            if (!((pb[k >> 5] >> (k & 31)) & 1u)) j->cmult[k] = j->nmin + k;
        j->nwalk = j->nmax - j->nmin;
    } else if (mode == PFC_PRIMORIAL) {
        j->qlist.assign(std::lower_bound(primes.begin(), primes.end(), j->nmin),
                        std::lower_bound(primes.begin(), primes.end(), j->nmax));
        j->nwalk = (uint32_t)j->qlist.size();
        j->qlist.resize(j->qlist.size() + 32, 1u);
    } else {
        j->nwalk = j->nmax - j->nmin;
    }
    j->use32 = j->pmin < kClassSplit;
    j->use64 = j->pmax > kClassSplit;
    const double e32 = est_cands(j->pmin, std::min<uint64_t>(j->pmax, kClassSplit));
    const double e64 = est_cands(std::max<uint64_t>(j->pmin, kClassSplit), j->pmax);
    j->cap32 = j->use32 ? (uint32_t)std::min(e32, 4.0e9) : 0;
    j->cap64 = j->use64 ? (uint32_t)std::min(e64, 4.0e9) : 0;
    j->tot32 = j->nsetup32 + j->nwalk;
    j->tot64 = j->nsetup64 + j->nwalk;
    j->prep_rc = PFC_OK;
}

template <class W>
static void free_vec(std::vector<W> &v) {
    std::vector<W>().swap(v);
}

}  // namespace pfc

using namespace pfc;

// a tensor-core setup tile of one candidate block (128 paired words x 32
// candidates, about 9,000 SM cycles) in the budget's units: multiplies at
// 64 per SM cycle
constexpr double kTcTileCost = 9000.0 * 64.0;
// share of a latency-policy iteration's budget given to setup chunks
constexpr double kTcChunkShare = 0.5;

// default work of one iteration in candidate-steps, per policy
constexpr double kThroughputIterWork = 1.6e12;
constexpr double kLatencyIterWork = 5e10;

struct pfc_batch {
    pfc_ctx *ctx = nullptr;
    static constexpr uint32_t kSlots = 4096;
    // one launch list per class group (class 32, class 64 below 2^64/3, other
    // class 64) and task kind, one stream per size class and kind
    static constexpr int kLists = 3, kKinds = 3, kStreams = 6;
    cudaStream_t st[kStreams] = {};
    cudaEvent_t ev = nullptr;
    DArr<BatchStats> stats;
    DArr<JobDev<uint32_t>> jobs32;
    DArr<JobDev<uint64_t>> jobs64;
    // task lists: class 32, class 64 below 2^63 (lazy walk), other class 64
    DArr<Window> wins[kLists][kKinds];
    DArr<pfc_factor> hits;
    DArr<uint32_t> tags;
    DArr<unsigned long long> hitcount;
    BatchStats *h_stats = nullptr;       // pinned mirror of `stats`
    unsigned long long *h_hitcount = nullptr;
    std::map<uint64_t, std::unique_ptr<BatchJob>> all;
    std::deque<BatchJob *> queued;       // kQueued and kPrepared, in arrival order
    std::vector<BatchJob *> ready;       // kReady: join the next iteration
    std::vector<BatchJob *> running;     // kRunning
    std::vector<uint32_t> free_slots;
    std::vector<uint32_t> prime_cache;   // primes up to cache_lim
    uint32_t cache_lim = 0;
    std::vector<Window> w[kLists][kKinds];   // this iteration's windows per launch
    uint64_t ctas[kLists][kKinds] = {};
    uint64_t next_id = 1;
    double work_per_iter = 0;            // candidate-steps per iteration (class 64 weighs 3); 0: the policy's
    int policy = PFC_BATCH_THROUGHPUT;
    uint64_t iterations = 0;
    // timing: kernel spans (CUDA events) and host phases (wall clock)
    cudaEvent_t ev_start = nullptr, ev_end[kStreams] = {};
    // tensor-core setups of admitted searches: their own streams, after the
    // uploads (ev_tc0 on the context stream); iterations do not wait for them
    static constexpr int kTcStreams = 4;
    double iter_budget = 0;              // this iteration's budget (multiplies), set by build_tasks
    cudaEvent_t ev_ck0 = nullptr, ev_ck1 = nullptr;   // around an iteration's setup chunks
    bool ck_pending = false;
    cudaStream_t tcst[kTcStreams] = {};
    cudaEvent_t ev_tc0 = nullptr;
    int tc_next = 0;
    double tc_s = 0;                     // summed durations of those setups
    double gpu_s = 0, gpu32_s = 0, gpu64_s = 0, prep_s = 0, admit_s = 0, step_s = 0;
    uint64_t tasks = 0;
    size_t t32_n = 0, t64_n = 0;   // task counts of the iteration in flight
    bool used[kStreams] = {};      // streams with launches in the iteration in flight
    uint32_t prio = 0;             // searches with their own window this iteration
    bool trace = false;            // PFCSIEVE_BATCH_TRACE: one stderr line per iteration
};

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

namespace {

// Build the host tables of the queued searches that have none yet, in
// parallel across searches: at most four per host thread per call (so the
// first iteration starts after a few searches are ready, and the rest are
// prepared while kernels run) and at most as many as there are free slots.
void prepare_queued(pfc_batch *b) {
    std::vector<BatchJob *> todo;
#ifdef _OPENMP
    const size_t per_call = 4 * (size_t)omp_get_max_threads();
#else
    const size_t per_call = 4;
#endif
    size_t room = std::min(b->free_slots.size(), per_call);
    for (BatchJob *j : b->queued) {
        if (todo.size() >= room) break;
        if (j->state == kQueued) todo.push_back(j);
    }
    if (todo.empty()) return;
    uint32_t lim = 0;
    for (BatchJob *j : todo) lim = std::max(lim, prime_limit(j));
    if (lim > b->cache_lim) {
        const uint32_t want = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(lim, 2ull * b->cache_lim), 0x7FFFFFFFu);
        b->prime_cache = primes_between(2, want);
        b->cache_lim = want;
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t k = 0; k < (int64_t)todo.size(); ++k) prepare_job(todo[k], b->prime_cache);
    for (BatchJob *j : todo) j->state = kPrepared;
}

void release_device(pfc_batch *b, BatchJob *j) {
    pfc_ctx *c = b->ctx;
    j->d_words32.release(c);
    j->d_words64.release(c);
    j->d_wordsw.release(c);
    j->d_tcgroups.release(c);
    j->d_tcsrc.release(c);
    j->d_tct.release(c);
    for (int k = 0; k < 2; ++k) {
        if (j->tc_ev0[k]) cudaEventDestroy(j->tc_ev0[k]);
        if (j->tc_ev1[k]) cudaEventDestroy(j->tc_ev1[k]);
        j->tc_ev0[k] = j->tc_ev1[k] = nullptr;
        j->tc_wait[k] = false;
    }
    j->d_segs32.release(c);
    j->d_segs64.release(c);
    j->d_cmult.release(c);
    j->d_qlist.release(c);
    j->c32.release(c);
    j->c64.release(c);
}

int launch_job_gen(pfc_batch *b, BatchJob *j) {
    pfc_ctx *c = b->ctx;
    BatchStats *st = b->stats.p + j->slot;
    CK(cudaMemsetAsync(st, 0, sizeof(BatchStats), c->st));
    GenArgs g;
    memset(&g, 0, sizeof(g));
    const uint64_t base = j->pmin | 1;
    g.base = base;
    g.nodd = j->pmax > base ? (j->pmax - base + 1) / 2 : 0;
    g.p32 = j->c32.p.p;
    g.p64 = j->c64.p.p;
    g.cap32 = j->use32 ? j->c32.cap : 0;
    g.cap64 = j->use64 ? j->c64.cap : 0;
    g.count = st->counts;
    g.pat = c->d_pat;
    static const uint32_t sp[kSmallPrimes] = {3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37,  41,  43,  47,  53,
                                              59, 61, 67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113};
    for (int k = 0; k < kSmallPrimes; ++k) g.bmod[k] = (uint32_t)(base % sp[k]);
    c->launches += launch_gen(g, c->sms, c->st);
    CK(cudaGetLastError());
    return PFC_OK;
}

// Device buffers, tables and candidate generation of one prepared search.
// PFC_ERR_NOMEM leaves nothing allocated.
int upload_job(pfc_batch *b, BatchJob *j) {
    pfc_ctx *c = b->ctx;
    cudaError_t e = j->d_words32.upload(c, j->words32);
    if (e == cudaSuccess) e = j->d_words64.upload(c, j->words64);
    if (e == cudaSuccess) e = j->d_wordsw.upload(c, j->wordsw);
    const uint64_t words = (uint64_t)j->tc_nw[0] + j->tc_nw[1];
    const bool tc = j->tc && c->setup_tc &&
                    ((j->use64 && words >= kTcMinWords64) || (j->use32 && words >= kTcMinWords32));
    const size_t tb = tc_tile_bytes(), nt = (size_t)j->tc_ntiles[0] + j->tc_ntiles[1];
    if (e == cudaSuccess && tc) e = j->d_tcgroups.upload(c, j->tcgroups);
    if (e == cudaSuccess && tc) e = j->d_tcsrc.upload(c, j->tcsrc);
    if (e == cudaSuccess && tc) e = j->d_tct.alloc(c, std::max<size_t>(nt * tb, 16));
    if (e == cudaSuccess) e = j->d_segs32.upload(c, j->segs32);
    if (e == cudaSuccess) e = j->d_segs64.upload(c, j->segs64);
    if (e == cudaSuccess) e = j->d_cmult.upload(c, j->cmult);
    if (e == cudaSuccess) e = j->d_qlist.upload(c, j->qlist);
    if (e == cudaSuccess) e = j->c32.ensure(c, j->cap32);
    if (e == cudaSuccess) e = j->c64.ensure(c, j->cap64);
    if (e != cudaSuccess) {
        release_device(b, j);
        return cuda_fail(e);
    }
    if (tc) {
        c->launches += launch_tc_pack(j->d_wordsw.p, j->d_tcsrc.p, j->tc_pw[0], j->tc_ntiles[0], j->d_tct.p, c->st);
        c->launches += launch_tc_pack(j->d_wordsw.p + j->tc_nw[0], j->d_tcsrc.p + j->tc_pw[0], j->tc_pw[1],
                                      j->tc_ntiles[1], j->d_tct.p + (size_t)j->tc_ntiles[0] * tb, c->st);
        CK(cudaGetLastError());
    }
    return launch_job_gen(b, j);
}

template <class W>
JobDev<W> job_view(pfc_batch *b, BatchJob *j, const DevClass<W> &cls, int which, const void *words,
                   const DArr<SetupSeg> &segs, size_t nsegs, uint64_t ca, uint64_t cb, uint32_t nsetup) {
    JobDev<W> d;
    memset(&d, 0, sizeof(d));
    d.mode = j->mode;
    d.nmin = j->nmin;
    d.nlast = j->nmax - 1;
    d.nsetup = nsetup;
    d.nwalk = j->nwalk;
    d.segs = segs.p;
    d.nsegs = (uint32_t)nsegs;
    d.words = words;
    d.corr_a = ca;
    d.corr_b = cb;
    d.cmult = j->d_cmult.p;
    d.qlist = j->d_qlist.p;
    d.c = cls.view(b->stats.p[j->slot].counts + which);
    d.termsum = &b->stats.p[j->slot].termsum;
    d.flags = &b->stats.p[j->slot].flags;
    return d;
}

// The tensor-core setup of one class of a search: candidate blocks
// [block0, block0 + n) (n 0: all), flags into the search's slot.
int tc_launch(pfc_batch *b, BatchJob *j, int cls, cudaStream_t st, uint32_t block0, uint32_t n) {
    BatchStats *bs = b->stats.p + j->slot;   // device address
    return cls ? launch_setup64w_tc(j->c64.view(bs->counts + 1), j->tc_args, j->tc_ta, j->tc_tb, &bs->flags, st, block0, n)
               : launch_setup32_tc(j->c32.view(bs->counts), j->tc_args, j->tc_ta, j->tc_tb, &bs->flags, st, block0, n);
}

// Move prepared searches onto the device while slots and the memory budget
// allow; on return their candidates exist and their blocks are laid out.
int admit_prepared(pfc_batch *b) {
    pfc_ctx *c = b->ctx;
    std::vector<BatchJob *> fresh;
    while (!b->queued.empty() && b->queued.front()->state == kPrepared && !b->free_slots.empty()) {
        BatchJob *j = b->queued.front();
        if (j->prep_rc != PFC_OK) {
            b->queued.pop_front();
            j->state = kDone;
            j->status = j->prep_rc;
            continue;
        }
        j->slot = b->free_slots.back();
        const int rc = upload_job(b, j);
        if (rc == PFC_ERR_NOMEM && !(b->running.empty() && b->ready.empty() && fresh.empty()))
            break;  // waits for running searches to free memory
        b->queued.pop_front();
        if (rc != PFC_OK) {
            release_device(b, j);
            j->state = kDone;
            j->status = rc;
            if (rc != PFC_ERR_NOMEM) return rc;
            continue;
        }
        b->free_slots.pop_back();
        fresh.push_back(j);
    }
    if (fresh.empty()) return PFC_OK;
    // candidate counts; regenerate with exact capacities where an estimate was short
    CK(cudaMemcpyAsync(b->h_stats, b->stats.p, sizeof(BatchStats) * pfc_batch::kSlots, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    bool regen = false;
    for (BatchJob *j : fresh) {
        const BatchStats &s = b->h_stats[j->slot];
        if ((j->use32 && s.counts[0] > j->c32.cap) || (j->use64 && s.counts[1] > j->c64.cap)) {
            CK(j->c32.ensure(c, j->use32 ? s.counts[0] + 1024 : 0));
            CK(j->c64.ensure(c, j->use64 ? s.counts[1] + 1024 : 0));
            const int g = launch_job_gen(b, j);
            if (g) return g;
            regen = true;
        }
    }
    if (regen) {
        CK(cudaMemcpyAsync(b->h_stats, b->stats.p, sizeof(BatchStats) * pfc_batch::kSlots, cudaMemcpyDeviceToHost,
                           c->st));
        CK(cudaStreamSynchronize(c->st));
    }
    std::vector<JobDev<uint32_t>> v32(fresh.size());
    std::vector<JobDev<uint64_t>> v64(fresh.size());
    for (size_t f = 0; f < fresh.size(); ++f) {
        BatchJob *j = fresh[f];
        const BatchStats &s = b->h_stats[j->slot];
        const uint32_t n32 = j->use32 ? s.counts[0] : 0;
        const uint32_t n64 = j->use64 ? s.counts[1] : 0;
        j->primecount = (uint64_t)n32 + n64;
        j->n32 = n32;
        j->n64 = n64;
        j->pos32 = n32 ? 0 : j->tot32;
        j->pos64 = n64 ? 0 : j->tot64;
        v32[f] = job_view<uint32_t>(b, j, j->c32, 0, j->d_words32.p, j->d_segs32, j->segs32.size(), j->c32a,
                                    j->c32b, j->nsetup32);
        const void *w64 = j->pmax <= kLazyEnd ? (const void *)j->d_wordsw.p : (const void *)j->d_words64.p;
        v64[f] = job_view<uint64_t>(b, j, j->c64, 1, w64, j->d_segs64, j->segs64.size(), j->c64a, j->c64b,
                                    j->nsetup64);
        CK(cudaMemcpyAsync(b->jobs32.p + j->slot, &v32[f], sizeof(v32[f]), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(b->jobs64.p + j->slot, &v64[f], sizeof(v64[f]), cudaMemcpyHostToDevice, c->st));
        c->h2d += sizeof(v32[f]) + sizeof(v64[f]);
    }
    CK(cudaStreamSynchronize(c->st));
    // setups of class 32 and of class 64 below 2^64/3 on the tensor cores.
    // The search's timeline of the class starts at its walk, which joins the
    // iterations once the setup has finished (build_tasks).  Throughput
    // policy: one setup launch per fresh search and class on the setup
    // streams, overlapping the iterations.  Latency policy: the setup runs in
    // chunks of candidate blocks ahead of each iteration (launch_iteration),
    // within a share of the iteration's budget, so that small searches are
    // not held up behind large setups.
    if (c->setup_tc) {
        bool waited[pfc_batch::kTcStreams] = {};
        CK(cudaEventRecord(b->ev_tc0, c->st));
        for (BatchJob *j : fresh) {
            // (a timeline without walk steps keeps its setup windows: the
            // window that ends it also adds the check terms)
            if (!j->d_tct.p || !j->nwalk) continue;
            SetupArgs<WideWord> &sw = j->tc_args;
            memset(&sw, 0, sizeof(sw));
            sw.mode = j->mode;
            Prog<WideWord> *pg[2] = {&sw.a, &sw.b};
            uint32_t goff = 0;
            for (int q = 0; q < 2; ++q) {   // the paired programs (the tiles hold their words)
                pg[q]->words = nullptr;
                pg[q]->groups = j->d_tcgroups.p + goff;
                pg[q]->ngroups = j->tc_ng[q];
                pg[q]->final_sq = j->tc_fsq[q];
                pg[q]->corr = j->tc_corr[q];
                goff += 3 * j->tc_ng[q];
            }
            j->tc_ta = TcTiles{j->d_tct.p, j->tc_ntiles[0]};
            j->tc_tb = TcTiles{j->d_tct.p + (size_t)j->tc_ntiles[0] * tc_tile_bytes(), j->tc_ntiles[1]};
            const uint64_t words = (uint64_t)j->tc_nw[0] + j->tc_nw[1];
            for (int cls = 0; cls < 2; ++cls) {
                const uint32_t n = cls ? j->n64 : j->n32;
                // small programs keep their setup windows (kernels.cuh kTcMinWords*)
                if (!n || words < (cls ? kTcMinWords64 : kTcMinWords32)) continue;
                j->tc_blocks[cls] = cls ? tc_setup_blocks(n) : tc_setup_blocks32(n);
                j->tc_block_cost[cls] = kTcTileCost * ((double)j->tc_ntiles[0] + j->tc_ntiles[1]);
                (cls ? j->pos64 : j->pos32) = cls ? j->nsetup64 : j->nsetup32;
                j->tc_wait[cls] = true;
                if (b->policy == PFC_BATCH_LATENCY) {
                    j->tc_block[cls] = 0;
                    continue;
                }
                const int si = b->tc_next++ % pfc_batch::kTcStreams;
                if (!waited[si]) CK(cudaStreamWaitEvent(b->tcst[si], b->ev_tc0, 0));
                waited[si] = true;
                CK(cudaEventCreate(&j->tc_ev0[cls]));
                CK(cudaEventCreate(&j->tc_ev1[cls]));
                CK(cudaEventRecord(j->tc_ev0[cls], b->tcst[si]));
                c->launches += tc_launch(b, j, cls, b->tcst[si], 0, 0);
                CK(cudaEventRecord(j->tc_ev1[cls], b->tcst[si]));
                j->tc_block[cls] = j->tc_blocks[cls];
            }
        }
        CK(cudaGetLastError());
    }
    for (BatchJob *j : fresh) {
        free_vec(j->tcgroups);
        free_vec(j->tcsrc);
        free_vec(j->words32);  // on the device now
        free_vec(j->words64);
        free_vec(j->wordsw);
        free_vec(j->segs32);
        free_vec(j->segs64);
        free_vec(j->cmult);
        free_vec(j->qlist);
        j->state = kReady;
        b->ready.push_back(j);
    }
    return PFC_OK;
}

// One task per unfinished block: a window of at most L timeline positions.
// Returns the window length used.
// Cost of timeline positions in IMAD-equivalent multiplies per candidate
// (measured multiply-pipe rates: class-32 step 6; class-64 lazy step 10.5
// plus its share of the block restore; an 896-bit setup word 32 wide
// multiply-adds and two rounds in class 32, 64 and three lazy rounds in
// class 64)
struct PosCost {
    double setup, walk;
};
static PosCost pos_cost(const BatchJob *j, bool cls64) {
    const double chains = j->mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL) ? 2.0 : 1.0;
    if (!cls64) return {85.0, 6.0 * chains};
    if (j->pmax <= kLazyEnd) return {175.0, 12.0 * chains};
    return {60.0, 30.0 * chains};
}

// remaining cost of n candidates at position pos of a timeline
static double class_cost(uint32_t n, uint32_t pos, uint32_t ns, uint32_t tot, PosCost c) {
    if (pos >= tot) return 0.0;
    const double setup = pos < ns ? (double)(ns - pos) : 0.0;
    const double walk = (double)tot - (double)std::max(pos, ns);
    return (double)n * (setup * c.setup + walk * c.walk);
}

// candidates per CTA of a class and task kind (as batch_kernel computes them)
static uint32_t per_cta(const BatchJob *j, bool cls64, int kind) {
    if (cls64) return 256u * Cls64L::NC;
    if (kind == kSetupTask) return 512u;
    return j->mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL) ? 256u : 256u * Cls32::NC;
}

// One window per search and class.  Throughput policy: every search advances
// a common window of L positions per iteration (all searches progress at the
// same pace, so the largest ones are never starved and the batch ends as
// early as the work allows).  Latency policy (shortest remaining work
// first): searches are taken in order of remaining cost, each gets its own
// window, as wide as keeps every one of its tasks within one CTA's share of
// the iteration (no single task outlasts the rest) and as the iteration's
// budget still open pays for; searches the budget cannot pay for wait, and
// one that has waited 32 iterations gets a minimal window.
// Windows are then ordered by the cost of one of their tasks, longest first.
// Host work is linear in the number of searches.  Returns L.
uint32_t build_tasks(pfc_batch *b) {
    for (BatchJob *j : b->ready) {
        j->state = kRunning;
        b->running.push_back(j);
    }
    b->ready.clear();
    // iteration length unless set: long for the throughput policy (every
    // iteration ends with a tail; on the 512-search mix 585 iterations of 1e11
    // candidate-steps took 41.3 s, 61 of 1.6e12 38.8 s), short for the
    // latency policy (arrivals join and results leave at iteration ends)
    const double per_iter = b->work_per_iter > 0
                                ? b->work_per_iter
                                : (b->policy == PFC_BATCH_LATENCY ? kLatencyIterWork : kThroughputIterWork);
    const double budget = per_iter * 6.0;   // candidate-steps -> multiplies
    b->iter_budget = budget;
    const double cta_share = budget / (3.0 * b->ctx->sms);
    for (BatchJob *j : b->running)   // tensor-core setups that have finished
        for (int k = 0; k < 2; ++k) {
            if (!j->tc_wait[k]) continue;
            if (!j->tc_ev1[k]) {   // chunks: done once the iteration that ran the last ones has finished
                if (j->tc_block[k] >= j->tc_blocks[k] && b->iterations > j->tc_iter[k]) j->tc_wait[k] = false;
                continue;
            }
            const cudaError_t q = cudaEventQuery(j->tc_ev1[k]);
            if (q == cudaErrorNotReady) continue;
            float ms = 0;
            if (q == cudaSuccess && cudaEventElapsedTime(&ms, j->tc_ev0[k], j->tc_ev1[k]) == cudaSuccess)
                b->tc_s += ms * 1e-3;
            j->tc_wait[k] = false;   // an error surfaces at the next synchronisation
        }
    std::vector<std::pair<double, BatchJob *>> order;
    order.reserve(b->running.size());
    for (BatchJob *j : b->running) {
        const double r = class_cost(j->n32, j->pos32, j->nsetup32, j->tot32, pos_cost(j, false)) +
                         class_cost(j->n64, j->pos64, j->nsetup64, j->tot64, pos_cost(j, true));
        order.push_back({r, j});
    }
    std::sort(order.begin(), order.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
    const bool latency = b->policy == PFC_BATCH_LATENCY;
    double prio_left = latency ? budget : 0.0, rate = 0;   // rate: cost per common-window position
    for (auto &o : order) {
        BatchJob *j = o.second;
        const PosCost c32 = pos_cost(j, false), c64 = pos_cost(j, true);
        double jrate = 0, worst = 0;
        if (j->pos32 < j->tot32 && !j->tc_wait[0]) {
            jrate += j->n32 * (j->pos32 < j->nsetup32 ? c32.setup : c32.walk);
            worst = std::max(worst, std::max(per_cta(j, false, kSetupTask) * c32.setup,
                                             per_cta(j, false, kWalkTask) * c32.walk));
        }
        if (j->pos64 < j->tot64 && !j->tc_wait[1]) {
            jrate += j->n64 * (j->pos64 < j->nsetup64 ? c64.setup : c64.walk);
            worst = std::max(worst, per_cta(j, true, kSetupTask) * std::max(c64.setup, c64.walk));
        }
        j->win = 0;
        j->wait = false;
        if (!latency) {
            rate += jrate;
            continue;
        }
        // as wide as one CTA's share of the iteration allows and as the budget
        // still open pays for; searches it cannot pay for wait, except that
        // one that has waited 32 iterations gets a minimal window
        const double w = std::min(cta_share / std::max(worst, 1.0), prio_left / std::max(jrate, 1.0));
        if (w >= 64.0 || j->waited >= 32 || &o == &order.front()) {  // the smallest always advances
            j->win = (uint32_t)std::min(std::max(w, 64.0), 4294967295.0);
            prio_left -= std::min(o.first, (double)j->win * jrate);
            j->waited = 0;
        } else {
            j->wait = true;
            ++j->waited;
        }
    }
    const double prio_work = latency ? budget - std::max(prio_left, 0.0) : 0.0;
    b->prio = 0;
    for (auto &o : order) b->prio += o.second->win ? 1u : 0u;
    const double Ld = std::max(64.0, std::min(std::max(budget - prio_work, 0.0) / std::max(rate, 1.0), 4194304.0));
    const uint32_t L = ((uint32_t)Ld + 15u) & ~15u;

    std::vector<std::pair<double, Window>> lists[pfc_batch::kLists][pfc_batch::kKinds];
    for (BatchJob *j : b->running) {
        j->next32 = j->pos32;
        j->next64 = j->pos64;
        for (int cls = 0; cls < 2; ++cls) {
            const uint32_t pos = cls ? j->pos64 : j->pos32, tot = cls ? j->tot64 : j->tot32;
            const uint32_t ns = cls ? j->nsetup64 : j->nsetup32, n = cls ? j->n64 : j->n32;
            if (pos >= tot || n == 0 || j->wait || j->tc_wait[cls]) continue;
            uint32_t hi = (uint32_t)std::min<uint64_t>((uint64_t)pos + (j->win ? j->win : L), tot);
            // a window that reaches the end of the setup stops there: the walk
            // starts in the next iteration, in the walk kernel, and the general
            // kernel (lower occupancy) only ends timelines without walk steps
            if (pos < ns && hi > ns) hi = ns;
            (cls ? j->next64 : j->next32) = hi;
            const PosCost c = pos_cost(j, cls != 0);
            const int kind = (hi <= ns && hi < tot) ? kSetupTask : (pos >= ns ? kWalkTask : kAnyTask);
            const uint32_t per = per_cta(j, cls != 0, kind);
            const double setup = pos < ns ? (double)(std::min(hi, ns) - pos) : 0.0;
            const double walk = hi > ns ? (double)(hi - std::max(pos, ns)) : 0.0;
            const double cost = (double)std::min(per, n) * (setup * c.setup + walk * c.walk);
            Window w{};
            w.nblocks = (n + per - 1) / per;
            w.slot = j->slot;
            w.ncand = n;
            w.lo = pos;
            w.hi = hi;
            const int l = cls == 0 ? 0 : (j->pmax <= kLazyEnd ? 1 : 2);
            lists[l][kind].push_back({cost, w});
        }
    }
    for (int l = 0; l < pfc_batch::kLists; ++l)
        for (int k = 0; k < pfc_batch::kKinds; ++k) {
            auto &lst = lists[l][k];
            std::sort(lst.begin(), lst.end(), [](const auto &x, const auto &y) { return x.first > y.first; });
            b->w[l][k].clear();
            uint64_t first = 0;
            for (auto &e : lst) {
                e.second.first_cta = (uint32_t)first;
                first += e.second.nblocks;
                b->w[l][k].push_back(e.second);
            }
            b->ctas[l][k] = first;
        }
    return L;
}

template <class T, int KIND>
static void launch_list(pfc_batch *b, int l, const JobDev<typename T::W> *jobs, const HitBuf &h) {
    const uint64_t n = b->ctas[l][KIND];
    if (!n) return;
    const int si = (l == 0 ? 0 : 3) + KIND;
    batch_kernel<T, KIND><<<(unsigned)n, task_threads<T, KIND>(), 0, b->st[si]>>>(
        b->wins[l][KIND].p, (uint32_t)b->w[l][KIND].size(), jobs, h);
    b->used[si] = true;
    b->ctx->launches++;
}

bool tc_chunks_pending(const pfc_batch *b) {
    for (const BatchJob *j : b->running)
        for (int k = 0; k < 2; ++k)
            if (j->tc_wait[k] && !j->tc_ev1[k] && j->tc_block[k] < j->tc_blocks[k]) return true;
    return false;
}

int launch_iteration(pfc_batch *b) {
    pfc_ctx *c = b->ctx;
    for (int l = 0; l < pfc_batch::kLists; ++l)
        for (int k = 0; k < pfc_batch::kKinds; ++k) {
            const size_t n = b->w[l][k].size();
            if (!n) continue;
            if (b->wins[l][k].n < n) CK(b->wins[l][k].alloc(c, n + n / 2 + 64));
            CK(cudaMemcpyAsync(b->wins[l][k].p, b->w[l][k].data(), n * sizeof(Window), cudaMemcpyHostToDevice, c->st));
            c->h2d += n * sizeof(Window);
        }
    // latency policy: chunks of pending tensor-core setups, smallest first,
    // ahead of the iteration's windows on the context stream
    if (tc_chunks_pending(b)) {
        struct Pend {
            double cost;
            BatchJob *j;
            int cls;
        };
        std::vector<Pend> pend;
        for (BatchJob *j : b->running)
            for (int k = 0; k < 2; ++k)
                if (j->tc_wait[k] && !j->tc_ev1[k] && j->tc_block[k] < j->tc_blocks[k])
                    pend.push_back({(j->tc_blocks[k] - j->tc_block[k]) * j->tc_block_cost[k], j, k});
        std::sort(pend.begin(), pend.end(), [](const Pend &x, const Pend &y) { return x.cost < y.cost; });
        double left = b->iter_budget * kTcChunkShare;
        CK(cudaEventRecord(b->ev_ck0, c->st));
        for (const Pend &pj : pend) {
            BatchJob *j = pj.j;
            const int k = pj.cls;
            if (left <= 0) break;
            const double fit = std::floor(left / std::max(j->tc_block_cost[k], 1.0));
            const uint32_t n =
                (uint32_t)std::min<double>(j->tc_blocks[k] - j->tc_block[k], std::max<double>(fit, c->sms));
            c->launches += tc_launch(b, j, k, c->st, j->tc_block[k], n);
            j->tc_block[k] += n;
            if (j->tc_block[k] >= j->tc_blocks[k]) j->tc_iter[k] = b->iterations;
            left -= n * j->tc_block_cost[k];
        }
        CK(cudaEventRecord(b->ev_ck1, c->st));
        b->ck_pending = true;
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(b->ev_start, c->st));
    for (int i = 0; i < pfc_batch::kStreams; ++i) {
        b->used[i] = false;
        CK(cudaStreamWaitEvent(b->st[i], b->ev_start, 0));
    }
    HitBuf h{};
    h.buf = b->hits.p;
    h.count = b->hitcount.p;
    h.cap = b->hits.n;
    h.tag = b->tags.p;
    // setup-only and general lists first: they hold the longest tasks
    launch_list<Cls32, kSetupTask>(b, 0, b->jobs32.p, h);
    launch_list<Cls32, kAnyTask>(b, 0, b->jobs32.p, h);
    launch_list<Cls32, kWalkTask>(b, 0, b->jobs32.p, h);
    launch_list<Cls64L, kSetupTask>(b, 1, b->jobs64.p, h);
    launch_list<Cls64L, kAnyTask>(b, 1, b->jobs64.p, h);
    launch_list<Cls64L, kWalkTask>(b, 1, b->jobs64.p, h);
    launch_list<Cls64, kSetupTask>(b, 2, b->jobs64.p, h);
    launch_list<Cls64, kAnyTask>(b, 2, b->jobs64.p, h);
    launch_list<Cls64, kWalkTask>(b, 2, b->jobs64.p, h);
    CK(cudaGetLastError());
    // the main stream waits for every list before the hit read-back
    for (int i = 0; i < pfc_batch::kStreams; ++i) {
        CK(cudaEventRecord(b->ev_end[i], b->st[i]));
        CK(cudaStreamWaitEvent(c->st, b->ev_end[i], 0));
    }
    uint64_t n32 = 0, n64 = 0;
    for (int k = 0; k < pfc_batch::kKinds; ++k) {
        n32 += b->ctas[0][k];
        n64 += b->ctas[1][k] + b->ctas[2][k];
    }
    b->tasks += n32 + n64;
    b->t32_n = n32;
    b->t64_n = n64;
    CK(cudaMemcpyAsync(b->h_hitcount, b->hitcount.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
    return PFC_OK;
}

// After the iteration: route the hits by slot (on overflow, every search of
// the iteration is redone alone at the end) and advance the positions.
int finish_iteration(pfc_batch *b, uint32_t L) {
    pfc_ctx *c = b->ctx;
    CK(cudaStreamSynchronize(c->st));
    ++b->iterations;
    if (b->ck_pending) {
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, b->ev_ck0, b->ev_ck1));
        b->tc_s += ms * 1e-3;
        b->ck_pending = false;
    }
    float ms32 = 0, ms64 = 0;
    for (int i = 0; i < pfc_batch::kStreams; ++i) {
        if (!b->used[i]) continue;
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, b->ev_start, b->ev_end[i]));
        (i < 3 ? ms32 : ms64) = std::max(i < 3 ? ms32 : ms64, ms);
    }
    b->gpu32_s += ms32 * 1e-3;
    b->gpu64_s += ms64 * 1e-3;
    b->gpu_s += std::max(ms32, ms64) * 1e-3;
    const unsigned long long nh = *b->h_hitcount;
    if (nh > b->hits.n) {
        for (BatchJob *j : b->running) j->rerun = true;
    } else if (nh) {
        std::vector<pfc_factor> hv(nh);
        std::vector<uint32_t> tv(nh);
        CK(cudaMemcpyAsync(hv.data(), b->hits.p, nh * sizeof(pfc_factor), cudaMemcpyDeviceToHost, c->st));
        CK(cudaMemcpyAsync(tv.data(), b->tags.p, nh * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        c->d2h += nh * (sizeof(pfc_factor) + sizeof(uint32_t));
        std::vector<BatchJob *> by_slot(pfc_batch::kSlots, nullptr);
        for (BatchJob *j : b->running) by_slot[j->slot] = j;
        for (unsigned long long i = 0; i < nh; ++i)
            if (tv[i] < pfc_batch::kSlots && by_slot[tv[i]]) by_slot[tv[i]]->hits.push_back(hv[i]);
    }
    if (nh) CK(cudaMemsetAsync(b->hitcount.p, 0, sizeof(unsigned long long), c->st));
    if (b->trace) {
        const float ms = std::max(ms32, ms64);
        fprintf(stderr, "batch iter %llu: running %zu prio %u L %u tasks %zu/%zu hits %llu gpu %.2f ms\n",
                (unsigned long long)b->iterations, b->running.size(), b->prio, L, b->t32_n, b->t64_n, nh, ms);
    }
    for (BatchJob *j : b->running) {  // the windows' ends (build_tasks)
        j->pos32 = j->next32;
        j->pos64 = j->next64;
    }
    return PFC_OK;
}

// a search whose hits overflowed the batch's hit buffer is redone on the
// per-job path
int rerun_alone(pfc_batch *b, BatchJob *j) {
    pfc_job *pj = nullptr;
    int rc = pfc_job_create(b->ctx, j->mode, j->nmin, j->nmax, j->pmin, j->pmax, &pj);
    if (rc) return rc;
    std::vector<pfc_factor> buf(1 << 16);
    size_t n = 0;
    for (;;) {
        rc = pfc_job_run(pj, buf.data(), buf.size(), &n);
        if (rc != PFC_ERR_HIT_OVERFLOW) break;
        pfc_job_destroy(pj);
        buf.resize(n + 1024);
        rc = pfc_job_create(b->ctx, j->mode, j->nmin, j->nmax, j->pmin, j->pmax, &pj);
        if (rc) return rc;
    }
    if (rc == PFC_OK) {
        buf.resize(n);
        j->hits = buf;
        uint64_t term = 0, count = 0;
        pfc_job_totals(pj, &term, &count);
        j->termsum = term;
        j->primecount = count;
        j->flags = 0;
    }
    pfc_job_destroy(pj);
    return rc;
}

int retire_finished(pfc_batch *b) {
    pfc_ctx *c = b->ctx;
    std::vector<BatchJob *> done, still;
    for (BatchJob *j : b->running) {
        const bool fin = j->pos32 >= j->tot32 && j->pos64 >= j->tot64;
        (fin ? done : still).push_back(j);
    }
    if (done.empty()) return PFC_OK;
    CK(cudaMemcpyAsync(b->h_stats, b->stats.p, sizeof(BatchStats) * pfc_batch::kSlots, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (BatchJob *j : done) {
        const BatchStats &s = b->h_stats[j->slot];
        j->termsum = s.termsum;
        j->flags = s.flags;
        release_device(b, j);
        b->free_slots.push_back(j->slot);
        j->state = kDone;
        if (j->rerun) {
            j->hits.clear();
            j->status = rerun_alone(b, j);
        } else if (j->flags & 1u) {
            j->status = PFC_ERR_VALIDATION;
        } else if (j->flags & 2u) {
            j->status = PFC_ERR_CUDA;   // a tensor-core setup wait gave up
        }
    }
    b->running.swap(still);
    return PFC_OK;
}

}  // namespace

// ====================================================================== C ABI

extern "C" int pfc_batch_destroy(pfc_batch *b);

extern "C" int pfc_batch_create(pfc_ctx *c, pfc_batch **out) {
    if (!c || !out) return PFC_ERR_ARG;
    *out = nullptr;
    CK(cudaSetDevice(c->device));
    pfc_batch *b = new (std::nothrow) pfc_batch();
    if (!b) return PFC_ERR_NOMEM;
    b->ctx = c;
    // iterations on the highest stream priority, tensor-core setups on the
    // lowest: a setup CTA holds a whole SM, and under priorities the block
    // scheduler gives freed SMs to pending iteration CTAs first, so setups
    // fill the iterations' tails and gaps instead of delaying small searches
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    for (int i = 0; i < pfc_batch::kStreams && e == cudaSuccess; ++i)
        e = cudaStreamCreateWithPriority(&b->st[i], cudaStreamNonBlocking, greatest);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev_start);
    for (int i = 0; i < pfc_batch::kStreams && e == cudaSuccess; ++i) e = cudaEventCreate(&b->ev_end[i]);
    for (int i = 0; i < pfc_batch::kTcStreams && e == cudaSuccess; ++i)
        e = cudaStreamCreateWithPriority(&b->tcst[i], cudaStreamNonBlocking, least);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_tc0, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev_ck0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev_ck1);
    if (e == cudaSuccess) e = b->stats.alloc(c, pfc_batch::kSlots);
    if (e == cudaSuccess) e = b->jobs32.alloc(c, pfc_batch::kSlots);
    if (e == cudaSuccess) e = b->jobs64.alloc(c, pfc_batch::kSlots);
    if (e == cudaSuccess) e = b->hits.alloc(c, 1u << 20);
    if (e == cudaSuccess) e = b->tags.alloc(c, 1u << 20);
    if (e == cudaSuccess) e = b->hitcount.alloc(c, 1);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&b->h_stats, sizeof(BatchStats) * pfc_batch::kSlots);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&b->h_hitcount, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemsetAsync(b->hitcount.p, 0, sizeof(unsigned long long), c->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->stats.p, 0, sizeof(BatchStats) * pfc_batch::kSlots, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) {
        pfc_batch_destroy(b);
        return cuda_fail(e);
    }
    for (uint32_t s = pfc_batch::kSlots; s-- > 0;) b->free_slots.push_back(s);
    const char *tr = getenv("PFCSIEVE_BATCH_TRACE");
    b->trace = tr && *tr && *tr != '0';
    *out = b;
    return PFC_OK;
}

extern "C" int pfc_batch_destroy(pfc_batch *b) {
    if (!b) return PFC_ERR_ARG;
    pfc_ctx *c = b->ctx;
    cudaSetDevice(c->device);
    for (int i = 0; i < pfc_batch::kStreams; ++i)
        if (b->st[i]) cudaStreamSynchronize(b->st[i]);
    for (int i = 0; i < pfc_batch::kTcStreams; ++i)
        if (b->tcst[i]) cudaStreamSynchronize(b->tcst[i]);
    cudaStreamSynchronize(c->st);
    for (auto &kv : b->all) release_device(b, kv.second.get());
    b->stats.release(c);
    b->jobs32.release(c);
    b->jobs64.release(c);
    for (auto &row : b->wins)
        for (auto &d : row) d.release(c);
    b->hits.release(c);
    b->tags.release(c);
    b->hitcount.release(c);
    if (b->h_stats) cudaFreeHost(b->h_stats);
    if (b->h_hitcount) cudaFreeHost(b->h_hitcount);
    if (b->ev) cudaEventDestroy(b->ev);
    if (b->ev_start) cudaEventDestroy(b->ev_start);
    if (b->ev_tc0) cudaEventDestroy(b->ev_tc0);
    if (b->ev_ck0) cudaEventDestroy(b->ev_ck0);
    if (b->ev_ck1) cudaEventDestroy(b->ev_ck1);
    for (int i = 0; i < pfc_batch::kTcStreams; ++i)
        if (b->tcst[i]) cudaStreamDestroy(b->tcst[i]);
    for (int i = 0; i < pfc_batch::kStreams; ++i) {
        if (b->ev_end[i]) cudaEventDestroy(b->ev_end[i]);
        if (b->st[i]) cudaStreamDestroy(b->st[i]);
    }
    delete b;
    return PFC_OK;
}

extern "C" int pfc_batch_submit(pfc_batch *b, const pfc_job_desc *d, uint64_t *id) {
    if (!b || !d || !id) return PFC_ERR_ARG;
    const unsigned mode = d->mode;
    const bool valid_mode = mode == PFC_FACTORIAL || mode == PFC_PRIMORIAL || mode == PFC_COMPOSITORIAL ||
                            mode == (PFC_FACTORIAL | PFC_COMPOSITORIAL);
    // the ranges of pfc_job_create, and at most 2^26 n per search (the
    // per-search multiplier table lives on the device for the whole search)
    if (!valid_mode || d->pmin < 3 || d->pmax <= d->pmin || d->nmin < 101 || d->nmax < d->nmin ||
        d->nmax > 0x7FFFFFFFu || d->nmax - d->nmin > (1u << 26))
        return PFC_ERR_ARG;
    // a batched search keeps all its candidates on the device at once:
    // at most 2^28 expected per size class (about 7.5 GB in class 64); larger
    // searches go through pfc_job_run, which walks the p range in segments
    const double e32 = est_cands(d->pmin, std::min<uint64_t>(d->pmax, kClassSplit));
    const double e64 = est_cands(std::max<uint64_t>(d->pmin, kClassSplit), d->pmax);
    if (e32 > (double)(1u << 28) || e64 > (double)(1u << 28)) return PFC_ERR_ARG;
    auto j = std::make_unique<BatchJob>();
    j->id = b->next_id++;
    j->mode = mode;
    j->nmin = d->nmin;
    j->nmax = d->nmax;
    j->pmin = d->pmin;
    j->pmax = d->pmax;
    b->queued.push_back(j.get());
    *id = j->id;
    b->all[j->id] = std::move(j);
    return PFC_OK;
}

// One iteration, pipelined with the host work of admission:
//   1. searches made ready by the previous call join; every running block
//      gets a task; both class kernels are launched (asynchronously);
//   2. while they run, the host tables of queued searches are built;
//   3. the iteration is finished (hits routed, blocks advanced) and finished
//      searches are retired, freeing slots and memory;
//   4. prepared searches are uploaded and their candidates generated while
//      the budget allows; they join at the next call.
// When nothing was running, the call admits and then runs at once.
extern "C" int pfc_batch_step(pfc_batch *b, uint32_t *active, uint32_t *queued) {
    if (!b) return PFC_ERR_ARG;
    CK(cudaSetDevice(b->ctx->device));
    const double ts = now_s();
    for (int pass = 0; pass < 2; ++pass) {
        uint32_t L = build_tasks(b);
        bool work = tc_chunks_pending(b);
        for (auto &row : b->ctas)
            for (uint64_t n : row) work |= n > 0;
        if (!work && pass == 0) {
            // everything running waits for a tensor-core setup: the call
            // returns after a short pause (searches submitted meanwhile are
            // admitted by the next call) instead of blocking on one setup
            for (BatchJob *j : b->running)
                if (j->tc_wait[0] || j->tc_wait[1]) {
                    std::this_thread::sleep_for(std::chrono::microseconds(200));
                    break;
                }
        }
        if (work) {
            const int rc = launch_iteration(b);
            if (rc) return rc;
        }
        const double tp = now_s();
        prepare_queued(b);
        b->prep_s += now_s() - tp;
        if (work) {
            int rc = finish_iteration(b, L);
            if (rc) return rc;
            rc = retire_finished(b);
            if (rc) return rc;
        }
        const double ta = now_s();
        const int rc = admit_prepared(b);
        b->admit_s += now_s() - ta;
        if (rc) return rc;
        if (work || b->ready.empty()) break;
    }
    b->step_s += now_s() - ts;
    if (active) *active = (uint32_t)(b->running.size() + b->ready.size());
    if (queued) *queued = (uint32_t)b->queued.size();
    return PFC_OK;
}

extern "C" int pfc_batch_result(pfc_batch *b, uint64_t id, pfc_batch_status *r) {
    if (!b || !r) return PFC_ERR_ARG;
    auto it = b->all.find(id);
    if (it == b->all.end()) return PFC_ERR_ARG;
    const BatchJob &j = *it->second;
    memset(r, 0, sizeof(*r));
    r->done = j.state == kDone;
    r->status = j.status;
    if (r->done) {
        r->term_checksum = j.termsum;
        r->primecount = j.primecount;
        r->pairs = j.primecount * (uint64_t)(j.nmax - j.nmin);
        r->hits = j.hits.size();
    }
    return PFC_OK;
}

extern "C" int pfc_batch_take_hits(pfc_batch *b, uint64_t id, pfc_factor *buf, size_t cap, size_t *n) {
    if (!b || !n || (!buf && cap)) return PFC_ERR_ARG;
    auto it = b->all.find(id);
    if (it == b->all.end() || it->second->state != kDone) return PFC_ERR_STATE;
    const std::vector<pfc_factor> &h = it->second->hits;
    *n = h.size();
    if (h.size() > cap) return PFC_ERR_HIT_OVERFLOW;
    if (!h.empty()) memcpy(buf, h.data(), h.size() * sizeof(pfc_factor));
    return PFC_OK;
}

extern "C" int pfc_batch_release(pfc_batch *b, uint64_t id) {
    if (!b) return PFC_ERR_ARG;
    auto it = b->all.find(id);
    if (it == b->all.end() || it->second->state != kDone) return PFC_ERR_STATE;
    b->all.erase(it);
    return PFC_OK;
}

extern "C" uint64_t pfc_batch_iterations(pfc_batch *b) { return b ? b->iterations : 0; }

extern "C" int pfc_batch_timing(pfc_batch *b, pfc_batch_times *t) {
    if (!b || !t) return PFC_ERR_ARG;
    t->step_s = b->step_s;
    t->gpu_s = b->gpu_s;
    t->gpu32_s = b->gpu32_s;
    t->gpu64_s = b->gpu64_s;
    t->prep_s = b->prep_s;
    t->admit_s = b->admit_s;
    t->setup_tc_s = b->tc_s;
    t->iterations = b->iterations;
    t->tasks = b->tasks;
    return PFC_OK;
}

extern "C" int pfc_batch_set_hit_capacity(pfc_batch *b, uint32_t records) {
    if (!b || records == 0 || !b->running.empty() || !b->ready.empty()) return b ? PFC_ERR_STATE : PFC_ERR_ARG;
    pfc_ctx *c = b->ctx;
    CK(cudaSetDevice(c->device));
    CK(cudaStreamSynchronize(c->st));
    CK(b->hits.alloc(c, records));
    CK(b->tags.alloc(c, records));
    return PFC_OK;
}

extern "C" int pfc_batch_set_policy(pfc_batch *b, int policy) {
    if (!b || (policy != PFC_BATCH_THROUGHPUT && policy != PFC_BATCH_LATENCY)) return PFC_ERR_ARG;
    b->policy = policy;
    return PFC_OK;
}

extern "C" int pfc_batch_set_iteration_work(pfc_batch *b, double candidate_steps) {
    if (!b || !(candidate_steps >= 1.0)) return PFC_ERR_ARG;
    b->work_per_iter = candidate_steps;
    return PFC_OK;
}
