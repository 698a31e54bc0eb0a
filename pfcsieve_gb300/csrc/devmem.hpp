// devmem.hpp -- the context record and budgeted device buffers shared by
// the C ABI implementations (api.cu, batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <utility>
#include <vector>

#include "host.hpp"
#include "kernels.cuh"
#include "pfcsieve.h"

struct pfc_ctx {
    int device = 0;
    cudaStream_t st = nullptr;
    // the context's buffers come from its own stream-ordered pool, allocated
    // and freed on `st`: freed blocks stay in the pool for the next job, so a
    // search does not pay for cudaMalloc and the device-wide synchronisation
    // of cudaFree each time (the pool is trimmed only when an allocation
    // would not fit, and released when the context is destroyed)
    cudaMemPool_t pool = nullptr;
    std::vector<void *> pinned_stats;   // spare pinned blocks for the jobs' segment stats
    int sms = 0;
    char name[256] = {0};
    uint64_t budget = 0, used = 0;
    uint64_t launches = 0;
    uint64_t h2d = 0, d2h = 0;   // bytes copied by this context
    uint64_t *d_pat = nullptr;
    int walk_var[3][2] = {{0, 0}, {0, 0}, {0, 0}};   // walk variant per size class and kind (fused)
    bool graphs = true;   // pfc_segment replays each job's segment body as a CUDA graph
    bool split = true;    // small candidate sets walk their n range in sub-ranges (split walks)
    bool setup_tc = true; // lazy class-64 setup folds its table words on the tensor cores
    // prime flags of [0, vbits_top] kept for pfc_verify_factors_device (one
    // bit per integer), rebuilt only when a call needs a larger range
    uint32_t *vbits = nullptr;
    uint32_t vbits_top = 0;
    size_t vbits_bytes = 0;
    // host tables kept between the context's jobs: the primes up to the
    // largest limit asked for so far, and the setup programs per (mode,
    // startN), oldest dropped first beyond kProgCacheBytes (searches of one n
    // range over many p ranges, and the split walks' boundaries, reuse them);
    // the prime list is shared, so a caller's copy of the pointer stays valid
    // when a later call replaces it with a longer one
    std::shared_ptr<const std::vector<uint32_t>> primes;
    uint32_t primes_lim = 0;
    std::map<std::pair<unsigned, uint32_t>, std::shared_ptr<pfc::ProgSet>> progs;
    std::deque<std::pair<unsigned, uint32_t>> prog_order;
    size_t prog_bytes = 0;
    static constexpr size_t kProgCacheBytes = 64u << 20;
};

namespace pfc {

// A buffer of the context's pool, ordered on the context stream (work on
// other streams must wait for that stream before using it; every caller
// synchronises it first).  Counted against the memory budget while held.
inline cudaError_t dalloc_bytes(pfc_ctx *c, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return cudaSuccess;
    if (c->used + bytes > c->budget) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, c->pool, c->st);
    if (e == cudaErrorMemoryAllocation) {
        // give the pool's idle blocks back to the device and try once more
        cudaGetLastError();
        e = cudaStreamSynchronize(c->st);
        if (e == cudaSuccess) e = cudaMemPoolTrimTo(c->pool, 0);
        if (e == cudaSuccess) e = cudaMallocFromPoolAsync(p, bytes, c->pool, c->st);
    }
    if (e == cudaSuccess) c->used += bytes;
    return e;
}

// Back to the pool after the work enqueued so far on the context stream.
// Buffers that other streams use are freed only when those streams are idle
// (the batch frees a search's buffers after its iteration has finished).
inline void dfree_bytes(pfc_ctx *c, void *p, size_t bytes) {
    if (!p) return;
    cudaFreeAsync(p, c->st);
    c->used -= bytes;
}

template <class T>
struct DArr {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t alloc(pfc_ctx *c, size_t count) {
        release(c);
        cudaError_t e = dalloc_bytes(c, (void **)&p, count * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    cudaError_t upload(pfc_ctx *c, const std::vector<T> &v) {
        cudaError_t e = alloc(c, std::max<size_t>(v.size(), 1));
        if (e != cudaSuccess) return e;
        if (v.empty()) return cudaMemsetAsync(p, 0, sizeof(T), c->st);
        c->h2d += v.size() * sizeof(T);
        return cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->st);
    }
    void release(pfc_ctx *c) {
        dfree_bytes(c, p, n * sizeof(T));
        p = nullptr;
        n = 0;
    }
};

template <class W>
struct DevProg {
    DArr<W> words;
    DArr<uint32_t> groups;
    Prog<W> view{};
    cudaError_t upload(pfc_ctx *c, const HostProg<W> &h) {
        cudaError_t e = words.upload(c, h.words);
        if (e == cudaSuccess) e = groups.upload(c, h.groups);
        view.words = words.p;
        view.groups = groups.p;
        view.ngroups = (uint32_t)(h.groups.size() / 3);
        view.final_sq = h.final_sq;
        view.corr = h.corr;
        return e;
    }
    void release(pfc_ctx *c) {
        words.release(c);
        groups.release(c);
    }
};

template <class W>
struct DevClass {
    DArr<W> p, s0, s1;
    DArr<uint32_t> nnext;
    uint32_t cap = 0;
    cudaError_t ensure(pfc_ctx *c, uint32_t want) {
        if (want <= cap && p.p) return cudaSuccess;
        release(c);
        const size_t n = std::max<uint32_t>(want, 256);
        cudaError_t e = p.alloc(c, n);
        if (e == cudaSuccess) e = s0.alloc(c, n);
        if (e == cudaSuccess) e = s1.alloc(c, n);
        if (e == cudaSuccess) e = nnext.alloc(c, n);
        if (e == cudaSuccess) cap = (uint32_t)n;
        return e;
    }
    void release(pfc_ctx *c) {
        p.release(c);
        s0.release(c);
        s1.release(c);
        nnext.release(c);
        cap = 0;
    }
    ClassBuf<W> view(const uint32_t *count) const {
        ClassBuf<W> b;
        b.p = p.p;
        b.s0 = s0.p;
        b.s1 = s1.p;
        b.nnext = nnext.p;
        b.cap = cap;
        b.count = count;
        return b;
    }
};

// small per-segment read-back block (pinned host mirror)
struct SegStats {
    uint32_t counts[2];
    uint32_t flags;
    uint32_t tc_err;     // set by the tensor-core setup when a wait gave up
    unsigned long long termsum;
    unsigned long long hits;
};

}  // namespace pfc


namespace pfc {

inline int cuda_fail(cudaError_t e) {
    if (e == cudaErrorMemoryAllocation) return PFC_ERR_NOMEM;
    return e == cudaSuccess ? PFC_OK : PFC_ERR_CUDA;
}
#define CK(x)                                    \
    do {                                         \
        cudaError_t e_ = (x);                    \
        if (e_ != cudaSuccess) return cuda_fail(e_); \
    } while (0)


}  // namespace pfc
