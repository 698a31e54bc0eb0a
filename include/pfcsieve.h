/*
 * pfcsieve.h -- C ABI of the GB300 (sm_103a) PFCSieve sieve path.
 *
 * This is the drop-in boundary between a host program (the pfcsieve CLI, a
 * BOINC wrapper, Python via ctypes) and the CUDA kernels.  Plain C types and
 * pointers only.  Every call returns PFC_OK (0) or a negative PFC_ERR_* code;
 * nothing in the library calls exit().
 *
 * Ownership: the context owns all device memory and its CUDA stream; the
 * caller owns every host buffer it passes (pointer + capacity).  One host
 * thread per context.
 *
 * The reference (mfl0p/PFCSieve 1.4, OpenCL) has no library API: its host
 * loop cl_sieve() (cl_sieve.cpp:1328-1761) binds OpenCL kernels by name and
 * sets positional arguments.  Each entry point below names the reference code
 * it replaces.
 */
#ifndef PFCSIEVE_H
#define PFCSIEVE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------- status codes */
#define PFC_OK                 0
#define PFC_ERR_ARG          (-1)  /* invalid argument (setupSearch checks, cl_sieve.cpp:600-641) */
#define PFC_ERR_CUDA         (-2)  /* a CUDA runtime call failed */
#define PFC_ERR_NOMEM        (-3)  /* allocation failed or the memory budget is exceeded */
#define PFC_ERR_HIT_OVERFLOW (-4)  /* more hits than the caller's buffer holds */
#define PFC_ERR_VALIDATION   (-5)  /* the n-counter check failed (kernels/check.cl:61-73) */
#define PFC_ERR_VERIFY       (-6)  /* CPU re-verification of a factor failed (cl_sieve.cpp:515-529) */
#define PFC_ERR_STATE        (-7)  /* call out of order (e.g. iterate before setup) */
#define PFC_ERR_CAND_OVERFLOW (-8) /* candidate buffer overflow (cl_sieve.cpp:462-472) */
#define PFC_ERR_NO_DEVICE    (-9)  /* no CUDA device, or not an sm_103 device */
#define PFC_ERR_IO          (-10)  /* file I/O (factors file, checkpoint) */

/* ------------------------------------------------------------------- modes */
/* Mode bits; PFC_FACTORIAL | PFC_COMPOSITORIAL is the combined search
 * (-! -c), every other combination except single bits is rejected
 * (cl_sieve.cpp:600-617). */
#define PFC_FACTORIAL     1u
#define PFC_PRIMORIAL     2u
#define PFC_COMPOSITORIAL 4u

/* factor types in pfc_factor.type (cl_sieve.h:4-6) */
#define PFC_TYPE_FACTORIAL     0
#define PFC_TYPE_PRIMORIAL     1
#define PFC_TYPE_COMPOSITORIAL 2

/* One hit: p divides n!-1, n#-1 or n!/n#-1 when nc = -n, and the +1 form
 * when nc = +n.  Same 16-byte layout as the reference `factor`
 * (cl_sieve.h:8-12). */
typedef struct {
    uint64_t p;
    int32_t nc;
    int32_t type;
} pfc_factor;

typedef struct pfc_ctx pfc_ctx;
typedef struct pfc_job pfc_job;

/* ----------------------------------------------------------------- context */

/* Select `device`, create the context's stream and its device buffers.
 * `mem_budget` caps the device memory the context's jobs and batches may hold
 * at once (0 = 90% of free memory).  Buffers come from a memory pool of the
 * context, allocated and freed in order on its stream: a freed buffer stays
 * in the pool for the next job (no cudaMalloc, and none of the device-wide
 * synchronisation of cudaFree, per search); the pool gives its idle memory
 * back to the device when an allocation would not fit, and all of it when
 * the context is destroyed.  Replaces the OpenCL platform/context/queue
 * set-up of main.cpp:245-297 and the buffer creation of
 * cl_sieve.cpp:1339-1350,1508-1519. */
int pfc_ctx_create(int device, uint64_t mem_budget, pfc_ctx **out);

/* Free everything the context owns (cleanup(), cl_sieve.cpp:77-103). */
int pfc_ctx_destroy(pfc_ctx *ctx);

/* The context's cudaStream_t (as void*), for callers that time the stages
 * with CUDA events on the launching stream. */
void *pfc_ctx_stream(pfc_ctx *ctx);

/* pfc_segment runs the part of a segment after candidate generation (setup,
 * walk launches, check, stats read-back) as a CUDA graph captured at the
 * job's second segment and replayed for the later ones (re-captured when a
 * buffer or a kernel choice changes; a job's first segment runs on the
 * stream, so one-segment searches pay no capture).  On by default; off (`on` = 0, or PFCSIEVE_CUDA_GRAPHS=0 in
 * the environment when the context is created) runs the same launches on the
 * stream.  Results are identical. */
int pfc_ctx_set_graphs(pfc_ctx *ctx, int on);

/* Split walks.  A segment whose candidates are too few to fill the GPU (a
 * walk of dependent multiplications per candidate leaves most SMs waiting on
 * latency) and whose whole n range fits one walk launch has that range cut
 * into up to 8 sub-ranges: the residue at each boundary b comes from a setup
 * program for (b-1)! (or (b-1)!/(b-1)#, or the primorial below the boundary's
 * prime), and one launch walks every (candidate, sub-range) pair.  Used only
 * when those programs cost under a sixth of the walk (a small nmin), in
 * pfc_segment and in a pfc_iterate call over the whole range.  No
 * counterpart in the reference, which walks each prime's n range in order
 * (kernels/iterate.cl:59-198).  On by default; off (`on` = 0, or
 * PFCSIEVE_SPLIT=0 in the environment when the context is created) walks
 * every candidate in one chain.  Results are identical. */
int pfc_ctx_set_split(pfc_ctx *ctx, int on);

/* Tensor-core setup.  The setup of class-32 candidates and of class-64
 * candidates below 2^64/3 folds each table word against the candidate's
 * position residues; this exact integer contraction runs on the tensor cores
 * (tcgen05, fp16 byte planes with fp32 sums kept below 2^24, so exact), on
 * 1792-bit words that are products of pairs of the program's 896-bit words,
 * and the CUDA cores do the Montgomery products, with the same result as the
 * integer-pipe setup.  No counterpart in the reference, whose setup
 * multiplies its power and product tables one entry at a time
 * (kernels/setup.cl:49-288).  On by default, in pfc_segment, the stage calls
 * and the batch, for searches whose setup programs hold at least 448
 * (class 32) or 480 (class 64) 896-bit words (pfc_setup_program_size);
 * smaller programs, and every program when off (`on` = 0, or
 * PFCSIEVE_SETUP_TC=0 in the environment when the context is created), use
 * the integer-pipe fold.  Results are identical. */
int pfc_ctx_set_setup_tc(pfc_ctx *ctx, int on);

/* Number of kernels this context has launched so far. */
uint64_t pfc_ctx_launch_count(pfc_ctx *ctx);

/* Bytes this context has copied host->device and device->host so far. */
int pfc_ctx_transfer_bytes(pfc_ctx *ctx, uint64_t *h2d, uint64_t *d2h);

/* Device name and SM count, for logs (main.cpp:299-335). */
int pfc_ctx_device_info(pfc_ctx *ctx, char *name, size_t name_cap, int *sm_count);

/* --------------------------------------------------------------------- job */

/* Validate a search and build its host tables: the factorial power table,
 * primorial and compositorial products and the prime lists of the n range
 * (setupSearch cl_sieve.cpp:596-665; setupPowerTable :842-984;
 * setupPrimeProducts :987-1148; setupCompositeProducts :1151-1326; prime list
 * :1494-1499), and upload them.  Range rules are the CLI's: 3 <= pmin < pmax,
 * 101 <= nmin <= nmax < 2^31 (main.cpp:58-72, cl_sieve.cpp:631-641). */
int pfc_job_create(pfc_ctx *ctx, unsigned mode, uint32_t nmin, uint32_t nmax,
                   uint64_t pmin, uint64_t pmax, pfc_job **out);

/* The same call under the name of the stage-call interface: a search of
 * `mode` over n in [nmin, nmax) and p in [pmin, pmax) is submitted to the
 * context that will run its stages (setupSearch, cl_sieve.cpp:596-665, and
 * the per-run table set-up that follows it).  Identical to pfc_job_create. */
int pfc_job_submit(pfc_ctx *ctx, unsigned mode, uint32_t nmin, uint32_t nmax,
                   uint64_t pmin, uint64_t pmax, pfc_job **out);
int pfc_job_destroy(pfc_job *job);

/* Suggest the end of the next p-segment starting at p_lo, sized to the
 * device budget (profileGPU's range, cl_sieve.cpp:669-769). */
int pfc_job_segment_end(pfc_job *job, uint64_t p_lo, uint64_t *p_hi);

/* ---- stage calls: enqueue on the context stream for the current p-segment */

/* Generate the candidate primes of [p_lo, p_hi): 3..113 and every base-2
 * strong probable prime with no factor <= 113.  Resets the segment state.
 * Replaces clearn + addsmallprimes + getsegprimes (cl_sieve.cpp:1572,
 * 1598-1615; kernels/addsmallprimes.cl, kernels/getsegprimes.cl). */
int pfc_gen_candidates(pfc_job *job, uint64_t p_lo, uint64_t p_hi);

/* Starting residues (nmin-1)!, (nmin-1)#, (nmin-1)!/(nmin-1)# mod p for every
 * candidate (the setup chunk loop cl_sieve.cpp:1655-1672; kernels/setup.cl). */
int pfc_setup(pfc_job *job);

/* Advance every candidate over n in [n_lo, n_hi) (primorial: over the primes
 * in that range), appending hits.  Calls must cover [nmin, nmax) in order
 * (the iterate chunk loop cl_sieve.cpp:1696-1719; kernels/iterate.cl). */
int pfc_iterate(pfc_job *job, uint32_t n_lo, uint32_t n_hi);

/* Fold the segment's checksum terms and candidate count into the job totals
 * and run the n-counter check (kernels/check.cl; cl_sieve.cpp:1722). */
int pfc_check(pfc_job *job);

/* gen + setup + iterate over the whole n range (in launches of bounded
 * length) + check for [p_lo, p_hi), enqueued on the context stream; grows the
 * buffers and re-runs on candidate or hit buffer overflow.  Synchronises.
 * The body of the reference's main loop, cl_sieve.cpp:1563-1726. */
int pfc_segment(pfc_job *job, uint64_t p_lo, uint64_t p_hi);

/* Wait for the context stream (waitOnEvent/sleepCPU, cl_sieve.cpp:248-365). */
int pfc_sync(pfc_job *job);

/* Copy the hits found since the last drain to `buf` (unsorted) and clear the
 * device hit list.  *n receives the number of hits; if it exceeds cap, only
 * cap are copied, nothing is cleared and PFC_ERR_HIT_OVERFLOW is returned
 * (the factor read-back of getResults, cl_sieve.cpp:479-494). */
int pfc_drain_hits(pfc_job *job, pfc_factor *buf, size_t cap, size_t *n);

/* Totals over all checked segments: the wrapping 64-bit sum of the
 * per-candidate checksum terms (kernels/check.cl:59,115,161) and the candidate
 * count (cl_sieve.cpp:452-460).  Factor terms are added by
 * pfc_finalize_factors. */
int pfc_job_totals(pfc_job *job, uint64_t *term_checksum, uint64_t *primecount);

/* Whole job [pmin, pmax) in segments; hits are drained into `buf` (capacity
 * cap, *n receives the total).  Returns PFC_ERR_HIT_OVERFLOW with *n set when
 * cap is too small (the caller re-runs with a larger buffer). */
int pfc_job_run(pfc_job *job, pfc_factor *buf, size_t cap, size_t *n);

/* Copy the current segment's candidates (class p < 2^32 first, then the
 * rest) with their residues in the reference's representation, Montgomery
 * with R = 2^64: s0 = the .s6 residue (factorial, primorial or compositorial),
 * s1 = the combined search's compositorial residue (.s4).  For inspection and
 * parity tests; synchronises.  Has no counterpart in the reference, whose
 * records stay on the device (cl_sieve.h:25-35). */
int pfc_segment_state(pfc_job *job, uint64_t *p, uint64_t *s0, uint64_t *s1, size_t cap, size_t *n);

/* (p, n) pairs of all checked segments: candidates x (nmax - nmin). */
uint64_t pfc_job_pairs(pfc_job *job);

/* Multiplications per candidate of the setup programs (class p < 2^32 when
 * cls64 = 0, else p >= 2^32), excluding the final correction. */
uint64_t pfc_job_setup_mulmods(pfc_job *job, int cls64);

/* Check the job's tables on the device against slow products, as the
 * reference checks its power and product tables once per run
 * (kernels/verifyslow.cl, kernels/verify.cl, cl_sieve.cpp:917-970,1100-1140,
 * 1270-1310).  Each setup-program form the job built is run by the setup
 * kernel on a test prime (2^31 - 1, 2^62 - 57, 2^64 - 59) and compared with
 * the products over k in [2, nmin - 1] of the primes and the composites,
 * found by a device Miller-Rabin test; the primorial's prime list and the
 * compositorial's prime flags of [nmin, nmax) are checked by product and
 * count.  PFC_ERR_VALIDATION on a mismatch; *table_bytes (may be NULL)
 * receives the size of the tables checked.  Synchronises. */
int pfc_job_verify_tables(pfc_job *job, uint64_t *table_bytes);

/* ------------------------------------------------- host-side post-processing */

/* Sort hits by (p, |n|, type), re-verify each on the CPU with naive products
 * when `verify` is set (verifyprime.cpp:199-268, OpenMP with `threads`),
 * drop hits whose p is not prime (exact Miller-Rabin with the same
 * verdicts as the reference's 7 bases, verifyprime.cpp:157-195; below 2^32
 * the bases 2, 7, 61) and add n+c of every kept factor to *checksum
 * (cl_sieve.cpp:496-589).  Kept factors are compacted to the front of f;
 * *kept receives their count. */
int pfc_finalize_factors(unsigned mode, uint32_t nmax, pfc_factor *f, size_t n,
                         int threads, int verify, size_t *kept, uint64_t *checksum);

/* The re-verification of pfc_finalize_factors for n hits at once on the GPU
 * of `ctx` (no counterpart in the reference, whose check runs on the CPU,
 * cl_sieve.cpp:509-540): each hit's product of verifyprime.cpp:199-268 -- the
 * start value of its type (34!, 101#, 44!/44#) times every k in [35, n] for a
 * factorial hit, or the list of the search's mode (primes in [103, nmax] for
 * n#, composites in [45, nmax) for n!/n#) up to n -- is formed modulo p as a
 * plain product split over the 256 threads of one CTA per hit, and must be 1
 * for a -1 hit and p - 1 for a +1 hit.  *failed receives the number of hits
 * that fail; bad (n bytes, may be NULL) receives 1 for each failing hit and 0
 * otherwise.  Returns PFC_ERR_VERIFY when any hit fails.  The records are not
 * reordered or changed: pass them to pfc_finalize_factors with verify = 0 for
 * the sort, the 2-PRP filter and the checksum.  At most 2^26 hits per call;
 * PFC_ERR_ARG for more, for a record with an even p or p < 3, n = 0 or a type
 * other than 0, 1, 2.  The prime flags of the verification lists stay in the
 * context for later calls.  Synchronises. */
int pfc_verify_factors_device(pfc_ctx *ctx, unsigned mode, uint32_t nmax, const pfc_factor *f, size_t n,
                              uint8_t *bad, size_t *failed);

/* Size of a search's setup programs, as pfc_job_create builds them (host
 * only, no GPU): *words table words and *squarings squarings per candidate,
 * with 896-bit words (wide = 1: class 32 and class 64 below 2^64/3) or 64-bit
 * words (wide = 0: class 64 above).  For counting the algorithmic work of a
 * run; no counterpart in the reference. */
int pfc_setup_program_size(unsigned mode, uint32_t nmin, int wide, uint64_t *words, uint64_t *squarings);

/* Host replay of a search's setup programs for one odd p (host only, no
 * GPU): the programs pfc_job_create builds, run as the device runs them
 * (each squaring and each product with a table word lowers the power of R,
 * the final correction restores it) in exact modular arithmetic, giving the
 * starting residues the setup must produce: *s0 = (nmin-1)!, (nmin-1)# or
 * (nmin-1)!/(nmin-1)# mod p, and for the combined search also
 * *s1 = (nmin-1)!/(nmin-1)# (else 0).  form 0: 64-bit words; 1: 896-bit
 * words; 2: 896-bit words multiplied in pairs as the tensor-core setup takes
 * them.  A check of the host-built programs against the definition
 * (kernels/setup.cl:49-288 computes the same residues); not used by the
 * sieve. */
int pfc_setup_program_eval(unsigned mode, uint32_t nmin, int form, uint64_t p, uint64_t *s0, uint64_t *s1);

/* Deterministic primality for 64-bit p (verifyprime.cpp:157-195). */
int pfc_is_prime(uint64_t p);

/* Format one factor line as factors.txt holds it (cl_sieve.cpp:565-581);
 * returns the length written (without NUL), or a negative code. */
int pfc_format_factor(const pfc_factor *f, char *buf, size_t cap);

/* --------------------------------------------------- allocation-free segment */

/* Size of the device array that pfc_segment_noalloc works in: 16 MiB, held by
 * every GPU that loads this library from its first use until the process
 * exits. */
#define PFC_NOALLOC_SCRATCH_BYTES (16u << 20)

/* One p-segment [p_lo, p_hi) of a search (the work of pfc_segment) without
 * allocating any device memory: for callers that cannot call cudaMalloc or
 * cudaFree while they run this path, such as a server that has reserved the
 * whole device under its own budget and admits work against it, or a host
 * that must not issue those calls while its other streams are busy (cudaFree
 * synchronises the device).  No counterpart in the reference.
 *
 * The caller passes device buffers: d_hits (capacity hit_cap records; hits
 * beyond it are counted, not written) and d_totals (4 x uint64): the wrapping
 * sum of the checksum terms, the candidate count, the hit count, and flags
 * (bit 0 candidate overflow, bit 1 n-counter validation failure).  Everything
 * else lives in one file-scope device array of PFC_NOALLOC_SCRATCH_BYTES.
 * Work is enqueued on `stream` (a cudaStream_t, 0 for the default stream) on
 * the current device, and the call returns after that stream has finished it.
 *
 * Limits (PFC_ERR_ARG beyond them): at most 2^18 expected candidates per size
 * class (p < 2^31 and p >= 2^31; roughly (p_hi - p_lo) / ln p_lo <= 2^18 / 1.25),
 * nmax - nmin <= 2^22, at most 2^18 primes in [nmin, nmax) for n#, and setup
 * tables of at most 2^12 896-bit words (p < 2^64/3) and 2^16 64-bit words
 * (p >= 2^64/3): nmin up to a few 10^5.  Requests whose nmin is far beyond
 * that are refused before any host table is built.
 *
 * The first call on each device resolves the device address of the array and
 * stores the sieve patterns in it; make that first call before any stream
 * capture.  The call copies tables from host memory that lives only for the
 * call and waits for `stream` before it returns, so a call on a stream that is
 * capturing returns PFC_ERR_STATE and enqueues nothing.  All calls on a device
 * share the array and it keeps the last call's contents (the call clears what
 * must start at zero): calls that overlap on the GPU race, so issue them one
 * at a time per device. */
int pfc_segment_noalloc(unsigned mode, uint32_t nmin, uint32_t nmax, uint64_t p_lo, uint64_t p_hi,
                        pfc_factor *d_hits, uint64_t hit_cap, uint64_t *d_totals, void *stream);

/* ------------------------------------------------------------------ batches */

/* Many searches on one device at once, with continuous batching.  The
 * reference runs one search per process (main.cpp:219-323); a queue of small
 * searches there leaves a large GPU mostly idle.  A batch takes searches as
 * they arrive; every pfc_batch_step admits queued searches while the memory
 * budget and the slots (4096) allow, runs one iteration in which each admitted
 * search advances a bounded stretch of its setup and walk, and retires the
 * searches that finished.  Results equal pfc_job_run's for the same search
 * (hits, checksum terms, candidate count).  No counterpart in the reference. */
typedef struct pfc_batch pfc_batch;

typedef struct {
    unsigned mode;          /* PFC_* mode bits, as for pfc_job_create */
    uint32_t nmin, nmax;    /* n range [nmin, nmax), nmin >= 101, nmax - nmin <= 2^26 */
    uint64_t pmin, pmax;    /* p range [pmin, pmax), pmin >= 3, at most ~2^28 candidates per
                               size class (a batched search keeps all its candidates on the
                               device; larger searches: pfc_job_run, which segments) */
} pfc_job_desc;

typedef struct {
    int done;               /* 1 once the search has finished */
    int status;             /* PFC_OK or the error that ended it */
    uint64_t term_checksum; /* wrapping sum of the checksum terms (as pfc_job_totals) */
    uint64_t primecount;    /* candidates sieved */
    uint64_t pairs;         /* candidates x (nmax - nmin) */
    uint64_t hits;          /* raw hits, before pfc_finalize_factors */
} pfc_batch_status;

int pfc_batch_create(pfc_ctx *ctx, pfc_batch **out);
int pfc_batch_destroy(pfc_batch *b);
/* Queue one search; *id names it in later calls. */
int pfc_batch_submit(pfc_batch *b, const pfc_job_desc *desc, uint64_t *id);
/* One iteration (admit, advance, retire); returns after the GPU finished it.
 * *active / *queued (either may be NULL) receive the searches still running
 * and still waiting. */
int pfc_batch_step(pfc_batch *b, uint32_t *active, uint32_t *queued);
int pfc_batch_result(pfc_batch *b, uint64_t id, pfc_batch_status *r);
/* Raw hits of a finished search (PFC_ERR_HIT_OVERFLOW with *n = the count
 * when cap is short). */
int pfc_batch_take_hits(pfc_batch *b, uint64_t id, pfc_factor *buf, size_t cap, size_t *n);
/* Forget a finished search. */
int pfc_batch_release(pfc_batch *b, uint64_t id);
/* Iterations run so far. */
uint64_t pfc_batch_iterations(pfc_batch *b);
/* Work of one iteration in candidate-steps (a class-64 candidate step counts
 * 3).  Default by policy: 1.6e12 for THROUGHPUT (about 0.6 s of GPU time:
 * every iteration ends with a tail, so long ones waste least), 5e10 for
 * LATENCY (arrivals join and finished searches leave at iteration ends).
 * Smaller values give new searches and finished results a shorter wait,
 * larger ones less tail and host overhead per step. */
int pfc_batch_set_iteration_work(pfc_batch *b, double candidate_steps);

/* Capacity of the batch's shared hit list per iteration (default 2^20
 * records), settable while no search is on the device.  When the hits of an
 * iteration exceed it, every search of that iteration is redone alone with
 * pfc_job_run after it finishes, so results never depend on this size. */
int pfc_batch_set_hit_capacity(pfc_batch *b, uint32_t records);

/* Scheduling policy.  THROUGHPUT (default): every search advances the same
 * number of positions per iteration; a batch submitted at once ends soonest.
 * LATENCY: searches are taken in order of least work left (shortest
 * remaining work first), each with a window that the iteration's budget still
 * pays for; the others wait, except that one that has waited 32 iterations
 * gets a minimal window and the smallest always advances.  For request
 * streams where the median wait matters. */
#define PFC_BATCH_THROUGHPUT 0
#define PFC_BATCH_LATENCY    1
int pfc_batch_set_policy(pfc_batch *b, int policy);

/* Where a batch's time went, summed over its steps. */
typedef struct {
    double step_s;          /* wall time inside pfc_batch_step */
    double gpu_s;           /* iteration kernels: span from launch to the last class finishing */
    double gpu32_s, gpu64_s;/* per size class (the two class kernels overlap) */
    double prep_s;          /* host tables of new searches (overlaps the kernels) */
    double admit_s;         /* uploads and candidate generation of new searches */
    double setup_tc_s;      /* tensor-core setups of new searches: summed GPU spans (throughput
                               policy: overlapping the iterations; latency: chunks before them) */
    uint64_t iterations, tasks;
} pfc_batch_times;
int pfc_batch_timing(pfc_batch *b, pfc_batch_times *t);

/* ------------------------------------------------------------ autotuning */

/* Walk variants: candidates per thread and block length of the walk kernel,
 * per size class (0: p < 2^31; 1: 2^31 <= p < 2^64/3, lazy arithmetic; 2: the
 * rest) and walk kind (fused = 1 for the combined search).  All variants give
 * the same results.  pfc_autotune times each variant of classes 0 and 1 on a
 * synthetic search on this device (about 0.1 s) and keeps the fastest in the
 * context; `report` (may be NULL) receives one line per variant.  Without it
 * the context uses variant 0, the fastest measured on GB300.  The reference
 * sizes its launches by timing the GPU too (profileGPU, cl_sieve.cpp:669-769)
 * but has no kernel variants. */
int pfc_autotune(pfc_ctx *ctx, char *report, size_t cap);
int pfc_ctx_set_walk_variant(pfc_ctx *ctx, int cls, int fused, int variant);
int pfc_ctx_walk_variant(pfc_ctx *ctx, int cls, int fused, int *variant, int *nc, int *block);

/* ------------------------------------------------------------ measurement */

/* Throughput of the integer pipes on `device`, in operations per second:
 * variant 0 = 32-bit multiply-add (IMAD), 1 = 32-bit multiply-high,
 * 2 = 32x32->64 multiply-add, 3 = 32-bit add/xor.  The roofline denominator
 * for the sieve kernels, which are integer-multiply bound.  No counterpart
 * in the reference. */
int pfc_bench_int_peak(int device, int variant, double *ops_per_s);

/* Static description of a status code. */
const char *pfc_status_string(int status);

#ifdef __cplusplus
}
#endif
#endif /* PFCSIEVE_H */
