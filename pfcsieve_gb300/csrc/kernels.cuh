// kernels.cuh -- device data layout and launch wrappers shared by the
// kernels (gen.cu, sieve.cu) and the C ABI implementation (api.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "host.hpp"
#include "pfcsieve.h"

namespace pfc {

constexpr int kSmallPrimes = 29;          // 3..113, the sieve bound of getsegprimes.cl
constexpr int kPatEntries = 1591;         // sum of the 29 primes: one 64-bit mask per residue

// Candidate list of one size class, structure of arrays in HBM.
//   p      : candidate primes
//   s0, s1 : residues (s0: factorial / primorial / compositorial-only;
//            s1: compositorial of the combined search)
//   nnext  : steps walked so far, summed over the candidate's chains; the
//            check kernel compares it with the steps the search needs
template <class W>
struct ClassBuf {
    W *p;
    W *s0;
    W *s1;
    uint32_t *nnext;
    uint32_t cap;
    const uint32_t *count;   // device counter written by the generator
};

struct HitBuf {
    pfc_factor *buf;
    unsigned long long *count;   // total hits (may exceed cap)
    uint64_t cap;
    uint32_t *tag;               // batches: job slot of each hit (else null)
    uint32_t tagval;
};

// Setup program for one quantity: a product of table words with squarings in
// between (Horner form of prod q^e over the bits of e), followed by one
// correction by a power of R.  groups[3k..3k+2] = {word_begin, word_end,
// squarings_before}; `final_sq` squarings follow the last group.
template <class W>
struct Prog {
    const W *words;
    const uint32_t *groups;
    uint32_t ngroups;
    uint32_t final_sq;
    uint64_t corr;           // apply *R^(corr+1) at the end (drift fix)
};

template <class W>
struct SetupArgs {
    unsigned mode;
    Prog<W> a;       // F: e-program; C: (e-1)-program; P: primorial words; FC: (e-1)-program
    Prog<W> b;       // FC only: primorial words continuing from a (factorial = comp * primorial)
    uint32_t nnext0; // nmin for n walks, 0 for the primorial prime index
};

// One walk launch over step indices [lo, hi).  The multiplier of step k is k
// itself (mult == nullptr: the factorial's n) or mult[k - base] (the
// compositorial's table of n at composite n and 1 at prime n, or the
// primorial's list of primes).  With mult2 set the launch also walks the
// candidate's second residue over mult2 (the compositorial chain of the
// combined search, fused with its factorial chain).  Hits record the
// multiplier.
struct WalkArgs {
    uint32_t lo, hi;
    const uint32_t *mult;
    const uint32_t *mult2;
    uint32_t base;      // index of mult[0] and mult2[0]
    int32_t type;       // factor type of chain-0 hits (PFC_TYPE_*)
    int32_t type2;      // factor type of the fused second chain
    int chain;          // single-chain walks: 0 -> residue s0, 1 -> residue s1
};

// A walk over n split into sub-ranges: candidate i's sub-range k covers steps
// [start[k], start[k+1]) and begins from the residue at start[k], which the
// setup kernel computed into s0/s1 + (k-1) * pitch for k >= 1 (sub-range 0
// begins from the candidate's own state).  One launch walks every (candidate,
// sub-range) pair (grid y = k); the last sub-range leaves the candidate's
// final residue in its state and every sub-range adds its steps to nnext.
// Candidate sets too small to fill the GPU get more chains this way.
constexpr int kMaxSplit = 8;
template <class W>
struct SplitArgs {
    uint32_t start[kMaxSplit + 1];
    uint32_t n;        // sub-ranges (1 = no split)
    uint32_t pitch;    // stride of the start-residue arrays (the class capacity)
    W *s0, *s1;        // start residues of sub-ranges 1 .. n-1
};

// the setup programs of a split walk's boundaries 1..n-1 (n <= kMaxSplit),
// evaluated in one launch (grid y = boundary - 1)
template <class SW>
struct SplitSetup {
    unsigned mode;
    uint32_t n;
    Prog<SW> a[kMaxSplit - 1];
    Prog<SW> b[kMaxSplit - 1];
};

// size classes: class 32 holds p < 2^31, class 64 the rest
constexpr uint64_t kClassSplit = 1ull << 31;
// class-64 segments whose candidates are all below kLazyEnd (3p < 2^64) set
// up with 896-bit table words and walk with lazy one-word steps
constexpr uint64_t kLazyEnd = 0x5555555555555556ull;
constexpr uint64_t kLazyWalkEnd = kLazyEnd;

struct CheckArgs {
    unsigned mode;
    uint32_t nlast;             // nmax - 1
    uint32_t nend;              // steps every candidate must have walked
    unsigned long long *termsum;
    uint32_t *flags;            // bit 0: n-counter validation failure
};

struct GenArgs {
    uint64_t base;     // first odd number of the segment
    uint64_t nodd;     // odd numbers in the segment
    uint32_t *p32;
    uint64_t *p64;
    uint32_t cap32, cap64;
    uint32_t *count;   // [0] class-32 count, [1] class-64 count (may exceed caps)
    const uint64_t *pat;      // kPatEntries sieve masks (device)
    uint32_t bmod[32];        // base mod each of the 29 small primes
    uint32_t share;           // threads per 64-bit word of odd numbers (1, 2 or 4; set by launch_gen)
};

// Launch wrappers (enqueue on `st`); return the number of kernels launched.
int launch_gen(const GenArgs &a, int sms, cudaStream_t st);
int launch_setup32(const ClassBuf<uint32_t> &c, const SetupArgs<WideWord> &a, cudaStream_t st);
int launch_setup64(const ClassBuf<uint64_t> &c, const SetupArgs<uint64_t> &a, cudaStream_t st);
// class 64 below 2^64/3 with 896-bit table words
int launch_setup64w(const ClassBuf<uint64_t> &c, const SetupArgs<WideWord> &a, cudaStream_t st);
// the same with the table-word fold on the tensor cores (setup_tc.cu): each
// program in its paired form (host.hpp TcProg: 1792-bit words, each the
// product of one or two 896-bit words, src[i] = first word | pair << 31)
// first packed once into fp16 byte tiles of tc_tile_words() words
// (tc_tile_bytes() each; tile i holds paired words 128 i ..), then the setup
// over those tiles with the paired programs' groups, final squarings and
// corrections in `a`; a wait that gives up sets *err (the segment then fails
// with PFC_ERR_CUDA)
struct TcTiles {
    const void *tiles;   // device, ntiles * tc_tile_bytes(), 16-byte aligned
    uint32_t ntiles;
};
size_t tc_tile_bytes();
uint32_t tc_tile_words();
int launch_tc_pack(const WideWord *words, const uint32_t *src, uint32_t nw, uint32_t ntiles, void *out,
                   cudaStream_t st);
// (candidate blocks of 64: [block0, block0 + nblocks), nblocks 0 to the end)
uint32_t tc_setup_blocks(uint32_t cands);
int launch_setup64w_tc(const ClassBuf<uint64_t> &c, const SetupArgs<WideWord> &a, const TcTiles &ta,
                       const TcTiles &tb, uint32_t *err, cudaStream_t st, uint32_t block0 = 0,
                       uint32_t nblocks = 0);
// class 32 on the same tiles (the class-32 and lazy class-64 programs are the same)
uint32_t tc_setup_blocks32(uint32_t cands);
// Smallest programs (896-bit words, both programs of the search) set up on the
// tensor cores: below them the kernel's fixed cost per CTA (the 224 position
// residues, TMEM, the first tile's copy and products, the final tree, tens of
// thousands of cycles) outweighs what it saves per word.  Measured on GB300
// (factorial searches, 4e6-wide p ranges), integer pipe against tensor cores:
// class 32 at 235 words 0.22 / 0.33 ms, at 460 words 0.41 / 0.40 ms; class 64
// at 460 words 0.79 / 0.80 ms, at 687 words 1.16 / 0.92 ms, at 20,330 words
// 33.4 / 8.0 ms.
constexpr uint64_t kTcMinWords32 = 448;
constexpr uint64_t kTcMinWords64 = 480;
int launch_setup32_tc(const ClassBuf<uint32_t> &c, const SetupArgs<WideWord> &a, const TcTiles &ta,
                      const TcTiles &tb, uint32_t *err, cudaStream_t st, uint32_t block0 = 0, uint32_t nblocks = 0);
// start residues of a split walk: boundary k's into s0/s1 + (k-1) * c.cap
int launch_split_setup32(const ClassBuf<uint32_t> &c, const SplitSetup<WideWord> &ss, uint32_t *s0, uint32_t *s1,
                         cudaStream_t st);
int launch_split_setup64(const ClassBuf<uint64_t> &c, const SplitSetup<uint64_t> &ss, uint64_t *s0, uint64_t *s1,
                         cudaStream_t st);
int launch_split_setup64w(const ClassBuf<uint64_t> &c, const SplitSetup<WideWord> &ss, uint64_t *s0, uint64_t *s1,
                          cudaStream_t st);
// walk launches: `variant` indexes the walk variants of the size class
// (0 = default; see walk_variant_shape)
// (sp: a split walk, null for the plain one; split walks use each class's
// default shape)
int launch_walk32(const ClassBuf<uint32_t> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st, int variant,
                  const SplitArgs<uint32_t> *sp = nullptr);
// lazy: every candidate is below 2^64/3 (the walk then takes lazy one-word steps)
int launch_walk64(const ClassBuf<uint64_t> &c, const WalkArgs &a, const HitBuf &h, cudaStream_t st, bool lazy,
                  int variant, const SplitArgs<uint64_t> *sp = nullptr);
// size class 0: p < 2^31, 1: lazy class 64 (p < 2^64/3), 2: other class 64
int walk_variant_count(int cls, bool fused);
int walk_variant_shape(int cls, bool fused, int variant, int *nc, int *b);
// compositorial multipliers of n in [lo, hi): n when composite, 1 when prime
// (bit k of primebits <-> n = nmin + k); `out` is padded with 1 to a multiple of
// 16; `ramp` (may be null) receives n itself, the factorial's multipliers
int launch_cmult(uint32_t *out, uint32_t *ramp, const uint32_t *primebits, uint32_t nmin, uint32_t lo, uint32_t hi,
                 cudaStream_t st);
int launch_check32(const ClassBuf<uint32_t> &c, const CheckArgs &a, cudaStream_t st);
int launch_check64(const ClassBuf<uint64_t> &c, const CheckArgs &a, cudaStream_t st);

// host helper: the sieve pattern table (kPatEntries masks) and prime list
void build_pattern_table(uint64_t *pat, uint32_t *primes29);

// Slow products over k in [lo, hi) modulo the self-check test primes
// (verify.cu): products of the primes and of the composites (plain residues)
// and the prime count.
constexpr int kVerifyPrimes = 3;
constexpr uint64_t kVerifyPrime[kVerifyPrimes] = {2147483647ull, 4611686018427387847ull, 18446744073709551557ull};
struct SlowProducts {
    uint64_t P[kVerifyPrimes], C[kVerifyPrimes], count;
};
}  // namespace pfc
struct pfc_ctx;
namespace pfc {
int slow_products(pfc_ctx *c, uint64_t lo, uint64_t hi, SlowProducts &out);


}  // namespace pfc
