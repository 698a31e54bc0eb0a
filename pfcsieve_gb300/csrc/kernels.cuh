// kernels.cuh -- device data layout and launch wrappers shared by the
// kernels (gen.cu, sieve.cu) and the C ABI implementation (api.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pfcsieve.h"

namespace pfc {

constexpr int kSmallPrimes = 29;          // 3..113, the sieve bound of getsegprimes.cl
constexpr int kPatEntries = 1591;         // sum of the 29 primes: one 64-bit mask per residue

// Candidate list of one size class, structure of arrays in HBM.
//   p      : candidate primes
//   s0, s1 : residues (s0: factorial / primorial / compositorial-only;
//            s1: compositorial of the combined search)
//   nnext  : next n (or prime index) each candidate will process; the
//            check kernel compares it with the end of the range
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

struct IterArgs {
    unsigned mode;
    uint32_t nmin;              // bit k of compbits <-> n = nmin + k
    uint32_t lo, hi;            // n range (or prime-index range for primorial)
    const uint32_t *primebits;  // prime flags over [nmin, nmax) (+ 2 pad words)
    const uint32_t *qlist;      // primorial: primes in [nmin, nmax)
};

struct CheckArgs {
    unsigned mode;
    uint32_t nlast;             // nmax - 1
    uint32_t nend;              // expected nnext: nmax, or the prime count
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
};

// Launch wrappers (enqueue on `st`); return the number of kernels launched.
int launch_gen(const GenArgs &a, int sms, cudaStream_t st);
int launch_setup32(const ClassBuf<uint32_t> &c, const SetupArgs<uint32_t> &a, cudaStream_t st);
int launch_setup64(const ClassBuf<uint64_t> &c, const SetupArgs<uint64_t> &a, cudaStream_t st);
int launch_iterate32(const ClassBuf<uint32_t> &c, const IterArgs &a, const HitBuf &h, cudaStream_t st);
int launch_iterate64(const ClassBuf<uint64_t> &c, const IterArgs &a, const HitBuf &h, cudaStream_t st);
int launch_check32(const ClassBuf<uint32_t> &c, const CheckArgs &a, cudaStream_t st);
int launch_check64(const ClassBuf<uint64_t> &c, const CheckArgs &a, cudaStream_t st);

// host helper: the sieve pattern table (kPatEntries masks) and prime list
void build_pattern_table(uint64_t *pat, uint32_t *primes29);

}  // namespace pfc
