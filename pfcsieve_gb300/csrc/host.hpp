// host.hpp -- host-side tables and post-processing for the sieve path.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace pfc {

// 896-bit setup table word (class 64 below 2^64/3): a product of primes as
// 32 little-endian limbs of 28 bits (each limb in the low bits of a u32),
// read on the device with eight 16-byte loads.  The 28-bit radix lets the
// device sum limb x residue products in 64-bit accumulators without carries.
constexpr int kWideLimbs = 32;
constexpr int kWideRadixBits = 28;
struct alignas(16) WideWord {
    uint32_t limb[kWideLimbs];
};

// primes p with lo <= p <= hi (segmented odd-only sieve; replaces the
// primesieve_generate_primes calls of cl_sieve.cpp:850,996,1000,1158,1472,
// 1476,1498)
std::vector<uint32_t> primes_between(uint32_t lo, uint32_t hi);

// Setup program on the host: words, groups {begin, end, squarings}, final
// squarings and the drift correction exponent (see kernels.cuh Prog).  Each
// word, of any width, lowers the power of R of the device value by one.
template <class W>
struct HostProg {
    std::vector<W> words;
    std::vector<uint32_t> groups;
    uint32_t final_sq = 0;
    uint64_t corr = 0;
    uint64_t mulmods() const;   // device multiplications per candidate (excl. correction)
};

// The tensor-core form of a 896-bit program: within each group, consecutive
// pairs of words are multiplied into one 1792-bit word (a group's odd last
// word stays alone), so the device multiplies half as many words into its
// accumulator.  src[i]: index of the first 896-bit word of word i, with bit 31
// set when the next word is multiplied in too.  groups, final_sq and corr are
// those of this word count (each word lowers the power of R by one).
struct TcProg {
    std::vector<uint32_t> src;
    std::vector<uint32_t> groups;
    uint32_t final_sq = 0;
    uint64_t corr = 0;
};
bool build_tc_prog(const HostProg<WideWord> &p, TcProg &out);

// The setup programs of one (mode, startN) in the two word types a context
// caches (a and b as pfc_job_create builds them; b only for the combined
// search), each built on first use.
struct ProgSet {
    HostProg<WideWord> wa, wb;
    HostProg<uint64_t> na, nb;
    bool has_wide = false, has_narrow = false;
    size_t bytes() const {
        return (wa.words.size() + wb.words.size()) * sizeof(WideWord) +
               (na.words.size() + nb.words.size()) * sizeof(uint64_t) +
               (wa.groups.size() + wb.groups.size() + na.groups.size() + nb.groups.size()) * sizeof(uint32_t);
    }
};

// prod over primes q <= startN of q^(e_q - sub), e_q = Legendre exponent of q
// in startN!, in Horner form over the bits of the exponent.  sub = 0 gives
// startN!, sub = 1 gives startN!/startN# (the product of the composites).
template <class W>
bool build_power_prog(uint32_t startN, uint32_t sub, const std::vector<uint32_t> &primes, HostProg<W> &out);

// plain product of the given factors packed into words (one group)
template <class W>
bool build_product_prog(const std::vector<uint32_t> &factors, HostProg<W> &out);

// prime flags for n in [nmin, nmax): bit k <-> nmin + k, plus 2 zero pad words
std::vector<uint32_t> prime_bitmap(uint32_t nmin, uint32_t nmax, const std::vector<uint32_t> &primes);

// 7-base deterministic Miller-Rabin (verifyprime.cpp:157-195)
bool is_prime_u64(uint64_t p);

// CPU re-verification of one factor by naive products (verifyprime.cpp:199-268)
bool verify_factor(uint64_t p, uint32_t n, int32_t c, int32_t type, const uint32_t *list, size_t listsize);

// start value of the verification product of a hit of `type` (34!, 101#,
// 44!/44#; verifyprime.cpp:205,222,241) reduced modulo p
uint64_t verify_start(int type, uint64_t p);

}  // namespace pfc
