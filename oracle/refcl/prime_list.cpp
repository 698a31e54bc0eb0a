/*
 * prime_list.cpp -- the prime-list calls of primesieve 12.3 that the reference
 * program makes (primesieve_generate_primes, primesieve_free,
 * primesieve_set_num_threads; cl_sieve.cpp:850,996,1000,1061,1158,1235,1472,
 * 1476,1498 and main.cpp:243), implemented with a plain segmented sieve of
 * Eratosthenes.  TEST INFRASTRUCTURE: linked only into
 * oracle/_ref/pfcsieve_ref; the prebuilt libprimesieve.a is never used.
 *
 * primesieve_generate_primes(start, stop, &size, type) returns the primes in
 * [start, stop] as a malloc'd array of the requested integer width; the
 * reference asks for UINT32_PRIMES below 2^31 only.
 */
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "primesieve.h"

namespace {

std::vector<uint64_t> primes_in(uint64_t lo, uint64_t hi) {
    std::vector<uint64_t> out;
    if (hi < 2 || lo > hi) return out;
    if (lo < 2) lo = 2;
    const uint64_t root = (uint64_t)std::sqrt((double)hi) + 1;
    std::vector<char> small(root + 1, 1);
    std::vector<uint64_t> base;
    for (uint64_t i = 2; i <= root; ++i) {
        if (!small[i]) continue;
        base.push_back(i);
        for (uint64_t j = i * i; j <= root; j += i) small[j] = 0;
    }
    const uint64_t seg = 1u << 20;
    std::vector<char> mark(seg);
    for (uint64_t a = lo; a <= hi; a += seg) {
        const uint64_t b = hi - a < seg - 1 ? hi : a + seg - 1;
        std::fill(mark.begin(), mark.begin() + (b - a + 1), 1);
        for (uint64_t q : base) {
            if (q * q > b) break;
            uint64_t m = (a + q - 1) / q * q;
            if (m < q * q) m = q * q;
            for (; m <= b; m += q) mark[m - a] = 0;
        }
        for (uint64_t x = a; x <= b; ++x)
            if (mark[x - a]) out.push_back(x);
        if (b == hi) break;
    }
    return out;
}

template <class T>
void *pack(const std::vector<uint64_t> &v) {
    T *p = (T *)std::malloc((v.size() ? v.size() : 1) * sizeof(T));
    if (!p) return nullptr;
    for (size_t i = 0; i < v.size(); ++i) p[i] = (T)v[i];
    return p;
}

}  // namespace

extern "C" void *primesieve_generate_primes(uint64_t start, uint64_t stop, size_t *size, int type) {
    const std::vector<uint64_t> v = primes_in(start, stop);
    if (size) *size = v.size();
    switch (type) {
        case UINT16_PRIMES: return pack<uint16_t>(v);
        case UINT32_PRIMES: return pack<uint32_t>(v);
        case UINT64_PRIMES: return pack<uint64_t>(v);
        default: return pack<unsigned>(v);
    }
}

extern "C" void primesieve_free(void *primes) { std::free(primes); }

extern "C" void primesieve_set_num_threads(int) {}
