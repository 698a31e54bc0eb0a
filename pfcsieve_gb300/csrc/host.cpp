// host.cpp -- host tables (prime lists, setup programs) and factor
// post-processing (re-verification, 2-PRP filter, checksum fold, formatting).
#include "host.hpp"

#include <algorithm>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "pfcsieve.h"

namespace pfc {

typedef unsigned __int128 u128;

// ----------------------------------------------------------------- primes

std::vector<uint32_t> primes_between(uint32_t lo, uint32_t hi) {
    std::vector<uint32_t> out;
    if (hi < 2 || hi < lo) return out;
    if (lo <= 2) out.push_back(2);
    const uint64_t root = (uint64_t)std::sqrt((double)hi) + 2;
    std::vector<uint8_t> comp(root + 1, 0);
    std::vector<uint32_t> base;
    for (uint64_t i = 3; i <= root; i += 2) {
        if (comp[i]) continue;
        base.push_back((uint32_t)i);
        for (uint64_t j = i * i; j <= root; j += 2 * i) comp[j] = 1;
    }
    const uint64_t first = std::max<uint64_t>(lo, 3) | 1;  // odd
    if (first > hi) return out;
    const uint64_t nodd = ((uint64_t)hi - first) / 2 + 1;
    const uint64_t seg = 1u << 21;
    const uint64_t nseg = (nodd + seg - 1) / seg;
    std::vector<std::vector<uint32_t>> parts(nseg);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t s = 0; s < (int64_t)nseg; ++s) {
        const uint64_t i0 = (uint64_t)s * seg;
        const uint64_t len = std::min(seg, nodd - i0);
        const uint64_t x0 = first + 2 * i0;  // odd, x_i = x0 + 2i
        std::vector<uint8_t> mark(len, 0);
        for (uint32_t q : base) {
            const uint64_t qq = (uint64_t)q * q;
            if (qq > x0 + 2 * (len - 1)) break;
            uint64_t start;
            if (qq >= x0) start = qq;
            else {
                start = (x0 + q - 1) / q * q;
                if (!(start & 1)) start += q;
            }
            for (uint64_t x = start; x < x0 + 2 * len; x += 2 * (uint64_t)q) mark[(x - x0) / 2] = 1;
        }
        std::vector<uint32_t> &v = parts[s];
        for (uint64_t i = 0; i < len; ++i)
            if (!mark[i] && x0 + 2 * i > 1) v.push_back((uint32_t)(x0 + 2 * i));
    }
    for (auto &v : parts) out.insert(out.end(), v.begin(), v.end());
    return out;
}

std::vector<uint32_t> prime_bitmap(uint32_t nmin, uint32_t nmax, const std::vector<uint32_t> &primes) {
    const uint64_t len = nmax > nmin ? (uint64_t)nmax - nmin : 0;
    std::vector<uint32_t> bits((len + 31) / 32 + 2, 0);
    auto it = std::lower_bound(primes.begin(), primes.end(), nmin);
    for (; it != primes.end() && *it < nmax; ++it) {
        const uint64_t k = *it - nmin;
        bits[k >> 5] |= 1u << (k & 31);
    }
    return bits;
}

// ------------------------------------------------------------ setup programs

template <class W>
uint64_t HostProg<W>::mulmods() const {
    uint64_t t = final_sq + words.size();
    for (size_t g = 0; g + 2 < groups.size(); g += 3) t += groups[g + 2];
    return t;
}

template <class W>
static inline u128 word_max() { return (u128)(W)~(W)0; }
template <class W>
static inline W to_word(u128 v) { return (W)v; }

// greedy: consecutive factors multiplied while the product fits a word
template <class W>
static void pack_words(const std::vector<uint32_t> &f, std::vector<W> &words) {
    const u128 lim = word_max<W>();
    size_t i = 0;
    while (i < f.size()) {
        u128 acc = f[i++];
        while (i < f.size() && acc <= lim / f[i]) acc *= f[i++];
        words.push_back(to_word<W>(acc));
    }
}

// 896-bit words: the product is built in 64-bit limbs over the limbs in use,
// two factors (< 2^62) per multiplication while both fit, then one, and the
// finished word is cut into 28-bit limbs
template <>
void pack_words<WideWord>(const std::vector<uint32_t> &f, std::vector<WideWord> &words) {
    constexpr int L64 = kWideLimbs * kWideRadixBits / 64;
    static_assert(L64 * 64 == kWideLimbs * kWideRadixBits, "whole 64-bit limbs");
    constexpr uint64_t mask = (1ull << kWideRadixBits) - 1u;
    size_t i = 0;
    while (i < f.size()) {
        uint64_t a[L64] = {};
        int used = 1;
        a[0] = f[i++];
        while (i < f.size()) {
            bool joined = false;
            for (int take = i + 1 < f.size() ? 2 : 1; take >= 1 && !joined; --take) {
                const uint64_t m = take == 2 ? (uint64_t)f[i] * f[i + 1] : (uint64_t)f[i];
                uint64_t b[L64];
                u128 carry = 0;
                for (int k = 0; k < used; ++k) {
                    const u128 t = (u128)a[k] * m + carry;
                    b[k] = (uint64_t)t;
                    carry = t >> 64;
                }
                int nu = used;
                if (carry) {
                    if (used == L64) continue;  // would not fit in 896 bits
                    b[nu++] = (uint64_t)carry;
                }
                std::copy(b, b + nu, a);
                used = nu;
                i += (size_t)take;
                joined = true;
            }
            if (!joined) break;
        }
        WideWord w{};
        for (int k = 0; k < kWideLimbs; ++k) {
            const int bit = k * kWideRadixBits, x = bit / 64, sh = bit % 64;
            uint64_t v = a[x] >> sh;
            if (sh + kWideRadixBits > 64 && x + 1 < L64) v |= a[x + 1] << (64 - sh);
            w.limb[k] = (uint32_t)(v & mask);
        }
        words.push_back(w);
    }
}

// drift bookkeeping: the device multiplies Montgomery values, so every
// reduction of a product with a plain table word lowers the power of R by
// one and every squaring maps d -> 2d - 1; the final correction multiplies
// by R^(corr+1) to come back to d = 1 (Montgomery form).
template <class W>
static bool finish_prog(HostProg<W> &p) {
    __int128 d = 1;
    const __int128 lim = (__int128)1 << 62;
    for (size_t g = 0; g + 2 < p.groups.size(); g += 3) {
        for (uint32_t k = 0; k < p.groups[g + 2]; ++k) {
            d = 2 * d - 1;
            if (-d > lim) return false;
        }
        d -= (__int128)(p.groups[g + 1] - p.groups[g]);
    }
    for (uint32_t k = 0; k < p.final_sq; ++k) {
        d = 2 * d - 1;
        if (-d > lim) return false;
    }
    p.corr = (uint64_t)(1 - d);
    return true;
}

bool build_tc_prog(const HostProg<WideWord> &p, TcProg &out) {
    out = TcProg();
    HostProg<uint64_t> shape;   // the groups of the paired words, for the drift correction
    for (size_t g = 0; g + 2 < p.groups.size(); g += 3) {
        const uint32_t b = p.groups[g], e = p.groups[g + 1];
        const uint32_t first = (uint32_t)out.src.size();
        for (uint32_t w = b; w < e; w += 2) out.src.push_back(w + 1 < e ? (w | 0x80000000u) : w);
        shape.groups.push_back(first);
        shape.groups.push_back((uint32_t)out.src.size());
        shape.groups.push_back(p.groups[g + 2]);
    }
    shape.final_sq = p.final_sq;
    if (!finish_prog(shape)) return false;
    out.groups = shape.groups;
    out.final_sq = shape.final_sq;
    out.corr = shape.corr;
    return true;
}

template <class W>
bool build_power_prog(uint32_t startN, uint32_t sub, const std::vector<uint32_t> &primes, HostProg<W> &out) {
    out = HostProg<W>();
    std::vector<std::vector<uint32_t>> bit(32);
    int top = -1;
    for (uint32_t q : primes) {
        if (q > startN) break;
        uint64_t e = 0;
        for (uint64_t qk = q; qk <= startN; qk *= q) e += startN / qk;   // Legendre, cl_sieve.cpp:824-833
        if (e < sub) continue;
        e -= sub;
        for (int j = 0; e; ++j, e >>= 1)
            if (e & 1) {
                bit[j].push_back(q);
                top = std::max(top, j);
            }
    }
    uint32_t pending = 0;
    bool started = false;
    for (int j = top; j >= 0; --j) {
        if (started) ++pending;
        if (bit[j].empty()) continue;
        const uint32_t b = (uint32_t)out.words.size();
        pack_words<W>(bit[j], out.words);
        out.groups.push_back(b);
        out.groups.push_back((uint32_t)out.words.size());
        out.groups.push_back(pending);
        pending = 0;
        started = true;
    }
    out.final_sq = pending;
    return finish_prog(out);
}

template <class W>
bool build_product_prog(const std::vector<uint32_t> &factors, HostProg<W> &out) {
    out = HostProg<W>();
    if (!factors.empty()) {
        pack_words<W>(factors, out.words);
        out.groups = {0u, (uint32_t)out.words.size(), 0u};
    }
    return finish_prog(out);
}

template struct HostProg<uint32_t>;
template struct HostProg<uint64_t>;
template struct HostProg<WideWord>;
template bool build_power_prog<uint32_t>(uint32_t, uint32_t, const std::vector<uint32_t> &, HostProg<uint32_t> &);
template bool build_power_prog<uint64_t>(uint32_t, uint32_t, const std::vector<uint32_t> &, HostProg<uint64_t> &);
template bool build_power_prog<WideWord>(uint32_t, uint32_t, const std::vector<uint32_t> &, HostProg<WideWord> &);
template bool build_product_prog<uint32_t>(const std::vector<uint32_t> &, HostProg<uint32_t> &);
template bool build_product_prog<uint64_t>(const std::vector<uint32_t> &, HostProg<uint64_t> &);
template bool build_product_prog<WideWord>(const std::vector<uint32_t> &, HostProg<WideWord> &);

// ------------------------------------------------------- host Montgomery

struct HMont {
    uint64_t p, q, one, r2;
    explicit HMont(uint64_t p_) : p(p_) {
        uint64_t x = p;
        for (int i = 0; i < 6; ++i) x *= 2 - p * x;
        q = x;
        one = (0 - p) % p;
        r2 = (uint64_t)(((u128)one * one) % p);
    }
    uint64_t mul(uint64_t a, uint64_t b) const {
        const u128 t = (u128)a * b;
        const uint64_t m = (uint64_t)t * q;
        const uint64_t u = (uint64_t)(((u128)m * p) >> 64);
        const uint64_t th = (uint64_t)(t >> 64);
        const uint64_t r = th - u;
        return th < u ? r + p : r;
    }
    uint64_t to(uint64_t x) const { return mul(x, r2); }
    // a + b and a - b mod p for a, b < p, without branches (the finite
    // differences take either side about half the time)
    uint64_t add(uint64_t a, uint64_t b) const {
        const uint64_t d = p - b, s = a - d;
        return s + (p & (0 - (uint64_t)(a < d)));
    }
    uint64_t sub(uint64_t a, uint64_t b) const { return a - b + (p & (0 - (uint64_t)(a < b))); }
};

// the same for p < 2^32 with R = 2^32: values below p held in 64-bit words,
// every product a plain 64-bit multiply (a b < p^2 < 2^64)
struct HMont32 {
    uint64_t p, one, r2;
    uint32_t q;   // p^-1 mod 2^32
    explicit HMont32(uint64_t p_) : p(p_) {
        uint32_t x = (uint32_t)p;
        for (int i = 0; i < 5; ++i) x *= 2u - (uint32_t)p * x;
        q = x;
        one = (1ull << 32) % p;
        r2 = one * one % p;
    }
    // a b 2^-32 mod p for a b < 2^32 p: m p = t (mod 2^32), so t - m p is
    // (hi(t) - hi(m p)) 2^32 exactly, with hi(t) - hi(m p) in (-p, p)
    uint64_t mul(uint64_t a, uint64_t b) const {
        const uint64_t t = a * b;
        const uint32_t m = (uint32_t)t * q;
        const uint64_t th = t >> 32, uh = ((uint64_t)m * p) >> 32;
        return th >= uh ? th - uh : th + p - uh;
    }
    uint64_t to(uint64_t x) const { return mul(x, r2); }   // x < 2^32
    // a + b and a - b mod p for a, b < p, without branches (the finite
    // differences take either side about half the time)
    uint64_t add(uint64_t a, uint64_t b) const {
        const uint64_t d = p - b, s = a - d;
        return s + (p & (0 - (uint64_t)(a < d)));
    }
    uint64_t sub(uint64_t a, uint64_t b) const { return a - b + (p & (0 - (uint64_t)(a < b))); }
};

template <class M>
static bool sprp_base(const M &m, uint32_t base, int t, uint64_t d) {
    const uint64_t nmo = m.p - m.one;
    const uint64_t b = m.to(base);
    uint64_t a = m.one;
    for (int k = 63 - __builtin_clzll(d); k >= 0; --k) {
        a = m.mul(a, a);
        if ((d >> k) & 1) a = m.mul(a, b);
    }
    if (a == m.one || a == nmo) return true;
    for (int s = 1; s < t; ++s) {
        a = m.mul(a, a);
        if (a == nmo) return true;
    }
    return false;
}

template <class M, size_t K>
static bool sprp_bases(uint64_t p, const uint32_t (&bases)[K]) {
    const M m(p);
    const int t = __builtin_ctzll(p - 1);
    const uint64_t d = (p - 1) >> t;
    for (uint32_t b : bases) {
        uint64_t bb = b;
        if (bb >= p) {
            bb %= p;
            if (!bb) continue;
        }
        if (!sprp_base(m, (uint32_t)bb, t, d)) return false;
    }
    return true;
}

// Exact primality, the reference's verdict (verifyprime.cpp:157-195 tests
// the seven bases below, a set with no strong pseudoprime under 2^64).
// Below 2^32 the bases 2, 7, 61 decide it as well (no composite under
// 4,759,123,141 is a strong probable prime to all three; Jaeschke 1993), so
// the verdict is the same with three 32-bit tests instead of seven 64-bit.
bool is_prime_u64(uint64_t p) {
    static const uint32_t bases64[7] = {2, 325, 9375, 28178, 450775, 9780504, 1795265022};
    static const uint32_t bases32[3] = {2, 7, 61};
    if (p < 2) return false;
    if (!(p & 1)) return p == 2;
    if (p < 9) return p > 1;
    return p < (1ull << 32) ? sprp_bases<HMont32>(p, bases32) : sprp_bases<HMont>(p, bases64);
}

// starting products of verifyprime.cpp:205,222,241: 34!, 101#, 44!/44#
static const u128 kStart[3] = {
    ((u128)0xde1bc4d19efcac82ull << 64) | 0x445da75b00000000ull,
    ((u128)0xaf2fa8f8a2d02a93ull << 64) | 0xae69c9f8987d5efeull,
    ((u128)0x98dcc10f185c0e67ull << 64) | 0x3c93ff0000000000ull};

// r * (cur+1) * ... * n in Montgomery form.  Long ranges in blocks of kBlock
// consecutive integers: the block at k = k0 + h j is a polynomial of degree
// kBlock in j, stepped by finite differences (kBlock modular additions and
// one product per block instead of kBlock products), in kChains chains of
// interleaved blocks; shorter ranges in eight interleaved chains of single
// terms (one chain is latency-bound; eight ran 2.7x faster than one on x86);
// the last terms one at a time.  The same residue as the plain product.
template <class M>
static uint64_t mul_range(const M &m, uint64_t r, uint64_t cur, uint64_t n) {
    constexpr int kBlock = 8, kChains = 2;
    constexpr uint64_t kSpan = (uint64_t)kBlock * kChains;   // terms per step of all chains
    const uint64_t steps = n > cur ? (n - cur) / kSpan : 0;
    if (steps >= 64) {
        uint64_t acc[kChains], q[kChains][kBlock + 1];   // q[c][i]: i-th difference at the current block
        for (int c = 0; c < kChains; ++c) {
            uint64_t v[kBlock + 1];   // blocks j = 0..kBlock of chain c: k = cur + 1 + kBlock (c + kChains j)
            for (int j = 0; j <= kBlock; ++j) {
                const uint64_t k = cur + 1 + (uint64_t)kBlock * (c + (uint64_t)kChains * j);
                uint64_t b = m.to(k % m.p);
                for (int i = 1; i < kBlock; ++i) b = m.mul(b, m.to((k + i) % m.p));
                v[j] = b;
            }
            for (int i = 0; i <= kBlock; ++i) {   // forward differences at j = 0
                q[c][i] = v[0];
                for (int j = 0; j < kBlock - i; ++j) v[j] = m.sub(v[j + 1], v[j]);
            }
            acc[c] = c ? m.one : r;
        }
        for (uint64_t t = 0; t < steps; ++t)
            for (int c = 0; c < kChains; ++c) {
                acc[c] = m.mul(acc[c], q[c][0]);
                for (int i = 0; i < kBlock; ++i) q[c][i] = m.add(q[c][i], q[c][i + 1]);
            }
        r = acc[0];
        for (int c = 1; c < kChains; ++c) r = m.mul(r, acc[c]);
        cur += steps * kSpan;
    }
    if (n >= cur + 16) {
        const uint64_t step = m.to(8 % m.p);
        uint64_t a[8], x[8];
        for (int j = 0; j < 8; ++j) {
            a[j] = j ? m.one : r;
            x[j] = m.to((cur + 1 + j) % m.p);
        }
        for (; cur + 8 <= n; cur += 8)
            for (int j = 0; j < 8; ++j) {
                a[j] = m.mul(a[j], x[j]);
                x[j] = m.add(x[j], step);
            }
        r = m.mul(m.mul(m.mul(a[0], a[1]), m.mul(a[2], a[3])), m.mul(m.mul(a[4], a[5]), m.mul(a[6], a[7])));
    }
    for (; cur < n; ++cur) r = m.mul(r, m.to((cur + 1) % m.p));
    return r;
}

// Mont(R^e) = R^(e+1) mod p (square-and-multiply from Mont(R) = R^2)
template <class M>
static uint64_t mont_R_pow(const M &m, uint64_t e) {
    uint64_t acc = m.one, base = m.r2;
    for (; e; e >>= 1, base = m.mul(base, base))
        if (e & 1) acc = m.mul(acc, base);
    return acc;
}

// r * prod list[i], i in [b, e) in Montgomery form: four interleaved chains
// multiply by the plain list values (each product lowers the power of R by
// one, list values < 2^32), and one product with Mont(R^count) restores it
template <class M>
static uint64_t mul_list(const M &m, uint64_t r, const uint32_t *list, size_t b, size_t e) {
    if (b >= e) return r;
    const uint64_t count = e - b;
    uint64_t a[4] = {r, m.one, m.one, m.one};
    for (; b + 4 <= e; b += 4)
        for (int j = 0; j < 4; ++j) a[j] = m.mul(a[j], list[b + j]);
    for (; b < e; ++b) a[0] = m.mul(a[0], list[b]);
    return m.mul(m.mul(m.mul(a[0], a[1]), m.mul(a[2], a[3])), mont_R_pow(m, count));
}

// One walk per (p, type) over the hits of one prime (sorted by |n|):
// the value of verifyprime.cpp:199-268 for each hit.
// Mont(x^-1) from Mont(x) for prime p: Mont(x)^(p-2) in Montgomery form;
// 0 when the product check fails (p composite, or x = 0 mod p)
template <class M>
static uint64_t mont_inverse(const M &m, uint64_t xm) {
    uint64_t y = m.one, b = xm;
    for (uint64_t e = m.p - 2; e; e >>= 1, b = m.mul(b, b))
        if (e & 1) y = m.mul(y, b);
    return m.mul(y, xm) == m.one ? y : 0;
}

template <class M>
static bool verify_group_m(const pfc_factor *h, size_t cnt, const uint32_t *list, size_t listsize,
                           const uint32_t *primes, size_t nprimes) {
    const uint64_t p = h[0].p;
    const M m(p);
    const uint64_t nmo = p - m.one;
    for (int type = 0; type < 3; ++type) {
        bool init = false;
        uint64_t r = 0;   // Montgomery running product
        uint64_t cur = type == 2 ? 44 : 34;   // last integer multiplied in (types 0 and 2)
        size_t li = 0;
        for (size_t k = 0; k < cnt; ++k) {
            if (h[k].type != type) continue;
            if (!init) {
                r = m.to((uint64_t)(kStart[type] % p));
                init = true;
            }
            const uint32_t n = (uint32_t)(h[k].nc < 0 ? -h[k].nc : h[k].nc);
            const int32_t c = h[k].nc < 0 ? -1 : 1;
            if (type == 0) {
                if (cur < n) {
                    r = mul_range(m, r, cur, n);
                    cur = n;
                }
            } else {
                const size_t e = (size_t)(std::upper_bound(list + li, list + listsize, n) - list);
                // the composites of (cur, n] are its integers over its primes: a
                // long range with n < p (no term 0 mod p) as a block product and
                // the inverse of the primes' product, else term by term
                uint64_t inv = 0, prm = m.one;
                if (type == 2 && primes && n < p && cur < n && n - cur >= 4096) {
                    const size_t pb = (size_t)(std::upper_bound(primes, primes + nprimes, (uint32_t)cur) - primes);
                    const size_t pe = (size_t)(std::upper_bound(primes, primes + nprimes, n) - primes);
                    prm = mul_list(m, m.one, primes, pb, pe);
                    inv = mont_inverse(m, prm);
                }
                if (inv) r = m.mul(mul_range(m, r, cur, n), inv);
                else r = mul_list(m, r, list, li, e);
                li = e;
                if (type == 2 && cur < n) cur = n;
            }
            if (!((r == m.one && c == -1) || (r == nmo && c == 1))) return false;
        }
    }
    return true;
}

// p < 2^32 in 32-bit Montgomery arithmetic (R = 2^32), else R = 2^64: the
// products are the same residues either way
// (primes: those of [45, nmax] for the compositorial, else null)
static bool verify_group(const pfc_factor *h, size_t cnt, const uint32_t *list, size_t listsize,
                         const uint32_t *primes = nullptr, size_t nprimes = 0) {
    return h[0].p < (1ull << 32) ? verify_group_m<HMont32>(h, cnt, list, listsize, primes, nprimes)
                                 : verify_group_m<HMont>(h, cnt, list, listsize, primes, nprimes);
}

uint64_t verify_start(int type, uint64_t p) { return (uint64_t)(kStart[type] % p); }

bool verify_factor(uint64_t p, uint32_t n, int32_t c, int32_t type, const uint32_t *list, size_t listsize) {
    pfc_factor f;
    f.p = p;
    f.nc = c < 0 ? -(int32_t)n : (int32_t)n;
    f.type = type;
    return verify_group(&f, 1, list, listsize);
}

}  // namespace pfc

// ==================================================================== C ABI

using namespace pfc;

static bool factor_less(const pfc_factor &a, const pfc_factor &b) {
    if (a.p != b.p) return a.p < b.p;
    const int32_t na = a.nc < 0 ? -a.nc : a.nc, nb = b.nc < 0 ? -b.nc : b.nc;
    if (na != nb) return na < nb;
    if (a.type != b.type) return a.type < b.type;
    return a.nc < b.nc;
}

extern "C" int pfc_finalize_factors(unsigned mode, uint32_t nmax, pfc_factor *f, size_t n, int threads,
                                    int verify, size_t *kept, uint64_t *checksum) {
    if ((!f && n) || !kept || !checksum) return PFC_ERR_ARG;
    std::sort(f, f + n, factor_less);
    // the hits of one p are adjacent: one verification walk and one
    // primality verdict per group
    std::vector<size_t> grp;
    for (size_t i = 0; i < n; ++i)
        if (i == 0 || f[i].p != f[i - 1].p) grp.push_back(i);
    grp.push_back(n);
    const int64_t ngrp = (int64_t)grp.size() - 1;
    std::vector<uint8_t> good((size_t)std::max<int64_t>(ngrp, 0), 0);
    if (verify && n) {
        // verification lists (cl_sieve.cpp:1468-1492)
        std::vector<uint32_t> list, pr;
        if (mode & PFC_PRIMORIAL) {
            list = primes_between(103, nmax);
        } else if (mode & PFC_COMPOSITORIAL) {
            pr = primes_between(45, nmax);
            size_t i = 0;
            for (uint32_t v = 45; v < nmax; ++v) {
                if (i < pr.size() && pr[i] == v) {
                    ++i;
                    continue;
                }
                list.push_back(v);
            }
        }
        int bad = 0;
#ifdef _OPENMP
        if (threads > 0) omp_set_num_threads(threads);
#else
        (void)threads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t g = 0; g < ngrp; ++g) {
            if (!verify_group(f + grp[g], grp[g + 1] - grp[g], list.data(), list.size(),
                              pr.empty() ? nullptr : pr.data(), pr.size())) {
#pragma omp atomic write
                bad = 1;
            }
            good[g] = is_prime_u64(f[grp[g]].p);
        }
        if (bad) return PFC_ERR_VERIFY;
    } else {
        for (int64_t g = 0; g < ngrp; ++g) good[g] = is_prime_u64(f[grp[g]].p);
    }
    // drop 2-PRP factors, fold n+c into the checksum (cl_sieve.cpp:555-589)
    size_t k = 0;
    for (int64_t g = 0; g < ngrp; ++g) {
        if (!good[g]) continue;
        for (size_t i = grp[g]; i < grp[g + 1]; ++i) {
            const uint32_t fn = (uint32_t)(f[i].nc < 0 ? -f[i].nc : f[i].nc);
            const int32_t fc = f[i].nc < 0 ? -1 : 1;
            *checksum += (uint32_t)(fn + (uint32_t)fc);
            f[k++] = f[i];
        }
    }
    *kept = k;
    return PFC_OK;
}

extern "C" int pfc_is_prime(uint64_t p) { return is_prime_u64(p) ? 1 : 0; }

extern "C" int pfc_format_factor(const pfc_factor *f, char *buf, size_t cap) {
    if (!f || !buf) return PFC_ERR_ARG;
    const uint32_t fn = (uint32_t)(f->nc < 0 ? -f->nc : f->nc);
    const int fc = f->nc < 0 ? -1 : 1;
    const char *sym = f->type == PFC_TYPE_FACTORIAL ? "!" : f->type == PFC_TYPE_PRIMORIAL ? "#" : "!/#";
    const int len = snprintf(buf, cap, "%" PRIu64 " | %u%s%+d", f->p, fn, sym, fc);
    return (len < 0 || (size_t)len >= cap) ? PFC_ERR_ARG : len;
}

extern "C" const char *pfc_status_string(int s) {
    switch (s) {
        case PFC_OK: return "ok";
        case PFC_ERR_ARG: return "invalid argument";
        case PFC_ERR_CUDA: return "CUDA runtime error";
        case PFC_ERR_NOMEM: return "out of memory or over the memory budget";
        case PFC_ERR_HIT_OVERFLOW: return "hit buffer overflow";
        case PFC_ERR_VALIDATION: return "gpu validation failure (n counter)";
        case PFC_ERR_VERIFY: return "CPU factor verification failed";
        case PFC_ERR_STATE: return "call out of order";
        case PFC_ERR_CAND_OVERFLOW: return "candidate buffer overflow";
        case PFC_ERR_NO_DEVICE: return "no usable CUDA device";
        case PFC_ERR_IO: return "file I/O error";
        default: return "unknown status";
    }
}
