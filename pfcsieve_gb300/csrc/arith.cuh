// arith.cuh -- modular arithmetic for the sieve kernels (sm_103a).
//
// Two size classes of candidate prime p:
//   class 32: p < 2^31, Montgomery with R = 2^32: one 32x32->64 multiply
//             (IMAD.WIDE) plus an IMAD and an IMAD.HI per multiplication;
//             walk residues are signed, in (-p, p) (redc31s).
//   class 64: p >= 2^31, Montgomery with R = 2^64; below 2^64/3 the walk
//             takes lazy one-word steps with R = 2^32 and residues in
//             [0, 2p) (redc64l), and the setup folds each 896-bit table
//             word into 96 bits and multiplies it in with three lazy
//             rounds (mul_wide_word).
//
// The reference keeps every residue in Montgomery form with R = 2^64
// (kernels/iterate.cl:44-50: m_mul(a,b) = a*b/2^64 mod p in [0,p)).  Values
// here are exact residues (canonical, or signed in (-p, p) inside class-32
// walks), so any representation maps back to the reference's by exact
// modular arithmetic; the checksum epilogue reduces and converts class-32
// residues to R = 2^64 before summing.
//
// "redc(a*b)" below always means a*b*R^-1 mod p for a*b < p*R; it is used
// with one operand in plain form (n, a prime q, a table word) so that the
// product drifts by a known power of R which the kernels track (see
// sieve.cu).
#pragma once
#include <cstdint>

namespace pfc {

// ------------------------------------------------------------------ class 32

// p^-1 mod 2^32 for odd p (Newton: x <- x(2 - p x); p*p = 1 mod 8 seeds 3 bits)
__device__ __forceinline__ uint32_t inv32(uint32_t p) {
    uint32_t x = p;
    x *= 2u - p * x;
    x *= 2u - p * x;
    x *= 2u - p * x;
    x *= 2u - p * x;
    return x;
}

// a*b*2^-32 mod p, requires a*b < p*2^32; result in [0,p)
__device__ __forceinline__ uint32_t redc32(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
    uint64_t t = (uint64_t)a * b;
    uint32_t m = (uint32_t)t * pinv;          // m*p = t (mod 2^32)
    uint32_t u = __umulhi(m, p);
    uint32_t th = (uint32_t)(t >> 32);
    uint32_t r = th - u;
    return (th < u) ? r + p : r;
}

// Signed Montgomery step for p < 2^31: x in (-p, p), n < 2^31 (as int32).
// m = lo(x*n) * p^-1 read as a signed 32-bit value, so |m*p| < 2^31 p and
// (x*n - m*p) / 2^32 = hi(x*n) - hi(m*p) lies in (-p, p): no correction step.
// Three multiplies (IMAD.WIDE, IMAD, IMAD.HI) and one subtract; result
// = x*n*2^-32 (mod p).
//
// hi(m*p) is taken from a full 32x32->64 product (mul.wide.s32) rather than a
// multiply-high: on this GPU the wide multiply-add issues at 8.95 Tops/s
// against 7.43 for the multiply-high, so it costs fewer multiply-pipe slots.
__device__ __forceinline__ int32_t redc31s(int32_t x, uint32_t n, int32_t p, uint32_t pinv) {
    const int64_t t = (int64_t)x * (int32_t)n;
    const int32_t m = (int32_t)((uint32_t)t * pinv);
    int64_t u;
    asm("mul.wide.s32 %0, %1, %2;" : "=l"(u) : "r"(m), "r"(p));
    return (int32_t)(t >> 32) - (int32_t)(u >> 32);
}

struct Mont32 {
    uint32_t p, pinv, one /* 2^32 mod p */, r2 /* 2^64 mod p */;
    __device__ __forceinline__ void init(uint32_t p_) {
        p = p_;
        pinv = inv32(p);
        one = (0u - p) % p;
        r2 = (uint32_t)(((uint64_t)one * one) % p);
    }
    __device__ __forceinline__ uint32_t mul(uint32_t a, uint32_t b) const { return redc32(a, b, p, pinv); }
    __device__ __forceinline__ uint32_t to_mont(uint32_t x) const { return redc32(x, r2, p, pinv); }
    // Mont(R^e) = R^(e+1) mod p by square-and-multiply on base Mont(R) = r2
    __device__ __forceinline__ uint32_t mont_R_pow(uint64_t e) const {
        uint32_t acc = one, base = r2;
        while (e) {
            if (e & 1) acc = mul(acc, base);
            base = mul(base, base);
            e >>= 1;
        }
        return acc;
    }
};

// ------------------------------------------------------------------ class 64

__device__ __forceinline__ uint64_t inv64(uint64_t p) {
    uint64_t x = p;
    x *= 2u - p * x;
    x *= 2u - p * x;
    x *= 2u - p * x;
    x *= 2u - p * x;
    x *= 2u - p * x;
    return x;
}

// a*b*2^-64 mod p, requires a*b < p*2^64; result in [0,p).  Same reduction
// as the reference m_mul (kernels/iterate.cl:44-50).
__device__ __forceinline__ uint64_t redc64(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv) {
    uint64_t tl = a * b;
    uint64_t th = __umul64hi(a, b);
    uint64_t m = tl * pinv;
    uint64_t u = __umul64hi(m, p);
    uint64_t r = th - u;
    return (th < u) ? r + p : r;
}

// s*n*2^-64 mod p for a 32-bit multiplier n (s < p): the 96-bit product
// s*n is formed with two 32x64 multiply-adds, then reduced as above.
__device__ __forceinline__ uint64_t redc64_u32(uint64_t s, uint32_t n, uint64_t p, uint64_t pinv) {
    uint64_t lo = (uint64_t)(uint32_t)s * n;
    uint64_t hi = (s >> 32) * (uint64_t)n;     // < 2^64
    uint64_t tl = lo + (hi << 32);
    uint64_t th = (hi >> 32) + (tl < lo ? 1u : 0u);
    uint64_t m = tl * pinv;
    uint64_t u = __umul64hi(m, p);
    uint64_t r = th - u;
    return (th < u) ? r + p : r;
}

__device__ __forceinline__ uint64_t addmod64(uint64_t a, uint64_t b, uint64_t p) {
    uint64_t c = (a >= p - b) ? p : 0;
    return a + b - c;
}

// Lazy walk step for 2^31 < p < 2^63: x*n*2^-32 (mod p) for x in [0, 2p) and
// n < 2^31, result again in [0, 2p), no conditional correction.  Montgomery
// reduction by one 32-bit word with m = lo(x*n) * (-p^-1) mod 2^32:
//   t = x*n = a0 + 2^32 B,  B = x1*n + hi(x0*n)
//   m*p = c0 + 2^32 D,      D = m*p1 + hi(m*p0), and a0 + c0 = 2^32 [a0 != 0]
//   (t + m*p) / 2^32 = B + D + [a0 != 0] < (2p*2^31 + 2^32 p) / 2^32 = 2p.
// Four 32x32->64 multiplies (hi(m*p0) from a wide product, which issues
// faster than a multiply-high on this GPU) and one multiply-low.
__device__ __forceinline__ uint64_t redc64l(uint64_t x, uint32_t n, uint64_t p, uint32_t q) {
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 x0, x1, a0, a1, b0, b1, m, c1, d0, d1, p0, p1, z;\n\t"
        ".reg .u64 A, Bv, D;\n\t"
        "mov.b64 {x0, x1}, %1;\n\t"
        "mov.b64 {p0, p1}, %3;\n\t"
        "mul.wide.u32 A, x0, %2;\n\t"
        "mov.b64 {a0, a1}, A;\n\t"
        "cvt.u64.u32 Bv, a1;\n\t"
        "mad.wide.u32 Bv, x1, %2, Bv;\n\t"
        "mul.lo.u32 m, a0, %4;\n\t"
        "mul.wide.u32 D, m, p0;\n\t"
        "mov.b64 {z, c1}, D;\n\t"
        "cvt.u64.u32 D, c1;\n\t"
        "mad.wide.u32 D, m, p1, D;\n\t"
        "mov.b64 {b0, b1}, Bv;\n\t"
        "mov.b64 {d0, d1}, D;\n\t"
        "add.cc.u32 z, a0, 0xffffffff;\n\t"
        "addc.cc.u32 b0, b0, d0;\n\t"
        "addc.u32 b1, b1, d1;\n\t"
        "mov.b64 %0, {b0, b1};\n\t"
        "}"
        : "=l"(r)
        : "l"(x), "r"(n), "l"(p), "r"(q));
    return r;
}

// One lazy Montgomery round with an accumulator, for multiplying by a
// multi-limb word (p < 2^64/3, s < 2p, c < 3p, any 32-bit limb w):
//   c' = (c + s*w + m*p) / 2^32,  m = lo(c + s*w) * (-p^-1) mod 2^32,
// c' < (3p + 2p*2^32 + 2^32 p) / 2^32 < 3p + 1, so c' < 3p again.
__device__ __forceinline__ uint64_t cios_round(uint64_t c, uint64_t s, uint32_t w, uint64_t p, uint32_t q) {
    uint64_t r;
    asm("{\n\t"
        ".reg .u32 s0, s1, c0, c1, a0, a1, b0, b1, m, h, d0, d1, p0, p1, z;\n\t"
        ".reg .u64 A, Bv, D, C1;\n\t"
        "mov.b64 {s0, s1}, %1;\n\t"
        "mov.b64 {c0, c1}, %2;\n\t"
        "mov.b64 {p0, p1}, %4;\n\t"
        "cvt.u64.u32 A, c0;\n\t"
        "mad.wide.u32 A, s0, %3, A;\n\t"
        "mov.b64 {a0, a1}, A;\n\t"
        "cvt.u64.u32 Bv, a1;\n\t"
        "mad.wide.u32 Bv, s1, %3, Bv;\n\t"
        "cvt.u64.u32 C1, c1;\n\t"
        "add.u64 Bv, Bv, C1;\n\t"
        "mul.lo.u32 m, a0, %5;\n\t"
        "mul.wide.u32 D, m, p0;\n\t"
        "mov.b64 {z, h}, D;\n\t"
        "cvt.u64.u32 D, h;\n\t"
        "mad.wide.u32 D, m, p1, D;\n\t"
        "mov.b64 {b0, b1}, Bv;\n\t"
        "mov.b64 {d0, d1}, D;\n\t"
        "add.cc.u32 z, a0, 0xffffffff;\n\t"
        "addc.cc.u32 b0, b0, d0;\n\t"
        "addc.u32 b1, b1, d1;\n\t"
        "mov.b64 %0, {b0, b1};\n\t"
        "}"
        : "=l"(r)
        : "l"(s), "l"(c), "r"(w), "l"(p), "r"(q));
    return r;
}

// s*W*2^(-32L) (mod p) for an L-limb word W (32-bit limbs, little-endian),
// s in [0, 2p), p < 2^64/3: one plain lazy round (c = 0) and L-1
// accumulating rounds, then one conditional subtraction: result in [0, 2p).
// The setup uses it with L = 3 on a table word already folded to 96 bits.
template <int L>
__device__ __forceinline__ uint64_t mul_wide_word(uint64_t s, const uint32_t (&w)[L], uint64_t p, uint32_t q) {
    uint64_t c = redc64l(s, w[0], p, q);
#pragma unroll
    for (int k = 1; k < L; ++k) c = cios_round(c, s, w[k], p, q);
    return c >= 2 * p ? c - p : c;
}

struct Mont64 {
    uint64_t p, pinv, one /* 2^64 mod p */, r2 /* 2^128 mod p */;
    uint32_t q32;  // -p^-1 mod 2^32 (lazy walk steps)
    __device__ __forceinline__ void init(uint64_t p_) {
        p = p_;
        pinv = inv64(p);
        q32 = 0u - (uint32_t)pinv;
        one = (0ull - p) % p;
        uint64_t two = addmod64(one, one, p);
        uint64_t x = addmod64(two, two, p);         // 4*2^64
        for (int i = 0; i < 5; ++i) x = redc64(x, x, p, pinv);  // 4^(2^5) * 2^64 = 2^128
        r2 = x;
    }
    __device__ __forceinline__ uint64_t mul(uint64_t a, uint64_t b) const { return redc64(a, b, p, pinv); }
    __device__ __forceinline__ uint64_t to_mont(uint64_t x) const { return redc64(x, r2, p, pinv); }
    __device__ __forceinline__ uint64_t mont_R_pow(uint64_t e) const {
        uint64_t acc = one, base = r2;
        while (e) {
            if (e & 1) acc = mul(acc, base);
            base = mul(base, base);
            e >>= 1;
        }
        return acc;
    }
};

// ------------------------------------------------ base-2 strong PRP (SPRP-2)
// Textbook strong probable-prime test to base 2 (the rule of
// kernels/getsegprimes.cl:79-108).  Doubling replaces multiplication by the
// base.  For odd n > 2 only.

__device__ __forceinline__ bool sprp2_32(uint32_t n) {
    Mont32 m;
    m.p = n;
    m.pinv = inv32(n);
    m.one = (0u - n) % n;
    uint32_t nmo = n - m.one;
    int t = __ffs(n - 1) - 1;
    uint32_t d = (n - 1) >> t;
    uint32_t a = m.one + m.one;                    // Mont(2), may be >= n
    if (a >= n || a < m.one) a -= n;
    if (d > 1) {
        int top = 31 - __clz(d);
        for (int b = top - 1; b >= 0; --b) {
            a = m.mul(a, a);
            if ((d >> b) & 1) {
                uint32_t a2 = a + a;
                a = (a2 >= n || a2 < a) ? a2 - n : a2;
            }
        }
    }
    if (a == m.one || a == nmo) return true;
    for (int s = 1; s < t; ++s) {
        a = m.mul(a, a);
        if (a == nmo) return true;
    }
    return false;
}

__device__ __forceinline__ bool sprp2_64(uint64_t n) {
    uint64_t pinv = inv64(n);
    uint64_t one = (0ull - n) % n;
    uint64_t nmo = n - one;
    int t = __ffsll((long long)(n - 1)) - 1;
    uint64_t d = (n - 1) >> t;
    uint64_t a = addmod64(one, one, n);
    if (d > 1) {
        int top = 63 - __clzll((long long)d);
        for (int b = top - 1; b >= 0; --b) {
            a = redc64(a, a, n, pinv);
            if ((d >> b) & 1) a = addmod64(a, a, n);
        }
    }
    if (a == one || a == nmo) return true;
    for (int s = 1; s < t; ++s) {
        a = redc64(a, a, n, pinv);
        if (a == nmo) return true;
    }
    return false;
}

}  // namespace pfc
