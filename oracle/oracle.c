/*
 * oracle.c -- CPU restatement of the PFCSieve sieve path (TEST INFRASTRUCTURE).
 *
 * This file is the checker for the CUDA implementation in pfcsieve_gb300/.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  It restates, routine by routine, what the reference computes; each
 * function names the reference file:line it follows.  It deliberately keeps
 * the reference's arithmetic shape (64-bit Montgomery, R = 2^64, direct
 * product tables, one mulmod per n) so that it is an independent check of
 * the faster algorithms used on the GPU.
 *
 * Parity pins: the reference's self-test triples (cl_sieve.cpp:1787-2080),
 * see tests/test_oracle.py; the reference kernels themselves compiled for the
 * CPU (oracle/ref_kernels.cpp -> oracle/_ref); and the factors.txt files the
 * reference's own OpenCL program wrote for two benchmark searches
 * (tests/test_gpu_configs.py).
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* ---------------------------------------------------------------- arithmetic */

/* Newton iteration for p^-1 mod 2^64 (verifyprime.cpp:73-78,
 * kernels/getsegprimes.cl:73-77) */
uint64_t orc_invert(uint64_t p)
{
    uint64_t inv = 1, prev = 0;
    while (inv != prev) {
        prev = inv;
        inv *= 2 - p * inv;
    }
    return inv;
}

/* Montgomery product a*b/2^64 mod p with q = p^-1 mod 2^64, result in [0,p)
 * whenever a*b < p*2^64 (verifyprime.cpp:81-97, kernels/iterate.cl:44-50) */
uint64_t orc_m_mul(uint64_t a, uint64_t b, uint64_t p, uint64_t q)
{
    u128 ab = (u128)a * b;
    uint64_t ab0 = (uint64_t)ab, ab1 = (uint64_t)(ab >> 64);
    uint64_t m = ab0 * q;
    uint64_t mp = (uint64_t)(((u128)m * p) >> 64);
    uint64_t r = ab1 - mp;
    return (ab1 < mp) ? r + p : r;
}

/* modular add for a, b < p (verifyprime.cpp:100-109, kernels/iterate.cl:52-57) */
uint64_t orc_add(uint64_t a, uint64_t b, uint64_t p)
{
    uint64_t c = (a >= p - b) ? p : 0;
    return a + b - c;
}

/* per-prime Montgomery constants, the record the reference builds in
 * kernels/getsegprimes.cl:214-221 and kernels/setup.cl:68-73 */
typedef struct {
    uint64_t p, q, one, two, nmo, r2;
} mont_t;

static mont_t mont_init(uint64_t p)
{
    mont_t m;
    m.p = p;
    m.q = orc_invert(p);
    m.one = (0 - p) % p;                 /* 2^64 mod p */
    m.nmo = p - m.one;                   /* Mont(-1) */
    m.two = orc_add(m.one, m.one, p);    /* Mont(2) */
    uint64_t r2 = orc_add(m.two, m.two, p);
    for (int i = 0; i < 5; ++i)          /* 4^(2^5) = 2^64 -> 2^128 mod p */
        r2 = orc_m_mul(r2, r2, p, m.q);
    m.r2 = r2;
    return m;
}

static inline uint64_t to_mont(const mont_t *m, uint64_t x)
{
    return orc_m_mul(x, m->r2, m->p, m->q);
}

/* Base-2 strong probable-prime test (kernels/getsegprimes.cl:79-108).
 * When n-1 is a power of two the reference shifts by 64; under OpenCL's
 * shift-count masking that squares 2^(2^64+1) instead of 2.  For every such
 * n below 2^64 that survives the sieve to 113 (257, 65537, 2^32+1, 2^40+1,
 * 2^48+1, 2^56+1) both forms give the same verdict, so the textbook form is
 * used here. */
int orc_strong_prp_two(uint64_t n)
{
    if (n < 3 || !(n & 1)) return n == 2;
    mont_t m = mont_init(n);
    int t = __builtin_ctzll(n - 1);
    uint64_t d = (n - 1) >> t;
    uint64_t a = m.two;
    if (d > 1) {
        uint64_t bit = 1ull << (62 - __builtin_clzll(d));
        while (bit) {
            a = orc_m_mul(a, a, n, m.q);
            if (d & bit) a = orc_add(a, a, n);
            bit >>= 1;
        }
    }
    if (a == m.one || a == m.nmo) return 1;
    for (int s = 1; s < t; ++s) {
        a = orc_m_mul(a, a, n, m.q);
        if (a == m.nmo) return 1;
    }
    return 0;
}

/* strong PRP to base `base` (verifyprime.cpp:116-154) */
static int strong_prp(uint32_t base, const mont_t *m, int t, uint64_t exp, uint64_t curbit)
{
    uint64_t a = to_mont(m, base);
    const uint64_t mbase = a;
    while (curbit) {
        a = orc_m_mul(a, a, m->p, m->q);
        if (exp & curbit) a = orc_m_mul(a, mbase, m->p, m->q);
        curbit >>= 1;
    }
    if (a == m->one || a == m->nmo) return 1;
    for (int s = 1; s < t; ++s) {
        a = orc_m_mul(a, a, m->p, m->q);
        if (a == m->nmo) return 1;
    }
    return 0;
}

/* deterministic 7-base Miller-Rabin for 64-bit p (verifyprime.cpp:157-195) */
int orc_is_prime(uint64_t p)
{
    static const uint32_t bases[7] = {2, 325, 9375, 28178, 450775, 9780504, 1795265022};
    if (p < 2) return 0;
    if (p % 2 == 0) return p == 2;
    if (p == 3) return 1;
    mont_t m = mont_init(p);
    int t = __builtin_ctzll(p - 1);
    uint64_t exp = p >> t;
    uint64_t curbit = (exp > 1) ? (1ull << (62 - __builtin_clzll(exp))) : 0;
    for (int i = 0; i < 7; ++i) {
        uint32_t base = bases[i];
        if (base >= p) {
            base %= p;
            if (base == 0) continue;
        }
        if (!strong_prp(base, &m, t, exp, curbit)) return 0;
    }
    return 1;
}

/* slow CPU verification of one factor (verifyprime.cpp:199-268): recompute
 * n!, n# or n!/n# mod p from 34!, 101# or 44!/44# by naive products */
int orc_verify(uint64_t p, uint32_t n, int32_t c, int32_t type,
               const uint32_t *list, size_t listsize)
{
    uint64_t r = 0;
    if (type == 0) {
        const u128 f34 = ((u128)0xde1bc4d19efcac82ull << 64) | 0x445da75b00000000ull;
        r = (uint64_t)(f34 % p);
        for (uint32_t i = 35; i <= n; ++i) r = (uint64_t)(((u128)r * i) % p);
    } else {
        const u128 c0 = (type == 1)
            ? (((u128)0xaf2fa8f8a2d02a93ull << 64) | 0xae69c9f8987d5efeull)   /* 101# */
            : (((u128)0x98dcc10f185c0e67ull << 64) | 0x3c93ff0000000000ull);  /* 44!/44# */
        r = (uint64_t)(c0 % p);
        for (size_t i = 0; i < listsize; ++i) {
            if (list[i] > n) break;
            r = (uint64_t)(((u128)r * list[i]) % p);
        }
    }
    if (r == 1 && c == -1) return 1;
    if (r == p - 1 && c == 1) return 1;
    return 0;
}

/* ------------------------------------------------------------ prime lists */

/* odd-only bit sieve: returns bits where bit i set <=> 2i+1 composite */
static uint8_t *odd_sieve(uint64_t limit)
{
    uint64_t nbits = limit / 2 + 1;
    uint8_t *bits = (uint8_t *)calloc((nbits + 7) / 8, 1);
    if (!bits) return NULL;
    bits[0] |= 1; /* 1 is not prime */
    for (uint64_t i = 3; i * i <= limit; i += 2) {
        if (bits[i >> 4] & (1u << ((i >> 1) & 7))) continue;
        for (uint64_t j = i * i; j <= limit; j += 2 * i)
            bits[j >> 4] |= (uint8_t)(1u << ((j >> 1) & 7));
    }
    return bits;
}

static inline int sieve_is_prime(const uint8_t *bits, uint64_t x)
{
    if (x < 2) return 0;
    if (!(x & 1)) return x == 2;
    return !(bits[x >> 4] & (1u << ((x >> 1) & 7)));
}

/* primes in [lo, hi] inclusive (primesieve_generate_primes semantics, as
 * called at cl_sieve.cpp:850,996,1000,1061,1158,1235,1472,1476,1498) */
uint64_t orc_primes_range(uint32_t lo, uint32_t hi, uint32_t *out, uint64_t cap)
{
    if (hi < lo) return 0;
    uint8_t *bits = odd_sieve(hi);
    if (!bits) return 0;
    uint64_t cnt = 0;
    for (uint64_t x = lo; x <= hi; ++x) {
        if (sieve_is_prime(bits, x)) {
            if (cnt < cap) out[cnt] = (uint32_t)x;
            ++cnt;
        }
    }
    free(bits);
    return cnt;
}

/* ------------------------------------------------------ candidate primes */

static const uint32_t k_small_primes[29] = {
    3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53,
    59, 61, 67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113};

/*
 * Candidates in [pmin, pmax): the primes 3..113 in range
 * (kernels/addsmallprimes.cl:25-38, cl_sieve.cpp:1599-1605), then every odd
 * x >= 114 with no prime factor <= 113 (the mod-30 wheel and bit tables of
 * kernels/getsegprimes.cl:110-197) that is a base-2 strong probable prime
 * (kernels/getsegprimes.cl:213-223).  Base-2 strong pseudoprimes with no
 * factor <= 113 are candidates, exactly as in the reference.
 */
#define SEG_ODDS (1u << 20)

uint64_t orc_candidates(uint64_t pmin, uint64_t pmax, uint64_t *out, uint64_t cap)
{
    uint64_t count = 0;
    for (int i = 0; i < 29; ++i) {
        uint64_t sp = k_small_primes[i];
        if (sp >= pmin && sp < pmax) {
            if (count < cap) out[count] = sp;
            ++count;
        }
    }
    uint64_t lo = pmin < 114 ? 114 : pmin;
    if (lo >= pmax) return count;
    uint64_t base0 = lo | 1;                       /* first odd >= lo */
    if (base0 >= pmax) return count;
    uint64_t nodd = (pmax - base0 + 1) / 2;        /* odds in [base0, pmax) */
    uint64_t nseg = (nodd + SEG_ODDS - 1) / SEG_ODDS;

    uint64_t **segv = (uint64_t **)calloc(nseg, sizeof(uint64_t *));
    uint64_t *segn = (uint64_t *)calloc(nseg, sizeof(uint64_t));
    if (!segv || !segn) { free(segv); free(segn); return 0; }

#pragma omp parallel for schedule(dynamic, 1)
    for (uint64_t s = 0; s < nseg; ++s) {
        uint64_t first = s * (uint64_t)SEG_ODDS;
        uint64_t len = nodd - first < SEG_ODDS ? nodd - first : SEG_ODDS;
        uint64_t base = base0 + 2 * first;         /* odd, x_i = base + 2i */
        uint8_t *mark = (uint8_t *)calloc(len, 1);
        uint64_t *vals = (uint64_t *)malloc(sizeof(uint64_t) * (len / 2 + 64));
        uint64_t nv = 0;
        for (int k = 0; k < 29; ++k) {
            uint64_t sp = k_small_primes[k];
            uint64_t r = base % sp;
            uint64_t off = r ? sp - r : 0;         /* base + off = multiple of sp */
            if (off & 1) off += sp;                /* make it odd (base is odd) */
            for (uint64_t i = off / 2; i < len; i += sp) mark[i] = 1;
        }
        for (uint64_t i = 0; i < len; ++i) {
            if (mark[i]) continue;
            uint64_t x = base + 2 * i;
            if (orc_strong_prp_two(x)) vals[nv++] = x;
        }
        free(mark);
        segv[s] = vals;
        segn[s] = nv;
    }
    for (uint64_t s = 0; s < nseg; ++s) {
        for (uint64_t i = 0; i < segn[s]; ++i) {
            if (count < cap) out[count] = segv[s][i];
            ++count;
        }
        free(segv[s]);
    }
    free(segv);
    free(segn);
    return count;
}

/* ------------------------------------------------------------ host tables */

typedef struct {
    uint64_t *prod;     /* products of table words */
    uint32_t *exp;      /* factorial power table: exponent (.s0) */
    uint32_t *curbit;   /* factorial power table: top-bit cursor (.s1) */
    uint64_t n;
} table_t;

static void table_free(table_t *t)
{
    free(t->prod);
    free(t->exp);
    free(t->curbit);
    memset(t, 0, sizeof(*t));
}

/* Legendre exponent of `prime` in startN! and its powmod start bit
 * (cl_sieve.cpp:824-839) */
static void get_power(uint32_t prime, uint32_t startN, uint32_t *e, uint32_t *cb)
{
    uint32_t total = 0;
    uint64_t cur = prime;
    uint32_t q = startN / (uint32_t)cur;
    for (;;) {
        total += q;
        cur *= prime;
        if (cur > startN) break;
        q = (uint32_t)(startN / cur);
    }
    uint32_t bit = 0x80000000u;
    if (total > 1) bit >>= (__builtin_clz(total) + 1);
    *e = total;
    *cb = bit;
}

/* factorial power table for (nmin-1)!: primes merged while the exponent is
 * equal and the product fits 64 bits (cl_sieve.cpp:842-888) */
static int build_power_table(uint32_t startN, table_t *t)
{
    uint64_t cap = startN + 1;
    uint32_t *pr = (uint32_t *)malloc(sizeof(uint32_t) * (cap / 2 + 16));
    if (!pr) return -3;
    uint64_t np = orc_primes_range(2, startN, pr, cap / 2 + 16);
    t->prod = (uint64_t *)malloc(sizeof(uint64_t) * (np + 1));
    t->exp = (uint32_t *)malloc(sizeof(uint32_t) * (np + 1));
    t->curbit = (uint32_t *)malloc(sizeof(uint32_t) * (np + 1));
    if (!t->prod || !t->exp || !t->curbit) { free(pr); return -3; }
    uint32_t e, cb;
    get_power(pr[0], startN, &e, &cb);
    t->prod[0] = pr[0];
    t->exp[0] = e;
    t->curbit[0] = cb;
    uint64_t m = 1;
    for (uint64_t i = 1; i < np; ++m) {
        get_power(pr[i], startN, &e, &cb);
        t->prod[m] = pr[i];
        t->exp[m] = e;
        t->curbit[m] = cb;
        for (++i; i < np; ++i) {
            uint32_t e2, cb2;
            get_power(pr[i], startN, &e2, &cb2);
            if (e2 != t->exp[m]) break;
            u128 pp = (u128)t->prod[m] * pr[i];
            if (pp > 0xFFFFFFFFFFFFFFFFull) break;
            t->prod[m] = (uint64_t)pp;
        }
    }
    t->n = m;
    free(pr);
    return 0;
}

/* greedy 64-bit packing of a list of factors (cl_sieve.cpp:1011-1020,
 * 1184-1193) */
static int pack_products(const uint32_t *v, uint64_t nv, table_t *t)
{
    t->prod = (uint64_t *)malloc(sizeof(uint64_t) * (nv + 1));
    if (!t->prod) return -3;
    uint64_t m = 0;
    for (uint64_t i = 0; i < nv; ++m) {
        t->prod[m] = v[i];
        for (++i; i < nv; ++i) {
            u128 pp = (u128)t->prod[m] * v[i];
            if (pp > 0xFFFFFFFFFFFFFFFFull) break;
            t->prod[m] = (uint64_t)pp;
        }
    }
    t->n = m;
    return 0;
}

/* primorial product table for (nmin-1)# (cl_sieve.cpp:991-1027) */
static int build_prime_products(uint32_t startN, table_t *t)
{
    uint64_t cap = startN / 2 + 16;
    uint32_t *pr = (uint32_t *)malloc(sizeof(uint32_t) * cap);
    if (!pr) return -3;
    uint64_t np = orc_primes_range(2, startN, pr, cap);
    int rc = pack_products(pr, np, t);
    free(pr);
    return rc;
}

/* compositorial product table for (nmin-1)!/(nmin-1)#: the composites
 * 4, 6, 8, 9, ... below nmin (cl_sieve.cpp:1155-1200) */
static int build_comp_products(uint32_t nmin, table_t *t)
{
    uint8_t *bits = odd_sieve(nmin);
    uint32_t *cv = (uint32_t *)malloc(sizeof(uint32_t) * (nmin + 1));
    if (!bits || !cv) { free(bits); free(cv); return -3; }
    uint64_t nc = 0;
    for (uint32_t n = 2; n < nmin; ++n)
        if (!sieve_is_prime(bits, n)) cv[nc++] = n;
    int rc = pack_products(cv, nc, t);
    free(bits);
    free(cv);
    return rc;
}

uint64_t orc_power_table(uint32_t startN, uint64_t *prod, uint32_t *exp_bit, uint64_t cap)
{
    table_t t = {0, 0, 0, 0};
    if (build_power_table(startN, &t)) { table_free(&t); return 0; }
    for (uint64_t i = 0; i < t.n && i < cap; ++i) {
        prod[i] = t.prod[i];
        exp_bit[2 * i] = t.exp[i];
        exp_bit[2 * i + 1] = t.curbit[i];
    }
    uint64_t n = t.n;
    table_free(&t);
    return n;
}

uint64_t orc_prime_products(uint32_t startN, uint64_t *prod, uint64_t cap)
{
    table_t t = {0, 0, 0, 0};
    if (build_prime_products(startN, &t)) { table_free(&t); return 0; }
    for (uint64_t i = 0; i < t.n && i < cap; ++i) prod[i] = t.prod[i];
    uint64_t n = t.n;
    table_free(&t);
    return n;
}

uint64_t orc_comp_products(uint32_t nmin, uint64_t *prod, uint64_t cap)
{
    table_t t = {0, 0, 0, 0};
    if (build_comp_products(nmin, &t)) { table_free(&t); return 0; }
    for (uint64_t i = 0; i < t.n && i < cap; ++i) prod[i] = t.prod[i];
    uint64_t n = t.n;
    table_free(&t);
    return n;
}

/* --------------------------------------------------- setup, iterate, check */

typedef struct {
    unsigned mode;
    uint32_t nmin, nmax;
    table_t pow, pprod, cprod;
    uint32_t *iterprimes;       /* primorial: primes in [nmin, nmax-1] */
    uint64_t niter;
    uint8_t *nbits;             /* odd sieve to nmax (compositorial skip) */
} plan_t;

static void plan_free(plan_t *pl)
{
    table_free(&pl->pow);
    table_free(&pl->pprod);
    table_free(&pl->cprod);
    free(pl->iterprimes);
    free(pl->nbits);
}

static int plan_init(plan_t *pl, unsigned mode, uint32_t nmin, uint32_t nmax)
{
    memset(pl, 0, sizeof(*pl));
    pl->mode = mode;
    pl->nmin = nmin;
    pl->nmax = nmax;
    int rc = 0;
    if (mode & ORC_FACTORIAL) rc |= build_power_table(nmin - 1, &pl->pow);
    if (mode & ORC_PRIMORIAL) {
        rc |= build_prime_products(nmin - 1, &pl->pprod);
        uint64_t cap = (uint64_t)(nmax - nmin) / 2 + 16;
        pl->iterprimes = (uint32_t *)malloc(sizeof(uint32_t) * cap);
        if (!pl->iterprimes) return -3;
        pl->niter = orc_primes_range(nmin, nmax - 1, pl->iterprimes, cap);
    }
    if (mode & ORC_COMPOSITORIAL) {
        rc |= build_comp_products(nmin, &pl->cprod);
        pl->nbits = odd_sieve(nmax);
        if (!pl->nbits) return -3;
    }
    return rc ? -3 : 0;
}

/* left-to-right powmod with the reference's cursor bit (setup.cl:96-110) */
static uint64_t powmod_table(const mont_t *m, uint64_t base, uint32_t e, uint32_t cb)
{
    if (e == 1) return base;
    uint64_t a = base;
    while (cb) {
        a = orc_m_mul(a, a, m->p, m->q);
        if (e & cb) a = orc_m_mul(a, base, m->p, m->q);
        cb >>= 1;
    }
    return a;
}

/* Mont((nmin-1)!) from the power table (setup.cl:65-112) */
static uint64_t setup_factorial(const mont_t *m, const table_t *t)
{
    /* entry 0 is the prime 2: powmod by doubling (setup.cl:78-88) */
    uint32_t e = t->exp[0], cb = t->curbit[0];
    uint64_t a = m->two;
    while (cb) {
        a = orc_m_mul(a, a, m->p, m->q);
        if (e & cb) a = orc_add(a, a, m->p);
        cb >>= 1;
    }
    uint64_t r = a;
    for (uint64_t i = 1; i < t->n; ++i) {
        uint64_t base = to_mont(m, t->prod[i]);
        r = orc_m_mul(r, powmod_table(m, base, t->exp[i], t->curbit[i]), m->p, m->q);
    }
    return r;
}

/* Mont(product of the table words) (setup.cl:143-152, 185-194) */
static uint64_t setup_products(const mont_t *m, const table_t *t)
{
    uint64_t r = 0;
    for (uint64_t i = 0; i < t->n; ++i) {
        uint64_t w = to_mont(m, t->prod[i]);
        r = i ? orc_m_mul(r, w, m->p, m->q) : w;
    }
    return r;
}

typedef struct {
    orc_factor *v;
    uint64_t n, cap;
} hitbuf_t;

static void hit_push(hitbuf_t *h, uint64_t p, int32_t nc, int32_t type)
{
    if (h->n == h->cap) {
        uint64_t nc2 = h->cap ? 2 * h->cap : 64;
        orc_factor *nv = (orc_factor *)realloc(h->v, nc2 * sizeof(orc_factor));
        if (!nv) return;
        h->v = nv;
        h->cap = nc2;
    }
    h->v[h->n].p = p;
    h->v[h->n].nc = nc;
    h->v[h->n].type = type;
    h->n++;
}

/* One candidate through setup + iterate + check.  Returns its checksum term
 * (check.cl:59 for !, !/#; :115 for #; :161 for ! with !/#). */
static uint64_t sieve_one(const plan_t *pl, uint64_t p, hitbuf_t *hits, uint64_t st[3])
{
    const mont_t m = mont_init(p);
    uint64_t s4 = 0, s6 = 0, s7 = 0;
    const unsigned mode = pl->mode;

    if (mode & ORC_PRIMORIAL) {
        /* primorial_setup (setup.cl:120-157), primorial_iterate
         * (iterate.cl:88-115): multiply Mont(q) at each prime q in [n, N) */
        s6 = setup_products(&m, &pl->pprod);
        for (uint64_t j = 0; j < pl->niter; ++j) {
            uint32_t q = pl->iterprimes[j];
            uint64_t mq = to_mont(&m, q);
            s6 = orc_m_mul(s6, mq, p, m.q);
            if (s6 == m.one || s6 == m.nmo)
                hit_push(hits, p, (s6 == m.one) ? -(int32_t)q : (int32_t)q, 1);
        }
        st[0] = s6; st[1] = 0; st[2] = 0;
        return s6;
    }

    s7 = to_mont(&m, pl->nmin - 1);          /* Mont(nmin-1), setup.cl:75 */
    const int fact = (mode & ORC_FACTORIAL) != 0;
    const int comp = (mode & ORC_COMPOSITORIAL) != 0;
    if (fact && comp) {
        s6 = setup_factorial(&m, &pl->pow);   /* combined_setup, setup.cl:202-288 */
        s4 = setup_products(&m, &pl->cprod);
    } else if (fact) {
        s6 = setup_factorial(&m, &pl->pow);
    } else {
        s6 = setup_products(&m, &pl->cprod);  /* compositorial_setup */
    }

    for (uint32_t n = pl->nmin; n < pl->nmax; ++n) {
        s7 = orc_add(s7, m.one, p);
        if (fact) {
            /* factorial_iterate (iterate.cl:72-80) / combined (:173-180) */
            s6 = orc_m_mul(s6, s7, p, m.q);
            if (s6 == m.one || s6 == m.nmo)
                hit_push(hits, p, (s6 == m.one) ? -(int32_t)n : (int32_t)n, 0);
        }
        if (comp) {
            /* compositorial_iterate skips prime n (iterate.cl:137-148,
             * 181-190) */
            if (sieve_is_prime(pl->nbits, n)) continue;
            uint64_t *rc = fact ? &s4 : &s6;
            *rc = orc_m_mul(*rc, s7, p, m.q);
            if (*rc == m.one || *rc == m.nmo)
                hit_push(hits, p, (*rc == m.one) ? -(int32_t)n : (int32_t)n, 2);
        }
    }
    st[0] = s6; st[1] = s7; st[2] = s4;
    if (fact && comp) return s4 + s6 + s7;
    return s6 + s7;
}

static int mode_ok(unsigned mode)
{
    if (mode == ORC_FACTORIAL || mode == ORC_PRIMORIAL || mode == ORC_COMPOSITORIAL) return 1;
    return mode == (ORC_FACTORIAL | ORC_COMPOSITORIAL);
}

/* setup + iterate + check for all candidates; the hits are returned in a
 * malloc'd array owned by the caller */
static int sieve_all(unsigned mode, uint32_t nmin, uint32_t nmax,
                     const uint64_t *cands, uint64_t ncand, int threads,
                     orc_factor **hits_out, uint64_t *nhits,
                     uint64_t *termsum, uint64_t *terms)
{
    if (!mode_ok(mode) || nmin < 2 || nmax <= nmin) return -1;
    plan_t pl;
    if (plan_init(&pl, mode, nmin, nmax)) { plan_free(&pl); return -3; }
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    uint64_t total = 0;
    hitbuf_t all = {0, 0, 0};
#pragma omp parallel
    {
        hitbuf_t hb = {0, 0, 0};
        uint64_t local = 0;
#pragma omp for schedule(dynamic, 8)
        for (uint64_t i = 0; i < ncand; ++i) {
            uint64_t st[3];
            uint64_t term = sieve_one(&pl, cands[i], &hb, st);
            local += term;
            if (terms) {
                terms[4 * i + 0] = st[0];
                terms[4 * i + 1] = st[1];
                terms[4 * i + 2] = st[2];
                terms[4 * i + 3] = term;
            }
        }
#pragma omp critical
        {
            total += local;
            for (uint64_t k = 0; k < hb.n; ++k)
                hit_push(&all, hb.v[k].p, hb.v[k].nc, hb.v[k].type);
        }
        free(hb.v);
    }
    plan_free(&pl);
    *hits_out = all.v;
    *nhits = all.n;
    *termsum = total;
    return 0;
}

int orc_sieve(unsigned mode, uint32_t nmin, uint32_t nmax,
              const uint64_t *cands, uint64_t ncand, int threads,
              orc_factor *hits, uint64_t hit_cap, uint64_t *nhits,
              uint64_t *termsum, uint64_t *terms)
{
    orc_factor *v = NULL;
    int rc = sieve_all(mode, nmin, nmax, cands, ncand, threads, &v, nhits, termsum, terms);
    if (rc == 0)
        for (uint64_t k = 0; k < *nhits && k < hit_cap; ++k) hits[k] = v[k];
    free(v);
    return rc;
}

/* The verdicts of orc_verify() for every hit of one prime p (hits sorted by
 * |n|), computed with one product walk per factor type instead of one walk per
 * hit; 64-bit arithmetic below 2^32 as verifyprime.cpp:209-217 does. */
static int verify_group(const orc_factor *h, uint64_t cnt, const uint32_t *vlist, uint64_t vsize)
{
    const uint64_t p = h[0].p;
    const int small = p < 0xFFFFFFFFull;
    for (int type = 0; type < 3; ++type) {
        uint64_t r = 0, cur = 34;
        size_t li = 0;
        int init = 0;
        for (uint64_t k = 0; k < cnt; ++k) {
            if (h[k].type != type) continue;
            if (!init) {
                const u128 c0 = (type == 0)
                    ? (((u128)0xde1bc4d19efcac82ull << 64) | 0x445da75b00000000ull)
                    : (type == 1)
                    ? (((u128)0xaf2fa8f8a2d02a93ull << 64) | 0xae69c9f8987d5efeull)
                    : (((u128)0x98dcc10f185c0e67ull << 64) | 0x3c93ff0000000000ull);
                r = (uint64_t)(c0 % p);
                init = 1;
            }
            uint32_t n = (uint32_t)(h[k].nc < 0 ? -h[k].nc : h[k].nc);
            int32_t c = h[k].nc < 0 ? -1 : 1;
            if (type == 0) {
                for (uint64_t i = cur + 1; i <= n; ++i)
                    r = small ? (r * i) % p : (uint64_t)(((u128)r * i) % p);
                if (n > cur) cur = n;
            } else {
                for (; li < vsize && vlist[li] <= n; ++li)
                    r = small ? (r * vlist[li]) % p : (uint64_t)(((u128)r * vlist[li]) % p);
            }
            if (!((r == 1 && c == -1) || (r == p - 1 && c == 1))) return 0;
        }
    }
    return 1;
}

/* ------------------------------------------------------------ whole job */

static int factor_cmp(const void *a, const void *b)
{
    const orc_factor *x = (const orc_factor *)a, *y = (const orc_factor *)b;
    if (x->p != y->p) return x->p < y->p ? -1 : 1;
    int32_t nx = x->nc < 0 ? -x->nc : x->nc, ny = y->nc < 0 ? -y->nc : y->nc;
    if (nx != ny) return nx < ny ? -1 : 1;
    if (x->type != y->type) return x->type < y->type ? -1 : 1;
    return x->nc < y->nc ? -1 : (x->nc > y->nc);
}

int orc_job(unsigned mode, uint32_t nmin, uint32_t nmax,
            uint64_t pmin, uint64_t pmax, int threads,
            orc_factor *factors, uint64_t fac_cap, orc_result *res)
{
    if (!mode_ok(mode) || nmin < 101 || nmax <= nmin || pmin < 3 || pmax <= pmin) return -1;
    memset(res, 0, sizeof(*res));

    uint64_t ncand = orc_candidates(pmin, pmax, NULL, 0);
    uint64_t *cands = (uint64_t *)malloc(sizeof(uint64_t) * (ncand + 1));
    if (!cands) return -3;
    orc_candidates(pmin, pmax, cands, ncand);

    uint64_t nh = 0, termsum = 0;
    orc_factor *hits = NULL;
    int rc = sieve_all(mode, nmin, nmax, cands, ncand, threads, &hits, &nh, &termsum, NULL);
    free(cands);
    if (rc) { free(hits); return rc; }
    res->primecount = ncand;
    res->checksum = termsum;
    res->hitcount = nh;
    res->pairs = ncand * (uint64_t)(nmax - nmin);

    /* verification lists (cl_sieve.cpp:1468-1492) */
    uint32_t *vlist = NULL;
    uint64_t vsize = 0;
    if (mode & ORC_PRIMORIAL) {
        uint64_t c = nmax / 2 + 16;
        vlist = (uint32_t *)malloc(sizeof(uint32_t) * c);
        vsize = orc_primes_range(103, nmax, vlist, c);
    } else if (mode & ORC_COMPOSITORIAL) {
        uint8_t *bits = odd_sieve(nmax);
        vlist = (uint32_t *)malloc(sizeof(uint32_t) * (nmax + 1));
        for (uint32_t n = 45; n < nmax; ++n)
            if (!sieve_is_prime(bits, n)) vlist[vsize++] = n;
        free(bits);
    }

    /* sort, verify, filter 2-PRPs, fold checksum (cl_sieve.cpp:496-589) */
    qsort(hits, nh, sizeof(orc_factor), factor_cmp);
    /* group boundaries: hits of one p are contiguous after the sort */
    uint64_t *grp = (uint64_t *)malloc(sizeof(uint64_t) * (nh + 1));
    uint64_t ng = 0;
    for (uint64_t i = 0; i < nh; ++i)
        if (i == 0 || hits[i].p != hits[i - 1].p) grp[ng++] = i;
    grp[ng] = nh;
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 4)
    for (uint64_t g = 0; g < ng; ++g) {
        if (!verify_group(hits + grp[g], grp[g + 1] - grp[g], vlist, vsize)) {
#pragma omp atomic write
            bad = 1;
        }
    }
    free(grp);
    free(vlist);
    if (bad) { free(hits); return -2; }

    uint64_t lastgood = 0, kept = 0;
    for (uint64_t i = 0; i < nh; ++i) {
        uint64_t fp = hits[i].p;
        if (fp == lastgood || orc_is_prime(fp)) {
            lastgood = fp;
            uint32_t fn = (uint32_t)(hits[i].nc < 0 ? -hits[i].nc : hits[i].nc);
            int32_t fc = hits[i].nc < 0 ? -1 : 1;
            res->checksum += (uint32_t)(fn + fc);
            if (kept < fac_cap) factors[kept] = hits[i];
            ++kept;
        }
    }
    res->factorcount = kept;
    free(hits);
    return 0;
}
