/*
 * oracle.h -- CPU restatement of the PFCSieve sieve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * it may be loaded by tests/, by __graft_entry__.smoke() and by the
 * cpu_baseline / reference leg of bench.py, never by the product library
 * (pfcsieve_gb300) or its CLI.
 *
 * Every routine restates the reference algorithm in plain C with 64-bit
 * Montgomery arithmetic exactly as the reference kernels do it, and cites the
 * reference file:line it follows.  Parity is pinned by the reference's own
 * self-test triples (cl_sieve.cpp:1787-2080) and by the reference kernels
 * compiled for the CPU by oracle/Makefile (oracle/_ref, where the reference
 * sources are available).
 */
#ifndef PFC_ORACLE_H
#define PFC_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* mode bits, one or more of them (factorial and compositorial may combine) */
#define ORC_FACTORIAL     1u
#define ORC_PRIMORIAL     2u
#define ORC_COMPOSITORIAL 4u

/* factor record, same layout as the reference's `factor` (cl_sieve.h:8-12):
 * type 0 = n!, 1 = n#, 2 = n!/n#; nc = -n for p | x-1, +n for p | x+1 */
typedef struct {
    uint64_t p;
    int32_t nc;
    int32_t type;
} orc_factor;

/* scalar primitives (verifyprime.cpp:73-109, kernels/getsegprimes.cl:73-108) */
uint64_t orc_invert(uint64_t p);
uint64_t orc_m_mul(uint64_t a, uint64_t b, uint64_t p, uint64_t q);
uint64_t orc_add(uint64_t a, uint64_t b, uint64_t p);
int orc_strong_prp_two(uint64_t n);
int orc_is_prime(uint64_t p);
int orc_verify(uint64_t p, uint32_t n, int32_t c, int32_t type,
               const uint32_t *verifylist, size_t verifylistsize);

/* candidate primes in [pmin, pmax), ascending; returns the total count (which
 * may exceed cap: only the first cap values are written) */
uint64_t orc_candidates(uint64_t pmin, uint64_t pmax, uint64_t *out, uint64_t cap);

/*
 * Run setup + iterate + check for the given candidates.
 *   hits     : factor records (unsorted), at most hit_cap written
 *   *nhits   : total number of hits found (may exceed hit_cap)
 *   *termsum : wrapping sum of the per-candidate checksum terms (check.cl)
 *   terms    : optional, 4 words per candidate: {s6, s7, s4, term}
 * Returns 0, or -1 on bad arguments.
 */
int orc_sieve(unsigned mode, uint32_t nmin, uint32_t nmax,
              const uint64_t *cands, uint64_t ncand, int threads,
              orc_factor *hits, uint64_t hit_cap, uint64_t *nhits,
              uint64_t *termsum, uint64_t *terms);

/*
 * Whole job as the reference's cl_sieve() computes it for one p-range:
 * candidates, residues, hits, CPU verification, 2-PRP filtering and the
 * checksum fold (cl_sieve.cpp:450-593).  `factors` receives the kept
 * (prime-p) factors sorted by (p, |n|, type); at most fac_cap written.
 * Returns 0, -1 bad arguments, -2 a hit failed CPU verification,
 * -3 out of memory.
 */
typedef struct {
    uint64_t checksum;
    uint64_t primecount;
    uint64_t factorcount;
    uint64_t hitcount;      /* hits before 2-PRP filtering */
    uint64_t pairs;         /* candidates x (nmax - nmin) */
} orc_result;

int orc_job(unsigned mode, uint32_t nmin, uint32_t nmax,
            uint64_t pmin, uint64_t pmax, int threads,
            orc_factor *factors, uint64_t fac_cap, orc_result *res);

/* host tables as cl_sieve.cpp builds them; each returns the entry count
 * (only the first cap entries are written):
 *   power table for startN! (cl_sieve.cpp:842-888): prod[i], exp_bit[2i] =
 *   exponent, exp_bit[2i+1] = powmod start bit;
 *   prime products for startN# (cl_sieve.cpp:991-1027);
 *   composite products for the composites below nmin (cl_sieve.cpp:1155-1200) */
uint64_t orc_power_table(uint32_t startN, uint64_t *prod, uint32_t *exp_bit, uint64_t cap);
uint64_t orc_prime_products(uint32_t startN, uint64_t *prod, uint64_t cap);
uint64_t orc_comp_products(uint32_t nmin, uint64_t *prod, uint64_t cap);

/* helper lists (the reference builds them with primesieve) */
uint64_t orc_primes_range(uint32_t lo, uint32_t hi, uint32_t *out, uint64_t cap);

#ifdef __cplusplus
}
#endif
#endif
