/*
 * ref_kernels.cpp -- runs the reference's own OpenCL kernels on the CPU.
 *
 * TEST INFRASTRUCTURE.  Built by `make -C oracle ref` into oracle/_ref/ only
 * where the reference sources exist (REF_DIR); nothing here is shipped.
 *
 * kernels/setup.cl and kernels/iterate.cl use no barriers or local memory, so
 * each work-item can run as a plain C++ call: a small shim maps the OpenCL C
 * types and built-ins (ulong, ulong2, uint2, ulong8, mul_hi, get_global_id,
 * atomic_inc, __kernel, __global) onto C++, and the .cl files are #included
 * unmodified from the reference tree.  Their non-NVIDIA branch of mul_wide
 * (a*b and mul_hi) is the one compiled.  verifyprime.cpp is included
 * unmodified as well.
 *
 * The host side restates, for one p-segment, what cl_sieve() does around the
 * kernels: the per-prime record written by getsegprimes
 * (kernels/getsegprimes.cl:214-221), setup launched over table chunks
 * (cl_sieve.cpp:1655-1672) and iterate launched over n chunks with the
 * compositorial prime cursor (cl_sieve.cpp:1696-1719).  The tables are passed
 * in by the caller (the oracle builds them the way cl_sieve.cpp:824-1326
 * does), so this harness pins the oracle's setup/iterate/check arithmetic
 * candidate by candidate against the reference's kernels.
 */
#include <cinttypes>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

/* ---- OpenCL C shim ---- */
typedef uint64_t ulong;
typedef uint32_t uint;
struct ulong2 { ulong s0, s1; };
struct uint2 { uint s0, s1; };
struct ulong8 { ulong s0, s1, s2, s3, s4, s5, s6, s7; };
static inline ulong mul_hi(ulong a, ulong b) { return (ulong)(((unsigned __int128)a * b) >> 64); }
static thread_local uint g_work_item;
static inline uint get_global_id(int) { return g_work_item; }
static inline uint atomic_inc(volatile uint *p) { return __atomic_fetch_add(p, 1u, __ATOMIC_RELAXED); }
#define __kernel
#define __global

namespace ref_setup {
#include "kernels/setup.cl"
}
namespace ref_iterate {
#include "kernels/iterate.cl"
}
namespace ref_vp {
#include "verifyprime.cpp"
}

/* the record getsegprimes/addsmallprimes append (getsegprimes.cl:214-221) */
static ulong8 make_record(uint64_t p)
{
    ulong q = ref_vp::invert(p);
    ulong one = (0 - p) % p;
    ulong nmo = p - one;
    ulong two = ref_vp::add(one, one, p);
    ulong8 r = {p, q, 0, one, two, nmo, 0, 0};
    return r;
}

extern "C" {

/* reference factor record (cl_sieve.h:8-12) */
typedef struct { uint64_t p; int32_t nc; int32_t type; } ref_factor;

int ref_is_prime(uint64_t p) { return ref_vp::isPrime(p) ? 1 : 0; }

int ref_verify(uint64_t p, uint32_t n, int32_t c, int32_t type, uint32_t *list, size_t listsize)
{
    return ref_vp::verify(p, n, c, type, list, listsize) ? 1 : 0;
}

uint64_t ref_m_mul(uint64_t a, uint64_t b, uint64_t p, uint64_t q) { return ref_vp::m_mul(a, b, p, q); }

/*
 * One p-segment through the reference's setup and iterate kernels.
 *   mode       : 1 factorial, 2 primorial, 4 compositorial, 5 both ! and !/#
 *   pow_prod/pow_exp_bit : factorial power table (u64 products, uint2 {exp, curBit})
 *   prod       : primorial prime products or compositorial composite products
 *   iterprimes : primorial: primes in [nmin, nmax-1]; compositorial: primes in
 *                [nmin, nmax+320]
 *   sstep/nstep: chunk sizes for the setup and iterate launches
 *   rec_out    : ncand x 8 words, the final ulong8 records
 *   hits       : factor records, capacity hit_cap; returns -2 if a chunk could
 *                overflow it (the kernels write without a bound)
 */
int ref_segment(unsigned mode, uint32_t nmin, uint32_t nmax,
                const uint64_t *cands, uint64_t ncand,
                const uint64_t *pow_prod, const uint32_t *pow_exp_bit, uint32_t powcount,
                const uint64_t *prod, uint32_t prodcount,
                const uint32_t *iterprimes, uint32_t itersize,
                uint32_t sstep, uint32_t nstep,
                uint64_t *rec_out, ref_factor *hits, uint64_t hit_cap, uint64_t *nhits)
{
    std::vector<ulong8> rec(ncand);
    for (uint64_t i = 0; i < ncand; ++i) rec[i] = make_record(cands[i]);
    std::vector<uint> counts(6, 0);
    counts[0] = (uint)ncand;
    const bool fact = mode & 1, prim = mode & 2, comp = mode & 4;
    uint startN = nmin - 1;
    ulong *pp = const_cast<ulong *>(pow_prod);
    uint2 *pe = reinterpret_cast<uint2 *>(const_cast<uint32_t *>(pow_exp_bit));
    ulong *pr = const_cast<ulong *>(prod);
    uint *ip = const_cast<uint *>(iterprimes);
    ref_iterate::factor *fac = reinterpret_cast<ref_iterate::factor *>(hits);

    /* setup over table chunks (cl_sieve.cpp:1642-1672) */
    uint32_t scount = fact && comp ? (powcount > prodcount ? powcount : prodcount)
                    : fact ? powcount : prodcount;
    for (uint32_t s = 0; s < scount; s += sstep) {
        uint32_t e = s + sstep > scount ? scount : s + sstep;
#pragma omp parallel for schedule(static)
        for (uint64_t g = 0; g < ncand; ++g) {
            g_work_item = (uint)g;
            if (fact && comp)
                ref_setup::combined_setup(rec.data(), counts.data(), pp, s, e, pe, startN, pr, powcount, prodcount);
            else if (fact)
                ref_setup::factorial_setup(rec.data(), counts.data(), pp, s, e, pe, startN);
            else if (prim)
                ref_setup::primorial_setup(rec.data(), counts.data(), pr, s, e);
            else
                ref_setup::compositorial_setup(rec.data(), counts.data(), pr, s, e, startN);
        }
    }

    /* iterate over n chunks (cl_sieve.cpp:1696-1719) */
    uint32_t nstart = prim ? 0 : nmin;
    uint32_t nlimit = prim ? itersize : nmax;
    uint32_t nextprimepos = 0;
    for (; nstart < nlimit; nstart += nstep) {
        uint32_t e = nstart + nstep > nlimit ? nlimit : nstart + nstep;
        if ((uint64_t)counts[2] + 2ull * ncand * (e - nstart) > hit_cap) return -2;
        if (comp)
            while (iterprimes[nextprimepos] < nstart) ++nextprimepos;
#pragma omp parallel for schedule(static)
        for (uint64_t g = 0; g < ncand; ++g) {
            g_work_item = (uint)g;
            if (fact && comp)
                ref_iterate::combined_iterate(rec.data(), counts.data(), fac, nstart, e, ip, nextprimepos);
            else if (fact)
                ref_iterate::factorial_iterate(rec.data(), counts.data(), fac, nstart, e);
            else if (prim)
                ref_iterate::primorial_iterate(rec.data(), counts.data(), fac, nstart, e, ip);
            else
                ref_iterate::compositorial_iterate(rec.data(), counts.data(), fac, nstart, e, ip, nextprimepos);
        }
    }
    *nhits = counts[2];
    memcpy(rec_out, rec.data(), sizeof(ulong8) * ncand);
    return 0;
}

} /* extern "C" */
