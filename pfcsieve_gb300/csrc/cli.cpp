// cli.cpp -- the pfcsieve command line, a drop-in for the reference's
// (main.cpp, cl_sieve.cpp) on top of the C ABI.
//
//   pfcsieve -! | -# | -c | -! -c  -n N0 -N N1 -p P0 -P P1 [-v threads] [-s] [-h]
//
// Same options, number suffixes, range checks, messages, factors.txt lines,
// checksum line and checkpoint files (stateA.ckp / stateB.ckp hold the
// reference's workStatus struct byte for byte, so a run can resume from a
// checkpoint either program wrote).
#include <getopt.h>

#include <cerrno>
#include <chrono>
#include <cinttypes>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "pfcsieve.h"

#define RESULTS_FILENAME "factors.txt"
#define STATE_FILENAME_A "stateA.ckp"
#define STATE_FILENAME_B "stateB.ckp"

// checkpoint record, same layout as the reference's workStatus (cl_sieve.h:14-18)
struct workStatus {
    uint64_t pmin, pmax, p, checksum, primecount, factorcount, last_trickle, state_sum;
    uint32_t nmin, nmax;
    bool factorial, primorial, compositorial;
};

struct Search {
    uint32_t threads = 2;
    bool test = false;
    int device = 0;
    bool write_state_a_next = true;
};

static void fail() { exit(EXIT_FAILURE); }

static void help() {
    printf("Welcome to PFCSieve, a CUDA program for GB300 to find factors of primorial, factorial, and "
           "compositorial prime candidates of the form n#+-1, n!+-1, and n!/#+-1\n");
    printf("Program usage:\n");
    printf("-!\tUse factorial mode\n");
    printf("-#\tUse primorial mode\n");
    printf("-c\tUse compositorial mode\n");
    printf("\t\tNote: -! -c can be used together to find factors of both at the same time.\n");
    printf("-n #\tStart primorial n#+-1, factorial n!+-1, or compositorial n!/#+-1\n");
    printf("-N #\tEnd primorial N#+-1, factorial N!+-1, or compositorial N!/#+-1\n");
    printf("\t\tN range is 101 <= -n < -N < 2^31, [-n, -N) exclusive\n");
    printf("-p #\tStarting prime factor p\n");
    printf("-P #\tEnd prime factor P\n");
    printf("\t\tP range is 3 <= -p < -P < 2^64, [-p, -P) exclusive\n");
    printf("\t\tNote for primorial and factorial there are no factors when p <= n\n");
    printf("\t\tNote N!+-1, N#+-1, and N!/#+-1 are not divisible by 2.\n");
    printf("-v #\tOptional, specify the number of CPU threads used to verify factors.  Default is 2, max is 128.\n");
    printf("-s \tPerform self test to verify proper operation of the program with the current GPU.\n");
    printf("-h\tPrint this help\n");
    fail();
}

// Number arguments: an integer (decimal, 0x hex or 0 octal) with at most one
// suffix that scales it.  The accepted suffixes are the reference's
// (putil.c:34-116): K M G T P scale by 1000^1..5, k m g t p by 1024^1..5,
// e<d> / E<d> by 10^d and b<d> / B<d> by 2^d, where d is a number that ends
// the text.  Each suffix is a (factor, repeat count) pair; the value is then
// scaled by one checked multiplication per repeat.
struct NumberSuffix {
    char letter;
    uint64_t factor;
    int repeats;  // -1: the repeat count is the number written after the letter
};

static const NumberSuffix kNumberSuffixes[] = {
    {'K', 1000, 1}, {'M', 1000, 2}, {'G', 1000, 3}, {'T', 1000, 4}, {'P', 1000, 5},
    {'k', 1024, 1}, {'m', 1024, 2}, {'g', 1024, 3}, {'t', 1024, 4}, {'p', 1024, 5},
    {'e', 10, -1},  {'E', 10, -1},  {'b', 2, -1},   {'B', 2, -1},
};

// 0: *out holds the value; -1: the text is not a number with an accepted
// suffix; -2: the number, or the number scaled, lies outside [lo, hi].
static int parse_u64(uint64_t *out, const char *s, uint64_t lo, uint64_t hi) {
    errno = 0;
    char *end = nullptr;
    uint64_t value = strtoull(s, &end, 0);
    if (errno != 0 || value > hi) return -2;

    uint64_t factor = 1, repeats = 0;
    if (*end != '\0') {
        const NumberSuffix *suffix = nullptr;
        for (const NumberSuffix &cand : kNumberSuffixes)
            if (cand.letter == *end) suffix = &cand;
        if (suffix == nullptr) return -1;
        const char *rest = end + 1;
        factor = suffix->factor;
        if (suffix->repeats >= 0) {
            repeats = (uint64_t)suffix->repeats;
        } else {
            char *after = nullptr;
            errno = 0;
            repeats = strtoull(rest, &after, 0);
            if (errno != 0) return -2;
            rest = after;
        }
        if (*rest != '\0') return -1;
    }

    for (uint64_t i = 0; i < repeats && value != 0; ++i) {
        if (value > hi / factor) return -2;
        value *= factor;
    }
    if (value < lo) return -2;
    *out = value;
    return 0;
}

static int parse_u32(uint32_t *out, const char *s, uint32_t lo, uint32_t hi) {
    uint64_t v = 0;
    int st = parse_u64(&v, s, lo, hi);
    if (st == 0) *out = (uint32_t)v;
    return st;
}

// option handling (main.cpp:50-112)
static int parse_option(int opt, const char *arg, workStatus &st, Search &sd) {
    switch (opt) {
        case 'p': return parse_u64(&st.pmin, arg, 3, 0xFFFFFFFFFFFFFFFFull - 1);
        case 'P': return parse_u64(&st.pmax, arg, 4, 0xFFFFFFFFFFFFFFFFull);
        case 'n': return parse_u32(&st.nmin, arg, 101, 0x7FFFFFFF - 1);
        case 'N': return parse_u32(&st.nmax, arg, 102, 0x7FFFFFFF);
        case 'v': return parse_u32(&sd.threads, arg, 1, 128);
        case 'd':             // --device: accepted, not used
        case 'f': return 0;   // accepted and ignored, as in the reference
        case 's':
            sd.test = true;
            fprintf(stderr, "Performing self test.\n");
            printf("Performing self test.\n");
            return 0;
        case '!':
            st.factorial = true;
            fprintf(stderr, "-! argument specified for factorial mode.\n");
            printf("\n-! argument specified for factorial mode.\n\n");
            return 0;
        case '#':
            st.primorial = true;
            fprintf(stderr, "-# argument specified for primorial mode.\n");
            printf("\n-# argument specified for primorial mode.\n\n");
            return 0;
        case 'c':
            st.compositorial = true;
            fprintf(stderr, "-c argument specified for compositorial mode.\n");
            printf("\n-c argument specified for compositorial mode.\n\n");
            return 0;
        case 'h':
        case '?':
            help();
            return 0;
        default: return -3;
    }
}

static const struct option long_opts[] = {
    {"device", optional_argument, 0, 'd'}, {"test", no_argument, 0, 's'}, {0, 0, 0, 0}};

static void process_args(int argc, char **argv, workStatus &st, Search &sd) {
    int ind = -1, opt;
    while ((opt = getopt_long(argc, argv, "p:P:n:N:v:s!#cfh", long_opts, &ind)) != -1) {
        const int r = parse_option(opt, optarg, st, sd);
        if (r == -1 || r == -2) {
            const char *what = r == -1 ? "invalid" : "out of range";
            if (ind == -1) {
                printf("%s: %s argument -%c %s\n", argv[0], what, opt, optarg ? optarg : "");
                fprintf(stderr, "%s: %s argument -%c %s\n", argv[0], what, opt, optarg ? optarg : "");
            } else {
                printf("%s: %s argument --%s %s\n", argv[0], what, long_opts[ind].name, optarg ? optarg : "");
                fprintf(stderr, "%s: %s argument --%s %s\n", argv[0], what, long_opts[ind].name,
                        optarg ? optarg : "");
            }
            fail();
        } else if (r != 0) {
            printf("unknown command line argument\n");
            fail();
        }
        ind = -1;
    }
    if (optind < argc) {
        fprintf(stderr, "%s: invalid non-option argument %s\n", argv[0], argv[optind]);
        fail();
    }
}

// ------------------------------------------------------------- checkpoint

static uint64_t state_sum(const workStatus &s) {
    return s.pmin + s.pmax + s.p + s.checksum + s.primecount + s.factorcount + s.last_trickle + s.nmin + s.nmax;
}

// cl_sieve.cpp:107-136
static void write_state(workStatus &st, Search &sd) {
    st.state_sum = state_sum(st);
    const char *fn = sd.write_state_a_next ? STATE_FILENAME_A : STATE_FILENAME_B;
    FILE *out = fopen(fn, "wb");
    if (!out) {
        fprintf(stderr, "Cannot open %s !!!\n", fn);
        return;
    }
    if (fwrite(&st, sizeof(workStatus), 1, out) != 1) {
        fprintf(stderr, "Cannot write checkpoint to file. Continuing...\n");
        fclose(out);
        return;
    }
    if (fclose(out) == 0) sd.write_state_a_next = !sd.write_state_a_next;
}

static bool read_one(const char *fn, const workStatus &want, workStatus &got) {
    FILE *in = fopen(fn, "rb");
    if (!in) return false;
    bool ok = true;
    if (fread(&got, sizeof(workStatus), 1, in) != 1) {
        fprintf(stderr, "Cannot parse %s !!!\n", fn);
        printf("Cannot parse %s !!!\n", fn);
        ok = false;
    } else if (got.pmin != want.pmin || got.pmax != want.pmax || got.nmin != want.nmin ||
               got.nmax != want.nmax || got.factorial != want.factorial || got.primorial != want.primorial ||
               got.compositorial != want.compositorial) {
        fprintf(stderr, "Invalid checkpoint file %s !!!\n", fn);
        printf("Invalid checkpoint file %s !!!\n", fn);
        ok = false;
    } else if (state_sum(got) != got.state_sum) {
        fprintf(stderr, "Checksum error in %s !!!\n", fn);
        printf("Checksum error in %s !!!\n", fn);
        ok = false;
    }
    fclose(in);
    return ok;
}

// cl_sieve.cpp:139-233: both files validated, the one with the larger p wins
static bool read_state(workStatus &st, Search &sd) {
    workStatus a, b;
    bool ga = read_one(STATE_FILENAME_A, st, a);
    bool gb = read_one(STATE_FILENAME_B, st, b);
    if (ga && gb) {
        if (a.p > b.p) gb = false;
        else ga = false;
    }
    if (ga) {
        st = a;
        sd.write_state_a_next = false;
        printf("Resuming from checkpoint in %s\n", STATE_FILENAME_A);
        return true;
    }
    if (gb) {
        st = b;
        sd.write_state_a_next = true;
        printf("Resuming from checkpoint in %s\n", STATE_FILENAME_B);
        return true;
    }
    return false;
}

static void checkpoint(workStatus &st, Search &sd) {
    write_state(st, sd);
    printf("Checkpoint, current p: %" PRIu64 "\n", st.p);
}

// ---------------------------------------------------------------- results

// drain, verify, filter and append (getResults, cl_sieve.cpp:450-593)
static int get_results(pfc_job *job, workStatus &st, const Search &sd, uint64_t &term_prev, uint64_t &count_prev) {
    uint64_t term = 0, count = 0;
    pfc_job_totals(job, &term, &count);
    st.checksum += term - term_prev;
    st.primecount += count - count_prev;
    term_prev = term;
    count_prev = count;
    std::vector<pfc_factor> buf(1 << 16);
    size_t n = 0;
    int rc;
    while ((rc = pfc_drain_hits(job, buf.data(), buf.size(), &n)) == PFC_ERR_HIT_OVERFLOW && n > buf.size())
        buf.resize(n);
    if (rc != PFC_OK) return rc;
    if (n == 0) return PFC_OK;
    printf("processing %zu factors on CPU\n", n);
    if (n > 1) printf("sorting factors\n");
    printf("Verifying factors on CPU...\n");
    const unsigned mode = (st.factorial ? PFC_FACTORIAL : 0u) | (st.primorial ? PFC_PRIMORIAL : 0u) |
                          (st.compositorial ? PFC_COMPOSITORIAL : 0u);
    size_t kept = 0;
    uint64_t add = 0;
    rc = pfc_finalize_factors(mode, st.nmax, buf.data(), n, (int)sd.threads, 1, &kept, &add);
    if (rc == PFC_ERR_VERIFY) {
        fprintf(stderr, "CPU factor verification failed!\n");
        printf("\nCPU factor verification failed!\n");
        return rc;
    }
    if (rc != PFC_OK) return rc;
    fprintf(stderr, "Verified %zu factors.\n", n);
    printf("\rVerified %zu factors.\n", n);
    if (kept < n) {
        fprintf(stderr, "discarded %zu 2-PRP factors\n", n - kept);
        printf("discarded %zu 2-PRP factors\n", n - kept);
    }
    FILE *res = fopen(RESULTS_FILENAME, "a");
    if (!res) {
        fprintf(stderr, "Cannot open %s !!!\n", RESULTS_FILENAME);
        return PFC_ERR_IO;
    }
    printf("writing factors to %s\n", RESULTS_FILENAME);
    char line[128];
    for (size_t i = 0; i < kept; ++i) {
        if (pfc_format_factor(&buf[i], line, sizeof(line)) < 0 || fprintf(res, "%s\n", line) < 0) {
            fprintf(stderr, "Cannot write to %s !!!\n", RESULTS_FILENAME);
            fclose(res);
            return PFC_ERR_IO;
        }
    }
    fclose(res);
    st.factorcount += kept;
    st.checksum += add;
    return PFC_OK;
}

// finalizeResults (cl_sieve.cpp:772-822)
static int finalize_results(const workStatus &st) {
    if (st.factorcount) {
        FILE *f = fopen(RESULTS_FILENAME, "r");
        if (!f) {
            fprintf(stderr, "Cannot open %s !!!\n", RESULTS_FILENAME);
            return PFC_ERR_IO;
        }
        char line[256];
        uint64_t lc = 0;
        while (fgets(line, sizeof(line), f)) ++lc;
        fclose(f);
        if (lc < st.factorcount) {
            fprintf(stderr, "ERROR: Missing factors in %s !!!\n", RESULTS_FILENAME);
            printf("ERROR: Missing factors in %s !!!\n", RESULTS_FILENAME);
            return PFC_ERR_IO;
        }
    }
    FILE *f = fopen(RESULTS_FILENAME, "a");
    if (!f) {
        fprintf(stderr, "Cannot open %s !!!\n", RESULTS_FILENAME);
        return PFC_ERR_IO;
    }
    int w = st.factorcount ? fprintf(f, "%016" PRIX64 "\n", st.checksum)
                           : fprintf(f, "no factors\n%016" PRIX64 "\n", st.checksum);
    fclose(f);
    return w < 0 ? PFC_ERR_IO : PFC_OK;
}

static bool truncate_results() {
    FILE *f = fopen(RESULTS_FILENAME, "w");
    if (!f) {
        fprintf(stderr, "Cannot open %s !!!\n", RESULTS_FILENAME);
        return false;
    }
    fclose(f);
    return true;
}

// ------------------------------------------------------------------ search

static unsigned mode_bits(const workStatus &st) {
    return (st.factorial ? PFC_FACTORIAL : 0u) | (st.primorial ? PFC_PRIMORIAL : 0u) |
           (st.compositorial ? PFC_COMPOSITORIAL : 0u);
}

// setupSearch's mode and range checks (cl_sieve.cpp:596-641)
static void setup_search(workStatus &st, bool announce = true) {
    st.p = st.pmin;
    int z = (int)st.factorial + (int)st.primorial + (int)st.compositorial;
    if (!z) {
        printf("\n-! or -# or -c argument is required\nuse -h for help\n");
        fprintf(stderr, "-! or -# or -c argument is required\nuse -h for help\n");
        fail();
    } else if (st.factorial && st.compositorial && !st.primorial) {
        if (announce) {
            printf("Sieving for factors of factorial and compositorial\n");
            fprintf(stderr, "Sieving for factors of factorial and compositorial\n");
        }
    } else if (z > 1 && st.primorial) {
        printf("\nSelect only one test type!\nuse -h for help\n");
        fprintf(stderr, "Select only one test type!\nuse -h for help\n");
        fail();
    }
    if (st.pmin == 0 || st.pmax == 0) {
        printf("\n-p and -P arguments are required\nuse -h for help\n");
        fprintf(stderr, "-p and -P arguments are required\n");
        fail();
    }
    if (st.nmin == 0 || st.nmax == 0) {
        printf("\n-n and -N arguments are required\nuse -h for help\n");
        fprintf(stderr, "-n and -N arguments are required\n");
        fail();
    }
    if (st.nmin > st.nmax) {
        printf("nmin <= nmax is required\nuse -h for help\n");
        fprintf(stderr, "nmin <= nmax is required\n");
        fail();
    }
    if (st.pmin > st.pmax) {
        printf("pmin <= pmax is required\nuse -h for help\n");
        fprintf(stderr, "pmin <= pmax is required\n");
        fail();
    }
    if (!announce) return;
    fprintf(stderr, "Starting sieve at p: %" PRIu64 " n: %u\nStopping sieve at P: %" PRIu64 " N: %u\n", st.pmin,
            st.nmin, st.pmax, st.nmax);
    printf("Starting sieve at p: %" PRIu64 " n: %u\nStopping sieve at P: %" PRIu64 " N: %u\n", st.pmin, st.nmin,
           st.pmax, st.nmax);
}

static void die_status(const char *where, int rc) {
    fprintf(stderr, "error: %s: %s\n", where, pfc_status_string(rc));
    printf("error: %s: %s\n", where, pfc_status_string(rc));
    fail();
}

// Validation, checkpoint and results-file handling that precede the sieve
// (cl_sieve.cpp:1336, 1406-1445).  Returns false when a checkpoint shows the
// work unit is already complete.
static bool prepare_search(workStatus &st, Search &sd) {
    setup_search(st);
    if (sd.test) {
        if (!truncate_results()) fail();
    } else if (read_state(st, sd)) {
        printf("Current p: %" PRIu64 "\n", st.p);
        fprintf(stderr, "Resuming from checkpoint, current p: %" PRIu64 "\n", st.p);
        if (st.p == st.pmax) {
            printf("Workunit complete.\n");
            fprintf(stderr, "Workunit complete.\n");
            return false;
        }
    } else {
        if (!truncate_results()) fail();
        st.last_trickle = (uint64_t)time(nullptr);
    }
    return true;
}

// Environment knobs: PFCSIEVE_CHECKPOINT_SECONDS (default 60, the reference's
// cadence, cl_sieve.cpp:1581), PFCSIEVE_SEGMENT_SPAN (p-range per segment;
// default: sized by the library to the device memory) and
// PFCSIEVE_EXIT_AFTER_CHECKPOINT=k, a host-side crash for resume tests: the
// process exits with status 3 right after writing its k-th checkpoint, when no
// kernel is in flight (the checkpoint follows a synchronising drain).
static double env_double(const char *name, double dflt) {
    const char *v = getenv(name);
    return (v && *v) ? strtod(v, nullptr) : dflt;
}

// the reference's cl_sieve() loop (cl_sieve.cpp:1328-1761), after
// prepare_search()
static void run_search(pfc_ctx *ctx, workStatus &st, Search &sd) {
    const auto t_start = std::chrono::steady_clock::now();
    pfc_job *job = nullptr;
    int rc = pfc_job_create(ctx, mode_bits(st), st.nmin, st.nmax, st.pmin, st.pmax, &job);
    if (rc == PFC_ERR_ARG && st.pmin == st.pmax) job = nullptr;   // empty p range: nothing to sieve
    else if (rc) die_status("pfc_job_create", rc);
    if (job) {
        // table self-check once per run (cl_sieve.cpp:917-973,1100-1137,1270-1307)
        uint64_t bytes = 0;
        rc = pfc_job_verify_tables(job, &bytes);
        const char *what = st.factorial && st.compositorial ? "factorial and compositorial"
                           : st.factorial                   ? "factorial power"
                           : st.primorial                   ? "primorial prime and product"
                                                            : "compositorial prime and product";
        if (rc == PFC_ERR_VALIDATION) {
            fprintf(stderr, "error: %s table verification failed\n", what);
            printf("error: %s table verification failed\n", what);
            exit(EXIT_FAILURE);
        }
        if (rc) die_status("pfc_job_verify_tables", rc);
        fprintf(stderr, "Verified %s tables (%" PRIu64 " bytes)\n", what, bytes);
        printf("Verified %s tables (%" PRIu64 " bytes)\n", what, bytes);
    }
    fprintf(stderr, "Starting Sieve...\n");
    printf("Starting Sieve...\n");
    uint64_t term_prev = 0, count_prev = 0;
    const double ckpt_secs = env_double("PFCSIEVE_CHECKPOINT_SECONDS", 60.0);
    const double span = env_double("PFCSIEVE_SEGMENT_SPAN", 0.0);
    const int exit_after = (int)env_double("PFCSIEVE_EXIT_AFTER_CHECKPOINT", 0.0);
    int ckpts = 0;
    auto last_progress = std::chrono::steady_clock::now(), last_ckpt = last_progress;
    const double irsize = 1.0 / (double)(st.pmax - st.pmin ? st.pmax - st.pmin : 1);
    while (job && st.p < st.pmax) {
        uint64_t hi = 0;
        rc = pfc_job_segment_end(job, st.p, &hi);
        if (rc) die_status("pfc_job_segment_end", rc);
        if (span >= 1.0 && (double)(hi - st.p) > span) hi = st.p + (uint64_t)span;
        rc = pfc_segment(job, st.p, hi);
        if (rc) die_status("pfc_segment", rc);
        st.p = hi;
        const auto now = std::chrono::steady_clock::now();
        if (std::chrono::duration<double>(now - last_progress).count() > 2.0) {
            printf("Sieve Progress: %.1f%%\n", (double)(st.p - st.pmin) * irsize * 100.0);
            last_progress = now;
        }
        if (std::chrono::duration<double>(now - last_ckpt).count() >= ckpt_secs && st.p < st.pmax) {
            rc = get_results(job, st, sd, term_prev, count_prev);
            if (rc) die_status("results", rc);
            if (!sd.test) checkpoint(st, sd);
            last_ckpt = now;
            if (exit_after > 0 && ++ckpts == exit_after) {
                fflush(stdout);
                exit(3);
            }
        }
    }
    st.p = st.pmax;
    printf("Sieve Progress: %.1f%%\n", 100.0);
    if (job) {
        rc = get_results(job, st, sd, term_prev, count_prev);
        if (rc) die_status("results", rc);
    }
    if (!sd.test) checkpoint(st, sd);
    if (finalize_results(st)) fail();
    if (job) pfc_job_destroy(job);
    fprintf(stderr, "Sieve complete.\nfactors %" PRIu64 ", prime count %" PRIu64 "\n", st.factorcount,
            st.primecount);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    printf("Sieve finished in %d sec.\n", (int)secs);
    printf("factors %" PRIu64 ", prime count %" PRIu64 ", checksum %016" PRIX64 "\n", st.factorcount, st.primecount,
           st.checksum);
}

// run_test (cl_sieve.cpp:1777-2095): the 16 self-test ranges and answers
struct TestCase {
    unsigned mode;
    uint64_t pmin, pmax;
    uint32_t nmin, nmax;
    uint64_t factors, primecount, checksum;
};
static const TestCase kTests[16] = {
    {1, 100000000ull, 101000000ull, 1000000, 2000000, 1071, 54211, 0x000004F844B5103Cull},
    {1, 1000000000000ull, 1000010000000ull, 10000, 2000000, 3, 361727, 0x0505A1C238896511ull},
    {1, 101ull, 100000ull, 101, 1000000, 42821, 9571, 0x0000000065DDB8A0ull},
    {1, 1000000000000ull, 1000001000000ull, 100000000, 110000000, 3, 36249, 0x00804FE7D7AA6C09ull},
    {2, 100000000ull, 101000000ull, 101, 25000000, 1703, 54211, 0x0000027EFF497990ull},
    {2, 101ull, 2000000ull, 101, 2000000, 24503, 148954, 0x000000027BF5B8E0ull},
    {2, 100000000000ull, 100005000000ull, 9000000, 110000000, 32, 197222, 0x0022FE7C09210B4Bull},
    {2, 1730720716000000ull, 1730720720000000ull, 600000, 30000000, 1, 114208, 0x5CDCB47F7E9532C2ull},
    {4, 200000000ull, 200010000ull, 101, 26000000, 127, 529, 0x0000001848D8AFBBull},
    {4, 101ull, 100000ull, 101, 1000000, 34271, 9571, 0x000000006FF88EAEull},
    {4, 200000000000ull, 200005000000ull, 15000000, 20000000, 13, 192386, 0x0088B59C23CD3E2Bull},
    {4, 1000000000000ull, 1000001000000ull, 700000, 25000000, 2, 36249, 0x0080997AF3BF42FEull},
    {5, 100000000000ull, 100010000000ull, 96000, 2000000, 27, 394403, 0x00D214CC0EF0ECB4ull},
    {5, 101ull, 110000ull, 101, 1000000, 84077, 10433, 0x00000000EFB634E9ull},
    {5, 10100000000ull, 10101000000ull, 11500000, 12500000, 19, 43374, 0x0002578EA9FD63C7ull},
    {5, 2000000000000ull, 2000020000000ull, 670000, 2460000, 3, 706162, 0x1D63BBC574E8D50Full},
};

static void run_test(pfc_ctx *ctx, Search &sd) {
    int good = 0;
    printf("Beginning self test of 16 ranges.\n");
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < 16; ++i) {
        const TestCase &t = kTests[i];
        workStatus st;
        memset(&st, 0, sizeof(st));
        st.factorial = t.mode & PFC_FACTORIAL;
        st.primorial = t.mode & PFC_PRIMORIAL;
        st.compositorial = t.mode & PFC_COMPOSITORIAL;
        st.pmin = t.pmin;
        st.pmax = t.pmax;
        st.nmin = t.nmin;
        st.nmax = t.nmax;
        prepare_search(st, sd);
        run_search(ctx, st, sd);
        if (st.factorcount == t.factors && st.primecount == t.primecount && st.checksum == t.checksum) {
            printf("test case %d passed.\n\n", i + 1);
            fprintf(stderr, "test case %d passed.\n", i + 1);
            ++good;
        } else {
            printf("test case %d failed.\n\n", i + 1);
            fprintf(stderr, "test case %d failed.\n", i + 1);
        }
    }
    if (good == 16) {
        printf("All test cases completed successfully!\n");
        fprintf(stderr, "All test cases completed successfully!\n");
    } else {
        printf("Self test FAILED!\n");
        fprintf(stderr, "Self test FAILED!\n");
    }
    printf("Elapsed time: %d sec.\n",
           (int)std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    if (good != 16) fail();
}

// GPU index from a BOINC-style init_data.xml if present (main.cpp:252-274)
static int device_from_init_data() {
    FILE *f = fopen("init_data.xml", "r");
    if (!f) {
        printf("init_data.xml not found, using device 0.\n");
        return 0;
    }
    char buf[4096];
    size_t n = fread(buf, 1, sizeof(buf) - 1, f);
    fclose(f);
    buf[n] = 0;
    const char *k = strstr(buf, "<gpu_device_num>");
    const int dev = k ? atoi(k + strlen("<gpu_device_num>")) : 0;
    printf("init_data.xml found, using device %d.\n", dev);
    return dev;
}

int main(int argc, char **argv) {
    setvbuf(stdout, nullptr, _IOLBF, 0);
    fprintf(stderr, "\nPFCSieve (GB300 CUDA build)\n");
    printf("\nPFCSieve (GB300 CUDA build)\n");
    fprintf(stderr, "Command line: ");
    for (int i = 0; i < argc; ++i) fprintf(stderr, "%s ", argv[i]);
    fprintf(stderr, "\n");
    workStatus st;
    memset(&st, 0, sizeof(st));
    Search sd;
    process_args(argc, argv, st, sd);
    // validation and checkpoint handling come before the GPU is touched
    if (!sd.test && !prepare_search(st, sd)) return EXIT_SUCCESS;
    sd.device = device_from_init_data();
    pfc_ctx *ctx = nullptr;
    int rc = pfc_ctx_create(sd.device, 0, &ctx);
    if (rc) die_status("pfc_ctx_create", rc);
    char name[256];
    int sms = 0;
    pfc_ctx_device_info(ctx, name, sizeof(name), &sms);
    printf("GPU Info:\n  Name: \t\t%s\n  Compute Units: \t%d\n", name, sms);
    // choose the walk kernels by timing them on this device (the reference
    // times the GPU to size its launches, profileGPU, cl_sieve.cpp:669-769)
    rc = pfc_autotune(ctx, nullptr, 0);
    if (rc) die_status("pfc_autotune", rc);
    if (sd.test) run_test(ctx, sd);
    else run_search(ctx, st, sd);
    pfc_ctx_destroy(ctx);
    return EXIT_SUCCESS;
}
