/*
 * boinc_api.h -- stand-in for the BOINC client API, for building the
 * reference program (mfl0p/PFCSieve) as a standalone run outside a BOINC
 * client.  TEST INFRASTRUCTURE: used only by the oracle/_ref/pfcsieve_ref
 * build recipe (oracle/Makefile `refcl`).
 *
 * The real BOINC headers bring in the C library's time and string headers,
 * which the reference program relies on; this one does too.
 *
 * Every call behaves as the BOINC library does when no client is attached
 * (standalone mode): file names resolve to themselves, progress, trickles and
 * critical sections are no-ops, and boinc_finish ends the process.
 */
#ifndef PFC_REFCL_BOINC_API_H
#define PFC_REFCL_BOINC_API_H

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <time.h>
#include <unistd.h>

struct BOINC_OPTIONS {
    bool normal_thread_priority = false;
};

struct APP_INIT_DATA {
    double starting_elapsed_time = 0;
};

inline void boinc_options_defaults(BOINC_OPTIONS &o) { o = BOINC_OPTIONS(); }
inline int boinc_init_options(BOINC_OPTIONS *) { return 0; }
inline int boinc_is_standalone() { return 1; }
inline int boinc_finish(int status) {
    fflush(stdout);
    exit(status);
}
inline void boinc_begin_critical_section() {}
inline void boinc_end_critical_section() {}
inline void boinc_checkpoint_completed() {}
inline double boinc_elapsed_time() { return 0; }
inline int boinc_fraction_done(double) { return 0; }
inline double boinc_get_fraction_done() { return 0; }
inline int boinc_wu_cpu_time(double &t) {
    t = 0;
    return 0;
}
inline int boinc_get_init_data(APP_INIT_DATA &d) {
    d = APP_INIT_DATA();
    return 0;
}
inline int boinc_send_trickle_up(char *, char *) { return 0; }
inline int boinc_resolve_filename(const char *name, char *out, int cap) {
    snprintf(out, (size_t)cap, "%s", name);
    return 0;
}
inline FILE *boinc_fopen(const char *path, const char *mode) { return fopen(path, mode); }

#endif
