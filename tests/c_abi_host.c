/* A C99 caller of include/pfcsieve.h: the header compiles as strict C and the
 * library links and answers its host-only entry points (no GPU).  Built and
 * run by tests/test_c_abi.py; prints "ok" and exits 0, else names the check
 * that failed and exits 1. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "pfcsieve.h"

#define CHECK(c)                                   \
    do {                                           \
        if (!(c)) {                                \
            printf("failed: %s\n", #c);            \
            return 1;                              \
        }                                          \
    } while (0)

int main(void) {
    const uint64_t p = 1000003; /* prime */
    pfc_ctx *ctx = NULL;
    pfc_factor f;
    char line[96];
    uint64_t w = 0, q = 0, s0 = 0, s1 = 0, fact = 1, add = 0;
    size_t kept = 0;
    uint32_t k;

    /* without a usable device the context is refused, never emulated */
    CHECK(pfc_ctx_create(0, 0, &ctx) == PFC_ERR_NO_DEVICE && ctx == NULL);
    CHECK(strlen(pfc_status_string(PFC_ERR_VERIFY)) > 0);

    CHECK(pfc_is_prime(p) == 1 && pfc_is_prime(1000001) == 0 && pfc_is_prime(4294967297ull) == 0);

    f.p = p;
    f.nc = -500;
    f.type = PFC_TYPE_FACTORIAL;
    CHECK(pfc_format_factor(&f, line, sizeof line) > 0 && strcmp(line, "1000003 | 500!-1") == 0);

    /* 999! mod p from the setup programs replayed on the host, every form */
    for (k = 2; k <= 999; ++k) fact = fact * k % p;
    CHECK(pfc_setup_program_size(PFC_FACTORIAL, 1000, 1, &w, &q) == PFC_OK && w > 0);
    for (k = 0; k < 3; ++k) {
        CHECK(pfc_setup_program_eval(PFC_FACTORIAL, 1000, (int)k, p, &s0, &s1) == PFC_OK);
        CHECK(s0 == fact && s1 == 0);
    }

    /* Wilson: (p-1)! = -1 (mod p), so p | (p-1)! + 1 is a true hit */
    f.nc = (int32_t)(p - 1);
    CHECK(pfc_finalize_factors(PFC_FACTORIAL, (uint32_t)p, &f, 1, 1, 1, &kept, &add) == PFC_OK && kept == 1);
    CHECK(add == (p - 1) + 1);
    f.nc = -(int32_t)(p - 1);
    CHECK(pfc_finalize_factors(PFC_FACTORIAL, (uint32_t)p, &f, 1, 1, 1, &kept, &add) == PFC_ERR_VERIFY);

    printf("ok\n");
    return 0;
}
