/* Command-line front end to the CPU oracle (test infrastructure only).
 *   kite_oracle_cli prp K N [L]      plain Fermat base-3 test: RES64, maxerr
 *   kite_oracle_cli llr K N [L]      Morrison/LLR test
 *   kite_oracle_cli time K N L SQ T  microseconds per squaring, T threads each on one test
 */
#include <inttypes.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "kite_oracle.h"

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s prp|llr|time K N [L] [SQ] [T]\n", argv[0]);
        return 2;
    }
    uint64_t k = strtoull(argv[2], 0, 10), n = strtoull(argv[3], 0, 10);
    uint32_t L = argc > 4 ? (uint32_t)strtoul(argv[4], 0, 10) : 0;
    if (!strcmp(argv[1], "prp")) {
        uint64_t r = 0;
        int prp = 0;
        double e = 0;
        int rc = ko_fermat(k, n, 3, L, &r, &prp, &e);
        printf("%" PRIu64 "*2^%" PRIu64 "-1 rc %d %s RES64 %016" PRIX64 " maxerr %.4f\n", k, n, rc,
               prp ? "PRP" : "composite", r, e);
        return rc != 0;
    }
    if (!strcmp(argv[1], "llr")) {
        uint32_t P = 0;
        uint64_t f = 0, r = 0;
        int pr = 0;
        double e = 0;
        int rc = ko_llr(k, n, L, &P, &f, &r, &pr, &e);
        printf("%" PRIu64 "*2^%" PRIu64 "-1 rc %d P %u factor %" PRIu64 " %s RES64 %016" PRIX64
               " maxerr %.4f\n", k, n, rc, P, f, pr ? "prime" : "composite", r, e);
        return rc != 0;
    }
    if (!strcmp(argv[1], "time")) {
        uint32_t sq = argc > 5 ? (uint32_t)atoi(argv[5]) : 20;
        int T = argc > 6 ? atoi(argv[6]) : 1;
        uint64_t *ks = malloc(T * 8), *ns = malloc(T * 8);
        uint32_t *Ls = malloc(T * 4);
        double *us = malloc(T * 8);
        for (int i = 0; i < T; i++) { ks[i] = k; ns[i] = n; Ls[i] = L; }
        ko_time_squarings(ks, ns, Ls, T, T, sq, us);
        for (int i = 0; i < T; i++) printf("test %d: %.1f us/sq\n", i, us[i]);
        return 0;
    }
    return 2;
}
