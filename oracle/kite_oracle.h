/* CPU oracle for the k*2^n-1 squaring path.  TEST INFRASTRUCTURE ONLY: the tests, the smoke
 * check and the CPU-baseline leg of the benchmark use it as the checker; the product never
 * links, loads or calls it.
 *
 * It restates, in plain C, the reference's `ref` backend and the exact integer layer around it
 * (reference project kite, paths relative to its root):
 *   - digit layout, exact fixed-point weights, FFT-length choice   src/ctx.c:17-221
 *   - balanced carry with the top fold                              src/ctx.c:345-407
 *   - digits <-> canonical limbs, RES64                             src/ctx.c:409-559
 *   - weighted full-length complex FFT squaring / multiplication    src/ref_fft.c:26-139
 *   - base^(N-1) from base^(N+1), also when gcd(base, N) > 1        src/prp.c:63-144
 *   - Morrison/LLR choice of P and the V-sequence                   src/llr.c:29-90, 150-184
 * A number is held as L doubles, each an exact balanced integer digit (the `ref` backend's
 * storage, src/ref_fft.c:76-82).
 */
#ifndef KITE_ORACLE_H
#define KITE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ko_ctx ko_ctx;

/* FFT-length helpers (src/ctx.c:17-148, without a tuning file). */
int ko_fft_len_ok(uint32_t L);
double ko_safe_bpw(uint32_t L, uint64_t k);
uint32_t ko_choose_fft_len(uint64_t k, uint64_t n);
uint32_t ko_next_fft_len(uint32_t L);

/* Context for N = k*2^n - 1 at FFT length L (0 = ko_choose_fft_len).  NULL on bad input. */
ko_ctx *ko_ctx_new(uint64_t k, uint64_t n, uint32_t L);
void ko_ctx_free(ko_ctx *c);
uint32_t ko_fft_len(const ko_ctx *c);
size_t ko_limbs(const ko_ctx *c);
/* bits[L], w[L], oscale[L]; meta = {lam, sL, top_t, top_st, top_m}. */
void ko_layout(const ko_ctx *c, uint8_t *bits, double *w, double *oscale, uint64_t *meta);

void ko_set_limbs(ko_ctx *c, double *x, const uint64_t *limbs);
void ko_get_limbs(ko_ctx *c, const double *x, uint64_t *limbs);
uint64_t ko_res64(ko_ctx *c, const double *x);
/* Integer digits (any magnitude below 2^62) -> canonical limbs of k*sum(d_j 2^s_j) mod N. */
void ko_digits_to_limbs(const ko_ctx *c, const int64_t *dig, uint64_t *limbs);
/* Balanced carry with the top fold, in place. */
void ko_carry_digits(const ko_ctx *c, int64_t *dig);

void ko_square(ko_ctx *c, double *x, uint64_t count);
void ko_mul(ko_ctx *c, double *x, const double *y);
void ko_mul_small(ko_ctx *c, double *x, int64_t m);
void ko_add(ko_ctx *c, double *x, const double *y);
void ko_sub(ko_ctx *c, double *x, const double *y);
double ko_maxerr(const ko_ctx *c);
void ko_reset_maxerr(ko_ctx *c);

/* y = base^(N+1) mod N (nl limbs) -> base^(N-1) mod N.  0, or -1 if unsupported. */
int ko_residue_nm1(uint64_t *y, const uint64_t *N, size_t nl, uint64_t base);

/* Plain Fermat test (no Gerbicz check): RES64 of base^(N-1) mod N. */
int ko_fermat(uint64_t k, uint64_t n, uint32_t base, uint32_t L, uint64_t *res64, int *is_prp,
              double *maxerr);
/* Morrison/LLR: P as PRST chooses it, factor if found. */
int ko_llr_choose_P(uint64_t k, uint64_t n, uint32_t *P, uint64_t *factor);
int ko_llr(uint64_t k, uint64_t n, uint32_t L, uint32_t *P, uint64_t *factor, uint64_t *res64,
           int *is_prime, double *maxerr);

/* CPU baseline: square each of ntests numbers (seeded by their index) `squarings` times, one
 * test per thread on `threads` threads; us_per_sq[i] receives each test's time per squaring. */
int ko_time_squarings(const uint64_t *k, const uint64_t *n, const uint32_t *L, int ntests,
                      int threads, uint32_t squarings, double *us_per_sq);

#ifdef __cplusplus
}
#endif
#endif
