/* Exact integer-NTT squaring engine modulo N = k*2^n - 1 on the GB300 (kn_*).
 *
 * The reference's GPU prototype squares modulo N with an integer number-theoretic transform
 * instead of the FP64 IBDWT (gpu/ntt.metal:121-166, gpu/ntt_reg.metal:90-246, gpu/sq.metal:23-192,
 * gpu/gpu_ctx.h:57-322): numbers in Montgomery form with R = 2^n, the product P = A + B*2^n
 * (A < 2^n) reduced as P*2^-n == B + k*A (mod N), residues modulo several word-size primes, a
 * Garner CRT back to integers.  This engine restates that arithmetic in CUDA for sm_103a.  It has
 * no round-off at all, so it cross-checks the FP64 engine bit for bit, and it runs on the integer
 * pipes, which GB300 has far more of than FP64 units.
 *
 * Representation: a number is W words of w bits (w <= 50) in 64-bit little-endian slots, value
 * x~ = x*2^n mod N up to a small multiple of N.  Three or four primes p < 2^30 with 2^20 | p-1 (per
 * n, whichever needs fewer prime-points); the transform length NP is a power of 2 >= 2W; every
 * convolution coefficient is below W*2^(2w) < the primes' product, so the CRT recovers it
 * exactly.
 *
 * Numbers live in device memory.  Operations queue on the engine's stream; kn_get_limbs and
 * kn_sync wait.  A CUDA failure is sticky: kn_error returns it and later calls do nothing.
 * The reference has no C interface for this path (its prototype is Objective-C over Metal);
 * these entry points are this library's own.
 */
#ifndef KITE_NTT_H
#define KITE_NTT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kn_engine kn_engine;

/* An engine for N = k*2^n - 1 (k odd, 1 <= k < 2^30, 8 <= n <= 2^26) on `device` (-1: the current
 * device); NULL if the GPU cannot be used or the sizes are out of range. */
kn_engine *kn_engine_new(uint64_t k, uint64_t n, int device);
void kn_engine_free(kn_engine *e);

uint32_t kn_num_words(const kn_engine *e);      /* W: 64-bit words per number */
uint32_t kn_word_bits(const kn_engine *e);      /* w */
uint32_t kn_transform_len(const kn_engine *e);  /* NP */

/* Device numbers of kn_num_words words; NULL on failure. */
uint64_t *kn_num_alloc(kn_engine *e);
void kn_num_free(kn_engine *e, uint64_t *x);

/* Canonical value in [0, N) as kite_limbs-many little-endian 64-bit limbs <-> device number. */
size_t kn_limbs(const kn_engine *e);
int kn_set_limbs(kn_engine *e, uint64_t *x, const uint64_t *limbs);
int kn_get_limbs(kn_engine *e, const uint64_t *x, uint64_t *limbs);

/* x <- x^(2^count) mod N; kn_square_add adds the constant c after every squaring
 * (x <- x^2 + c, the LLR step with c = -2).  x <- x*y mod N. */
int kn_square(kn_engine *e, uint64_t *x, uint64_t count);
int kn_square_add(kn_engine *e, uint64_t *x, uint64_t count, int64_t c);
int kn_mul(kn_engine *e, uint64_t *x, const uint64_t *y);
int kn_copy(kn_engine *e, uint64_t *dst, const uint64_t *src);

int kn_error(const kn_engine *e);
int kn_sync(kn_engine *e);

/* Host-only, no GPU needed: the engine's sizes for N = k*2^n - 1 -- the primes in use (3 or 4: the
 * choice with the fewest prime-points), the word size, the words, the transform length -- (0, or -1
 * if out of range), and the conversions between a canonical value in [0, N) (kn_limbs-many limbs:
 * (n + 127) / 64) and the engine's W words in Montgomery form x~ = x*2^n mod N. */
int kn_layout(uint64_t k, uint64_t n, uint32_t *primes, uint32_t *w, uint32_t *W, uint32_t *NP);
int kn_limbs_to_words(uint64_t k, uint64_t n, const uint64_t *limbs, uint64_t *words);
int kn_words_to_limbs(uint64_t k, uint64_t n, const uint64_t *words, uint64_t *limbs);

/* Groups: one launch set per squaring advances every member at once (many tests on one GPU, as
 * the reference's prototype keeps B numbers in flight, gpu/gpu_ctx.h:57-77).  A member is an
 * engine with the number it squares; engines may differ in k and n but not repeat, since each
 * owns its scratch.  Squarings run as CUDA graphs of 8.  gpu_ms (optional) receives the GPU time
 * of the call, measured with events on the group's stream. */
typedef struct kn_group kn_group;
kn_group *kn_group_new(int device);
void kn_group_free(kn_group *g);
int kn_group_add(kn_group *g, kn_engine *e, uint64_t *x);
int kn_group_square(kn_group *g, uint64_t count, float *gpu_ms);
/* kn_group_square of ng groups of the same device at once (no counterpart in the reference's
 * prototype, which squares one group per command buffer): each group's graphs go to its own
 * stream, so one group's latency-bound reduction overlaps another's transforms.  gpu_ms
 * receives the time from the common start to the last group's end. */
int kn_groups_square(kn_group *const *gs, int ng, uint64_t count, float *gpu_ms);
/* Every member's number times ys[i] (members in the order they were added; ys[i] a number of
 * member i's engine, distinct from its own number). */
int kn_group_mul(kn_group *g, const uint64_t *const *ys, float *gpu_ms);
int kn_group_error(const kn_group *g);

#ifdef __cplusplus
}
#endif
#endif
