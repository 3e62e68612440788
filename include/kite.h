/* kite public C API, served by the GB300 engine.
 *
 * Modular squaring and multiplication modulo N = k*2^n - 1, Fermat PRP and Morrison/LLR tests.
 * This header declares the same types, names, argument meanings and error conventions as the
 * reference library's include/kite.h (kite 0.1.8, include/kite.h:17-169), so code written
 * against that header links against libkite_gb300.so unchanged.  The one addition is
 * KITE_BACKEND_CUDA, the value the reference's `--backend cuda` selects, and KITE_BACKEND_CUDA_NTT,
 * an exact integer-transform engine for cross-checks.
 *
 * Numbers are opaque: a kite_num lives in GPU memory in the engine's transformed
 * representation.  Every entry point here is host-callable; none needs a CUDA context from the
 * caller.
 */
#ifndef KITE_H
#define KITE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KITE_VERSION "0.1.8"
#define KITE_GB300_VERSION "0.1.0"

typedef struct kite_ctx kite_ctx;
typedef struct kite_num kite_num;

/* Backend selector (reference include/kite.h:20-26).  This library implements the CUDA backend
 * only: AUTO and CUDA select it; REF, NEON, SME and C2P are the reference's CPU backends and
 * make kite_ctx_new return NULL.  There is no CPU fallback. */
typedef enum {
    KITE_BACKEND_AUTO = 0,
    KITE_BACKEND_REF = 1,
    KITE_BACKEND_NEON = 2,
    KITE_BACKEND_SME = 3,
    KITE_BACKEND_C2P = 4,
    KITE_BACKEND_CUDA = 5,
    /* The exact integer-NTT engine (include/kite_ntt.h): the arithmetic of the reference's GPU
     * prototype (gpu/sq.metal), no round-off; kite_max_roundoff stays 0. */
    KITE_BACKEND_CUDA_NTT = 6,
} kite_backend;

/* Context options (reference include/kite.h:28-35). */
typedef struct {
    kite_backend backend;
    uint32_t fft_len;    /* 0: choose from n and k */
    uint32_t threads;    /* accepted for compatibility; the GPU grid replaces CPU threads */
    uint32_t plan_order; /* 0: engine default; else 1 + stage-order bits, as the reference */
} kite_opts;

/* ---- contexts and numbers (reference include/kite.h:37-69) ----------------------------------- */

/* c must be -1.  NULL when k is even or >= 2^30, n < 8, the FFT length is unusable, the backend
 * is not CUDA/AUTO, or the GPU cannot be initialised. */
kite_ctx *kite_ctx_new(uint64_t k, uint64_t n, int32_t c, const kite_opts *o);
void kite_ctx_free(kite_ctx *ctx);
uint32_t kite_fft_len(const kite_ctx *ctx);
const char *kite_backend_name(const kite_ctx *ctx);

kite_num *kite_num_new(kite_ctx *ctx);
void kite_num_free(kite_ctx *ctx, kite_num *x);
void kite_copy(kite_ctx *ctx, kite_num *dst, const kite_num *src);
void kite_set_u64(kite_ctx *ctx, kite_num *x, uint64_t v);

/* Operations are queued on the context's stream and return at once; results are read back by
 * kite_get_limbs / kite_res64 / kite_max_roundoff, which wait for the queue. */
void kite_square(kite_ctx *ctx, kite_num *x);
void kite_square_n(kite_ctx *ctx, kite_num *x, uint64_t count);
void kite_mul(kite_ctx *ctx, kite_num *x, const kite_num *y);  /* x = x*y */
void kite_mul_small(kite_ctx *ctx, kite_num *x, int64_t m);    /* x = x*m, |m| < 2^20 */
/* x = x + y, x = x - y on the transformed arrays; the digits stay unbalanced until the next
 * product, so use at most one add or sub between products. */
void kite_add(kite_ctx *ctx, kite_num *x, const kite_num *y);
void kite_sub(kite_ctx *ctx, kite_num *x, const kite_num *y);

/* Largest |rounded - exact| since the last reset, 0..0.5.  A CUDA failure on this context is
 * reported as 1.0 (and by kite_ctx_error), which sends the drivers down their retry path. */
double kite_max_roundoff(const kite_ctx *ctx);
void kite_reset_roundoff(kite_ctx *ctx);
void kite_set_roundoff_check(kite_ctx *ctx, uint32_t every);

size_t kite_limbs(const kite_ctx *ctx);
void kite_get_limbs(kite_ctx *ctx, const kite_num *x, uint64_t *limbs); /* canonical, [0, N) */
void kite_set_limbs(kite_ctx *ctx, kite_num *x, const uint64_t *limbs);
uint64_t kite_res64(kite_ctx *ctx, const kite_num *x);

/* ---- Fermat PRP test (reference include/kite.h:71-118) ------------------------------------- */

typedef struct {
    kite_opts fft;
    uint32_t gerbicz_block;   /* 0: ~sqrt(n) in [32, 2000] */
    uint32_t gerbicz_blocks;  /* 0: max(block/4, 8) */
    double max_roundoff;      /* 0: 0.40 */
    const char *checkpoint;   /* verified state file, or NULL */
    double checkpoint_secs;   /* 0: 600 */
    const char *checkpoint_unverified; /* unverified state file, or NULL */
    double unverified_secs;            /* 0: 60 */
    void (*progress)(void *arg, uint64_t iter, uint64_t n, double maxerr);
    void *progress_arg;
    uint64_t inject_fault_at; /* testing: add 1 to one digit after this squaring (0: never) */
    const uint32_t *points;   /* ascending proof-point iterations */
    uint32_t npoints;
    int (*on_point)(void *arg, uint32_t index, uint64_t iter, const uint64_t *limbs);
    void *point_arg;
    volatile int *abort_flag;
} kite_prp_opts;

enum { KITE_PRP_ABORTED = -5, KITE_PRP_POINT_FAILED = -6 };

typedef struct {
    uint64_t res64; /* low 64 bits of base^(N-1) mod N */
    int is_prp;
    uint32_t fft_len;
    double maxerr;
    uint32_t gerbicz_errors;
    uint32_t roundoff_retries;
    int resumed;
    uint64_t resumed_at;
    double seconds;
} kite_prp_result;

/* 0 on success; -1 setup, -2 no longer FFT, -3 repeated failures, -4 residue, -5 aborted,
 * -6 a proof-point callback failed. */
int kite_prp(uint64_t k, uint64_t n, uint32_t base, const kite_prp_opts *o, kite_prp_result *res);

/* ---- LLR (Morrison) test (reference include/kite.h:120-166) --------------------------------- */

typedef struct {
    kite_opts fft;
    double max_roundoff;
    const char *checkpoint;
    double checkpoint_secs;
    void (*progress)(void *arg, uint64_t iter, uint64_t total, double maxerr);
    void (*on_confirm)(void *arg, int run);
    void *progress_arg;
    volatile int *abort_flag;
    uint64_t inject_fault_at;
    uint32_t inject_fault_runs;
    uint64_t inject_roundoff_at;
    int inject_roundoff_ladder;
} kite_llr_opts;

typedef struct {
    int is_prime;
    uint64_t factor;
    uint64_t res64;
    uint32_t P;
    uint32_t fft_len;
    double maxerr;
    uint32_t roundoff_retries;
    uint32_t confirm_runs;
    int resumed;
    uint64_t resumed_at;
    double seconds;
} kite_llr_result;

enum { KITE_LLR_ABORTED = -5 };

int kite_llr(uint64_t k, uint64_t n, const kite_llr_opts *o, kite_llr_result *res);
int kite_llr_choose_P(uint64_t k, uint64_t n, uint32_t *P, uint64_t *factor);
int kite_llr_checkpoint_iter(const char *path, uint64_t k, uint64_t n, uint64_t *iter, int *run);
int kite_prp_checkpoint_iter(const char *path, uint64_t k, uint64_t n, uint32_t base,
                             uint64_t *iter);

/* Testing hook (reference include/kite.h:168-169): add 1 to digit L/3 of x, a valid encoding of
 * a wrong value that only the Gerbicz check can catch. */
void kite_debug_corrupt(kite_ctx *ctx, kite_num *x);

/* ---- additions of this library ----------------------------------------------------------------- */

/* Sticky CUDA error recorded on the context (0 when none).  Not in the reference API: there
 * square/mul return void and a failure can only surface as round-off. */
int kite_ctx_error(const kite_ctx *ctx);
/* Block until the context's queued work is done; returns kite_ctx_error(). */
int kite_ctx_sync(kite_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
