/* C ABI of the GB300 squaring engine: the boundary a kite backend binds.
 *
 * The reference selects an arithmetic backend through a vtable (src/internal.h:57-66,
 * struct kite_backend_ops {init, free, to_digits, from_digits, square, mul, mul_small}),
 * dispatched in kite_ctx_new (src/ctx.c:256-280).  Each entry point below replaces one hook
 * of that vtable, or one of the host loops in src/ctx.c that assume numbers live in host
 * memory (kite_copy/add/sub, src/ctx.c:323-343; kite_max_roundoff, src/ctx.c:300).  Arguments
 * are plain pointers and sizes; numbers are device pointers returned by kc_num_alloc.
 *
 * Errors: entry points returning int give 0 on success and a negative value after a CUDA
 * failure.  A failure is sticky on the engine: kc_error() reports it and kc_maxerr() returns
 * 1.0 from then on, which sends the reference's drivers down their retry path.  No entry point
 * aborts the process.
 */
#ifndef KITE_CUDA_H
#define KITE_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kc_engine kc_engine;

/* Replaces kite_backend_ops.init (src/internal.h:60; e.g. src/ref_fft.c:50-65).  The layout is
 * the context's own (src/internal.h:31-54: bits, w, oscale, top_t, top_st, top_m, sL); the
 * engine copies it to the device.  device < 0: the current CUDA device.  NULL on failure. */
kc_engine *kc_engine_new(uint64_t k, uint64_t n, uint32_t L, const uint8_t *bits, const double *w,
                         const double *oscale, uint32_t top_t, uint64_t top_st, uint32_t top_m,
                         uint64_t sL, int device);
/* Replaces kite_backend_ops.free (src/internal.h:61). */
void kc_engine_free(kc_engine *e);
/* Doubles per number (the reference's ctx->num_doubles, src/internal.h:53). */
size_t kc_num_doubles(const kc_engine *e);

/* Number storage in device memory: replaces kite_alloc/kite_free_aligned as used by
 * kite_num_new/kite_num_free (src/ctx.c:305-321).  The new number is zero. */
double *kc_num_alloc(kc_engine *e);
void kc_num_free(kc_engine *e, double *x);

/* Replace kite_backend_ops.from_digits / to_digits (src/internal.h:62-63): L balanced integer
 * digits in host memory <-> the device number.  to_digits waits for the engine's queue. */
int kc_from_digits(kc_engine *e, double *x, const int64_t *digits);
int kc_to_digits(kc_engine *e, const double *x, int64_t *digits);

/* Replace kite_backend_ops.square / mul (src/internal.h:64-65) and the loop of kite_square_n
 * (src/ctx.c:329-331).  Queued on the engine's stream; return without waiting. */
int kc_square(kc_engine *e, double *x, uint64_t count);
int kc_mul(kc_engine *e, double *x, const double *y);
/* x <- x^2 + c (c a small signed constant in value terms, e.g. -2 for the LLR step
 * V <- V^2 - 2, src/llr.c:395-406), the constant folded into the carry: no extra pass. */
int kc_square_add(kc_engine *e, double *x, uint64_t count, int64_t c);

/* a == b (mod N)?  Replaces the canonical comparison of the reference's drivers (nums_equal,
 * src/prp.c:291-296, used by the Gerbicz check at src/prp.c:470-474 and the tail at :538),
 * which converts both numbers to limbs on the host.  Here the digits of a and b are formed on
 * the device, their difference is carried exactly with the top fold, and only the verdict (4
 * bytes) comes back.  Waits for the queue.  1 equal, 0 different, or a negative CUDA error. */
int kc_equal(kc_engine *e, const double *a, const double *b);

/* Replace the host loops of kite_copy / kite_add / kite_sub (src/ctx.c:323-343). */
int kc_copy(kc_engine *e, double *dst, const double *src);
int kc_add(kc_engine *e, double *x, const double *y);
int kc_sub(kc_engine *e, double *x, const double *y);

/* Round-off: replaces the reads and writes of ctx->maxerr (src/ctx.c:300-302) and the sampling
 * of src/neon.c:779.  kc_maxerr waits for the queue. */
double kc_maxerr(kc_engine *e);
void kc_reset_maxerr(kc_engine *e);
void kc_set_roundoff_check(kc_engine *e, uint32_t every);

/* Sticky CUDA error (0 if none); kc_sync waits for the queue and returns kc_error(). */
int kc_error(const kc_engine *e);
int kc_sync(kc_engine *e);
/* The engine's CUDA stream (a cudaStream_t), for callers that time or order work on it. */
void *kc_stream(kc_engine *e);
/* Four-step shape chosen for the engine's length: H = R * C complex points. */
void kc_shape(const kc_engine *e, uint32_t *R, uint32_t *C);
/* Columns per column-pass work unit (2, 4 or 8): an engine created by kc_engine_new spreads each
 * pass of one squaring over the SMs; batch slots use 8. */
int kc_group_width(const kc_engine *e);
/* Self-test of the bounded waits of the persistent squaring kernel that batches run (no
 * counterpart in the reference, whose host threads never wait on one another on a device).
 * Launches that kernel over engine e's column items without its row items, so every item waits
 * for work that is not in the queue; each wait gives up after wait_cycles SM cycles, raises the
 * launch's timeout word and the launch ends.  Nothing is written to e's numbers.  Returns 1 if
 * the timeout was raised (the expected outcome), 0 if not, or a negative CUDA error.  The
 * context stays usable afterwards. */
int kc_engine_wait_selftest(kc_engine *e, uint64_t wait_cycles);

/* ---- a squaring that allocates nothing ---------------------------------------------------
 * No counterpart in the reference (its backends run on the host and never allocate device
 * memory).  y = x^2 mod N (x == y allowed) on engine e, like kc_square(e, y, 1) after copying x
 * to y, but calling no cudaMalloc, cudaFree or other allocating routine.  It is for callers that
 * cannot allocate when they need the product: a plugin whose host owns the device memory
 * through its own pool (a cudaMalloc of its own would fail or evict the host's data), or a
 * latency-bound loop that cannot afford the device synchronisation an allocation brings.  Its
 * scratch is one static device array of about 0.65 MB that every GPU loading this library
 * reserves until the process exits.
 *   - lengths above KC_NOALLOC_MAX_WORDS words are refused with KC_NOALLOC_TOO_LARGE;
 *   - the first call on a device looks up the array's device address (cudaGetSymbolAddress)
 *     with that device current and keeps it for the life of the process; after a
 *     cudaDeviceReset of that device the kept address is stale, so do not call it there again;
 *   - all calls share the array, which keeps the last call's contents; calls that overlap on
 *     the GPU (different streams, engines or threads) race and corrupt each other's result:
 *     serialise them;
 *   - round-off is tracked on every call into the engine's kc_maxerr.
 * Returns 0, KC_NOALLOC_TOO_LARGE, KC_NOALLOC_BAD_ARGUMENT (a null argument, or a device this
 * library cannot address), or a negated CUDA error code (also recorded on e).  The two named
 * codes lie below -10000, outside the range of negated CUDA errors. */
#define KC_NOALLOC_MAX_WORDS 65536
#define KC_NOALLOC_TOO_LARGE (-10001)
#define KC_NOALLOC_BAD_ARGUMENT (-10002)
int kc_square_noalloc(kc_engine *e, const double *x, double *y);

/* ---- batched engine ------------------------------------------------------------------------
 * Many independent tests advanced together on one GPU.  The reference's form of concurrent
 * tests is one context per test on CPU threads (`kite throughput`, tools/kite.c:65-105); a batch
 * replaces those contexts: each test is a slot with its own modulus and FFT length.  A Gerbicz
 * block of every slot's squarings is one CUDA graph: the slots in three parts of about equal
 * work, each part's pass launches on its own stream (KITE_GB300_BATCH_SPLIT=P for P parts), or
 * with KITE_GB300_BATCH_PERSISTENT=1 a persistent kernel over one queue of every slot's work
 * whose waits between CTAs are bounded (a wait that runs out fails the step with
 * -cudaErrorLaunchTimeout).  Fermat slots run the Gerbicz-checked driver of
 * src/prp.c:407-567 (block B, check every M blocks, rollback, longer FFT on round-off above
 * 0.40, doubled tail); LLR slots run the doubling V <- V^2 - 2 of src/llr.c:395-406 after the
 * Lucas ladder.  Results are bit-identical to a test run alone. */
typedef struct kc_batch kc_batch;

enum { KC_TEST_FERMAT = 0, KC_TEST_LLR = 1 };

typedef struct {
    int kind;                  /* KC_TEST_FERMAT or KC_TEST_LLR */
    int rc;                    /* 0, or the kite_prp / kite_llr error code */
    uint64_t k, n;
    uint64_t res64;            /* Fermat: low word of base^(N-1); LLR: of V_{k 2^(n-1)} */
    int is_prp;                /* Fermat: PRP; LLR: the final V is 0 (prime) */
    uint32_t fft_len;
    double maxerr;
    uint32_t gerbicz_errors;
    uint32_t roundoff_retries;
    uint64_t squarings;        /* modular products done, checks and retries included */
    double seconds;            /* admission to verdict */
    uint32_t P;                /* LLR */
    uint64_t factor;           /* LLR: small factor found while choosing P */
    uint64_t iter;             /* last verified iteration */
    uint64_t position;         /* squarings of x done so far (n once finished) */
} kc_test_result;

/* gerbicz_block 0: 1000; gerbicz_blocks 0: max(block/4, 8); mem_budget 0: 80% of free memory. */
kc_batch *kc_batch_new(int device, uint32_t gerbicz_block, uint32_t gerbicz_blocks, size_t mem_budget);
void kc_batch_free(kc_batch *b);
/* Admit a test (fft_len 0: chosen as kite_ctx_new does).  Returns the slot id, -1 for an
 * invalid test, -2 when the memory budget is full. */
int kc_batch_add_fermat(kc_batch *b, uint64_t k, uint64_t n, uint32_t base, uint32_t fft_len);
int kc_batch_add_llr(kc_batch *b, uint64_t k, uint64_t n, uint32_t fft_len);
/* Spread the Gerbicz checks of the Fermat slots admitted from now on: the first round of the
 * j-th admitted slot is 1 + (j mod M) blocks instead of M, so in a batch admitted at once the
 * slots' checks fall on different blocks, as they do in a batch refilled over time.  Every round
 * still ends in the reference's check (src/prp.c:407-517); a shorter first round only adds one.
 * Verdicts do not change.  Off by default. */
void kc_batch_stagger_checks(kc_batch *b, int on);
/* Advance every active slot by `blocks` Gerbicz blocks (B squarings each, plus the block's
 * product or check).  *gpu_ms receives the CUDA-event time of the work.  Returns the number of
 * slots still active, or a negative CUDA error. */
int kc_batch_step(kc_batch *b, uint32_t blocks, double *gpu_ms);
/* 0 running, 1 finished (result valid), 2 failed (rc set), -1 no such slot. */
int kc_batch_result(const kc_batch *b, int slot, kc_test_result *out);
/* Canonical limbs (kite_limbs words) of the slot's current x, read back from the device. */
int kc_batch_read(kc_batch *b, int slot, uint64_t *limbs);
/* Write the slot's last verified state to `path` in the reference's checkpoint formats:
 * KITECKP1 (x and d limbs, src/prp.c:158-192) for Fermat slots, KITELLR1 (V limbs, run 0,
 * src/llr.c:106-121) for LLR slots.  0, or -1 on failure. */
int kc_batch_checkpoint(kc_batch *b, int slot, const char *path);
/* Testing hook, the batch's form of kite_debug_corrupt (src/prp.c:28-34): adds 1 to digit L/3
 * of the slot's current x, a valid encoding of a wrong value that only the Gerbicz check (or the
 * tail's comparison) catches.  0, or -1 when the slot is not running. */
int kc_batch_debug_corrupt(kc_batch *b, int slot);
/* Host<->device bytes moved by the last kc_batch_step (slot tables, work lists, round-off). */
void kc_batch_last_transfer(const kc_batch *b, uint64_t *h2d, uint64_t *d2h);
/* Free a slot's device memory (its number becomes reusable by later admissions). */
void kc_batch_release(kc_batch *b, int slot);
int kc_batch_active(const kc_batch *b);
size_t kc_batch_bytes_in_use(const kc_batch *b);
size_t kc_batch_budget(const kc_batch *b);
int kc_batch_error(const kc_batch *b);
/* What the last failed kc_batch_step failed at ("" if nothing failed). */
const char *kc_batch_error_string(const kc_batch *b);

/* Per-kernel timing of the batched squaring: copies each running Fermat slot's x into its
 * scratch number t and squares t `squarings` times with the three pass kernels launched one by
 * one, CUDA events around each (on the batch stream).  ms[0..2] receive the mean duration of one
 * launch of the row pass, the column inverse pass and the column forward pass; flops[0..2] the
 * algorithmic FP64 operations one launch of each performs over all slots (the per-squaring count
 * F(L) = 5 L log2(L/2) + 24 L split as 10 H log2 C + 10 L, 5 H log2 R + 7 L, 5 H log2 R + 7 L).
 * Only valid while no slot is in its check or tail (it uses t).  0 or a negative CUDA error. */
int kc_batch_profile(kc_batch *b, uint32_t squarings, double *ms, double *flops);
/* The same measurement for the form kc_batch_step runs: one persistent launch (k_squarings) of
 * `squarings` squarings of every running Fermat slot's copy t, after one warm-up launch, timed
 * with CUDA events on the batch stream.  *ms receives the launch's duration and *flops its
 * algorithmic FP64 operations (F(L) per slot per squaring).  Same preconditions; 0, -1 if a
 * wait inside the kernel timed out, or a negative CUDA error. */
int kc_batch_profile_steps(kc_batch *b, uint32_t squarings, double *ms, double *flops);

/* Measured FP64 FMA throughput of `device` in FLOP/s (2 per FMA), from a dependent-chain DFMA
 * kernel timed with CUDA events: the roofline denominator of this FP64-bound path. */
double kc_fp64_peak(int device);
/* The same probe in other shapes, for checking that kc_fp64_peak is the pipe's rate and not the
 * probe's: blocks_per_sm x threads (128 or 256) per SM, `chains` independent chains per thread
 * (4, 8 or 16 for DFMA, 8 for the others) of opcode op (0 DFMA, 1 DMUL, 2 DADD).  Returns FP64
 * lane operations per second (an FMA counts once), or -1. */
double kc_fp64_probe_rate(int device, int blocks_per_sm, int threads, int chains, int op);

/* ---- per-length tuning (replaces `kite tune`, tools/kite.c:274-326 and src/ctx.c:35-92) ------
 * The four-step shape H = R*C of each FFT length can be chosen by measurement instead of the
 * default (rows about four times as long as columns).  A tuning file has lines "L us R C":
 * the length, its measured microseconds per squaring (batched throughput), and the shape; the
 * times also drive the length choice among the safe lengths within 30 %, as the reference's
 * tuning file does.  Plans built before a change keep their shape. */
/* Use R rows for length L (R = 0: back to the default).  0, or -1 if the shape is unusable. */
int kc_set_fft_shape(uint32_t L, uint32_t R);
/* Record the measured time of length L (us <= 0 forgets it). */
void kc_set_fft_time(uint32_t L, double us);
/* Candidate shapes of length L near balance: up to `max` (R, C) pairs; returns the count. */
int kc_fft_shape_candidates(uint32_t L, uint32_t *R, uint32_t *C, int max);
/* The shape length L gets now. 0, or -1. */
int kc_fft_shape(uint32_t L, uint32_t *R, uint32_t *C);
/* Shape of one test run alone (latency mode, kc_engine_new with throughput 0) at length L:
 * R rows and column groups of G in {2, 4, 8} (R = 0: back to the built-in model).  Used for
 * every number whose digits allow groups of G.  0, or -1 if the shape is unusable. */
int kc_set_latency_shape(uint32_t L, uint32_t R, int G);
/* Load a tuning file (shapes and times).  Lines "L us R C G" (five fields) are latency shapes
 * (kc_set_latency_shape; their times, single-test microseconds, do not steer the length
 * choice).  Returns the number of lines read, -1 if unreadable.  The library also loads
 * $KITE_GB300_TUNING, if set, when it plans its first length. */
int kc_tuning_load(const char *path);
/* Largest round-off of `squarings` squarings of a seeded residue mod k*2^n-1 at length L on the
 * current GPU (the reference's tools/sweep_err.c measurement); negative on failure. */
double kc_roundoff_probe(uint64_t k, uint64_t n, uint32_t L, uint32_t squarings, uint64_t seed);

/* ---- host-only helpers (no GPU needed) ---------------------------------------------------
 * The exact integer layer the engine's callers use, exported so a host can check or reuse it:
 * kc_layout fills the digit layout of (k, n, L) as the reference's build_layout does
 * (src/ctx.c:198-221): bits[L], w[L], oscale[L] and meta = {lam, sL, top_t, top_st, top_m};
 * kc_digits_to_limbs / kc_limbs_to_digits convert as kite_get_limbs / kite_set_limbs
 * (src/ctx.c:497-544); kc_carry_digits is kite_carry_digits (src/ctx.c:378-407).  Each returns
 * 0, or -1 when (k, n, L) cannot be laid out. */
int kc_layout(uint64_t k, uint64_t n, uint32_t L, uint8_t *bits, double *w, double *oscale,
              uint64_t *meta);
int kc_digits_to_limbs(uint64_t k, uint64_t n, uint32_t L, const int64_t *digits, uint64_t *limbs);
int kc_limbs_to_digits(uint64_t k, uint64_t n, uint32_t L, const uint64_t *limbs, int64_t *digits);
int kc_carry_digits(uint64_t k, uint64_t n, uint32_t L, int64_t *digits);
/* FFT length the engine picks for (k, n) (src/ctx.c:107-141), 0 if none. */
uint32_t kc_choose_fft_len(uint64_t k, uint64_t n);

#ifdef __cplusplus
}
#endif
#endif
