/* PRST-compatible Fermat proofs for k*2^n-1 on the GB300 engine.
 *
 * The same entry points, argument meanings, file names and file bytes as the reference's proof
 * module (src/prstproof.h:1-57, the "smooth" path of PRST 14.1: x_0 = a^k, then n squarings,
 * points at PRST's positions, products compressed with MD5 challenges, a certificate that
 * `prst -proof cert` verifies).  Every product, power and certificate squaring runs on the GPU
 * through the kite_* calls of kite.h; files and hashes are host work.
 *
 * File layout (src/prstproof.c:91-109, PRST's TaskState): little-endian 32-bit words
 *   magic 0x9f2b3cd4, app id 4 | type << 16, [fingerprint if non-zero], iteration,
 *   then per value: its word count and its words (no leading zero words),
 * written through "<path>.tmp" and a rename, with a "<path>.md5" sidecar holding the lowercase
 * hex MD5 of the file.  Point files are "<prefix>.proof.<i>", products "<prefix>.prod.<j>", the
 * certificate "<prefix>.cert"; prefix is "prst_<N mod 3417905339>".
 */
#ifndef KITE_PROOF_H
#define KITE_PROOF_H

#include <stdint.h>

#include "kite.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A non-negative integer as PRST stores it: little-endian 32-bit words, no leading zeros
 * (src/prstproof.h:11-15).  Giants returned by this library are freed with pp_giant_free. */
typedef struct {
    uint32_t *w;
    int32_t len;
} pp_giant;

void pp_giant_free(pp_giant *g);

enum { PP_TYPE_VALUE = 1, PP_TYPE_PRODUCT = 3, PP_TYPE_CERT = 4 };

/* (k*2^n - 1) mod 3417905339 (src/prstproof.c:34-40). */
uint32_t pp_fingerprint(uint64_t k, uint64_t n);
/* The first little-endian word of MD5(fp as 4 bytes || id) (src/prstproof.c:42-50). */
uint32_t pp_unique_fingerprint(uint32_t fp, const char *id);
/* The fingerprint inside point and product files: unique(fp, "<a>.<n>") (src/prstproof.c:52-56). */
uint32_t pp_proof_fingerprint(uint64_t k, uint64_t n, uint32_t a);

/* Write a state file and its .md5 sidecar; 0 on success (src/prstproof.c:91-109). */
int pp_write(const char *path, int type, uint32_t fingerprint, int32_t iteration,
             const pp_giant *g, int ng);
/* Read a state file: magic, app id, type, fingerprint (when non-zero) and a present .md5
 * sidecar are checked.  Fills up to maxg giants; trailing giants the file lacks are left empty.
 * 0 on success (src/prstproof.c:126-180). */
int pp_read(const char *path, int type, uint32_t fingerprint, int32_t *iteration, pp_giant *g,
            int maxg);

/* Positions of the count+1 proof points along `iterations` squarings (count a power of 2);
 * returns PRST's spacing M (src/prstproof.c:191-207). */
int pp_points(uint32_t iterations, int count, uint32_t *pos);

/* Conversions between a number and a giant holding its value in [0, N)
 * (src/prstproof.c:209-237). */
void pp_from_num(kite_ctx *ctx, const kite_num *x, pp_giant *g);
void pp_to_num(kite_ctx *ctx, const pp_giant *g, kite_num *x);
uint64_t pp_res64(const pp_giant *g);

/* Save step (src/prstproof.c:317-429): points 0..count are on disk under `prefix`; writes the
 * products and the raw certificate RES64.  Deletes points 1..count-1 unless keep.  Products
 * left by an interrupted run are reused.  Returns PP_ABORTED when *abort_flag turns non-zero
 * between points. */
enum { PP_ABORTED = -2 };
int pp_save_products(kite_ctx *ctx, uint64_t k, uint64_t n, uint32_t a, int count,
                     const char *prefix, int keep, volatile int *abort_flag, uint64_t *raw_res64);
/* Build step (src/prstproof.c:500-597): checks point 0 = a^k and, for a composite result, the
 * roots-of-unity condition; writes <prefix>.cert and returns the certificate RES64.  Deletes
 * points 0 and count and the products unless keep. */
int pp_build_cert(kite_ctx *ctx, uint64_t k, uint64_t n, uint32_t a, int count,
                  const char *prefix, int keep, uint64_t *cert_res64);
/* Verify (src/prstproof.c:600-666): squares the certificate's value M times with a Gerbicz
 * check and returns the RES64 PRST prints as "certificate RES64". */
int pp_verify_cert(kite_ctx *ctx, uint64_t k, uint64_t n, const char *path, uint64_t *cert_res64,
                   uint32_t *M);

#ifdef __cplusplus
}
#endif
#endif
