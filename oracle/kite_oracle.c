/* CPU oracle for the k*2^n-1 squaring path.  TEST INFRASTRUCTURE ONLY (see kite_oracle.h):
 * it is the checker for the tests, the smoke check and the CPU-baseline leg of the benchmark,
 * never part of the product.
 *
 * Each function cites the reference function whose behaviour it restates (kite, paths relative
 * to the project root).  The arithmetic is written out here independently; where a step has to
 * produce the same bits as the reference (the 64-bit log2 fraction, the digit boundaries and the
 * weights) the method is the same published one and says so.
 */
#include "kite_oracle.h"

#include <complex.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef unsigned __int128 u128;
typedef __int128 i128;
typedef double complex cplx;

struct ko_ctx {
    uint64_t k, n;
    uint32_t L;
    uint64_t lam;    /* frac(log2 k) * 2^64 */
    u128 tfix;       /* T' * 2^64 = (n + floor(log2 k)) * 2^64 + lam */
    uint64_t *s;     /* s[j] = ceil(j T'/L), j = 0..L */
    uint8_t *bits;   /* s[j+1] - s[j] */
    double *w, *oscale;
    uint32_t top_t, top_m;
    uint64_t top_st, sL;
    size_t nlimbs;
    uint64_t *Nl;
    double maxerr;
    uint32_t nrad, rad[48];
    cplx *tw;        /* tw[j] = exp(-2 pi i j / L) */
    cplx *fa, *fb, *fc;
    int64_t *dig;
};

/* ---- FFT-length helpers: src/ctx.c:17-33, 94-148 ------------------------------------------ */

int ko_fft_len_ok(uint32_t L) {
    if (L < 16 || (L & 1)) return 0;
    static const uint32_t primes[4] = {2, 3, 5, 7};
    for (int i = 0; i < 4; i++)
        while (L % primes[i] == 0) L /= primes[i];
    return L == 1;
}

/* Fitted safe bits per word, less the 0.2 margin (src/ctx.c:26-33). */
double ko_safe_bpw(uint32_t L, uint64_t k) {
    return 21.44 - 0.305 * (log2((double)L) - 12.0) - 0.5 * log2((double)k) - 0.2;
}

/* Relative cost used when no tuning file exists (src/ctx.c:94-103). */
static double heuristic_cost(uint32_t L) {
    double c = log2((double)L);
    uint32_t m = L;
    for (; m % 3 == 0; m /= 3) c += 0.6;
    for (; m % 5 == 0; m /= 5) c += 1.0;
    for (; m % 7 == 0; m /= 7) c += 1.4;
    return (double)L * c;
}

static int usable(uint32_t L) { return L % 64 == 0 && ko_fft_len_ok(L); }

/* src/ctx.c:107-141 without a tuning file: the first safe usable length, then the cheapest
 * usable length up to 30% above it by the heuristic. */
uint32_t ko_choose_fft_len(uint64_t k, uint64_t n) {
    if (n < 2048) {
        for (uint32_t L = 16; L <= n; L *= 2)
            if ((double)n / L <= ko_safe_bpw(L, k)) return L;
        return 0;
    }
    uint32_t first = 0;
    for (uint32_t L = 64; L < (1u << 28); L += 64) {
        if (usable(L) && (double)n / L <= ko_safe_bpw(L, k)) {
            first = L;
            break;
        }
    }
    if (!first) return 0;
    uint32_t best = first;
    double bestc = INFINITY;
    for (uint32_t L = first; L <= first + first / 10 * 3; L += 64) {
        if (!usable(L)) continue;
        double cst = heuristic_cost(L);
        if (cst < bestc) {
            bestc = cst;
            best = L;
        }
    }
    return best;
}

/* src/ctx.c:143-148 */
uint32_t ko_next_fft_len(uint32_t L) {
    for (uint32_t M = (L / 64 + 1) * 64; M < (1u << 28); M += 64)
        if (ko_fft_len_ok(M)) return M;
    return 0;
}

/* ---- exact layout: src/ctx.c:150-221 -------------------------------------------------------- */

/* frac(log2 k) to 64 bits by the classic bit-at-a-time squaring method (as src/ctx.c:153-167,
 * 62 fractional bits of fixed point, truncating), so that the layout is bit-identical. */
static uint64_t log2_fraction(uint64_t k) {
    int e = 63 - __builtin_clzll(k);
    u128 y = (u128)k << (62 - e); /* y/2^62 in [1, 2) */
    uint64_t f = 0;
    for (int i = 0; i < 64; i++) {
        y = (y * y) >> 62;
        f <<= 1;
        if (y >> 63) {
            f |= 1;
            y >>= 1;
        }
    }
    return f;
}

/* twiddle exp(-2 pi i j / m) with the angle reduced exactly in integers to [0, pi/4] */
static cplx cis_neg(uint64_t j, uint64_t m) {
    j %= m;
    /* angle = pi * x, x = num/den = 2j/m in [0, 2) */
    uint64_t num = 2 * j, den = m;
    double cs = 1, sn = 1; /* signs */
    int swap = 0;
    if (num > den) { /* x in (1, 2): x-1, both negate */
        num -= den;
        cs = -cs;
        sn = -sn;
    }
    if (2 * num > den) { /* x in (1/2, 1]: 1-x, cos negates */
        num = den - num;
        cs = -cs;
    }
    if (4 * num > den) { /* x in (1/4, 1/2]: 1/2-x, cos<->sin */
        num = den - 2 * num;
        den = 2 * den;
        swap = 1;
    }
    long double th = 3.14159265358979323846264338327950288L * (long double)num / (long double)den;
    double c = (double)cosl(th), s = (double)sinl(th);
    if (swap) {
        double t = c;
        c = s;
        s = t;
    }
    return cs * c - I * (sn * s);
}

static int factor_radices(uint32_t L, uint32_t *rad) {
    int m = 0;
    while (L % 4 == 0) { rad[m++] = 4; L /= 4; }
    static const uint32_t pr[4] = {2, 3, 5, 7};
    for (int i = 0; i < 4; i++)
        while (L % pr[i] == 0) { rad[m++] = pr[i]; L /= pr[i]; }
    return L == 1 ? m : -1;
}

ko_ctx *ko_ctx_new(uint64_t k, uint64_t n, uint32_t L) {
    /* argument checks as src/ctx.c:224-235 */
    if (k == 0 || !(k & 1) || k >= (1ull << 30) || n < 8) return NULL;
    if (!L) L = ko_choose_fft_len(k, n);
    if (!ko_fft_len_ok(L) || L > n) return NULL;
    ko_ctx *c = calloc(1, sizeof *c);
    if (!c) return NULL;
    c->k = k;
    c->n = n;
    c->L = L;
    c->lam = log2_fraction(k);
    uint64_t e = (uint64_t)(63 - __builtin_clzll(k));
    c->tfix = ((u128)(n + e) << 64) + c->lam;
    c->s = malloc((size_t)(L + 1) * sizeof(uint64_t));
    c->bits = malloc(L);
    c->w = malloc((size_t)L * sizeof(double));
    c->oscale = malloc((size_t)L * sizeof(double));
    c->nlimbs = (n + 64 + 63) / 64;
    c->Nl = calloc(c->nlimbs, sizeof(uint64_t));
    c->tw = malloc((size_t)L * sizeof(cplx));
    c->fa = malloc((size_t)L * sizeof(cplx));
    c->fb = malloc((size_t)L * sizeof(cplx));
    c->fc = malloc((size_t)L * sizeof(cplx));
    c->dig = malloc((size_t)L * sizeof(int64_t));
    if (!c->s || !c->bits || !c->w || !c->oscale || !c->Nl || !c->tw || !c->fa || !c->fb ||
        !c->fc || !c->dig)
        goto fail;
    u128 den = (u128)L << 64;
    for (uint32_t j = 0; j <= L; j++) {
        u128 num = (u128)j * c->tfix; /* < 2^118 for the sizes accepted above */
        c->s[j] = (uint64_t)((num + den - 1) / den);
    }
    c->top_t = L;
    for (uint32_t j = 0; j < L; j++) {
        uint64_t d = c->s[j + 1] - c->s[j];
        if (d > 40 || d == 0) goto fail;
        c->bits[j] = (uint8_t)d;
        if (c->top_t == L && c->s[j + 1] > n) c->top_t = j;
        /* w_j = 2^{s_j - j T'/L}: the exponent is (s_j L 2^64 - j T' 2^64) / (L 2^64) in [0,1);
         * its top 64 bits, rounded to double, then exp2 (src/ctx.c:186-196) */
        u128 r = (u128)c->s[j] * den - (u128)j * c->tfix;
        double frac = (double)(uint64_t)(r / L) / 18446744073709551616.0;
        c->w[j] = exp2(frac);
        c->oscale[j] = (double)k / c->w[j];
    }
    c->sL = c->s[L];
    c->top_st = c->top_t < L ? c->s[c->top_t] : c->sL;
    c->top_m = (uint32_t)(n - c->top_st);
    if (c->sL - c->top_st > 100 || c->top_t == 0) goto fail;
    /* N = k*2^n - 1 */
    c->Nl[n / 64] = k << (n % 64);
    if (n % 64 && n / 64 + 1 < c->nlimbs) c->Nl[n / 64 + 1] = k >> (64 - n % 64);
    for (size_t i = 0; i < c->nlimbs; i++)
        if (c->Nl[i]--) break;
    int m = factor_radices(L, c->rad);
    if (m < 0) goto fail;
    c->nrad = (uint32_t)m;
    for (uint32_t j = 0; j < L; j++) c->tw[j] = cis_neg(j, L);
    return c;
fail:
    ko_ctx_free(c);
    return NULL;
}

void ko_ctx_free(ko_ctx *c) {
    if (!c) return;
    free(c->s);
    free(c->bits);
    free(c->w);
    free(c->oscale);
    free(c->Nl);
    free(c->tw);
    free(c->fa);
    free(c->fb);
    free(c->fc);
    free(c->dig);
    free(c);
}

uint32_t ko_fft_len(const ko_ctx *c) { return c->L; }
size_t ko_limbs(const ko_ctx *c) { return c->nlimbs; }
double ko_maxerr(const ko_ctx *c) { return c->maxerr; }
void ko_reset_maxerr(ko_ctx *c) { c->maxerr = 0; }

void ko_layout(const ko_ctx *c, uint8_t *bits, double *w, double *oscale, uint64_t *meta) {
    if (bits) memcpy(bits, c->bits, c->L);
    if (w) memcpy(w, c->w, (size_t)c->L * sizeof(double));
    if (oscale) memcpy(oscale, c->oscale, (size_t)c->L * sizeof(double));
    if (meta) {
        meta[0] = c->lam;
        meta[1] = c->sL;
        meta[2] = c->top_t;
        meta[3] = c->top_st;
        meta[4] = c->top_m;
    }
}

/* ---- balanced carry and the top fold: src/ctx.c:345-407 -------------------------------------- */

static inline int64_t balance(int64_t v, unsigned b, int64_t *q) {
    int64_t h = (int64_t)1 << (b - 1);
    *q = (v + h) >> b; /* floor division by 2^b (arithmetic shift) */
    return v - (*q << b);
}

static i128 floor_div(i128 a, i128 b) { /* b > 0 */
    i128 q = a / b;
    if ((a % b) != 0 && a < 0) q -= 1;
    return q;
}

/* The value above 2^n -- the top digits t..L-1 plus the carry cy at 2^{s_L} -- is H*2^{s_t}.
 * With m = n - s_t: H = lo + 2^m*hi, hi = q*k + r, and k*2^n == 1 (mod N), so the region keeps
 * lo + r*2^m (re-centred to [-k 2^m/2, k 2^m/2)) and q moves to digit 0. */
static int64_t fold_top(const ko_ctx *c, int64_t *d, int64_t cy) {
    uint32_t L = c->L, t = c->top_t;
    i128 H = (i128)cy << (c->sL - c->top_st);
    unsigned pos = 0;
    for (uint32_t j = t; j < L; j++) {
        H += (i128)d[j] << pos;
        pos += c->bits[j];
    }
    unsigned m = c->top_m;
    i128 lo = H & (((i128)1 << m) - 1);
    i128 hi = H >> m;
    i128 K = (i128)c->k;
    i128 q = floor_div(hi, K);
    i128 top = lo + ((hi - q * K) << m);
    i128 span = K << m;
    if (2 * top >= span) {
        top -= span;
        q += 1;
    }
    for (uint32_t j = t; j + 1 < L; j++) {
        unsigned b = c->bits[j];
        i128 qq = (top + ((i128)1 << (b - 1))) >> b;
        d[j] = (int64_t)(top - (qq << b));
        top = qq;
    }
    if (t < L) d[L - 1] = (int64_t)top;
    return (int64_t)q;
}

void ko_carry_digits(const ko_ctx *c, int64_t *d) {
    uint32_t L = c->L;
    int64_t cy = 0;
    for (uint32_t j = 0; j < L; j++) d[j] = balance(d[j] + cy, c->bits[j], &cy);
    for (int pass = 0; pass < 64; pass++) {
        cy = fold_top(c, d, cy);
        for (uint32_t j = 0; j < c->top_t && cy; j++) d[j] = balance(d[j] + cy, c->bits[j], &cy);
        if (!cy) return;
        if (c->top_t < L) {
            d[c->top_t] += cy;
            cy = 0;
        }
    }
}

/* ---- big-integer helpers (little-endian u64 limbs) ------------------------------------------- */

static void big_add_at(uint64_t *a, size_t na, uint64_t pos, uint64_t v) {
    size_t w = pos / 64;
    unsigned sh = pos % 64;
    if (w >= na) return;
    u128 t = (u128)v << sh;
    u128 s = (u128)a[w] + (uint64_t)t;
    a[w] = (uint64_t)s;
    uint64_t carry = (uint64_t)(s >> 64) + (uint64_t)(t >> 64);
    for (size_t i = w + 1; carry && i < na; i++) {
        s = (u128)a[i] + carry;
        a[i] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
    }
}

static int big_cmp(const uint64_t *a, const uint64_t *b, size_t n) {
    for (size_t i = n; i-- > 0;)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}

static void big_sub(uint64_t *a, const uint64_t *b, size_t n) { /* a -= b, a >= b */
    uint64_t br = 0;
    for (size_t i = 0; i < n; i++) {
        u128 d = (u128)a[i] - b[i] - br;
        a[i] = (uint64_t)d;
        br = (uint64_t)(d >> 64) & 1;
    }
}

static void big_add(uint64_t *a, const uint64_t *b, size_t n) {
    uint64_t cy = 0;
    for (size_t i = 0; i < n; i++) {
        u128 s = (u128)a[i] + b[i] + cy;
        a[i] = (uint64_t)s;
        cy = (uint64_t)(s >> 64);
    }
}

static void big_mul_small(uint64_t *a, size_t n, uint64_t m) {
    u128 cy = 0;
    for (size_t i = 0; i < n; i++) {
        cy += (u128)a[i] * m;
        a[i] = (uint64_t)cy;
        cy >>= 64;
    }
}

/* a /= m in place, returns the remainder */
static uint64_t big_div_small(uint64_t *a, size_t n, uint64_t m) {
    u128 r = 0;
    for (size_t i = n; i-- > 0;) {
        r = (r << 64) | a[i];
        a[i] = (uint64_t)(r / m);
        r %= m;
    }
    return (uint64_t)r;
}

static uint64_t big_mod_small(const uint64_t *a, size_t n, uint64_t m) {
    u128 r = 0;
    for (size_t i = n; i-- > 0;) r = ((r << 64) | a[i]) % m;
    return (uint64_t)r;
}

static int big_is_zero(const uint64_t *a, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (a[i]) return 0;
    return 1;
}

/* Reduce a (na >= nlimbs limbs, value below 2^(64 na)) into [0, N), using k*2^n == 1: write
 * a = lo + 2^n*hi with hi = q*k + r; then a == lo + r*2^n + q.  Result in a[0..nlimbs). */
static void reduce_mod_N(const ko_ctx *c, uint64_t *a, size_t na) {
    uint64_t n = c->n;
    size_t w0 = n / 64;
    unsigned sh = n % 64;
    size_t nh = na - w0 + 1;
    uint64_t *hi = calloc(nh, sizeof(uint64_t));
    for (;;) {
        /* hi = a >> n */
        memset(hi, 0, nh * sizeof(uint64_t));
        for (size_t i = w0; i < na; i++) {
            size_t o = i - w0;
            hi[o] |= sh ? a[i] >> sh : a[i];
            if (sh && o > 0) hi[o - 1] |= a[i] << (64 - sh);
        }
        /* stop once hi < k */
        int small = 1;
        for (size_t i = 1; i < nh; i++)
            if (hi[i]) small = 0;
        if (small && hi[0] < c->k) break;
        uint64_t r = big_div_small(hi, nh, c->k);
        /* a = lo */
        if (sh) a[w0] &= ((uint64_t)1 << sh) - 1;
        else a[w0] = 0;
        for (size_t i = w0 + 1; i < na; i++) a[i] = 0;
        big_add_at(a, na, n, r);
        for (size_t i = 0; i < nh; i++) big_add_at(a, na, 64 * (uint64_t)i, hi[i]);
    }
    free(hi);
    for (size_t i = c->nlimbs; i < na; i++)
        if (a[i]) { /* cannot happen: a < k 2^n < 2^(64 nlimbs) */ }
    if (big_cmp(a, c->Nl, c->nlimbs) >= 0) big_sub(a, c->Nl, c->nlimbs);
}

/* x = k * sum(d_j 2^{s_j}) mod N, for integer digits of any sign (src/ctx.c:477-517) */
void ko_digits_to_limbs(const ko_ctx *c, const int64_t *dig, uint64_t *limbs) {
    size_t na = (c->sL + 64 + 40) / 64 + 3;
    if (na < c->nlimbs + 2) na = c->nlimbs + 2;
    uint64_t *P = calloc(na, sizeof(uint64_t)), *M = calloc(na, sizeof(uint64_t));
    for (uint32_t j = 0; j < c->L; j++) {
        int64_t v = dig[j];
        if (v > 0) big_add_at(P, na, c->s[j], (uint64_t)v);
        else if (v < 0) big_add_at(M, na, c->s[j], (uint64_t)(-(v + 1)) + 1);
    }
    big_mul_small(P, na, c->k);
    big_mul_small(M, na, c->k);
    reduce_mod_N(c, P, na);
    reduce_mod_N(c, M, na);
    if (big_cmp(P, M, c->nlimbs) < 0) big_add(P, c->Nl, c->nlimbs);
    big_sub(P, M, c->nlimbs);
    memcpy(limbs, P, c->nlimbs * sizeof(uint64_t));
    free(P);
    free(M);
}

static uint64_t big_get_bits(const uint64_t *a, size_t na, uint64_t pos, unsigned cnt) {
    size_t w = pos / 64;
    unsigned sh = pos % 64;
    if (w >= na) return 0;
    u128 v = a[w];
    if (w + 1 < na) v |= (u128)a[w + 1] << 64;
    v >>= sh;
    return cnt >= 64 ? (uint64_t)v : (uint64_t)v & (((uint64_t)1 << cnt) - 1);
}

/* limbs x in [0, N) -> stored value V = x/k == x*2^n (mod N) as balanced digits
 * (src/ctx.c:519-544) */
static void limbs_to_digits(const ko_ctx *c, const uint64_t *limbs, int64_t *d) {
    size_t na = c->nlimbs + 2;
    uint64_t *a = calloc(na, sizeof(uint64_t));
    memcpy(a, limbs, c->nlimbs * sizeof(uint64_t));
    uint64_t r = big_div_small(a, na, c->k); /* a = q, x = q k + r */
    big_add_at(a, na, c->n, r);              /* V = q + r 2^n <= N */
    if (big_cmp(a, c->Nl, c->nlimbs) >= 0 && !a[c->nlimbs] && !a[c->nlimbs + 1])
        big_sub(a, c->Nl, c->nlimbs);
    for (uint32_t j = 0; j + 1 < c->L; j++) d[j] = (int64_t)big_get_bits(a, na, c->s[j], c->bits[j]);
    d[c->L - 1] = (int64_t)big_get_bits(a, na, c->s[c->L - 1], 64);
    free(a);
    ko_carry_digits(c, d);
}

void ko_set_limbs(ko_ctx *c, double *x, const uint64_t *limbs) {
    limbs_to_digits(c, limbs, c->dig);
    for (uint32_t j = 0; j < c->L; j++) x[j] = (double)c->dig[j];
}

void ko_get_limbs(ko_ctx *c, const double *x, uint64_t *limbs) {
    for (uint32_t j = 0; j < c->L; j++) c->dig[j] = (int64_t)x[j];
    ko_digits_to_limbs(c, c->dig, limbs);
}

uint64_t ko_res64(ko_ctx *c, const double *x) {
    uint64_t *l = malloc(c->nlimbs * sizeof(uint64_t));
    ko_get_limbs(c, x, l);
    uint64_t r = l[0];
    free(l);
    return r;
}

/* ---- weighted full-length FFT arithmetic: src/ref_fft.c:26-139 ------------------------------ */

/* Forward DFT (exp(-2 pi i jk/L)) of src into dst by a Stockham decimation-in-time sweep;
 * src is used as scratch. */
static void dft_forward(const ko_ctx *c, cplx *src, cplx *dst) {
    uint32_t L = c->L, Lp = 1;
    cplx *in = src, *out = dst;
    for (uint32_t st = 0; st < c->nrad; st++) {
        uint32_t p = c->rad[st], Lt = Lp * p, r = L / Lt, step = L / p;
        for (uint32_t i = 0; i < r; i++) {
            for (uint32_t kk = 0; kk < Lp; kk++) {
                cplx t[8];
                for (uint32_t q = 0; q < p; q++) {
                    cplx v = in[(size_t)(i + r * q) * Lp + kk];
                    t[q] = q && kk ? v * c->tw[(size_t)q * kk * r] : v;
                }
                cplx *o = out + (size_t)i * Lt + kk;
                if (p == 4) {
                    cplx a = t[0] + t[2], b = t[0] - t[2], e = t[1] + t[3];
                    cplx f = (t[1] - t[3]) * -I;
                    o[0] = a + e;
                    o[Lp] = b + f;
                    o[2 * Lp] = a - e;
                    o[3 * Lp] = b - f;
                } else if (p == 2) {
                    o[0] = t[0] + t[1];
                    o[Lp] = t[0] - t[1];
                } else {
                    for (uint32_t s = 0; s < p; s++) {
                        cplx acc = t[0];
                        for (uint32_t q = 1; q < p; q++) acc += t[q] * c->tw[(size_t)((q * s) % p) * step];
                        o[(size_t)s * Lp] = acc;
                    }
                }
            }
        }
        cplx *tmp = in;
        in = out;
        out = tmp;
        Lp = Lt;
    }
    if (in != dst) memcpy(dst, in, (size_t)L * sizeof(cplx));
}

static void weighted_forward(ko_ctx *c, const double *x, cplx *dst) {
    for (uint32_t j = 0; j < c->L; j++) c->fc[j] = x[j] * c->w[j];
    dft_forward(c, c->fc, dst);
}

/* prod holds the pointwise product; inverse transform, unweight (times k / L), round, track the
 * round-off, carry (src/ref_fft.c:92-112) */
static void inverse_round_carry(ko_ctx *c, cplx *prod, double *x) {
    uint32_t L = c->L;
    for (uint32_t j = 0; j < L; j++) prod[j] = conj(prod[j]);
    dft_forward(c, prod, c->fb);
    double inv = 1.0 / L, me = c->maxerr;
    for (uint32_t j = 0; j < L; j++) {
        double v = creal(c->fb[j]) * inv * c->oscale[j];
        double r = rint(v);
        double e = fabs(v - r);
        if (e > me) me = e;
        c->dig[j] = (int64_t)r;
    }
    c->maxerr = me;
    ko_carry_digits(c, c->dig);
    for (uint32_t j = 0; j < L; j++) x[j] = (double)c->dig[j];
}

void ko_square(ko_ctx *c, double *x, uint64_t count) {
    for (uint64_t i = 0; i < count; i++) {
        weighted_forward(c, x, c->fa);
        for (uint32_t j = 0; j < c->L; j++) c->fa[j] *= c->fa[j];
        inverse_round_carry(c, c->fa, x);
    }
}

void ko_mul(ko_ctx *c, double *x, const double *y) {
    uint32_t L = c->L;
    cplx *fy = malloc((size_t)L * sizeof(cplx));
    weighted_forward(c, y, fy);
    weighted_forward(c, x, c->fa);
    for (uint32_t j = 0; j < L; j++) c->fa[j] *= fy[j];
    free(fy);
    inverse_round_carry(c, c->fa, x);
}

void ko_mul_small(ko_ctx *c, double *x, int64_t m) {
    for (uint32_t j = 0; j < c->L; j++) c->dig[j] = (int64_t)x[j] * m;
    ko_carry_digits(c, c->dig);
    for (uint32_t j = 0; j < c->L; j++) x[j] = (double)c->dig[j];
}

/* element-wise, as src/ctx.c:336-343: digits are left unbalanced until the next product */
void ko_add(ko_ctx *c, double *x, const double *y) {
    for (uint32_t j = 0; j < c->L; j++) x[j] += y[j];
}
void ko_sub(ko_ctx *c, double *x, const double *y) {
    for (uint32_t j = 0; j < c->L; j++) x[j] -= y[j];
}

/* ---- base^(N-1) from base^(N+1): src/prp.c:63-144 ------------------------------------------- */

/* a = a / d mod m (a < m, gcd(d, m) = 1, d small): add t*m with a + t m == 0 (mod d), divide */
static void div_small_mod(uint64_t *a, const uint64_t *m, size_t n, uint64_t d) {
    if (n == 0 || n > ((size_t)1 << 40)) return;
    uint64_t am = big_mod_small(a, n, d), mm = big_mod_small(m, n, d), t = 0;
    while ((am + (u128)t * mm) % d) t++;
    uint64_t *tmp = calloc(n + 1, sizeof(uint64_t));
    memcpy(tmp, m, n * sizeof(uint64_t));
    big_mul_small(tmp, n + 1, t);
    uint64_t *acc = calloc(n + 1, sizeof(uint64_t));
    memcpy(acc, a, n * sizeof(uint64_t));
    big_add(acc, tmp, n + 1);
    big_div_small(acc, n + 1, d);
    memcpy(a, acc, n * sizeof(uint64_t));
    free(tmp);
    free(acc);
}

int ko_residue_nm1(uint64_t *y, const uint64_t *N, size_t nl, uint64_t base) {
    /* N = Q * M, Q collecting the primes of base that divide N */
    uint64_t Q = 1, b = base;
    uint64_t *M = calloc(nl + 1, sizeof(uint64_t));
    memcpy(M, N, nl * sizeof(uint64_t));
    for (uint64_t p = 2; b > 1; p++) {
        if (b % p) continue;
        while (b % p == 0) b /= p;
        while (big_mod_small(M, nl, p) == 0) {
            if (Q > (1ull << 40)) {
                free(M);
                return -1;
            }
            Q *= p;
            big_div_small(M, nl, p);
        }
    }
    if (Q == 1) {
        div_small_mod(y, N, nl, base);
        div_small_mod(y, N, nl, base);
        free(M);
        return 0;
    }
    /* r = y mod M, then r / base^2 mod M; the answer is the x == 0 (mod Q), x == r (mod M) */
    uint64_t *r = calloc(nl + 1, sizeof(uint64_t));
    memcpy(r, y, nl * sizeof(uint64_t));
    while (big_cmp(r, M, nl + 1) >= 0) big_sub(r, M, nl + 1); /* y < N = Q M: < Q rounds */
    div_small_mod(r, M, nl, base);
    div_small_mod(r, M, nl, base);
    uint64_t rm = big_mod_small(r, nl, Q), mm = big_mod_small(M, nl, Q), u = 0;
    while ((rm + (u128)mm * u) % Q) u++;
    uint64_t *t = calloc(nl + 1, sizeof(uint64_t));
    memcpy(t, M, nl * sizeof(uint64_t));
    big_mul_small(t, nl + 1, u);
    big_add(r, t, nl + 1);
    memcpy(y, r, nl * sizeof(uint64_t));
    free(t);
    free(r);
    free(M);
    return 0;
}

/* ---- drivers ------------------------------------------------------------------------------- */

/* x0 = base^k mod N: exact when base^k < N, else by square-and-multiply (src/prp.c:298-327) */
static void power_base_k(ko_ctx *c, double *x, uint64_t base) {
    size_t nl = c->nlimbs;
    uint64_t *l = calloc(nl, sizeof(uint64_t));
    if ((double)c->k * log2((double)base) + 2 < (double)c->n) {
        l[0] = 1;
        for (uint64_t i = 0; i < c->k; i++) big_mul_small(l, nl, base);
        ko_set_limbs(c, x, l);
    } else {
        l[0] = 1;
        ko_set_limbs(c, x, l);
        for (int b = 63; b >= 0; b--) {
            if (c->k >> b == 0) continue;
            ko_square(c, x, 1);
            if ((c->k >> b) & 1) ko_mul_small(c, x, (int64_t)base);
        }
    }
    free(l);
}

int ko_fermat(uint64_t k, uint64_t n, uint32_t base, uint32_t L, uint64_t *res64, int *is_prp,
              double *maxerr) {
    ko_ctx *c = ko_ctx_new(k, n, L);
    if (!c) return -1;
    double *x = calloc(c->L, sizeof(double));
    size_t nl = c->nlimbs;
    uint64_t *y = calloc(nl, sizeof(uint64_t));
    power_base_k(c, x, base);
    ko_square(c, x, n);
    ko_get_limbs(c, x, y);
    int prp = y[0] == (uint64_t)base * base;
    for (size_t i = 1; i < nl; i++) prp &= y[i] == 0;
    int rc = ko_residue_nm1(y, c->Nl, nl, base);
    if (res64) *res64 = y[0];
    if (is_prp) *is_prp = prp;
    if (maxerr) *maxerr = c->maxerr;
    free(x);
    free(y);
    ko_ctx_free(c);
    return rc ? -4 : 0;
}

static uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); }

static uint64_t N_mod(uint64_t k, uint64_t n, uint64_t m) { /* (k 2^n - 1) mod m */
    uint64_t r = 1 % m, b = 2 % m;
    for (uint64_t e = n; e; e >>= 1, b = mulmod64(b, b, m))
        if (e & 1) r = mulmod64(r, b, m);
    return (mulmod64(k % m, r, m) + m - 1 % m) % m;
}

static int jacobi_small(uint64_t a, uint64_t m) { /* m odd */
    int s = 1;
    a %= m;
    while (a) {
        while (!(a & 1)) {
            a >>= 1;
            uint64_t r = m & 7;
            if (r == 3 || r == 5) s = -s;
        }
        uint64_t t = a;
        a = m;
        m = t;
        if ((a & 3) == 3 && (m & 3) == 3) s = -s;
        a %= m;
    }
    return m == 1 ? s : 0;
}

/* Jacobi(a | N) for small a by quadratic reciprocity against N mod a (src/llr.c:58-69) */
static int jacobi_N(uint64_t a, uint64_t k, uint64_t n) {
    int s = 1;
    uint64_t n8 = N_mod(k, n, 8);
    while (a && !(a & 1)) {
        a >>= 1;
        if (n8 == 3 || n8 == 5) s = -s;
    }
    if (a == 1) return s;
    if ((a & 3) == 3 && (n8 & 3) == 3) s = -s;
    return s * jacobi_small(N_mod(k, n, a), a);
}

static uint64_t gcd64(uint64_t a, uint64_t b) {
    while (b) {
        uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

/* smallest P >= 1 with Jacobi(P^2+4 | N) != 1, and a common factor of 4P(P^2+4) with N
 * (src/llr.c:80-90) */
int ko_llr_choose_P(uint64_t k, uint64_t n, uint32_t *P, uint64_t *factor) {
    uint32_t p = 1;
    while (jacobi_N((uint64_t)p * p + 4, k, n) == 1)
        if (++p > 1000000) return -1;
    *P = p;
    uint64_t d = 4ull * p * ((uint64_t)p * p + 4);
    uint64_t g = gcd64(d, N_mod(k, n, d));
    *factor = g > 1 ? g : 0;
    return 0;
}

int ko_llr(uint64_t k, uint64_t n, uint32_t L, uint32_t *Pout, uint64_t *factor, uint64_t *res64,
           int *is_prime, double *maxerr) {
    uint32_t P;
    uint64_t f;
    if (n < 3 || !(k & 1) || ko_llr_choose_P(k, n, &P, &f)) return -1;
    if (Pout) *Pout = P;
    if (factor) *factor = f;
    if (f) return 0;
    ko_ctx *c = ko_ctx_new(k, n, L);
    if (!c) return -1;
    size_t nl = c->nlimbs;
    uint64_t *l = calloc(nl, sizeof(uint64_t));
    double *v0 = calloc(c->L, sizeof(double)), *v1 = calloc(c->L, sizeof(double));
    double *cP = calloc(c->L, sizeof(double)), *c2 = calloc(c->L, sizeof(double));
    double *t = calloc(c->L, sizeof(double));
    l[0] = P;
    ko_set_limbs(c, cP, l);
    l[0] = 2;
    ko_set_limbs(c, c2, l);
    /* Lucas ladder for V_k(P, -1): (V_m, V_{m+1}) from m = 0 (src/llr.c:150-184) */
    memcpy(v0, c2, c->L * sizeof(double));
    memcpy(v1, cP, c->L * sizeof(double));
    uint64_t m = 0;
    int top = 63;
    while (top > 0 && !((k >> top) & 1)) top--;
    for (int b = top; b >= 0; b--) {
        int odd = (int)(m & 1);
        memcpy(t, v0, c->L * sizeof(double)); /* V_{2m+1} = V_m V_{m+1} - P Q^m */
        ko_mul(c, t, v1);
        if (odd) ko_add(c, t, cP);
        else ko_sub(c, t, cP);
        if ((k >> b) & 1) { /* (V_{2m+1}, V_{2m+2}), V_{2m+2} = V_{m+1}^2 - 2 Q^{m+1} */
            ko_square(c, v1, 1);
            if (odd) ko_sub(c, v1, c2);
            else ko_add(c, v1, c2);
            memcpy(v0, t, c->L * sizeof(double));
            m = 2 * m + 1;
        } else { /* (V_{2m}, V_{2m+1}), V_{2m} = V_m^2 - 2 Q^m */
            ko_square(c, v0, 1);
            if (odd) ko_add(c, v0, c2);
            else ko_sub(c, v0, c2);
            memcpy(v1, t, c->L * sizeof(double));
            m = 2 * m;
        }
    }
    /* V_{2k} = V_k^2 + 2 (k odd), then V <- V^2 - 2 up to V_{k 2^(n-1)} */
    for (uint64_t i = 0; i + 1 < n; i++) {
        ko_square(c, v0, 1);
        if (i == 0) ko_add(c, v0, c2);
        else ko_sub(c, v0, c2);
    }
    ko_get_limbs(c, v0, l);
    if (res64) *res64 = l[0];
    if (is_prime) *is_prime = big_is_zero(l, nl);
    if (maxerr) *maxerr = c->maxerr;
    free(l);
    free(v0);
    free(v1);
    free(cP);
    free(c2);
    free(t);
    ko_ctx_free(c);
    return 0;
}

/* ---- CPU baseline timing ------------------------------------------------------------------- */

typedef struct {
    const uint64_t *k, *n;
    const uint32_t *L;
    int ntests;
    uint32_t squarings;
    double *us;
    int next;
    pthread_mutex_t mu;
} time_job;

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

static void *time_worker(void *arg) {
    time_job *j = arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int i = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (i >= j->ntests) return NULL;
        ko_ctx *c = ko_ctx_new(j->k[i], j->n[i], j->L[i]);
        if (!c) {
            j->us[i] = -1;
            continue;
        }
        double *x = calloc(c->L, sizeof(double));
        uint64_t *l = calloc(c->nlimbs, sizeof(uint64_t));
        uint64_t s = 0x9E3779B97F4A7C15ull ^ (uint64_t)(i + 1);
        for (size_t q = 0; q + 1 < c->nlimbs; q++) { /* below 2^(64(nlimbs-1)) < N */
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            l[q] = s;
        }
        ko_set_limbs(c, x, l);
        ko_square(c, x, 2);
        double t0 = now_s();
        ko_square(c, x, j->squarings);
        j->us[i] = (now_s() - t0) * 1e6 / j->squarings;
        free(x);
        free(l);
        ko_ctx_free(c);
    }
}

int ko_time_squarings(const uint64_t *k, const uint64_t *n, const uint32_t *L, int ntests,
                      int threads, uint32_t squarings, double *us_per_sq) {
    if (threads < 1) threads = 1;
    if (threads > 1024) threads = 1024;
    time_job j = {k, n, L, ntests, squarings ? squarings : 1, us_per_sq, 0,
                  PTHREAD_MUTEX_INITIALIZER};
    pthread_t th[1024];
    for (int t = 0; t < threads; t++) pthread_create(&th[t], NULL, time_worker, &j);
    for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
    return 0;
}
