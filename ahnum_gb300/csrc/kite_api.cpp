// The kite public API (include/kite.h) on top of the GB300 engine: contexts and numbers, the
// exact host conversions, and the element-wise operations.  Behaviour follows the reference's
// src/ctx.c:223-559 with the arithmetic backend replaced by kc_* calls.
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/kite.h"
#include "../../include/kite_cuda.h"
#include "kite_internal.h"

using kg::Layout;

extern "C" {

kite_ctx *kite_ctx_new(uint64_t k, uint64_t n, int32_t c, const kite_opts *o) {
    if (c != -1 || k == 0 || !(k & 1) || n < 8 || k >= (1ull << 30)) return nullptr;
    const kite_backend b = o ? o->backend : KITE_BACKEND_AUTO;
    if (b != KITE_BACKEND_AUTO && b != KITE_BACKEND_CUDA) return nullptr;  // no CPU backends here
    kite_ctx *ctx = new (std::nothrow) kite_ctx();
    if (!ctx) return nullptr;
    const uint32_t L = o && o->fft_len ? o->fft_len : kg::choose_fft_len(k, n);
    if (!L || !ctx->lay.build(k, n, L)) {
        delete ctx;
        return nullptr;
    }
    const Layout &y = ctx->lay;
    ctx->eng = kc_engine_new(k, n, L, y.bits.data(), y.w.data(), y.oscale.data(), y.top_t, y.top_st,
                             y.top_m, y.sL, -1);
    if (!ctx->eng) {
        delete ctx;
        return nullptr;
    }
    ctx->dig.resize(L);
    return ctx;
}

void kite_ctx_free(kite_ctx *ctx) {
    if (!ctx) return;
    kc_engine_free(ctx->eng);
    delete ctx;
}

uint32_t kite_fft_len(const kite_ctx *ctx) { return ctx->lay.L; }
const char *kite_backend_name(const kite_ctx *ctx) {
    (void)ctx;
    return "cuda";
}

kite_num *kite_num_new(kite_ctx *ctx) {
    kite_num *x = new (std::nothrow) kite_num();
    if (!x) return nullptr;
    x->d = kc_num_alloc(ctx->eng);
    if (!x->d) {
        delete x;
        return nullptr;
    }
    return x;
}

void kite_num_free(kite_ctx *ctx, kite_num *x) {
    if (!x) return;
    kc_num_free(ctx->eng, x->d);
    delete x;
}

void kite_copy(kite_ctx *ctx, kite_num *dst, const kite_num *src) { kc_copy(ctx->eng, dst->d, src->d); }
void kite_square(kite_ctx *ctx, kite_num *x) { kc_square(ctx->eng, x->d, 1); }
void kite_square_n(kite_ctx *ctx, kite_num *x, uint64_t count) { kc_square(ctx->eng, x->d, count); }
void kite_mul(kite_ctx *ctx, kite_num *x, const kite_num *y) { kc_mul(ctx->eng, x->d, y->d); }
void kite_add(kite_ctx *ctx, kite_num *x, const kite_num *y) { kc_add(ctx->eng, x->d, y->d); }
void kite_sub(kite_ctx *ctx, kite_num *x, const kite_num *y) { kc_sub(ctx->eng, x->d, y->d); }

// x*m on the digits (src/ref_fft.c:133-139): exact integer product, carried on the host
void kite_mul_small(kite_ctx *ctx, kite_num *x, int64_t m) {
    int64_t *d = ctx->dig.data();
    if (kc_to_digits(ctx->eng, x->d, d)) return;
    for (uint32_t j = 0; j < ctx->lay.L; j++) d[j] *= m;
    ctx->lay.carry(d);
    kc_from_digits(ctx->eng, x->d, d);
}

double kite_max_roundoff(const kite_ctx *ctx) { return kc_maxerr(ctx->eng); }
void kite_reset_roundoff(kite_ctx *ctx) { kc_reset_maxerr(ctx->eng); }
void kite_set_roundoff_check(kite_ctx *ctx, uint32_t every) { kc_set_roundoff_check(ctx->eng, every); }
size_t kite_limbs(const kite_ctx *ctx) { return ctx->lay.nlimbs; }

void kite_get_limbs(kite_ctx *ctx, const kite_num *x, uint64_t *limbs) {
    int64_t *d = ctx->dig.data();
    if (kc_to_digits(ctx->eng, x->d, d)) {
        std::memset(limbs, 0, ctx->lay.nlimbs * sizeof(uint64_t));
        return;
    }
    ctx->lay.digits_to_limbs(d, limbs);
}

void kite_set_limbs(kite_ctx *ctx, kite_num *x, const uint64_t *limbs) {
    int64_t *d = ctx->dig.data();
    ctx->lay.limbs_to_digits(limbs, d);
    kc_from_digits(ctx->eng, x->d, d);
}

void kite_set_u64(kite_ctx *ctx, kite_num *x, uint64_t v) {
    std::vector<uint64_t> l(ctx->lay.nlimbs, 0);
    l[0] = v;
    kite_set_limbs(ctx, x, l.data());
}

uint64_t kite_res64(kite_ctx *ctx, const kite_num *x) {
    std::vector<uint64_t> l(ctx->lay.nlimbs);
    kite_get_limbs(ctx, x, l.data());
    return l[0];
}

void kite_debug_corrupt(kite_ctx *ctx, kite_num *x) {
    int64_t *d = ctx->dig.data();
    if (kc_to_digits(ctx->eng, x->d, d)) return;
    d[ctx->lay.L / 3] += 1;
    kc_from_digits(ctx->eng, x->d, d);
}

int kite_ctx_error(const kite_ctx *ctx) { return kc_error(ctx->eng); }
int kite_ctx_sync(kite_ctx *ctx) { return kc_sync(ctx->eng); }

}  // extern "C"
