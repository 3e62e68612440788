// The kite public API (include/kite.h) on top of the GB300 engines: contexts and numbers, the
// exact host conversions, and the element-wise operations.  Behaviour follows the reference's
// src/ctx.c:223-559 with the arithmetic backend replaced by kc_* calls (the FP64 IBDWT engine)
// or kn_* calls (the integer-NTT engine, KITE_BACKEND_CUDA_NTT).
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/kite.h"
#include "../../include/kite_cuda.h"
#include "../../include/kite_ntt.h"
#include "kite_internal.h"

using kg::Layout;

namespace {

double *fp(const kite_num *x) { return static_cast<double *>(x->d); }
uint64_t *wd(const kite_num *x) { return static_cast<uint64_t *>(x->d); }

// NTT numbers: exact host arithmetic on balanced digits (the Layout's carry and fold), for the
// operations the drivers use a handful of times per test (add, sub, mul_small, corrupt)
template <typename F>
void ntt_digit_op(kite_ctx *ctx, kite_num *x, F &&f) {
    const Layout &y = ctx->lay;
    std::vector<uint64_t> l(y.nlimbs);
    if (kn_get_limbs(ctx->ntt, wd(x), l.data())) return;
    int64_t *d = ctx->dig.data();
    y.limbs_to_digits(l.data(), d);
    f(d);
    y.carry(d);
    y.digits_to_limbs(d, l.data());
    kn_set_limbs(ctx->ntt, wd(x), l.data());
}

}  // namespace

int kite_square_add_internal(kite_ctx *ctx, kite_num *x, uint64_t count, int64_t c) {
    return ctx->ntt ? kn_square_add(ctx->ntt, wd(x), count, c) : kc_square_add(ctx->eng, fp(x), count, c);
}

int kite_equal_internal(kite_ctx *ctx, const kite_num *a, const kite_num *b) {
    if (!ctx->ntt) return kc_equal(ctx->eng, fp(a), fp(b));
    std::vector<uint64_t> la(ctx->lay.nlimbs), lb(ctx->lay.nlimbs);
    const int rc = kn_get_limbs(ctx->ntt, wd(a), la.data());
    if (rc) return rc;
    const int rc2 = kn_get_limbs(ctx->ntt, wd(b), lb.data());
    if (rc2) return rc2;
    return la == lb ? 1 : 0;
}

extern "C" {

kite_ctx *kite_ctx_new(uint64_t k, uint64_t n, int32_t c, const kite_opts *o) {
    if (c != -1 || k == 0 || !(k & 1) || n < 8 || k >= (1ull << 30)) return nullptr;
    const kite_backend b = o ? o->backend : KITE_BACKEND_AUTO;
    if (b != KITE_BACKEND_AUTO && b != KITE_BACKEND_CUDA && b != KITE_BACKEND_CUDA_NTT)
        return nullptr;  // no CPU backends here
    kite_ctx *ctx = new (std::nothrow) kite_ctx();
    if (!ctx) return nullptr;
    const bool ntt = b == KITE_BACKEND_CUDA_NTT;
    // the NTT engine sizes its own transform; the digit layout only serves host conversions
    const uint32_t L = o && o->fft_len && !ntt ? o->fft_len : kg::choose_fft_len(k, n);
    if (!L || !ctx->lay.build(k, n, L)) {
        delete ctx;
        return nullptr;
    }
    const Layout &y = ctx->lay;
    if (ntt)
        ctx->ntt = kn_engine_new(k, n, -1);
    else
        ctx->eng = kc_engine_new(k, n, L, y.bits.data(), y.w.data(), y.oscale.data(), y.top_t, y.top_st,
                                 y.top_m, y.sL, -1);
    if (!ctx->eng && !ctx->ntt) {
        delete ctx;
        return nullptr;
    }
    ctx->dig.resize(L);
    return ctx;
}

void kite_ctx_free(kite_ctx *ctx) {
    if (!ctx) return;
    kc_engine_free(ctx->eng);
    kn_engine_free(ctx->ntt);
    delete ctx;
}

uint32_t kite_fft_len(const kite_ctx *ctx) { return ctx->ntt ? kn_transform_len(ctx->ntt) : ctx->lay.L; }
const char *kite_backend_name(const kite_ctx *ctx) { return ctx->ntt ? "cuda-ntt" : "cuda"; }

kite_num *kite_num_new(kite_ctx *ctx) {
    kite_num *x = new (std::nothrow) kite_num();
    if (!x) return nullptr;
    x->d = ctx->ntt ? (void *)kn_num_alloc(ctx->ntt) : (void *)kc_num_alloc(ctx->eng);
    if (!x->d) {
        delete x;
        return nullptr;
    }
    return x;
}

void kite_num_free(kite_ctx *ctx, kite_num *x) {
    if (!x) return;
    if (ctx->ntt)
        kn_num_free(ctx->ntt, wd(x));
    else
        kc_num_free(ctx->eng, fp(x));
    delete x;
}

void kite_copy(kite_ctx *ctx, kite_num *dst, const kite_num *src) {
    if (ctx->ntt)
        kn_copy(ctx->ntt, wd(dst), wd(src));
    else
        kc_copy(ctx->eng, fp(dst), fp(src));
}

void kite_square(kite_ctx *ctx, kite_num *x) { kite_square_n(ctx, x, 1); }

void kite_square_n(kite_ctx *ctx, kite_num *x, uint64_t count) {
    if (ctx->ntt)
        kn_square(ctx->ntt, wd(x), count);
    else
        kc_square(ctx->eng, fp(x), count);
}

void kite_mul(kite_ctx *ctx, kite_num *x, const kite_num *y) {
    if (ctx->ntt)
        kn_mul(ctx->ntt, wd(x), wd(y));
    else
        kc_mul(ctx->eng, fp(x), fp(y));
}

void kite_add(kite_ctx *ctx, kite_num *x, const kite_num *y) {
    if (!ctx->ntt) {
        kc_add(ctx->eng, fp(x), fp(y));
        return;
    }
    std::vector<int64_t> dy(ctx->lay.L);
    std::vector<uint64_t> l(ctx->lay.nlimbs);
    if (kn_get_limbs(ctx->ntt, wd(y), l.data())) return;
    ctx->lay.limbs_to_digits(l.data(), dy.data());
    ntt_digit_op(ctx, x, [&](int64_t *d) {
        for (uint32_t j = 0; j < ctx->lay.L; j++) d[j] += dy[j];
    });
}

void kite_sub(kite_ctx *ctx, kite_num *x, const kite_num *y) {
    if (!ctx->ntt) {
        kc_sub(ctx->eng, fp(x), fp(y));
        return;
    }
    std::vector<int64_t> dy(ctx->lay.L);
    std::vector<uint64_t> l(ctx->lay.nlimbs);
    if (kn_get_limbs(ctx->ntt, wd(y), l.data())) return;
    ctx->lay.limbs_to_digits(l.data(), dy.data());
    ntt_digit_op(ctx, x, [&](int64_t *d) {
        for (uint32_t j = 0; j < ctx->lay.L; j++) d[j] -= dy[j];
    });
}

// x*m on the digits (src/ref_fft.c:133-139): exact integer product, carried on the host
void kite_mul_small(kite_ctx *ctx, kite_num *x, int64_t m) {
    if (ctx->ntt) {
        ntt_digit_op(ctx, x, [&](int64_t *d) {
            for (uint32_t j = 0; j < ctx->lay.L; j++) d[j] *= m;
        });
        return;
    }
    int64_t *d = ctx->dig.data();
    if (kc_to_digits(ctx->eng, fp(x), d)) return;
    for (uint32_t j = 0; j < ctx->lay.L; j++) d[j] *= m;
    ctx->lay.carry(d);
    kc_from_digits(ctx->eng, fp(x), d);
}

// The NTT engine is exact: no round-off to report.
double kite_max_roundoff(const kite_ctx *ctx) { return ctx->ntt ? 0.0 : kc_maxerr(ctx->eng); }
void kite_reset_roundoff(kite_ctx *ctx) {
    if (!ctx->ntt) kc_reset_maxerr(ctx->eng);
}
void kite_set_roundoff_check(kite_ctx *ctx, uint32_t every) {
    if (!ctx->ntt) kc_set_roundoff_check(ctx->eng, every);
}
size_t kite_limbs(const kite_ctx *ctx) { return ctx->lay.nlimbs; }

void kite_get_limbs(kite_ctx *ctx, const kite_num *x, uint64_t *limbs) {
    if (ctx->ntt) {
        if (kn_get_limbs(ctx->ntt, wd(x), limbs)) std::memset(limbs, 0, ctx->lay.nlimbs * sizeof(uint64_t));
        return;
    }
    int64_t *d = ctx->dig.data();
    if (kc_to_digits(ctx->eng, fp(x), d)) {
        std::memset(limbs, 0, ctx->lay.nlimbs * sizeof(uint64_t));
        return;
    }
    ctx->lay.digits_to_limbs(d, limbs);
}

void kite_set_limbs(kite_ctx *ctx, kite_num *x, const uint64_t *limbs) {
    if (ctx->ntt) {
        kn_set_limbs(ctx->ntt, wd(x), limbs);
        return;
    }
    int64_t *d = ctx->dig.data();
    ctx->lay.limbs_to_digits(limbs, d);
    kc_from_digits(ctx->eng, fp(x), d);
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

// +1 on digit L/3 (src/prp.c:28-34): a valid encoding of a wrong value, on either engine
void kite_debug_corrupt(kite_ctx *ctx, kite_num *x) {
    if (ctx->ntt) {
        ntt_digit_op(ctx, x, [&](int64_t *d) { d[ctx->lay.L / 3] += 1; });
        return;
    }
    int64_t *d = ctx->dig.data();
    if (kc_to_digits(ctx->eng, fp(x), d)) return;
    d[ctx->lay.L / 3] += 1;
    kc_from_digits(ctx->eng, fp(x), d);
}

int kite_ctx_error(const kite_ctx *ctx) { return ctx->ntt ? kn_error(ctx->ntt) : kc_error(ctx->eng); }
int kite_ctx_sync(kite_ctx *ctx) { return ctx->ntt ? kn_sync(ctx->ntt) : kc_sync(ctx->eng); }

}  // extern "C"
