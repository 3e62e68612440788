// LLR (Morrison, Q = -1) driver (kite_llr) on the GPU engine.
//
// Semantics of the reference's src/llr.c:29-534, which computes the test as PRST does: P is the
// smallest P >= 1 with Jacobi(P^2+4 | N) != 1 (a common factor of 4P(P^2+4) and N is reported);
// V_k(P, -1) comes from a Lucas ladder, V_{2k} = V_k^2 + 2 (k odd), then n-2 steps V <- V^2 - 2
// give V_{k 2^(n-1)}; N is prime iff that is 0, else RES64 is its low word.  Round-off is
// checked every step; a step over the limit redoes the run from its last verified state at a
// longer FFT; a composite result is confirmed by a second run at the next length, and a third
// decides if they disagree.
//
// The doubling V <- V^2 - 2 runs entirely on the device: the -2 is added to the rounded digits
// inside the normaliser (kc_square_add; the NTT engine adds it in its reduction), so a step is
// one squaring with no extra pass.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/kite.h"
#include "../../include/kite_cuda.h"
#include "kite_internal.h"
#include "persist.h"

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((unsigned __int128)a * b % m); }

uint64_t n_mod(uint64_t k, uint64_t n, uint64_t m) {  // (k 2^n - 1) mod m
    uint64_t r = 1 % m, b = 2 % m;
    for (uint64_t e = n; e; e >>= 1, b = mulmod(b, b, m))
        if (e & 1) r = mulmod(r, b, m);
    return (mulmod(k % m, r, m) + m - 1 % m) % m;
}

int jacobi(uint64_t a, uint64_t m) {  // m odd
    int s = 1;
    a %= m;
    while (a) {
        while (!(a & 1)) {
            a >>= 1;
            if ((m & 7) == 3 || (m & 7) == 5) s = -s;
        }
        std::swap(a, m);
        if ((a & 3) == 3 && (m & 3) == 3) s = -s;
        a %= m;
    }
    return m == 1 ? s : 0;
}

int jacobi_N(uint64_t a, uint64_t k, uint64_t n) {
    int s = 1;
    const uint64_t n8 = n_mod(k, n, 8);
    while (a && !(a & 1)) {
        a >>= 1;
        if (n8 == 3 || n8 == 5) s = -s;
    }
    if (a == 1) return s;
    if ((a & 3) == 3 && (n8 & 3) == 3) s = -s;
    return s * jacobi(n_mod(k, n, a), a);
}

uint64_t gcd(uint64_t a, uint64_t b) {
    while (b) {
        uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// V_k(P, -1) into x by the Lucas ladder on the bits of k (src/llr.c:150-184)
void lucas_vk(kite_ctx *ctx, uint64_t k, kite_num *x, kite_num *v1, kite_num *t, kite_num *cP, kite_num *c2) {
    kite_set_u64(ctx, x, 2);
    kite_copy(ctx, v1, cP);
    uint64_t m = 0;
    int top = 63;
    while (top > 0 && !((k >> top) & 1)) top--;
    for (int b = top; b >= 0; b--) {
        const bool odd = m & 1;  // Q^m = -1 when m is odd
        kite_copy(ctx, t, x);    // V_{2m+1} = V_m V_{m+1} - P Q^m
        kite_mul(ctx, t, v1);
        if (odd) kite_add(ctx, t, cP);
        else kite_sub(ctx, t, cP);
        if ((k >> b) & 1) {  // (V_{2m+1}, V_{2m+2}); V_{2m+2} = V_{m+1}^2 - 2 Q^{m+1}
            kite_square(ctx, v1);
            if (odd) kite_sub(ctx, v1, c2);
            else kite_add(ctx, v1, c2);
            kite_copy(ctx, x, t);
            m = 2 * m + 1;
        } else {  // (V_{2m}, V_{2m+1}); V_{2m} = V_m^2 - 2 Q^m
            kite_square(ctx, x);
            if (odd) kite_add(ctx, x, c2);
            else kite_sub(ctx, x, c2);
            kite_copy(ctx, v1, t);
            m = 2 * m;
        }
    }
}

bool all_zero(const std::vector<uint64_t> &l) {
    for (uint64_t v : l)
        if (v) return false;
    return true;
}

// One complete run from its checkpoint (if any) to V_{k 2^(n-1)}; 0 and the value in `out`.
int llr_run(uint64_t k, uint64_t n, uint32_t P, const kite_llr_opts &o, uint32_t fft_len, int run,
            const uint64_t prev[2], std::vector<uint64_t> &out, kite_llr_result *res) {
    kite_opts fo = o.fft;
    if (fft_len) fo.fft_len = fft_len;
    const double maxround = o.max_roundoff > 0 ? o.max_roundoff : 0.40;
    const double ck_secs = o.checkpoint_secs > 0 ? o.checkpoint_secs : 600;
    const uint64_t total = n - 1;  // doublings
    bool fault_due = o.inject_fault_at && (((o.inject_fault_runs ? o.inject_fault_runs : 1u) >> run) & 1);
    bool roundoff_due = run == 0 && (o.inject_roundoff_at || o.inject_roundoff_ladder);
    for (int attempt = 0;; attempt++) {
        kite_ctx *ctx = kite_ctx_new(k, n, -1, &fo);
        if (!ctx) return -1;
        kite_set_roundoff_check(ctx, 1);
        const size_t nl = kite_limbs(ctx);
        std::vector<uint64_t> vx(nl);
        kite_num *x = kite_num_new(ctx), *v1 = kite_num_new(ctx), *t = kite_num_new(ctx);
        kite_num *cP = kite_num_new(ctx), *c2 = kite_num_new(ctx);
        kite_set_u64(ctx, cP, P);
        kite_set_u64(ctx, c2, 2);
        uint64_t vi = 0;
        int rc = 0;
        bool round_fail = false, have_state = false;
        kg::LlrCheckpointHeader h{};
        std::vector<uint64_t> cx;
        if (o.checkpoint && kg::llr_checkpoint_read(o.checkpoint, nl, h, cx) && h.k == k && h.n == n &&
            h.P == P && h.run == (uint64_t)run && h.iter <= total) {
            vi = h.iter;
            vx = cx;
            if (!res->resumed) {
                res->resumed = 1;
                res->resumed_at = vi;
            }
            kite_set_limbs(ctx, x, vx.data());
            have_state = true;
        } else {
            kite_reset_roundoff(ctx);
            lucas_vk(ctx, k, x, v1, t, cP, c2);
            const double e = kite_max_roundoff(ctx);
            if (e > res->maxerr && e < 1.0) res->maxerr = e;
            if (e > maxround || (roundoff_due && o.inject_roundoff_ladder)) {
                roundoff_due = false;
                round_fail = true;
            } else {
                kite_get_limbs(ctx, x, vx.data());
                have_state = true;
            }
        }
        double last_ck = now_s();
        uint64_t i = vi;
        const uint64_t B = 1000;  // doublings between verified in-memory states
        while (!round_fail && i < total) {
            kite_reset_roundoff(ctx);
            const uint64_t stop = i + B < total ? i + B : total;
            while (i < stop) {
                if (i == 0) {  // V_{2k} = V_k^2 + 2
                    kite_square_add_internal(ctx, x, 1, 2);
                    i++;
                    continue;
                }
                uint64_t upto = stop;
                if (fault_due && o.inject_fault_at > i && o.inject_fault_at < upto) upto = o.inject_fault_at;
                kite_square_add_internal(ctx, x, upto - i, -2);
                i = upto;
                if (fault_due && i == o.inject_fault_at) {
                    kite_debug_corrupt(ctx, x);
                    fault_due = false;
                }
            }
            const double e = kite_max_roundoff(ctx);
            if (e > res->maxerr && e < 1.0) res->maxerr = e;
            if (e > maxround || (roundoff_due && o.inject_roundoff_at && stop >= o.inject_roundoff_at)) {
                roundoff_due = false;
                round_fail = true;
                break;
            }
            kite_get_limbs(ctx, x, vx.data());
            vi = i;
            if (o.progress) o.progress(o.progress_arg, vi, total, e);
            const bool stop_now = o.abort_flag && *o.abort_flag;
            if (o.checkpoint && (stop_now || now_s() - last_ck > ck_secs)) {
                kg::LlrCheckpointHeader w{};
                w.k = k;
                w.n = n;
                w.P = P;
                w.iter = vi;
                w.fft_len = kite_fft_len(ctx);
                w.run = (uint64_t)run;
                w.prev[0] = prev[0];
                w.prev[1] = prev[1];
                kg::llr_checkpoint_write(o.checkpoint, w, vx);
                last_ck = now_s();
            }
            if (stop_now) {
                rc = KITE_LLR_ABORTED;
                break;
            }
        }
        const uint32_t L = kite_fft_len(ctx);
        if (!round_fail && rc == 0) {
            out = vx;
            res->fft_len = L;
        }
        kite_num_free(ctx, x);
        kite_num_free(ctx, v1);
        kite_num_free(ctx, t);
        kite_num_free(ctx, cP);
        kite_num_free(ctx, c2);
        kite_ctx_free(ctx);
        if (!round_fail) return rc;
        if (o.checkpoint && have_state) {
            kg::LlrCheckpointHeader w{};
            w.k = k;
            w.n = n;
            w.P = P;
            w.iter = vi;
            w.fft_len = L;
            w.run = (uint64_t)run;
            w.prev[0] = prev[0];
            w.prev[1] = prev[1];
            kg::llr_checkpoint_write(o.checkpoint, w, vx);
        }
        fo.fft_len = kg::next_fft_len(L + L / 25);
        res->roundoff_retries++;
        if (!fo.fft_len || attempt > 8) return -2;
    }
}

}  // namespace

extern "C" int kite_llr_choose_P(uint64_t k, uint64_t n, uint32_t *P, uint64_t *factor) {
    uint32_t p = 1;
    while (jacobi_N((uint64_t)p * p + 4, k, n) == 1)
        if (++p > 1000000) return -1;
    *P = p;
    const uint64_t d = 4ull * p * ((uint64_t)p * p + 4);
    const uint64_t g = gcd(d, n_mod(k, n, d));
    *factor = g > 1 ? g : 0;
    return 0;
}

extern "C" int kite_llr_checkpoint_iter(const char *path, uint64_t k, uint64_t n, uint64_t *iter, int *run) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return -1;
    kg::LlrCheckpointHeader h;
    bool ok = std::fread(&h, sizeof h, 1, f) == 1 && !std::memcmp(h.magic, "KITELLR1", 8) && h.k == k && h.n == n;
    std::fclose(f);
    if (!ok) return -1;
    *iter = h.iter;
    if (run) *run = (int)h.run;
    return 0;
}

extern "C" int kite_llr(uint64_t k, uint64_t n, const kite_llr_opts *opts, kite_llr_result *res) {
    kite_llr_opts o = opts ? *opts : kite_llr_opts{};
    std::memset(res, 0, sizeof *res);
    const double t0 = now_s();
    if (n < 3 || !(k & 1)) return -1;
    uint32_t P;
    uint64_t factor;
    if (kite_llr_choose_P(k, n, &P, &factor)) return -1;
    res->P = P;
    if (factor) {
        res->factor = factor;
        res->seconds = now_s() - t0;
        return 0;
    }
    kite_ctx *probe = kite_ctx_new(k, n, -1, &o.fft);
    if (!probe) return -1;
    const size_t nl = kite_limbs(probe);
    const uint32_t L0 = kite_fft_len(probe);
    kite_ctx_free(probe);

    uint64_t res64[3] = {0, 0, 0};
    bool zero[3] = {false, false, false};
    int rc = 0, run = 0, final_run = 0;
    uint32_t L = 0;
    {
        kg::LlrCheckpointHeader h;
        std::vector<uint64_t> tmp;
        if (o.checkpoint && kg::llr_checkpoint_read(o.checkpoint, nl, h, tmp) && h.k == k && h.n == n &&
            h.P == P && h.run < 3) {
            run = (int)h.run;
            res64[0] = h.prev[0];
            res64[1] = h.prev[1];
            zero[0] = run > 0 && res64[0] == 0;
            zero[1] = run > 1 && res64[1] == 0;
            if (run > 0) L = (uint32_t)h.fft_len;
        }
    }
    std::vector<uint64_t> out(nl);
    auto agree = [&](int a, int b) { return res64[a] == res64[b] && zero[a] == zero[b]; };
    for (; run < 3; run++) {
        if (run > 0) {
            res->confirm_runs = (uint32_t)run;
            if (o.on_confirm) o.on_confirm(o.progress_arg, run);
        }
        rc = llr_run(k, n, P, o, L, run, res64, out, res);
        if (rc) break;
        res64[run] = out[0];
        zero[run] = all_zero(out);
        if (run == 0 && zero[0]) break;  // prime
        if (run == 1 && agree(1, 0)) break;
        if (run == 2) {
            if (agree(2, 1)) final_run = 1;
            else if (agree(2, 0)) final_run = 0;
            else rc = -3;
            break;
        }
        const uint32_t base_len = res->fft_len ? res->fft_len : L0;
        L = kg::next_fft_len(base_len + 1);
        if (!L) {
            rc = -2;
            break;
        }
    }
    if (rc == 0) {
        res->is_prime = zero[final_run];
        res->res64 = res64[final_run];
    }
    if (o.checkpoint && rc != KITE_LLR_ABORTED) std::remove(o.checkpoint);
    res->seconds = now_s() - t0;
    return rc;
}
