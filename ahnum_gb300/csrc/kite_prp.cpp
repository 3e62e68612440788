// Fermat PRP driver (kite_prp) with the Gerbicz check, on the GPU engine.
//
// Semantics of the reference's src/prp.c:298-583: x_0 = base^k, x_{i+1} = x_i^2, so
// x_n = base^(N+1); the residue is base^(N-1) and N is a PRP iff x_n == base^2.  The Gerbicz
// product d_t = prod x_{jB} obeys d_{t+1} = x_0 * d_t^(2^B); every M blocks it is checked with
// B extra squarings of the saved t, and a mismatch rolls back to the last verified state.
// Round-off above the limit restarts from the verified state at a longer FFT.  The squarings,
// the running product d*x and the check's squarings and product all run on the device; only
// the canonical comparison of the check reads numbers back.
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/kite.h"
#include "kite_internal.h"
#include "persist.h"

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct PrpState {
    kite_ctx *ctx = nullptr;
    kite_num *x = nullptr, *d = nullptr, *x0 = nullptr, *t = nullptr;
    ~PrpState() { reset(); }
    void reset() {
        if (!ctx) return;
        kite_num_free(ctx, x);
        kite_num_free(ctx, d);
        kite_num_free(ctx, x0);
        kite_num_free(ctx, t);
        kite_ctx_free(ctx);
        ctx = nullptr;
        x = d = x0 = t = nullptr;
    }
    bool open(uint64_t k, uint64_t n, const kite_opts &o) {
        reset();
        ctx = kite_ctx_new(k, n, -1, &o);
        if (!ctx) return false;
        kite_set_roundoff_check(ctx, 4);  // sample every 4th operation (src/prp.c:281-283)
        x = kite_num_new(ctx);
        d = kite_num_new(ctx);
        x0 = kite_num_new(ctx);
        t = kite_num_new(ctx);
        return x && d && x0 && t;
    }
};

// x0 = base^k: exact while base^k < N, else square-and-multiply (src/prp.c:298-327)
void power_start(PrpState &s, uint64_t k, uint32_t base, std::vector<uint64_t> &l) {
    kite_ctx *ctx = s.ctx;
    const size_t nl = kite_limbs(ctx);
    kite_set_u64(ctx, s.x0, 1);
    for (int b = 63; b >= 0; b--) {
        if (k >> b == 0) continue;
        kite_square(ctx, s.x0);
        if ((k >> b) & 1) kite_mul_small(ctx, s.x0, base);
    }
    if ((double)k * std::log2((double)base) + 2 < (double)ctx->lay.n) {
        std::fill(l.begin(), l.end(), 0);
        l[0] = 1;
        size_t used = 1;
        for (uint64_t i = 0; i < k; i++) {
            unsigned __int128 c = 0;
            for (size_t j = 0; j < used; j++) {
                c += (unsigned __int128)l[j] * base;
                l[j] = (uint64_t)c;
                c >>= 64;
            }
            if (c && used < nl) l[used++] = (uint64_t)c;
        }
        kite_set_limbs(ctx, s.x0, l.data());
    }
}

struct Pending {
    std::vector<uint32_t> index;
    std::vector<std::vector<uint64_t>> limbs;
    void clear() {
        index.clear();
        limbs.clear();
    }
    void add(kite_ctx *ctx, uint32_t i, const kite_num *x) {
        index.push_back(i);
        limbs.emplace_back(kite_limbs(ctx));
        kite_get_limbs(ctx, x, limbs.back().data());
    }
    int flush(const kite_prp_opts &o) {
        int rc = 0;
        for (size_t i = 0; i < index.size() && !rc; i++)
            rc = o.on_point(o.point_arg, index[i], o.points[index[i]], limbs[i].data());
        clear();
        return rc;
    }
};

bool equal(kite_ctx *ctx, const kite_num *a, const kite_num *b, std::vector<uint64_t> &la,
           std::vector<uint64_t> &lb) {
    kite_get_limbs(ctx, a, la.data());
    kite_get_limbs(ctx, b, lb.data());
    return la == lb && !kite_ctx_error(ctx);
}

}  // namespace

extern "C" int kite_prp_checkpoint_iter(const char *path, uint64_t k, uint64_t n, uint32_t base,
                                        uint64_t *iter) {
    kg::PrpCheckpointHeader h;
    if (!kg::prp_checkpoint_header(path, h) || h.k != k || h.n != n || h.base != base) return -1;
    *iter = h.iter;
    return 0;
}

extern "C" int kite_prp(uint64_t k, uint64_t n, uint32_t base, const kite_prp_opts *opts,
                        kite_prp_result *res) {
    kite_prp_opts o = opts ? *opts : kite_prp_opts{};
    std::memset(res, 0, sizeof *res);
    const double t_start = now_s();
    uint32_t B = o.gerbicz_block;
    if (!B) {
        B = (uint32_t)std::sqrt((double)n);
        B = B < 32 ? 32 : B > 2000 ? 2000 : B;
    }
    const uint32_t M = o.gerbicz_blocks ? o.gerbicz_blocks : (B / 4 > 8 ? B / 4 : 8);
    const double maxround = o.max_roundoff > 0 ? o.max_roundoff : 0.40;
    const double ck_secs = o.checkpoint_secs > 0 ? o.checkpoint_secs : 600;
    const double u_secs = o.unverified_secs > 0 ? o.unverified_secs : 60;

    PrpState s;
    if (!s.open(k, n, o.fft)) return -1;
    const size_t nl = kite_limbs(s.ctx);
    std::vector<uint64_t> la(nl), lb(nl), vx(nl), vd(nl), ux, ud;
    uint64_t vi = 0, ui = 0;
    int rc = 0;
    Pending pend;

    power_start(s, k, base, la);
    kite_get_limbs(s.ctx, s.x0, vx.data());
    vd = vx;
    {
        uint32_t Lv = 0, Lu = 0;
        if (o.checkpoint && kg::prp_checkpoint_read(o.checkpoint, k, n, base, nl, vi, Lv, vx, vd))
            res->resumed = 1;
        if (o.checkpoint_unverified) {
            ux.resize(nl);
            ud.resize(nl);
            if (!kg::prp_checkpoint_read(o.checkpoint_unverified, k, n, base, nl, ui, Lu, ux, ud) || ui <= vi)
                ui = 0;
            else {
                res->resumed = 1;
                if (Lu > Lv) Lv = Lu;
            }
        }
        if (Lv > kite_fft_len(s.ctx)) {  // the saved run had moved to a longer FFT
            kite_opts fo = o.fft;
            fo.fft_len = Lv;
            if (!s.open(k, n, fo)) {
                res->seconds = now_s() - t_start;
                return -1;
            }
            power_start(s, k, base, la);
        }
    }
    const uint64_t full = n / B * B;
    double last_ck = now_s(), last_u = last_ck;
    int consecutive_fail = 0;
    res->resumed_at = ui ? ui : vi;
    uint32_t vp = 0, up = 0;
    if (o.on_point) {
        while (vp < o.npoints && o.points[vp] < vi + (vi > 0)) vp++;
        if (vp < o.npoints && o.points[vp] == 0) {  // x_0 itself, checked by power_start
            kite_set_limbs(s.ctx, s.x, vx.data());
            pend.add(s.ctx, vp++, s.x);
            if (pend.flush(o)) {
                res->seconds = now_s() - t_start;
                return KITE_PRP_POINT_FAILED;
            }
        }
        up = vp;
        while (up < o.npoints && o.points[up] < ui + 1) up++;
    }
    for (;;) {
        const bool from_u = ui > vi;
        kite_set_limbs(s.ctx, s.x, from_u ? ux.data() : vx.data());
        kite_set_limbs(s.ctx, s.d, from_u ? ud.data() : vd.data());
        kite_reset_roundoff(s.ctx);
        const uint64_t start = from_u ? ui : vi;
        uint64_t i = start;
        uint32_t pi = from_u ? up : vp;
        ui = 0;  // an unverified state is used once
        bool failed = false, round_fail = false;
        pend.clear();
        if (o.abort_flag && *o.abort_flag) {
            if (o.checkpoint) kg::prp_checkpoint_write(o.checkpoint, k, n, base, vi, kite_fft_len(s.ctx), vx, vd);
            rc = KITE_PRP_ABORTED;
            break;
        }
        uint64_t check_at = start + (uint64_t)B * M;
        if (check_at > full) check_at = full;
        while (i < check_at) {
            if (o.abort_flag && *o.abort_flag) break;
            // squarings up to the next event (fault injection or proof point) are queued at once
            uint64_t block_end = i + B;
            while (i < block_end) {
                uint64_t stop = block_end;
                if (o.inject_fault_at > i && o.inject_fault_at < stop) stop = o.inject_fault_at;
                if (o.on_point && pi < o.npoints && o.points[pi] > i && o.points[pi] < stop) stop = o.points[pi];
                kite_square_n(s.ctx, s.x, stop - i);
                i = stop;
                if (o.inject_fault_at && i == o.inject_fault_at) {
                    kite_debug_corrupt(s.ctx, s.x);
                    o.inject_fault_at = 0;
                }
                if (o.on_point && pi < o.npoints && o.points[pi] == i) pend.add(s.ctx, pi++, s.x);
            }
            kite_copy(s.ctx, s.t, s.d);
            kite_mul(s.ctx, s.d, s.x);
            if (kite_max_roundoff(s.ctx) > maxround) {
                round_fail = true;
                break;
            }
            if (o.progress) o.progress(o.progress_arg, i, n, kite_max_roundoff(s.ctx));
            if (o.checkpoint_unverified && now_s() - last_u > u_secs && i < check_at) {
                if (!pend.index.empty() && pend.flush(o)) {
                    rc = KITE_PRP_POINT_FAILED;
                    goto out;
                }
                kite_get_limbs(s.ctx, s.x, la.data());
                kite_get_limbs(s.ctx, s.d, lb.data());
                kg::prp_checkpoint_write(o.checkpoint_unverified, k, n, base, i, kite_fft_len(s.ctx), la, lb);
                last_u = now_s();
            }
        }
        {
            const bool stopping = o.abort_flag && *o.abort_flag;
            if (stopping && i == start) continue;  // nothing new; saved at the top of the loop
            if (!round_fail && i > start) {
                // verify d == x0 * t^(2^B), on the device
                kite_square_n(s.ctx, s.t, B);
                kite_mul(s.ctx, s.t, s.x0);
                if (kite_max_roundoff(s.ctx) > maxround) round_fail = true;
                else failed = !equal(s.ctx, s.t, s.d, la, lb);
            }
            const double e = kite_max_roundoff(s.ctx);
            if (e > res->maxerr && e < 1.0) res->maxerr = e;
            if ((round_fail || failed) && o.checkpoint_unverified) std::remove(o.checkpoint_unverified);
            if (round_fail) {
                const uint32_t L = kite_fft_len(s.ctx);
                kite_opts fo = o.fft;
                fo.fft_len = kg::next_fft_len(L + L / 25);
                if (!fo.fft_len || !s.open(k, n, fo)) {
                    rc = -2;
                    goto out;
                }
                power_start(s, k, base, la);
                res->roundoff_retries++;
                continue;
            }
            if (failed) {
                res->gerbicz_errors++;
                if (++consecutive_fail > 5) {
                    rc = -3;
                    goto out;
                }
                continue;
            }
            consecutive_fail = 0;
            kite_get_limbs(s.ctx, s.x, vx.data());
            kite_get_limbs(s.ctx, s.d, vd.data());
            vi = i;
            vp = pi;
            if (!pend.index.empty() && pend.flush(o)) {
                rc = KITE_PRP_POINT_FAILED;
                goto out;
            }
            if (o.checkpoint && (now_s() - last_ck > ck_secs || vi == full || stopping)) {
                kg::prp_checkpoint_write(o.checkpoint, k, n, base, vi, kite_fft_len(s.ctx), vx, vd);
                last_ck = now_s();
            }
            if (stopping) {
                rc = KITE_PRP_ABORTED;
                goto out;
            }
            if (vi >= full) break;
        }
    }
    if (rc) goto out;
    // the tail (< B squarings) is computed twice and compared (src/prp.c:520-551)
    for (int attempt = 0;; attempt++) {
        kite_set_limbs(s.ctx, s.x, vx.data());
        kite_set_limbs(s.ctx, s.t, vx.data());
        uint64_t i = full;
        uint32_t pi = vp;
        pend.clear();
        while (i < n) {
            uint64_t next = n;
            if (o.on_point && pi < o.npoints && o.points[pi] > i && o.points[pi] < next) next = o.points[pi];
            kite_square_n(s.ctx, s.x, next - i);
            kite_square_n(s.ctx, s.t, next - i);
            i = next;
            if (o.on_point && pi < o.npoints && o.points[pi] == i) pend.add(s.ctx, pi++, s.x);
        }
        if (equal(s.ctx, s.x, s.t, la, lb)) {
            if (!pend.index.empty() && pend.flush(o)) {
                rc = KITE_PRP_POINT_FAILED;
                goto out;
            }
            break;
        }
        if (attempt > 5) {
            rc = -3;
            goto out;
        }
        res->gerbicz_errors++;
    }
    {
        // la = x_n = base^(N+1); PRP iff x_n == base^2; residue base^(N-1) = x_n / base^2
        bool is_prp = la[0] == (uint64_t)base * base;
        for (size_t j = 1; j < nl; j++) is_prp &= la[j] == 0;
        if (kg::residue_nm1(la.data(), s.ctx->lay.Nl.data(), nl, base)) rc = -4;
        res->res64 = la[0];
        res->is_prp = is_prp;
    }
    res->fft_len = kite_fft_len(s.ctx);
    {
        const double e = kite_max_roundoff(s.ctx);
        if (e > res->maxerr && e < 1.0) res->maxerr = e;
    }
out:
    res->seconds = now_s() - t_start;
    return rc;
}
