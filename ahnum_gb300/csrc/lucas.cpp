// LLR (Morrison, Q = -1) test of N = k*2^n - 1 (kite_llr, include/kite.h) on the GPU.
//
// What is computed -- the reference's test (src/llr.c:1-13), which is PRST's Morrison test: P is
// the smallest P >= 1 with Jacobi((P^2+4) | N) != 1, and a common factor of 4P(P^2+4) and N is
// reported as a factor; V_k(P, -1) comes from a Lucas ladder, V_2k = V_k^2 + 2 (k odd), and
// n - 2 doublings V <- V^2 - 2 reach V_{k 2^(n-1)}, which is 0 exactly when N is prime (else
// its low word is the RES64).  No Gerbicz check covers the doublings, so a composite verdict is
// confirmed by a second complete run at a longer FFT, and a third run settles a disagreement.
//
// How a run is organised here.  Its anchor -- the value after the ladder, then every 1000
// doublings whose round-off stayed under the limit -- is kept as a device copy.  The doublings
// are kite_square_add_internal calls: the constant is added to the rounded digits inside the
// normaliser, so a step is one squaring and a stretch of them one queued call.  Round-off above
// the limit moves the run to a context at the next length at least 4% longer, where it goes on
// from the anchor (the ladder is redone only if it failed itself).  KITELLR1 checkpoint files
// are written from the anchor.
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/kite.h"
#include "drivers.h"
#include "layout.h"
#include "persist.h"

namespace {

using kd::Number;
using u128 = unsigned __int128;

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); }

// (k*2^n - 1) mod m, for m > 1
uint64_t n_mod(uint64_t k, uint64_t n, uint64_t m) {
    uint64_t p = 1 % m, sq = 2 % m;
    for (uint64_t e = n; e; e >>= 1) {
        if (e & 1) p = mulmod(p, sq, m);
        sq = mulmod(sq, sq, m);
    }
    return (mulmod(k % m, p, m) + m - 1) % m;
}

// Jacobi symbol (a | m) for odd m > 0, by the binary algorithm (reciprocity and the rule for 2).
int jacobi(uint64_t a, uint64_t m) {
    a %= m;
    int sign = 1;
    while (a != 0) {
        const int twos = __builtin_ctzll(a);
        a >>= twos;
        if ((twos & 1) && (m % 8 == 3 || m % 8 == 5)) sign = -sign;
        if (a % 4 == 3 && m % 4 == 3) sign = -sign;
        const uint64_t r = m % a;
        m = a;
        a = r;
    }
    return m == 1 ? sign : 0;
}

uint64_t gcd(uint64_t a, uint64_t b) {
    while (b) {
        const uint64_t r = a % b;
        a = b;
        b = r;
    }
    return a;
}

// Jacobi((P^2 + 4) | N).  For odd n > 0 the symbol (a | n) depends only on n mod 4a, so it is
// (a | N mod 4a): a word-size symbol, with no reciprocity steps on N itself.
int jacobi_of_N(uint64_t a, uint64_t k, uint64_t n) { return jacobi(a, n_mod(k, n, 4 * a)); }

struct Vote {
    uint64_t res64 = 0;
    bool zero = false;
    bool operator==(const Vote &o) const { return res64 == o.res64 && zero == o.zero; }
};

// One complete run: V_{k 2^(n-1)} at a given FFT length, from the run's checkpoint if there is
// one.
class LucasRun {
  public:
    LucasRun(uint64_t k, uint64_t n, uint32_t P, const kite_llr_opts &o, int run, const Vote prev[2],
             kite_llr_result *res)
        : k_(k), n_(n), P_(P), o_(o), run_(run), res_(res) {
        prev_[0] = prev[0].res64;
        prev_[1] = prev[1].res64;
        limit_ = o.max_roundoff > 0 ? o.max_roundoff : 0.40;
        save_every_ = o.checkpoint_secs > 0 ? o.checkpoint_secs : 600;
        total_ = n - 1;
        fault_at_ = o.inject_fault_at && (((o.inject_fault_runs ? o.inject_fault_runs : 1u) >> run) & 1)
                        ? o.inject_fault_at
                        : 0;
        injected_roundoff_ = run == 0 && (o.inject_roundoff_at || o.inject_roundoff_ladder);
    }

    // 0 and the final value's limbs, or an error code
    int go(uint32_t fft_len, std::vector<uint64_t> &out);

  private:
    struct Lane {
        kite_ctx *ctx = nullptr;
        Number v, anchor, cP, c2, s1, s2;
        ~Lane() {
            for (Number *p : {&v, &anchor, &cP, &c2, &s1, &s2}) p->reset();
            kite_ctx_free(ctx);
        }
    };
    bool open(uint32_t fft_len);
    void ladder();
    bool stretch_failed(uint64_t &i);
    void save(uint64_t iter);
    void note(double e) {
        if (e > res_->maxerr && e < 1.0) res_->maxerr = e;
    }

    const uint64_t k_, n_;
    const uint32_t P_;
    const kite_llr_opts &o_;
    const int run_;
    kite_llr_result *res_;
    uint64_t prev_[2];
    double limit_, save_every_;
    uint64_t total_;
    uint64_t fault_at_;
    bool injected_roundoff_;
    std::unique_ptr<Lane> lane_;
};

bool LucasRun::open(uint32_t fft_len) {
    lane_.reset();
    auto lane = std::make_unique<Lane>();
    kite_opts fo = o_.fft;
    if (fft_len) fo.fft_len = fft_len;
    lane->ctx = kite_ctx_new(k_, n_, -1, &fo);
    if (!lane->ctx) return false;
    kite_set_roundoff_check(lane->ctx, 1);  // every step: no other check protects the chain
    for (Number *p : {&lane->v, &lane->anchor, &lane->cP, &lane->c2, &lane->s1, &lane->s2}) {
        *p = Number(lane->ctx);
        if (!*p) return false;
    }
    kite_set_u64(lane->ctx, lane->cP, P_);
    kite_set_u64(lane->ctx, lane->c2, 2);
    lane_ = std::move(lane);
    return true;
}

// V_k(P, -1) into v.  The ladder keeps the pair (V_m, V_{m+1}) and reads the bits of k from the
// top: V_{2m} = V_m^2 - 2 Q^m, V_{2m+1} = V_m V_{m+1} - P Q^m, V_{2m+2} = V_{m+1}^2 - 2 Q^{m+1},
// with Q = -1 (the reference's lucas_vk, src/llr.c:150-184).  V_2k = V_k^2 + 2 follows as the
// first doubling.
void LucasRun::ladder() {
    kite_ctx *ctx = lane_->ctx;
    kite_num *lo = lane_->v, *hi = lane_->s1, *mid = lane_->s2;
    kite_set_u64(ctx, lo, 2);        // V_0
    kite_copy(ctx, hi, lane_->cP);   // V_1
    int bit = 63;
    while (bit > 0 && !((k_ >> bit) & 1)) bit--;
    bool m_odd = false;  // m = 0
    for (; bit >= 0; bit--) {
        // mid = V_{2m+1} = lo * hi - P Q^m
        kite_copy(ctx, mid, lo);
        kite_mul(ctx, mid, hi);
        (m_odd ? kite_add : kite_sub)(ctx, mid, lane_->cP);
        if ((k_ >> bit) & 1) {
            // m <- 2m+1: (V_{2m+1}, V_{2m+2}), V_{2m+2} = hi^2 - 2 Q^{m+1}
            kite_square(ctx, hi);
            (m_odd ? kite_sub : kite_add)(ctx, hi, lane_->c2);
            std::swap(lo, mid);
            m_odd = true;
        } else {
            // m <- 2m: (V_2m, V_{2m+1}), V_2m = lo^2 - 2 Q^m
            kite_square(ctx, lo);
            (m_odd ? kite_add : kite_sub)(ctx, lo, lane_->c2);
            std::swap(hi, mid);
            m_odd = false;
        }
    }
    if (lo != lane_->v.get()) kite_copy(ctx, lane_->v, lo);
}

void LucasRun::save(uint64_t iter) {
    kg::LlrCheckpointHeader h{};
    h.k = k_;
    h.n = n_;
    h.P = P_;
    h.iter = iter;
    h.fft_len = kite_fft_len(lane_->ctx);
    h.run = (uint64_t)run_;
    h.prev[0] = prev_[0];
    h.prev[1] = prev_[1];
    kg::llr_checkpoint_write(o_.checkpoint, h, kd::limbs_of(lane_->ctx, lane_->anchor));
}

int LucasRun::go(uint32_t fft_len, std::vector<uint64_t> &out) {
    bool have_anchor = false;  // an anchor from an earlier attempt, carried as limbs
    uint64_t anchor_iter = 0;
    std::vector<uint64_t> carried;
    for (int attempt = 0;; attempt++) {
        if (!open(fft_len)) return -1;
        kite_ctx *ctx = lane_->ctx;
        const size_t nl = kite_limbs(ctx);
        bool failed = false;
        if (have_anchor) {
            kite_set_limbs(ctx, lane_->anchor, carried.data());
            // the reference re-reads the checkpoint it wrote before the retry
            if (o_.checkpoint && !res_->resumed) {
                res_->resumed = 1;
                res_->resumed_at = anchor_iter;
            }
        } else {
            kg::LlrCheckpointHeader h{};
            std::vector<uint64_t> saved;
            if (o_.checkpoint && kg::llr_checkpoint_read(o_.checkpoint, nl, h, saved) && h.k == k_ && h.n == n_ &&
                h.P == P_ && h.run == (uint64_t)run_ && h.iter <= total_) {
                anchor_iter = h.iter;
                if (!res_->resumed) {
                    res_->resumed = 1;
                    res_->resumed_at = anchor_iter;
                }
                kite_set_limbs(ctx, lane_->anchor, saved.data());
                have_anchor = true;
            } else {
                // the ladder's round-off is checked like a stretch's: a bad V_k would spoil every
                // doubling after it
                kite_reset_roundoff(ctx);
                ladder();
                const double e = kite_max_roundoff(ctx);
                note(e);
                if (e > limit_ || (injected_roundoff_ && o_.inject_roundoff_ladder)) {
                    injected_roundoff_ = false;
                    failed = true;
                } else {
                    kite_copy(ctx, lane_->anchor, lane_->v);
                    anchor_iter = 0;
                    have_anchor = true;
                }
            }
        }
        if (!failed) {
            kite_copy(ctx, lane_->v, lane_->anchor);
            double last_save = kd::clock_s();
            uint64_t i = anchor_iter;
            while (i < total_) {
                if (stretch_failed(i)) {
                    failed = true;
                    break;
                }
                kite_copy(ctx, lane_->anchor, lane_->v);
                anchor_iter = i;
                if (o_.progress) o_.progress(o_.progress_arg, i, total_, kite_max_roundoff(ctx));
                const bool stop = o_.abort_flag && *o_.abort_flag;
                if (o_.checkpoint && (stop || kd::clock_s() - last_save > save_every_)) {
                    save(anchor_iter);
                    last_save = kd::clock_s();
                }
                if (stop) return KITE_LLR_ABORTED;
            }
            if (!failed) {
                out = kd::limbs_of(ctx, lane_->anchor);
                res_->fft_len = kite_fft_len(ctx);
                return 0;
            }
        }
        // round-off above the limit: on to a longer FFT, from the anchor (or the ladder again)
        const uint32_t L = kite_fft_len(ctx);
        if (have_anchor) {
            carried = kd::limbs_of(ctx, lane_->anchor);
            if (o_.checkpoint) save(anchor_iter);
        }
        fft_len = kg::next_fft_len(L + L / 25);
        res_->roundoff_retries++;
        if (!fft_len || attempt > 8) return -2;
    }
}

// Up to 1000 doublings from i (V_2k = V_k^2 + 2 first, then V <- V^2 - 2), split only at an
// injected fault; true when the stretch's round-off is above the limit.
bool LucasRun::stretch_failed(uint64_t &i) {
    kite_ctx *ctx = lane_->ctx;
    kite_reset_roundoff(ctx);
    const uint64_t end = std::min<uint64_t>(i + 1000, total_);
    while (i < end) {
        const int64_t c = i == 0 ? 2 : -2;
        uint64_t to = i == 0 ? 1 : end;
        if (fault_at_ > i && fault_at_ < to) to = fault_at_;
        kite_square_add_internal(ctx, lane_->v, to - i, c);
        i = to;
        if (fault_at_ && i == fault_at_) {
            kite_debug_corrupt(ctx, lane_->v);  // testing hook: once per run
            fault_at_ = 0;
        }
    }
    const double e = kite_max_roundoff(ctx);
    note(e);
    if (e > limit_ || (injected_roundoff_ && o_.inject_roundoff_at && end >= o_.inject_roundoff_at)) {
        injected_roundoff_ = false;
        return true;
    }
    return false;
}

}  // namespace

extern "C" int kite_llr_choose_P(uint64_t k, uint64_t n, uint32_t *P, uint64_t *factor) {
    uint32_t p = 1;
    while (jacobi_of_N((uint64_t)p * p + 4, k, n) == 1)
        if (++p > 1000000) return -1;
    *P = p;
    const uint64_t d = 4ull * p * ((uint64_t)p * p + 4);
    const uint64_t g = gcd(d, n_mod(k, n, d));
    *factor = g > 1 ? g : 0;
    return 0;
}

extern "C" int kite_llr_checkpoint_iter(const char *path, uint64_t k, uint64_t n, uint64_t *iter, int *run) {
    kg::LlrCheckpointHeader h;
    if (!kg::llr_checkpoint_header(path, h) || h.k != k || h.n != n) return -1;
    *iter = h.iter;
    if (run) *run = (int)h.run;
    return 0;
}

extern "C" int kite_llr(uint64_t k, uint64_t n, const kite_llr_opts *opts, kite_llr_result *res) {
    std::memset(res, 0, sizeof *res);
    const double t0 = kd::clock_s();
    const kite_llr_opts o = opts ? *opts : kite_llr_opts{};
    if (n < 3 || !(k & 1)) return -1;
    uint32_t P = 0;
    uint64_t factor = 0;
    if (kite_llr_choose_P(k, n, &P, &factor)) return -1;
    res->P = P;
    if (factor) {
        res->factor = factor;
        res->seconds = kd::clock_s() - t0;
        return 0;
    }
    size_t nl;
    uint32_t first_len;
    {
        kite_ctx *probe = kite_ctx_new(k, n, -1, &o.fft);
        if (!probe) return -1;
        nl = kite_limbs(probe);
        first_len = kite_fft_len(probe);
        kite_ctx_free(probe);
    }
    // Runs 0, 1, 2 vote by RES64 and zero-ness: run 0 decides a prime; a non-zero run 0 needs
    // run 1 (the next length) to agree; otherwise run 2 (the length after) sides with one of
    // them.  A checkpoint says which run was under way and what the earlier ones gave.
    Vote votes[3];
    int run = 0;
    uint32_t L = 0;
    {
        kg::LlrCheckpointHeader h{};
        std::vector<uint64_t> ignored;
        if (o.checkpoint && kg::llr_checkpoint_read(o.checkpoint, nl, h, ignored) && h.k == k && h.n == n &&
            h.P == P && h.run < 3) {
            run = (int)h.run;
            for (int r = 0; r < run && r < 2; r++) {
                votes[r].res64 = h.prev[r];
                votes[r].zero = h.prev[r] == 0;  // a non-zero value with RES64 0 has probability 2^-64
            }
            if (run > 0) L = (uint32_t)h.fft_len;
        }
    }
    int rc = 0, decided = -1;
    std::vector<uint64_t> out;
    for (; run < 3 && decided < 0 && rc == 0; run++) {
        if (run > 0) {
            res->confirm_runs = (uint32_t)run;
            if (o.on_confirm) o.on_confirm(o.progress_arg, run);
        }
        {
            LucasRun r(k, n, P, o, run, votes, res);
            rc = r.go(L, out);
        }
        if (rc) break;
        votes[run].res64 = out[0];
        votes[run].zero = kd::limbs_equal_word(out, 0);
        if (run == 0 && votes[0].zero) decided = 0;
        else if (run == 1 && votes[1] == votes[0]) decided = 0;
        else if (run == 2) decided = votes[2] == votes[1] ? 1 : votes[2] == votes[0] ? 0 : -2;
        if (decided == -2) rc = -3;  // three different answers
        if (decided != -1) break;
        L = kg::next_fft_len((res->fft_len ? res->fft_len : first_len) + 1);
        if (!L) rc = -2;
    }
    if (rc == 0 && decided >= 0) {
        res->is_prime = votes[decided].zero;
        res->res64 = votes[decided].res64;
    }
    if (o.checkpoint && rc != KITE_LLR_ABORTED) std::remove(o.checkpoint);
    res->seconds = kd::clock_s() - t0;
    return rc;
}
