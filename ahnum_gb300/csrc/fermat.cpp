// Fermat PRP test of N = k*2^n - 1 (kite_prp, include/kite.h), Gerbicz-checked, on the GPU.
//
// The walk x_{i+1} = x_i^2 starts at x_0 = base^k and reaches x_n = base^(N+1): N is a probable
// prime when x_n == base^2, and the residue reported is base^(N-1) = x_n / base^2 -- the
// semantics of the reference's driver (src/prp.c:1-11, 329-583), whose options, results, error
// codes and checkpoint files this one keeps.
//
// How the walk is organised here.  The state a check has confirmed -- the anchor: an iteration
// i, x_i and the Gerbicz product d_i -- stays on the device as two numbers of the context.  A
// round starts from the anchor (or, once, from a newer unverified save) and advances block by
// block: B squarings of x queued as a few kite_square_n calls (split only where a proof point or
// an injected fault falls), then t <- d and d <- d*x.  After M blocks, at the end of the checked
// part n - n mod B, or at a stop request, the round is closed by the check x0 * t^(2^B) == d,
// decided on the device (kite_equal_internal: the digits of both numbers carried exactly there,
// one word read back).  A closed round becomes the anchor, device to device; a failed check
// returns to the anchor; round-off above the limit moves the walk to the next FFT length at
// least 4% longer and returns to the anchor there (the only time the anchor travels as limbs).
// Proof points met in a round are kept as device copies until the round is closed, then handed
// to the caller.  The n mod B squarings after the checked part are computed twice and compared.
#include <cmath>
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

// The numbers of the walk in one context: the walk itself (x, d), the start x0, the check's
// scratch t, and the anchor (ax, ad).
struct Lane {
    kite_ctx *ctx = nullptr;
    Number x, d, x0, t, ax, ad;
    Lane() = default;
    Lane(const Lane &) = delete;
    Lane &operator=(const Lane &) = delete;
    ~Lane() {
        for (Number *p : {&x, &d, &x0, &t, &ax, &ad}) p->reset();
        kite_ctx_free(ctx);
    }
};

// A proof point captured in the current round: its index and a device copy of x there.
struct Captured {
    uint32_t index;
    Number value;
};

enum class RoundEnd { Blocks, RoundOff, PointFailed };

class FermatWalk {
  public:
    FermatWalk(uint64_t k, uint64_t n, uint32_t base, const kite_prp_opts &o, kite_prp_result *res)
        : k_(k), n_(n), base_(base), o_(o), res_(res) {
        B_ = o.gerbicz_block;
        if (!B_) B_ = (uint32_t)std::fmin(2000.0, std::fmax(32.0, std::floor(std::sqrt((double)n))));
        M_ = o.gerbicz_blocks ? o.gerbicz_blocks : std::max<uint32_t>(B_ / 4, 8);
        limit_ = o.max_roundoff > 0 ? o.max_roundoff : 0.40;
        verified_every_ = o.checkpoint_secs > 0 ? o.checkpoint_secs : 600;
        unverified_every_ = o.unverified_secs > 0 ? o.unverified_secs : 60;
        checked_end_ = n / B_ * B_;
        fault_at_ = o.inject_fault_at;
    }

    int run();

  private:
    bool open(uint32_t fft_len);
    uint32_t fft_len() const { return kite_fft_len(lane_->ctx); }
    bool stop_requested() const { return o_.abort_flag && *o_.abort_flag; }
    void note_roundoff() {
        const double e = kite_max_roundoff(lane_->ctx);
        if (e > res_->maxerr && e < 1.0) res_->maxerr = e;
    }
    uint32_t first_point_after(uint64_t iter, uint32_t from) const {
        while (from < o_.npoints && o_.points[from] <= iter) from++;
        return from;
    }
    void capture(uint32_t index, const kite_num *x);
    bool hand_over_points();
    bool save_anchor();
    RoundEnd advance(uint64_t &i, uint32_t &next, uint64_t end);
    bool move_to_longer_fft();
    int tail();

    const uint64_t k_, n_;
    const uint32_t base_;
    const kite_prp_opts o_;
    kite_prp_result *res_;
    uint32_t B_, M_;
    double limit_, verified_every_, unverified_every_;
    uint64_t checked_end_;
    uint64_t fault_at_;
    std::unique_ptr<Lane> lane_;
    // the anchor's iteration and the first proof point after it
    uint64_t anchor_iter_ = 0;
    uint32_t anchor_point_ = 0;
    // an unverified save ahead of the anchor, used for one round
    bool ahead_ = false;
    uint64_t ahead_iter_ = 0;
    uint32_t ahead_point_ = 0;
    std::vector<uint64_t> ahead_x_, ahead_d_;
    std::vector<Captured> pending_;
    double last_verified_save_ = 0, last_unverified_save_ = 0;
};

bool FermatWalk::open(uint32_t fft_len) {
    pending_.clear();
    lane_.reset();
    auto lane = std::make_unique<Lane>();
    kite_opts fo = o_.fft;
    if (fft_len) fo.fft_len = fft_len;
    lane->ctx = kite_ctx_new(k_, n_, -1, &fo);
    if (!lane->ctx) return false;
    // round-off sampled on every 4th operation: enough to see a length that is too short; the
    // Gerbicz check catches arithmetic errors (src/prp.c:281-283)
    kite_set_roundoff_check(lane->ctx, 4);
    for (Number *p : {&lane->x, &lane->d, &lane->x0, &lane->t, &lane->ax, &lane->ad}) {
        *p = Number(lane->ctx);
        if (!*p) return false;
    }
    kd::power_of_base(lane->ctx, lane->x0, k_, base_, n_);
    lane_ = std::move(lane);
    return true;
}

void FermatWalk::capture(uint32_t index, const kite_num *x) {
    Captured c{index, Number(lane_->ctx)};
    kite_copy(lane_->ctx, c.value, x);
    pending_.push_back(std::move(c));
}

// The points of a closed round (or before an unverified save) go to the caller in order;
// false when the caller refuses one.
bool FermatWalk::hand_over_points() {
    bool ok = true;
    for (Captured &c : pending_) {
        if (!ok) break;
        const std::vector<uint64_t> l = kd::limbs_of(lane_->ctx, c.value);
        ok = o_.on_point(o_.point_arg, c.index, o_.points[c.index], l.data()) == 0;
    }
    pending_.clear();
    return ok;
}

bool FermatWalk::save_anchor() {
    const std::vector<uint64_t> x = kd::limbs_of(lane_->ctx, lane_->ax), d = kd::limbs_of(lane_->ctx, lane_->ad);
    return kg::prp_checkpoint_write(o_.checkpoint, k_, n_, base_, anchor_iter_, fft_len(), x, d);
}

// Blocks from iteration i up to `end` (or a stop request, or round-off above the limit).
RoundEnd FermatWalk::advance(uint64_t &i, uint32_t &next, uint64_t end) {
    kite_ctx *ctx = lane_->ctx;
    while (i < end) {
        // a round holds up to B*M squarings, minutes at large n: a stop is honoured per block
        if (stop_requested()) break;
        const uint64_t block_end = i + B_;
        while (i < block_end) {
            uint64_t to = block_end;
            if (fault_at_ > i && fault_at_ < to) to = fault_at_;
            if (o_.on_point && next < o_.npoints && o_.points[next] > i && o_.points[next] < to)
                to = o_.points[next];
            kite_square_n(ctx, lane_->x, to - i);
            i = to;
            if (fault_at_ && i == fault_at_) {
                kite_debug_corrupt(ctx, lane_->x);  // testing hook: once per call
                fault_at_ = 0;
            }
            if (o_.on_point && next < o_.npoints && o_.points[next] == i) capture(next++, lane_->x);
        }
        // t keeps d from before the update, at every block, so a stop part way through a round
        // can close the round at the block it reached
        kite_copy(ctx, lane_->t, lane_->d);
        kite_mul(ctx, lane_->d, lane_->x);
        const double e = kite_max_roundoff(ctx);
        if (e > limit_) return RoundEnd::RoundOff;
        if (o_.progress) o_.progress(o_.progress_arg, i, n_, e);
        // an unverified save for a test killed without the chance to stop; the points so far go
        // to the caller first, so a resume from the save has them
        if (o_.checkpoint_unverified && kd::clock_s() - last_unverified_save_ > unverified_every_ && i < end) {
            if (!pending_.empty() && !hand_over_points()) return RoundEnd::PointFailed;
            kg::prp_checkpoint_write(o_.checkpoint_unverified, k_, n_, base_, i, fft_len(),
                                     kd::limbs_of(ctx, lane_->x), kd::limbs_of(ctx, lane_->d));
            last_unverified_save_ = kd::clock_s();
        }
    }
    return RoundEnd::Blocks;
}

// Round-off above the limit: the anchor moves, as limbs, to a context at the next length at
// least 4% longer.
bool FermatWalk::move_to_longer_fft() {
    const uint32_t L = fft_len();
    const uint32_t next = kg::next_fft_len(L + L / 25);
    if (!next) return false;
    const std::vector<uint64_t> x = kd::limbs_of(lane_->ctx, lane_->ax), d = kd::limbs_of(lane_->ctx, lane_->ad);
    if (!open(next)) return false;
    kite_set_limbs(lane_->ctx, lane_->ax, x.data());
    kite_set_limbs(lane_->ctx, lane_->ad, d.data());
    return true;
}

// The squarings after the checked part, twice from the anchor, compared (src/prp.c:520-551).
int FermatWalk::tail() {
    kite_ctx *ctx = lane_->ctx;
    for (int attempt = 0;; attempt++) {
        kite_copy(ctx, lane_->x, lane_->ax);
        kite_copy(ctx, lane_->t, lane_->ax);
        pending_.clear();
        uint64_t i = checked_end_;
        uint32_t next = anchor_point_;
        while (i < n_) {
            uint64_t to = n_;
            if (o_.on_point && next < o_.npoints && o_.points[next] > i && o_.points[next] < to) to = o_.points[next];
            kite_square_n(ctx, lane_->x, to - i);
            kite_square_n(ctx, lane_->t, to - i);
            i = to;
            if (o_.on_point && next < o_.npoints && o_.points[next] == i) capture(next++, lane_->x);
        }
        if (kite_equal_internal(ctx, lane_->x, lane_->t) == 1) {
            if (!pending_.empty() && !hand_over_points()) return KITE_PRP_POINT_FAILED;
            return 0;
        }
        if (attempt > 5) return -3;
        res_->gerbicz_errors++;
    }
}

int FermatWalk::run() {
    if (!open(0)) return -1;
    kite_ctx *ctx = lane_->ctx;
    const size_t nl = kite_limbs(ctx);
    // ---- resume from the verified checkpoint and, if ahead of it, the unverified one
    {
        std::vector<uint64_t> vx(nl), vd(nl);
        uint64_t vi = 0;
        uint32_t saved_len = 0, ahead_len = 0;
        const bool verified = o_.checkpoint &&
                              kg::prp_checkpoint_read(o_.checkpoint, k_, n_, base_, nl, vi, saved_len, vx, vd);
        if (verified) res_->resumed = 1;
        if (o_.checkpoint_unverified) {
            ahead_x_.assign(nl, 0);
            ahead_d_.assign(nl, 0);
            ahead_ = kg::prp_checkpoint_read(o_.checkpoint_unverified, k_, n_, base_, nl, ahead_iter_, ahead_len,
                                             ahead_x_, ahead_d_) &&
                     ahead_iter_ > vi;
            if (ahead_) {
                res_->resumed = 1;
                saved_len = std::max(saved_len, ahead_len);
            } else {
                ahead_iter_ = 0;
            }
        }
        if (saved_len > fft_len() && !open(saved_len)) return -1;  // the saved run had moved on
        ctx = lane_->ctx;
        if (verified) {
            kite_set_limbs(ctx, lane_->ax, vx.data());
            kite_set_limbs(ctx, lane_->ad, vd.data());
        } else {
            kite_copy(ctx, lane_->ax, lane_->x0);
            kite_copy(ctx, lane_->ad, lane_->x0);
        }
        anchor_iter_ = vi;
        res_->resumed_at = ahead_ ? ahead_iter_ : vi;
    }
    // ---- proof points: after the anchor; x_0 itself is handed over at once
    if (o_.on_point) {
        anchor_point_ = anchor_iter_ ? first_point_after(anchor_iter_, 0) : 0;
        if (anchor_point_ < o_.npoints && o_.points[anchor_point_] == 0) {
            capture(anchor_point_++, lane_->ax);
            if (!hand_over_points()) return KITE_PRP_POINT_FAILED;
        }
        ahead_point_ = first_point_after(ahead_iter_, anchor_point_);
    }
    last_verified_save_ = last_unverified_save_ = kd::clock_s();
    int failures_in_a_row = 0;
    // ---- rounds until a closed round puts the anchor at the end of the checked part
    while (true) {
        ctx = lane_->ctx;
        const bool from_ahead = ahead_;
        ahead_ = false;  // used once: a failure below returns to the anchor
        const uint64_t start = from_ahead ? ahead_iter_ : anchor_iter_;
        if (from_ahead) {
            kite_set_limbs(ctx, lane_->x, ahead_x_.data());
            kite_set_limbs(ctx, lane_->d, ahead_d_.data());
        } else {
            kite_copy(ctx, lane_->x, lane_->ax);
            kite_copy(ctx, lane_->d, lane_->ad);
        }
        kite_reset_roundoff(ctx);
        pending_.clear();
        if (stop_requested()) {
            if (o_.checkpoint) save_anchor();
            return KITE_PRP_ABORTED;
        }
        uint64_t i = start;
        uint32_t next = from_ahead ? ahead_point_ : anchor_point_;
        const uint64_t end = std::min(start + (uint64_t)B_ * M_, checked_end_);
        const RoundEnd how = advance(i, next, end);
        if (how == RoundEnd::PointFailed) return KITE_PRP_POINT_FAILED;
        const bool stopping = stop_requested();
        if (stopping && i == start) continue;  // nothing new: saved and returned above
        bool roundoff = how == RoundEnd::RoundOff, mismatch = false;
        if (!roundoff && i > start) {
            // close the round: d == x0 * t^(2^B), decided on the device
            kite_square_n(ctx, lane_->t, B_);
            kite_mul(ctx, lane_->t, lane_->x0);
            if (kite_max_roundoff(ctx) > limit_)
                roundoff = true;
            else
                mismatch = kite_equal_internal(ctx, lane_->t, lane_->d) != 1;
        }
        note_roundoff();
        // an unverified save from this round, or the one resumed from, may hold the error
        if ((roundoff || mismatch) && o_.checkpoint_unverified) std::remove(o_.checkpoint_unverified);
        if (roundoff) {
            if (!move_to_longer_fft()) return -2;
            res_->roundoff_retries++;
            continue;
        }
        if (mismatch) {
            res_->gerbicz_errors++;
            if (++failures_in_a_row > 5) return -3;
            continue;
        }
        failures_in_a_row = 0;
        kite_copy(ctx, lane_->ax, lane_->x);
        kite_copy(ctx, lane_->ad, lane_->d);
        anchor_iter_ = i;
        anchor_point_ = next;
        if (!pending_.empty() && !hand_over_points()) return KITE_PRP_POINT_FAILED;
        if (o_.checkpoint &&
            (kd::clock_s() - last_verified_save_ > verified_every_ || anchor_iter_ == checked_end_ || stopping)) {
            save_anchor();
            last_verified_save_ = kd::clock_s();
        }
        if (stopping) return KITE_PRP_ABORTED;
        if (anchor_iter_ >= checked_end_) break;
    }
    // ---- the unchecked tail, then the verdict from x_n = base^(N+1)
    const int rc = tail();
    if (rc) return rc;
    ctx = lane_->ctx;
    std::vector<uint64_t> xn = kd::limbs_of(ctx, lane_->x);
    const bool prp = kd::limbs_equal_word(xn, (uint64_t)base_ * base_);
    int out = 0;
    if (kg::residue_nm1(xn.data(), ctx->lay.Nl.data(), nl, base_)) out = -4;
    res_->res64 = xn[0];
    res_->is_prp = prp;
    res_->fft_len = fft_len();
    note_roundoff();
    return out;
}

}  // namespace

extern "C" int kite_prp_checkpoint_iter(const char *path, uint64_t k, uint64_t n, uint32_t base, uint64_t *iter) {
    kg::PrpCheckpointHeader h;
    if (!kg::prp_checkpoint_header(path, h) || h.k != k || h.n != n || h.base != base) return -1;
    *iter = h.iter;
    return 0;
}

extern "C" int kite_prp(uint64_t k, uint64_t n, uint32_t base, const kite_prp_opts *opts, kite_prp_result *res) {
    std::memset(res, 0, sizeof *res);
    const double t0 = kd::clock_s();
    const kite_prp_opts o = opts ? *opts : kite_prp_opts{};
    int rc;
    {
        FermatWalk walk(k, n, base, o, res);
        rc = walk.run();
    }
    res->seconds = kd::clock_s() - t0;
    return rc;
}
