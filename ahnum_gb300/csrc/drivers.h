// Pieces shared by the test drivers built on the kite API (the Fermat test, the LLR test and the
// PRST proof steps): scoped numbers, limb helpers and a monotonic clock.
#pragma once

#include <chrono>
#include <cstdint>
#include <utility>
#include <vector>

#include "../../include/kite.h"
#include "kite_internal.h"

namespace kd {

inline double clock_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// A kite number freed when it goes out of scope; its context must outlive it.
class Number {
  public:
    Number() = default;
    explicit Number(kite_ctx *c) : ctx_(c), x_(c ? kite_num_new(c) : nullptr) {}
    ~Number() { reset(); }
    Number(Number &&o) noexcept : ctx_(o.ctx_), x_(std::exchange(o.x_, nullptr)) {}
    Number &operator=(Number &&o) noexcept {
        if (this != &o) {
            reset();
            ctx_ = o.ctx_;
            x_ = std::exchange(o.x_, nullptr);
        }
        return *this;
    }
    Number(const Number &) = delete;
    Number &operator=(const Number &) = delete;
    void reset() {
        if (x_) kite_num_free(ctx_, x_);
        x_ = nullptr;
    }
    kite_num *get() const { return x_; }
    operator kite_num *() const { return x_; }
    explicit operator bool() const { return x_ != nullptr; }

  private:
    kite_ctx *ctx_ = nullptr;
    kite_num *x_ = nullptr;
};

// Canonical limbs (kite_limbs words) of x.
inline std::vector<uint64_t> limbs_of(kite_ctx *ctx, const kite_num *x) {
    std::vector<uint64_t> l(kite_limbs(ctx));
    kite_get_limbs(ctx, x, l.data());
    return l;
}

// Whether the limbs hold the small value v.
inline bool limbs_equal_word(const std::vector<uint64_t> &l, uint64_t v) {
    if (l.empty()) return v == 0;
    if (l[0] != v) return false;
    for (size_t i = 1; i < l.size(); i++)
        if (l[i]) return false;
    return true;
}

// x = base^k mod N.  While base^k stays below N/4 the value is formed exactly in limbs on the
// host; otherwise it is raised on the device by left-to-right binary powering (squarings and
// multiplications by the small base).  Either way the value equals the reference's starting
// value x_0 = base^k (src/prp.c:298-327).
inline void power_of_base(kite_ctx *ctx, kite_num *x, uint64_t k, uint32_t base, uint64_t n) {
    const size_t nl = kite_limbs(ctx);
    double bits = 0;
    for (uint32_t b = base; b > 1; b >>= 1) bits += 1;  // floor(log2 base) + 1 >= log2 base
    if ((double)k * bits + 2 < (double)n) {
        std::vector<uint64_t> v(nl, 0);
        v[0] = 1;
        size_t top = 1;
        for (uint64_t i = 0; i < k; i++) {
            unsigned __int128 carry = 0;
            for (size_t j = 0; j < top; j++) {
                carry += (unsigned __int128)v[j] * base;
                v[j] = (uint64_t)carry;
                carry >>= 64;
            }
            if (carry && top < nl) v[top++] = (uint64_t)carry;
        }
        kite_set_limbs(ctx, x, v.data());
        return;
    }
    kite_set_u64(ctx, x, 1);
    int hi = 63;
    while (hi > 0 && !((k >> hi) & 1)) hi--;
    for (int b = hi; b >= 0; b--) {
        kite_square(ctx, x);
        if ((k >> b) & 1) kite_mul_small(ctx, x, base);
    }
}

}  // namespace kd
