// Host-only entry points of include/kite_cuda.h: the exact layout and conversions, callable
// without a GPU.
#include <cstring>

#include "../../include/kite_cuda.h"
#include "layout.h"

extern "C" {

int kc_layout(uint64_t k, uint64_t n, uint32_t L, uint8_t *bits, double *w, double *oscale,
              uint64_t *meta) {
    kg::Layout y;
    if (!y.build(k, n, L)) return -1;
    if (bits) std::memcpy(bits, y.bits.data(), L);
    if (w) std::memcpy(w, y.w.data(), L * sizeof(double));
    if (oscale) std::memcpy(oscale, y.oscale.data(), L * sizeof(double));
    if (meta) {
        meta[0] = y.lam;
        meta[1] = y.sL;
        meta[2] = y.top_t;
        meta[3] = y.top_st;
        meta[4] = y.top_m;
    }
    return 0;
}

int kc_digits_to_limbs(uint64_t k, uint64_t n, uint32_t L, const int64_t *digits, uint64_t *limbs) {
    kg::Layout y;
    if (!y.build(k, n, L)) return -1;
    y.digits_to_limbs(digits, limbs);
    return 0;
}

int kc_limbs_to_digits(uint64_t k, uint64_t n, uint32_t L, const uint64_t *limbs, int64_t *digits) {
    kg::Layout y;
    if (!y.build(k, n, L)) return -1;
    y.limbs_to_digits(limbs, digits);
    return 0;
}

int kc_carry_digits(uint64_t k, uint64_t n, uint32_t L, int64_t *digits) {
    kg::Layout y;
    if (!y.build(k, n, L)) return -1;
    y.carry(digits);
    return 0;
}

uint32_t kc_choose_fft_len(uint64_t k, uint64_t n) { return kg::choose_fft_len(k, n); }

}  // extern "C"
