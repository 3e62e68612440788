// Exact host-side arithmetic of the k-scaled irrational-base DWT for N = k*2^n - 1.
//
// Representation (the same as the reference's, src/internal.h:3-17):
//   T' = n + log2(k) held as a 64-bit binary fraction; s_j = ceil(j*T'/L), j = 0..L;
//   digit j has width bits[j] = s_{j+1} - s_j; a number V = sum_j x_j 2^{s_j};
//   weights w_j = 2^{s_j - j*T'/L} in [1, 2); outputs are scaled by oscale_j = k / w_j;
//   the stored value is V = x/k (mod N), so that squaring the digits yields k*V^2 == (x^2)/k.
// The digit boundaries and the weights are bit-identical to the reference (src/ctx.c:150-221)
// because they are derived by the same exact integer method.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace kg {

bool fft_len_ok(uint32_t L);
double safe_bpw(uint32_t L, uint64_t k);
uint32_t choose_fft_len(uint64_t k, uint64_t n);
uint32_t next_fft_len(uint32_t L);
// Record (us > 0) or forget the measured time per squaring of length L (autotuner results).
void set_tuned_time(uint32_t L, double us);

struct Layout {
    uint64_t k = 0, n = 0;
    uint32_t L = 0;
    uint64_t lam = 0;        // frac(log2 k) * 2^64
    uint64_t sL = 0;         // s_L
    uint32_t top_t = 0;      // first digit with s_{j+1} > n (L if none)
    uint64_t top_st = 0;     // s_{top_t}
    uint32_t top_m = 0;      // n - s_{top_t}
    std::vector<uint64_t> s; // L + 1 boundaries
    std::vector<uint8_t> bits;
    std::vector<double> w, oscale;
    size_t nlimbs = 0;       // limbs of a value in [0, N)
    std::vector<uint64_t> Nl;

    // false when (k, n, L) cannot be laid out (the reference rejects the same cases)
    bool build(uint64_t k, uint64_t n, uint32_t L);

    // Balanced carry (digit in [-2^(b-1), 2^(b-1))) with the top fold, in place.  Digits may
    // be any integers below 2^62 in magnitude.
    void carry(int64_t *d) const;
    // Canonical limbs in [0, N) of k * sum(d_j 2^{s_j}) for integer digits of any sign.
    void digits_to_limbs(const int64_t *d, uint64_t *limbs) const;
    // Limbs in [0, N) -> balanced digits of the stored value x/k (mod N).
    void limbs_to_digits(const uint64_t *limbs, int64_t *d) const;
    // Sparse digits of the stored form of the small signed constant c (i.e. c/k mod N), as
    // (index, value) pairs with non-zero value; at most `cap` pairs, returns the count or -1.
    int constant_digits(int64_t c, uint32_t *idx, int64_t *val, int cap) const;

  private:
    int64_t fold_top(int64_t *d, int64_t cy) const;
    void reduce_mod_N(uint64_t *a, size_t na) const;
};

// y = base^(N+1) mod N (nl limbs) -> base^(N-1) mod N, also when gcd(base, N) > 1.
// 0, or -1 when the base-prime part of N does not fit a word.
int residue_nm1(uint64_t *y, const uint64_t *N, size_t nl, uint64_t base);

}  // namespace kg
