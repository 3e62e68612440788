// Per-length tuning (include/kite_cuda.h): shapes and measured times per FFT length, set
// directly or loaded from a tuning file, and the round-off probe used to report each length's
// largest round-off.
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "../../include/kite_cuda.h"
#include "layout.h"
#include "plan.h"

extern "C" {

int kc_set_fft_shape(uint32_t L, uint32_t R) { return kg::set_shape_override(L, R) ? 0 : -1; }

int kc_set_latency_shape(uint32_t L, uint32_t R, int G) { return kg::set_latency_override(L, R, G) ? 0 : -1; }

void kc_set_fft_time(uint32_t L, double us) { kg::set_tuned_time(L, us); }

int kc_fft_shape_candidates(uint32_t L, uint32_t *R, uint32_t *C, int max) {
    if (L % 2) return 0;
    return kg::shape_candidates(L / 2, R, C, max);
}

int kc_fft_shape(uint32_t L, uint32_t *R, uint32_t *C) {
    uint32_t r = 0, c = 0;
    if (L % 2 || !kg::choose_shape(L / 2, r, c)) return -1;
    if (R) *R = r;
    if (C) *C = c;
    return 0;
}

int kc_tuning_load(const char *path) {
    FILE *f = path ? std::fopen(path, "r") : nullptr;
    if (!f) return -1;
    char line[256];
    int count = 0;
    while (std::fgets(line, sizeof line, f)) {
        unsigned L = 0, R = 0, C = 0;
        int G = 0;
        double us = 0;
        int got = std::sscanf(line, "%u %lf %u %u %d", &L, &us, &R, &C, &G);
        if (got < 2 || line[0] == '#') continue;
        if (got == 5) {
            if ((uint64_t)R * C == L / 2) kg::set_latency_override(L, R, G);
        } else {
            if (us > 0) kg::set_tuned_time(L, us);
            if (got == 4 && (uint64_t)R * C == L / 2) kg::set_shape_override(L, R);
        }
        count++;
    }
    std::fclose(f);
    return count;
}

double kc_roundoff_probe(uint64_t k, uint64_t n, uint32_t L, uint32_t squarings, uint64_t seed) {
    kg::Layout lay;
    if (!lay.build(k, n, L)) return -1;
    kc_engine *e = kc_engine_new(k, n, L, nullptr, nullptr, nullptr, 0, 0, 0, 0, -1);
    if (!e) return -2;
    double *x = kc_num_alloc(e);
    double r = -3;
    if (x) {
        // a seeded value below 2^(n-1) < N, as limbs
        std::vector<uint64_t> l(lay.nlimbs, 0);
        uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
        for (uint64_t bit = 0; bit + 64 <= n - 1; bit += 64) {
            s ^= s << 13;
            s ^= s >> 7;
            s ^= s << 17;
            l[bit / 64] = s;
        }
        kc_set_roundoff_check(e, 1);
        std::vector<int64_t> d(L);
        lay.limbs_to_digits(l.data(), d.data());
        if (!kc_from_digits(e, x, d.data()) && !kc_square(e, x, squarings)) r = kc_maxerr(e);
        kc_num_free(e, x);
    }
    kc_engine_free(e);
    return r;
}

}  // extern "C"
