// Per-FFT-length plans: four-step shape, mixed-radix stage plans and the twiddle tables, built
// once per (device, L) on the host and kept resident on the device.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "device.h"

namespace kg {

struct LengthPlan {
    uint32_t L = 0, H = 0, R = 0, C = 0;
    FftPlan rp, cp;                   // row plan (C points), column plan (R points)
    std::vector<int> rev_r, pos_r;    // DIF output position <-> frequency, column transform
    std::vector<int> rev_c, pos_c;    // same for the row transform
    std::vector<int2> pairs;          // row pairs (p, p'), p <= p'
    // device copies
    int device = -1;
    double2 *twr = nullptr, *twc = nullptr, *t4 = nullptr, *sw = nullptr;
    int *dposr = nullptr, *dposc = nullptr;
    int2 *dpairs = nullptr;
    size_t device_bytes = 0;
    ~LengthPlan();
};

// H = R*C with C a multiple of kGroup; the autotuned shape of this length if one was set, else
// rows about four times as long as columns.  false if no usable shape exists.
bool choose_shape(uint32_t H, uint32_t &R, uint32_t &C);
// Use R rows for FFT length L from now on (R = 0: back to the default); false if unusable.
bool set_shape_override(uint32_t L, uint32_t R);
// Usable shapes of H = R*C near balance, at most `max`; returns the count.
int shape_candidates(uint32_t H, uint32_t *R, uint32_t *C, int max);
// Radices for a length-n transform in DIF order; false if n has a prime factor above 7.
bool make_fft_plan(int n, FftPlan &pl);

// exp(-2 pi i j / m) with the angle reduced exactly in integer arithmetic
double2 cis_neg(uint64_t j, uint64_t m);

// Shape and column-group width for one test run alone: spread every pass over the SMs so the
// squaring's latency, not its total FP64 work, is smallest.  Throughput (batched) use takes
// choose_shape and G = kGroup instead.  min_bits: the narrowest digit; top_digits: L - top_t.
// An autotuned shape of the length (set_latency_override) comes first wherever the number's
// digits allow its group width.
bool choose_latency_shape(uint32_t H, int nsm, unsigned min_bits, unsigned top_digits, uint32_t &R,
                          uint32_t &C, int &G);
// Use R rows and column groups of G for one test alone at FFT length L from now on (R = 0: back
// to the model); false if the shape is unusable.
bool set_latency_override(uint32_t L, uint32_t R, int G);

// Cached plan for (current device, L, R) (R = 0: choose_shape); nullptr if L cannot be planned or
// the device upload fails.  Thread-safe.
std::shared_ptr<LengthPlan> get_plan(uint32_t L, uint32_t R = 0);
// Host tables only (no device upload).
std::shared_ptr<LengthPlan> build_plan_host(uint32_t L, uint32_t R, std::vector<double2> *twr,
                                            std::vector<double2> *twc, std::vector<double2> *t4,
                                            std::vector<double2> *sw);

}  // namespace kg
