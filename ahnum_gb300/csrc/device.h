// Structures shared by the host code and the sm_103a kernels.
//
// One squaring of a number of L real words uses a complex transform of H = L/2 points arranged
// four-step as R rows x C columns, element m = r*C + c (row-major):
//   stored form  S[k_r][c] = (column transform over r of u, times w_H^{c*k_r}), rows in natural
//                frequency order, where u_m = x_{2m} w_{2m} + i x_{2m+1} w_{2m+1} are the
//                weighted digits;
//   row pass     forward row transform (C points), real-split square or product, inverse row
//                transform;
//   column pass  conj twiddle, inverse column transform, unweight/round/carry, reweight,
//                forward column transform, twiddle.
// This is the pass structure of the reference's two-pass backend (src/fast2p.c:1-19); the
// kernels that implement it are written for the GPU.
#pragma once

#include <cstdint>
#include <vector_types.h>

namespace kg {

constexpr int kMaxStages = 12;
constexpr int kGroup = 8;        // widest column group (16 digits per row segment); C is a multiple of it
constexpr int kMaxAddend = 4;    // sparse constant digits folded into the normaliser

// In-place mixed-radix decimation-in-time transform of length n, unnormalised, input in the
// digit-reversed order pos() of the plan.  Stage i has radix rad[i] and span
// span[i] = n / (rad[0]*...*rad[i]); stages run from i = nst-1 (span 1) to 0.  Stage i's
// twiddle records start at tw + off[i]: for each j < span, rad-1 double2 -- tangent form
// {tau1, c1} (radix 2), {tau1, tau2}, {tau3, c1}, {c2, c3/c1} (radix 4), or the complex
// twiddles w^{t*j}, t = 1..rad-1 (odd radices), of w = exp(-2 pi i / (rad*span)).
struct FftPlan {
    int n = 0;
    int nst = 0;
    int rad[kMaxStages] = {};
    int span[kMaxStages] = {};
    int off[kMaxStages] = {};
};

// Everything a kernel needs for one test (one modulus).  Lives in device memory; a kernel copies
// the descriptor of the item it works on into shared memory (16-byte chunks, hence alignas).
struct alignas(16) TestDesc {
    // shape
    int L, H, R, C, NG;      // NG = C / G column groups
    int G;                   // columns per column group: 2, 4 or 8 (2G digits per row segment)
    FftPlan rp, cp;          // row plan (length C), column plan (length R)
    const double2 *twr;      // row stage twiddles
    const double2 *twc;      // column stage twiddles
    const double2 *t4;       // [k_r][c] four-step twiddle w_H^{c * k_r}
    const double2 *sw;       // [k_r][k_c] real-split twiddle w_H^{k_r + R * k_c}
    const int *posr;         // [r] digit-reversed position of the column transform
    const int *posc;         // [c] digit-reversed position of the row transform
    const int2 *pairs;       // row pairs (k_r, (R - k_r) mod R), k_r <= its partner
    int npairs;
    // per-modulus tables
    const uint8_t *bits;     // [L]
    const double *w;         // [L] weights
    const double *osc;       // [L] k / (w_j * 4H): unweight and scale after a product
    const double *idig;      // [L] 1 / (R * w_j): unweight after the column inverse alone
    // scratch
    long long *dig;          // [L] integer digits between the two column kernels
    long long *slot;         // [NG * R] carry into segment (g, r), index g*R + r
    unsigned long long *maxerr;  // bits of the largest round-off (non-negative double)
    int *status;             // sticky device-side error flags
    // top fold
    unsigned long long k;
    int top_t, top_m, top_shift; // top_shift = s_L - s_t
    // constant digits added before the carry (LLR: -2), (index, value)
    int nadd;
    int addj[kMaxAddend];
    long long addv[kMaxAddend];
    // operands of the current operation
    double2 *x;
    const double2 *y;
    int count;      // steps of the current launch sequence this test takes part in
    int err_every;  // round-off is tracked on steps that are multiples of this
};

// A unit of work: the test and the row pair or column group it covers.
struct WorkItem {
    int test;
    int unit;
};

}  // namespace kg
