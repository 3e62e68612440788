// Structures shared by the host code and the sm_103a kernels.
//
// One squaring of a number of L real words uses a complex transform of H = L/2 points arranged
// four-step as R rows x C columns, element m = r*C + c (row-major):
//   stored form  S[p][c] = (column DIF over r of u, times w_H^{c*k_r}), p = pos_R(k_r), where
//                u_m = x_{2m} w_{2m} + i x_{2m+1} w_{2m+1} are the weighted digits;
//   row pass     forward row DIF (C points), real-split square or product, inverse row DIT;
//   column pass  conj twiddle, inverse column DIT, unweight/round/carry, reweight, forward
//                column DIF, twiddle.
// This is the pass structure of the reference's two-pass backend (src/fast2p.c:1-19); the
// kernels that implement it are written for the GPU.
#pragma once

#include <cstdint>
#include <vector_types.h>

namespace kg {

constexpr int kMaxStages = 12;
constexpr int kGroup = 8;        // columns per column-pass work unit (16 digits per row segment)
constexpr int kMaxAddend = 4;    // sparse constant digits folded into the normaliser

// In-place mixed-radix DIF (forward) / DIT (inverse) of length n, unnormalised.
// Stage i has radix rad[i] and span span[i] = n / (rad[0]*...*rad[i]); its twiddles
// w_{rad[i]*span[i]}^{t*j} (t < rad, j < span) start at tw + off[i], index t*span + j.
struct FftPlan {
    int n = 0;
    int nst = 0;
    int rad[kMaxStages] = {};
    int span[kMaxStages] = {};
    int off[kMaxStages] = {};
};

// Everything a kernel needs for one test (one modulus).  Lives in device memory.
struct TestDesc {
    // shape
    int L, H, R, C, NG;      // NG = C / kGroup column groups
    FftPlan rp, cp;          // row plan (length C), column plan (length R)
    const double2 *twr;      // row stage twiddles
    const double2 *twc;      // column stage twiddles
    const double2 *t4;       // [p][c] four-step twiddle w_H^{c * k_r(p)}
    const double2 *sw;       // [p][q] real-split twiddle w_H^{k_r(p) + R * k_c(q)}
    const int *part0;        // [q] partner column position in the row with k_r = 0
    const int *part1;        // [q] partner column position for k_r != 0: pos(C-1-k_c(q))
    const int2 *pairs;       // row pairs (p, p') with k_r(p') = R - k_r(p), p <= p'
    int npairs;
    int prow0;               // position of row k_r = 0 (always 0)
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
