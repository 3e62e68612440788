// Exact integer-NTT squaring modulo N = k*2^n - 1 (include/kite_ntt.h).
//
// One modular squaring is four kernels over a test's W words of w bits:
//   kn_col_fwd   per group of G columns of the R x C four-step layout: words -> residues modulo
//                four primes, forward column NTT (decimation in frequency, natural order in,
//                bit-reversed out), times the four-step twiddle w_NP^(k_r c).
//   kn_rows      per row: forward row NTT (DIF), pointwise Montgomery square or product,
//                inverse row NTT (decimation in time, bit-reversed in, natural out).
//   kn_col_inv   per column group: times w_NP^(-k_r c) 2^32 / NP, inverse column NTT (DIT),
//                Garner CRT of the four residues into the exact coefficients (< 2^120), and the
//                carry through each row's 8 consecutive coefficients: 8 words of the product P
//                and one segment carry.
//   kn_reduce    per test, one block: the segment carries into the words of P = x^2, Montgomery
//                reduction P 2^-n == B + k A (mod N) for P = A + B 2^n, A < 2^n, plus an
//                optional constant, carry, and the top fold T 2^n == q + r 2^n for T = q k + r.
// Reference: gpu/ntt_reg.metal:90-246 (the four-step NTT passes), gpu/sq.metal:23-192 (residues,
// Garner CRT, carry, REDC, fold), gpu/gpu_ctx.h:57-322 (tables and the pass sequence).
//
// Modular arithmetic (p < 2^30, so 4p < 2^32): residues stay in [0, 2p) between operations
// (Harvey's lazy butterflies); a twiddle w is applied as Shoup's x*w - floor(x*w'/2^32)*p with
// w' = floor(w*2^32/p); pointwise products use Montgomery's reduction by 2^32, whose 2^-32 the
// inverse twiddles undo.  Every kernel is integer-only: IMAD, IADD3, IMNMX, LOP3 on the
// integer pipes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/kite_ntt.h"

namespace kn {

using u128 = unsigned __int128;

constexpr int kPrimes = 4;
// p = m 2^e + 1 below 2^30 with 15 | m and e >= 20: transforms of length 2^a, 3 2^a, 5 2^a for
// a <= 20 exist modulo every one; their product is 2^119.36.
constexpr uint32_t kP[kPrimes] = {1053818881u, 975175681u, 943718401u, 880803841u};
constexpr int kG = 8;                // columns per column group
constexpr int kColThreads = 256;
constexpr int kRowThreads = 256;
constexpr int kReduceThreads = 256;

struct Prime {
    uint32_t p;
    uint32_t pinv;  // -p^-1 mod 2^32
    uint2 one;      // Shoup pair of 1: reduces any 32-bit value to [0, 2p)
    uint2 r32;      // Shoup pair of 2^32 mod p
};

struct Tables {
    const uint2 *twr_f[kPrimes], *twr_i[kPrimes];  // length-R level tables, [s + j] = w_2s^(+-j)
    const uint2 *twc_f[kPrimes], *twc_i[kPrimes];  // length-C level tables
    const uint2 *t4_f[kPrimes], *t4_i[kPrimes];    // [pos_r * C + c], storage order
};

// Garner constants: Shoup pairs of p_i^-1 mod p_j
struct Crt {
    uint2 inv01, inv02, inv12, inv03, inv13, inv23;
};

struct Desc {
    uint32_t NP, R, C;
    uint32_t np;                // primes in use: 3, or 4 when the coefficients need them
    uint32_t W, w, WN0, BN0;    // words, word bits, n / w, n % w
    uint64_t k;
    uint64_t *x;                // operand and result
    const uint64_t *y;          // second operand of a product
    uint32_t *res, *res2;       // 4 NP residues each
    ulonglong2 *seg;            // NP / 8 carries out of the product's 8-word segments (lo, hi)
    uint64_t *pw;               // NP words of the product
    const uint64_t *addend;     // W words added after the reduction, or null
    int *status;                // non-zero: a carry left the number (cannot happen for valid input)
    Prime pr[kPrimes];
    Crt crt;
    Tables tb;
};

// ---- device arithmetic ------------------------------------------------------------------------

__device__ __forceinline__ uint32_t red2(uint32_t v, uint32_t m) { return min(v, v - m); }  // [0,2m) -> [0,m)

__device__ __forceinline__ uint32_t shoup(uint32_t x, uint2 w, uint32_t p) {
    const uint32_t q = __umulhi(x, w.y);
    return x * w.x - q * p;  // in [0, 2p) for any 32-bit x
}

__device__ __forceinline__ uint32_t montmul(uint32_t a, uint32_t b, uint32_t p, uint32_t pinv) {
    const uint64_t t = (uint64_t)a * b;  // a, b < 2p: t < 4p^2 < 2^62
    const uint32_t m = (uint32_t)t * pinv;
    return (uint32_t)((t + (uint64_t)m * p) >> 32);  // a b 2^-32 mod p, in [0, 2p)
}

__device__ __forceinline__ uint32_t residue(uint64_t word, const Prime &P) {
    const uint32_t lo = (uint32_t)word, hi = (uint32_t)(word >> 32);
    return red2(shoup(lo, P.one, P.p) + shoup(hi, P.r32, P.p), 2 * P.p);
}

__device__ __forceinline__ int log2i(uint32_t x) { return 31 - __clz(x); }

// A length n = A*B transform runs as two register passes (Bailey's split of the levels):
//   the "wide" levels, half-sizes n/2 .. B, pair elements B apart: a unit holds the A values at
//   t + B m (m < A) for one t < B;
//   the "narrow" levels, half-sizes B/2 .. 1, stay inside blocks of B consecutive elements: a
//   unit holds one block, B t2 + m (m < B).
// Between the passes the values go through shared memory once, with element e stored at
// e + (e >> log2 B) so that both access patterns are free of bank conflicts.
//
// DIF levels over register values at positions c0 + m*stride: level s pairs m with m + s/stride
// and multiplies the difference by w_2s^(c mod s) = tw[s + (c mod s)].  NARROW: stride 1 and c0 a
// multiple of A, so c mod s = m mod s is known at compile time and the butterflies whose twiddle
// is 1 (m mod s = 0: all of level 1, half of level 2, ...) skip the multiplication.
// UPPER_ZERO: the values at m >= A/2 are zero (the padding half of an acyclic product's input),
// so the first level only multiplies: (u, 0) -> (u, u w).
template <int A, bool NARROW, bool UPPER_ZERO = false>
__device__ __forceinline__ void dif_regs(uint32_t (&x)[A], int c0, int stride, const uint2 *tw, uint32_t p) {
    const uint32_t p2 = 2 * p;
#pragma unroll
    for (int half = A / 2; half >= 1; half >>= 1) {
        const int s = NARROW ? half : stride * half;
#pragma unroll
        for (int m = 0; m < A; m++) {
            if (m & half) continue;
            if (UPPER_ZERO && half == A / 2) {
                const int c = NARROW ? m : c0 + m * stride;
                x[m + half] = shoup(x[m] + p2, __ldg(&tw[s + (c & (s - 1))]), p);
                continue;
            }
            const uint32_t u = x[m], v = x[m + half];
            x[m] = red2(u + v, p2);
            if (NARROW && (m & (half - 1)) == 0) {
                x[m + half] = red2(u - v + p2, p2);
            } else {
                const int c = NARROW ? m : c0 + m * stride;
                x[m + half] = shoup(u - v + p2, __ldg(&tw[s + (c & (s - 1))]), p);
            }
        }
    }
}

// DIT levels (inverse), ascending: (u, v) -> (u + v w, u - v w), w = w_2s^-(c mod s)
template <int A, bool NARROW>
__device__ __forceinline__ void dit_regs(uint32_t (&x)[A], int c0, int stride, const uint2 *tw, uint32_t p) {
    const uint32_t p2 = 2 * p;
#pragma unroll
    for (int half = 1; half < A; half <<= 1) {
        const int s = NARROW ? half : stride * half;
#pragma unroll
        for (int m = 0; m < A; m++) {
            if (m & half) continue;
            const uint32_t u = x[m];
            uint32_t v = x[m + half];
            if (!(NARROW && (m & (half - 1)) == 0)) {
                const int c = NARROW ? m : c0 + m * stride;
                v = shoup(v, __ldg(&tw[s + (c & (s - 1))]), p);
            }
            x[m] = red2(u + v, p2);
            x[m + half] = red2(u - v + p2, p2);
        }
    }
}

template <int X>
__host__ __device__ constexpr int clog2() { return X <= 1 ? 0 : 1 + clog2<X / 2>(); }

// ---- pass kernels -----------------------------------------------------------------------------

// Column layout in shared memory: [prime][padded r][l], l < kG.
template <int B>
__device__ __forceinline__ int col_addr(int i, int rp_len, int e, int l) {
    return ((i * rp_len + e + (e >> clog2<B>())) << 3) + l;
}

template <int A, int B>
__device__ __forceinline__ void col_fwd_item(uint32_t *sm, const Desc &D, int g, const uint64_t *src, uint32_t *dst) {
    constexpr int R = A * B, RP = R + R / B;
    const int C = (int)D.C;
    const int np = (int)D.np;
    // NP >= 2W: the words at r C + c >= W, hence every row r >= R/2, are the product's zero
    // padding; only the lower half is converted and stored
    for (int e = threadIdx.x; e < (R / 2) * kG; e += blockDim.x) {
        const int r = e >> 3, l = e & 7;
        const uint32_t j = (uint32_t)r * C + g * kG + l;
        const uint64_t word = j < D.W ? src[j] : 0;
        for (int i = 0; i < np; i++) sm[col_addr<B>(i, RP, r, l)] = residue(word, D.pr[i]);
    }
    __syncthreads();
    for (int u = threadIdx.x; u < np * B * kG; u += blockDim.x) {
        const int l = u & 7, t = (u >> 3) & (B - 1), i = u >> (3 + clog2<B>());
        uint32_t x[A];
#pragma unroll
        for (int m = 0; m < A / 2; m++) x[m] = sm[col_addr<B>(i, RP, t + B * m, l)];
        dif_regs<A, false, true>(x, t, B, D.tb.twr_f[i], D.pr[i].p);
#pragma unroll
        for (int m = 0; m < A; m++) sm[col_addr<B>(i, RP, t + B * m, l)] = x[m];
    }
    __syncthreads();
    for (int u = threadIdx.x; u < np * A * kG; u += blockDim.x) {
        const int l = u & 7, t2 = (u >> 3) & (A - 1), i = u >> (3 + clog2<A>());
        uint32_t x[B];
#pragma unroll
        for (int m = 0; m < B; m++) x[m] = sm[col_addr<B>(i, RP, B * t2 + m, l)];
        dif_regs<B, true>(x, B * t2, 1, D.tb.twr_f[i], D.pr[i].p);
        const uint32_t p = D.pr[i].p;
#pragma unroll
        for (int m = 0; m < B; m++) {
            const uint32_t mm = (uint32_t)(B * t2 + m) * C + g * kG + l;  // storage position B t2 + m
            dst[(size_t)i * D.NP + mm] = shoup(x[m], __ldg(&D.tb.t4_f[i][mm]), p);
        }
    }
    __syncthreads();
}

// src overrides the test's operand (x, or y for the second operand of a product)
__global__ void __launch_bounds__(kColThreads) kn_col_fwd(const Desc *descs, const int2 *items, int nitems,
                                                          int second, const uint64_t *src_o) {
    extern __shared__ uint32_t sm[];
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 wi = items[it];
        const Desc &D = descs[wi.x];
        const uint64_t *src = src_o ? src_o : (second ? D.y : D.x);
        uint32_t *dst = second ? D.res2 : D.res;
        switch (log2i(D.R)) {
        case 3: col_fwd_item<2, 4>(sm, D, wi.y, src, dst); break;
        case 4: col_fwd_item<4, 4>(sm, D, wi.y, src, dst); break;
        case 5: col_fwd_item<4, 8>(sm, D, wi.y, src, dst); break;
        case 6: col_fwd_item<8, 8>(sm, D, wi.y, src, dst); break;
        case 7: col_fwd_item<8, 16>(sm, D, wi.y, src, dst); break;
        case 8: col_fwd_item<16, 16>(sm, D, wi.y, src, dst); break;
        case 9: col_fwd_item<16, 32>(sm, D, wi.y, src, dst); break;
        default: col_fwd_item<32, 32>(sm, D, wi.y, src, dst); break;
        }
    }
}

// Row layout in shared memory: [operand][prime][padded c].
template <int A, int B, bool MUL>
__device__ __forceinline__ void row_item(uint32_t *sm, const Desc &D, int pos) {
    constexpr int C = A * B, CP = C + C / B, lB = clog2<B>(), lA = clog2<A>();
    constexpr int nops = MUL ? 2 : 1;
    const int np = (int)D.np;
    // wide forward levels straight from global memory
    for (int u = threadIdx.x; u < nops * np * B; u += blockDim.x) {
        const int t = u & (B - 1), q = u >> lB, op = q >= np, i = q - op * np;
        const uint32_t *src = op ? D.res2 : D.res;
        const size_t base = (size_t)i * D.NP + (size_t)pos * C + t;
        uint32_t x[A];
#pragma unroll
        for (int m = 0; m < A; m++) x[m] = src[base + B * m];
        dif_regs<A, false>(x, t, B, D.tb.twc_f[i], D.pr[i].p);
        uint32_t *row = sm + (op * np + i) * CP;
#pragma unroll
        for (int m = 0; m < A; m++) row[t + B * m + m] = x[m];
    }
    __syncthreads();
    // narrow forward levels, the pointwise product, narrow inverse levels
    for (int u = threadIdx.x; u < np * A; u += blockDim.x) {
        const int t2 = u & (A - 1), i = u >> lA;
        uint32_t *row = sm + i * CP + (B + 1) * t2;
        const uint32_t p = D.pr[i].p, pinv = D.pr[i].pinv;
        uint32_t x[B];
#pragma unroll
        for (int m = 0; m < B; m++) x[m] = row[m];
        dif_regs<B, true>(x, B * t2, 1, D.tb.twc_f[i], p);
        if (MUL) {
            const uint32_t *rowy = sm + (np + i) * CP + (B + 1) * t2;
            uint32_t y[B];
#pragma unroll
            for (int m = 0; m < B; m++) y[m] = rowy[m];
            dif_regs<B, true>(y, B * t2, 1, D.tb.twc_f[i], p);
#pragma unroll
            for (int m = 0; m < B; m++) x[m] = montmul(x[m], y[m], p, pinv);
        } else {
#pragma unroll
            for (int m = 0; m < B; m++) x[m] = montmul(x[m], x[m], p, pinv);
        }
        dit_regs<B, true>(x, B * t2, 1, D.tb.twc_i[i], p);
#pragma unroll
        for (int m = 0; m < B; m++) row[m] = x[m];
    }
    __syncthreads();
    // wide inverse levels straight to global memory
    for (int u = threadIdx.x; u < np * B; u += blockDim.x) {
        const int t = u & (B - 1), i = u >> lB;
        const uint32_t *row = sm + i * CP;
        uint32_t x[A];
#pragma unroll
        for (int m = 0; m < A; m++) x[m] = row[t + B * m + m];
        dit_regs<A, false>(x, t, B, D.tb.twc_i[i], D.pr[i].p);
        const size_t base = (size_t)i * D.NP + (size_t)pos * C + t;
#pragma unroll
        for (int m = 0; m < A; m++) D.res[base + B * m] = x[m];
    }
    __syncthreads();
}

template <bool MUL>
__global__ void __launch_bounds__(kRowThreads) kn_rows(const Desc *descs, const int2 *items, int nitems) {
    extern __shared__ uint32_t sm[];
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 wi = items[it];
        const Desc &D = descs[wi.x];
        switch (log2i(D.C)) {
        case 3: row_item<2, 4, MUL>(sm, D, wi.y); break;
        case 4: row_item<4, 4, MUL>(sm, D, wi.y); break;
        case 5: row_item<4, 8, MUL>(sm, D, wi.y); break;
        case 6: row_item<8, 8, MUL>(sm, D, wi.y); break;
        case 7: row_item<8, 16, MUL>(sm, D, wi.y); break;
        case 8: row_item<16, 16, MUL>(sm, D, wi.y); break;
        case 9: row_item<16, 32, MUL>(sm, D, wi.y); break;
        default: row_item<32, 32, MUL>(sm, D, wi.y); break;
        }
    }
}

__device__ __forceinline__ uint32_t sub_mod(uint32_t a, uint32_t b, uint32_t p) {  // a, b in [0, p)
    return red2(a + p - b, p);
}

// exact coefficient from residues v_i in [0, p_i) (Garner's mixed radix)
__device__ __forceinline__ ulonglong2 garner(const uint32_t *v, const Desc &D) {
    const uint32_t p0 = D.pr[0].p, p1 = D.pr[1].p, p2 = D.pr[2].p, p3 = D.pr[3].p;
    const uint32_t x0 = v[0];
    const uint32_t x1 = red2(shoup(sub_mod(v[1], red2(x0, p1), p1), D.crt.inv01, p1), p1);
    uint32_t t = red2(shoup(sub_mod(v[2], red2(x0, p2), p2), D.crt.inv02, p2), p2);
    const uint32_t x2 = red2(shoup(sub_mod(t, red2(x1, p2), p2), D.crt.inv12, p2), p2);
    if (D.np == 3) {  // c = x0 + p0 (x1 + p1 x2) < 2^90
        const u128 c = (u128)x0 + (u128)p0 * ((u128)x1 + (u128)p1 * x2);
        return make_ulonglong2((unsigned long long)c, (unsigned long long)(c >> 64));
    }
    t = red2(shoup(sub_mod(v[3], red2(x0, p3), p3), D.crt.inv03, p3), p3);
    t = red2(shoup(sub_mod(t, red2(x1, p3), p3), D.crt.inv13, p3), p3);
    const uint32_t x3 = red2(shoup(sub_mod(t, red2(x2, p3), p3), D.crt.inv23, p3), p3);
    const uint64_t h = x2 + (uint64_t)p2 * x3;                 // < 2^60
    u128 c = (u128)x1 + (u128)p1 * h;                          // < 2^90
    c = (u128)x0 + (u128)p0 * c;                               // < 2^120
    return make_ulonglong2((unsigned long long)c, (unsigned long long)(c >> 64));
}

template <int A, int B>
__device__ __forceinline__ void col_inv_item(uint32_t *sm, const Desc &D, int g) {
    constexpr int R = A * B, RP = R + R / B;
    const int C = (int)D.C, np = (int)D.np;
    // narrow inverse levels straight from global memory, after the inverse four-step twiddle
    for (int u = threadIdx.x; u < np * A * kG; u += blockDim.x) {
        const int l = u & 7, t2 = (u >> 3) & (A - 1), i = u >> (3 + clog2<A>());
        const uint32_t p = D.pr[i].p;
        uint32_t x[B];
#pragma unroll
        for (int m = 0; m < B; m++) {
            const uint32_t mm = (uint32_t)(B * t2 + m) * C + g * kG + l;
            x[m] = shoup(D.res[(size_t)i * D.NP + mm], __ldg(&D.tb.t4_i[i][mm]), p);
        }
        dit_regs<B, true>(x, B * t2, 1, D.tb.twr_i[i], p);
#pragma unroll
        for (int m = 0; m < B; m++) sm[col_addr<B>(i, RP, B * t2 + m, l)] = x[m];
    }
    __syncthreads();
    // wide inverse levels
    for (int u = threadIdx.x; u < np * B * kG; u += blockDim.x) {
        const int l = u & 7, t = (u >> 3) & (B - 1), i = u >> (3 + clog2<B>());
        uint32_t x[A];
#pragma unroll
        for (int m = 0; m < A; m++) x[m] = sm[col_addr<B>(i, RP, t + B * m, l)];
        dit_regs<A, false>(x, t, B, D.tb.twr_i[i], D.pr[i].p);
#pragma unroll
        for (int m = 0; m < A; m++) sm[col_addr<B>(i, RP, t + B * m, l)] = x[m];
    }
    __syncthreads();
    // Row r of the group holds the coefficients r C + 8 g .. + 7, one per lane of an 8-lane group
    // of a warp.  Each lane splits its coefficient c_l < W 2^2w into w-bit parts lo + mid 2^w +
    // hi 2^2w (hi < W <= 2^20); word l of the segment collects s_l = lo_l + mid_(l-1) + hi_(l-2)
    // < 2^(w+2), so the carries between lanes are at most 3 and settle in 7 shuffle rounds.
    // Lane 7 also keeps what leaves the segment: mid_7 + hi_6 + hi_7 2^w plus its carry.
    const uint32_t w = D.w;
    const uint64_t M = (1ull << w) - 1;
    for (int e = threadIdx.x; e < R * kG; e += blockDim.x) {  // whole warps: R * kG is a multiple of 32
        const int r = e >> 3, l = e & 7;
        uint32_t v[kPrimes];
#pragma unroll
        for (int i = 0; i < kPrimes; i++) v[i] = i < np ? red2(sm[col_addr<B>(i, RP, r, l)], D.pr[i].p) : 0;
        const ulonglong2 c2 = garner(v, D);
        const u128 c = ((u128)c2.y << 64) | c2.x;
        const uint64_t lo = (uint64_t)c & M, mid = (uint64_t)(c >> w) & M;
        const uint32_t hi = (uint32_t)(c >> (2 * w));
        const uint32_t mid_lo = __shfl_up_sync(0xffffffffu, (uint32_t)mid, 1, kG);
        const uint32_t mid_hi = __shfl_up_sync(0xffffffffu, (uint32_t)(mid >> 32), 1, kG);
        const uint32_t hi1 = __shfl_up_sync(0xffffffffu, hi, 1, kG);
        const uint32_t hi2 = __shfl_up_sync(0xffffffffu, hi, 2, kG);
        const uint64_t sl = lo + (l >= 1 ? ((uint64_t)mid_hi << 32 | mid_lo) : 0) + (l >= 2 ? hi2 : 0);
        const uint64_t rl = sl & M;
        const uint32_t gl = (uint32_t)(sl >> w);
        uint32_t cout = gl;
#pragma unroll
        for (int round = 0; round < kG - 1; round++) {
            const uint32_t cin = __shfl_up_sync(0xffffffffu, cout, 1, kG);
            cout = gl + (uint32_t)((rl + (l ? cin : 0)) >> w);
        }
        const uint32_t cin = __shfl_up_sync(0xffffffffu, cout, 1, kG);
        const uint32_t j = (uint32_t)r * C + g * kG + l;
        D.pw[j] = (rl + (l ? cin : 0)) & M;
        if (l == kG - 1) {
            const u128 out = (u128)mid + hi1 + cout + ((u128)hi << w);
            D.seg[j >> 3] = make_ulonglong2((unsigned long long)out, (unsigned long long)(out >> 64));
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kColThreads) kn_col_inv(const Desc *descs, const int2 *items, int nitems) {
    extern __shared__ uint32_t sm[];
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int2 wi = items[it];
        const Desc &D = descs[wi.x];
        switch (log2i(D.R)) {
        case 3: col_inv_item<2, 4>(sm, D, wi.y); break;
        case 4: col_inv_item<4, 4>(sm, D, wi.y); break;
        case 5: col_inv_item<4, 8>(sm, D, wi.y); break;
        case 6: col_inv_item<8, 8>(sm, D, wi.y); break;
        case 7: col_inv_item<8, 16>(sm, D, wi.y); break;
        case 8: col_inv_item<16, 16>(sm, D, wi.y); break;
        case 9: col_inv_item<16, 32>(sm, D, wi.y); break;
        default: col_inv_item<32, 32>(sm, D, wi.y); break;
        }
    }
}

// Carries pending at chunk boundaries: co[t] is the carry out of chunk t (S words at t S) into
// chunk t + 1.  Adds them in until none is left; returns (in every thread) the carry that left
// the top of v.  A carry moves up at least one chunk per round, so T + 1 rounds always suffice;
// the loop stops there in any case and reports bit 4 in *status if carries were still pending.
__device__ u128 resolve_chunks(uint64_t *v, uint32_t len, uint32_t S, uint32_t w, u128 *co, u128 *top,
                               int *status) {
    const int t = threadIdx.x, T = blockDim.x;
    const uint64_t M = (w == 64) ? ~0ull : ((1ull << w) - 1);
    if (t == 0) *top = 0;
    for (int round = 0;; round++) {
        if (round > T + 1) {
            if (t == 0) atomicOr(status, 4);
            break;
        }
        __syncthreads();
        const u128 cin = t > 0 ? co[t - 1] : 0;
        if (t == T - 1) *top += co[T - 1];
        __syncthreads();
        u128 acc = cin;
        uint32_t j = (uint32_t)t * S;
        const uint32_t e = min(len, j + S);
        for (; acc != 0 && j < e; j++) {
            acc += v[j];
            v[j] = (uint64_t)acc & M;
            acc >>= w;
        }
        co[t] = acc;
        if (!__syncthreads_or(acc != 0)) break;
    }
    __syncthreads();
    return *top;
}

// x_o, add_o override the test's result array and addend
__global__ void __launch_bounds__(kReduceThreads) kn_reduce(const Desc *descs, const int *tests, uint64_t *x_o,
                                                            const uint64_t *add_o) {
    __shared__ u128 co[kReduceThreads];
    __shared__ u128 top;
    const Desc &D = descs[tests[blockIdx.x]];
    uint64_t *X = x_o ? x_o : D.x;
    const uint64_t *addend = x_o ? add_o : D.addend;
    const int t = threadIdx.x, T = blockDim.x;
    const uint32_t w = D.w;
    const uint64_t M = (1ull << w) - 1;
    // The descriptor's fields are read once: the stores below go through global pointers the
    // compiler cannot tell apart from the descriptor.
    const uint32_t NP = D.NP, Wn = D.W, WN0 = D.WN0, BN0 = D.BN0;
    const uint64_t kk = D.k;
    const ulonglong2 *__restrict__ seg = D.seg;
    uint64_t *__restrict__ pw = D.pw;
    int *status = D.status;
    constexpr int U = 8;  // loads in flight per thread
    // 1. product words: the transform kernels left P as 8-word segments, each normalised, with
    //    the carry out of segment s in seg[s]; add every segment's carry into the next one
    {
        const uint32_t nseg = NP >> 3, per = (nseg + T - 1) / T;
        const uint32_t s0 = (uint32_t)t * per, s1 = min(nseg, s0 + per);
        ulonglong2 *__restrict__ pw2 = reinterpret_cast<ulonglong2 *>(pw);
        u128 acc = 0;
        // A segment's carry (< 2^(w+20)) almost always settles within the segment's first two
        // words.  So SB segments at a time, their carries and first two words are loaded
        // together before the carry walks through them: a thread waits for memory about once
        // per batch instead of once per word; the rare longer carries continue word by word.
        constexpr int SB = 4;
        for (uint32_t sb = s0; sb < s1; sb += SB) {
            ulonglong2 c[SB], v[SB];
#pragma unroll
            for (int q = 0; q < SB; q++) {
                const uint32_t sg = sb + q;
                const bool in = sg < s1;
                c[q] = in && sg > s0 ? seg[sg - 1] : make_ulonglong2(0, 0);
                v[q] = in ? pw2[sg * 4] : make_ulonglong2(0, 0);
            }
#pragma unroll
            for (int q = 0; q < SB; q++) {
                const uint32_t sg = sb + q;
                if (sg >= s1) break;
                acc += ((u128)c[q].y << 64) | c[q].x;
                if (acc == 0) continue;  // words below 2^w: a zero carry leaves them as they are
                acc += v[q].x;
                v[q].x = (uint64_t)acc & M;
                acc >>= w;
                acc += v[q].y;
                v[q].y = (uint64_t)acc & M;
                acc >>= w;
                pw2[sg * 4] = v[q];
                for (uint32_t j = (sg << 3) + 2; acc != 0 && j < (sg << 3) + 8; j++) {
                    acc += pw[j];
                    pw[j] = (uint64_t)acc & M;
                    acc >>= w;
                }
            }
        }
        if (s1 > s0) {
            const ulonglong2 c = seg[s1 - 1];
            acc += ((u128)c.y << 64) | c.x;
        }
        co[t] = acc;
        if (resolve_chunks(pw, NP, per << 3, w, co, &top, status) != 0 && t == 0) atomicOr(status, 1);
    }
    // 2. Montgomery reduction E = B + k A (+ addend), P = A + B 2^n
    {
        const uint32_t S = (Wn + T - 1) / T;
        const uint64_t lowmask = (1ull << BN0) - 1;
        u128 acc = 0;
        const uint32_t j0 = (uint32_t)t * S, e = min(Wn, j0 + S);
        for (uint32_t j = j0; j < e; j += U) {
            uint64_t a[U], bw[U + 1], ad[U];
#pragma unroll
            for (int q = 0; q < U; q++) {
                const uint32_t jj = j + q;
                a[q] = jj < WN0 ? pw[jj] : (jj == WN0 ? (pw[jj] & lowmask) : 0);
                ad[q] = addend && jj < e ? addend[jj] : 0;
            }
#pragma unroll
            for (int q = 0; q <= U; q++) {
                const uint32_t s2 = WN0 + j + q;
                bw[q] = s2 < NP ? pw[s2] : 0;
            }
#pragma unroll
            for (int q = 0; q < U; q++) {
                if (j + q >= e) break;
                const uint64_t b = BN0 ? (((bw[q] >> BN0) | (bw[q + 1] << (w - BN0))) & M) : bw[q];
                acc += (u128)b + (u128)kk * a[q] + ad[q];
                X[j + q] = (uint64_t)acc & M;
                acc >>= w;
            }
        }
        co[t] = acc;
        if (resolve_chunks(X, Wn, S, w, co, &top, status) != 0 && t == 0) atomicOr(status, 2);
    }
    // 3. top fold: T = x >> n = q k + r; x <- x mod 2^n + q + r 2^n
    if (t == 0) {
        uint64_t *x = X;
        u128 Tv = x[WN0] >> BN0;
        uint32_t sh = w - BN0;
        for (uint32_t j = WN0 + 1; j < Wn; j++) {
            if (x[j]) {
                if (sh >= 128 || (sh > 64 && (x[j] >> (128 - sh)) != 0)) atomicOr(status, 4);
                else Tv |= (u128)x[j] << sh;
            }
            sh += w;
            x[j] = 0;
        }
        x[WN0] &= (1ull << BN0) - 1;
        u128 q;
        uint64_t r;
        if ((uint64_t)(Tv >> 64) == 0) {  // always for k < 2^30: T < 2^(2 log2 k + 3)
            const uint64_t t64 = (uint64_t)Tv;
            q = t64 / kk;
            r = t64 - (uint64_t)q * kk;
        } else {
            q = Tv / kk;
            r = (uint64_t)(Tv - q * kk);
        }
        u128 add = (u128)r << BN0;
        for (uint32_t j = WN0; add != 0 && j < Wn; j++) {
            add += x[j];
            x[j] = (uint64_t)add & M;
            add >>= w;
        }
        if (add) atomicOr(status, 8);
        add = q;
        for (uint32_t j = 0; add != 0 && j < Wn; j++) {
            add += x[j];
            x[j] = (uint64_t)add & M;
            add >>= w;
        }
        if (add) atomicOr(status, 8);
    }
}

// ---- host tables ------------------------------------------------------------------------------

uint32_t mulmod(uint32_t a, uint32_t b, uint32_t p) { return (uint32_t)((uint64_t)a * b % p); }
uint32_t powmod(uint32_t a, uint64_t e, uint32_t p) {
    uint32_t r = 1 % p;
    for (; e; e >>= 1, a = mulmod(a, a, p))
        if (e & 1) r = mulmod(r, a, p);
    return r;
}
uint32_t invmod(uint32_t a, uint32_t p) { return powmod(a % p, p - 2, p); }
uint2 shoup_pair(uint32_t w, uint32_t p) { return make_uint2(w, (uint32_t)(((uint64_t)w << 32) / p)); }

// a generator of the multiplicative group mod p (p - 1 = m 2^e with m's prime factors small)
uint32_t generator(uint32_t p) {
    std::vector<uint32_t> f;
    uint32_t m = p - 1;
    for (uint32_t q = 2; q * q <= m; q++)
        if (m % q == 0) {
            f.push_back(q);
            while (m % q == 0) m /= q;
        }
    if (m > 1) f.push_back(m);
    for (uint32_t g = 2;; g++) {
        bool ok = true;
        for (uint32_t q : f)
            if (powmod(g, (p - 1) / q, p) == 1) {
                ok = false;
                break;
            }
        if (ok) return g;
    }
}

uint32_t bitrev(uint32_t x, int bits) {
    uint32_t r = 0;
    for (int b = 0; b < bits; b++) r |= ((x >> b) & 1u) << (bits - 1 - b);
    return r;
}

int ilog2(uint32_t x) {
    int b = 0;
    while ((1u << b) < x) b++;
    return b;
}

// shared memory of the transform kernels for a length-n transform split A x B (B = 2^ceil(log2 n / 2)),
// stored padded: n + n / B elements
size_t padded_len(uint32_t n) {
    const int l = ilog2(n);
    return (size_t)n + (n >> ((l + 1) / 2));
}
size_t col_smem_bytes(uint32_t R) { return (size_t)kPrimes * padded_len(R) * kG * 4; }
size_t row_smem_bytes(uint32_t C) { return (size_t)kPrimes * padded_len(C) * 4; }

struct Plan {
    uint32_t NP = 0, R = 0, C = 0;
    uint2 *d_tables = nullptr;  // one allocation for every table
    Tables tb{};
    ~Plan() {
        if (d_tables) cudaFree(d_tables);
    }
};

// level tables of a length-n transform: [s + j] = w_2s^(dir j), s = 1, 2, .., n/2, j < s
void level_table(std::vector<uint2> &out, uint32_t n, uint32_t wn, uint32_t p) {
    // wn: a primitive n-th root; w_2s = wn^(n / 2s)
    out.assign(n, make_uint2(0, 0));
    for (uint32_t s = 1; s < n; s <<= 1) {
        const uint32_t w2s = powmod(wn, n / (2 * s), p);
        uint32_t v = 1;
        for (uint32_t j = 0; j < s; j++, v = mulmod(v, w2s, p)) out[s + j] = shoup_pair(v, p);
    }
}

std::mutex g_plan_mu;
std::map<std::pair<int, uint32_t>, std::shared_ptr<Plan>> g_plans;

std::shared_ptr<Plan> get_plan(int device, uint32_t NP) {
    std::lock_guard<std::mutex> lock(g_plan_mu);
    auto key = std::make_pair(device, NP);
    auto itp = g_plans.find(key);
    if (itp != g_plans.end()) return itp->second;
    auto P = std::make_shared<Plan>();
    P->NP = NP;
    const int a = ilog2(NP);
    P->R = 1u << (a / 2);
    P->C = NP / P->R;
    const uint32_t R = P->R, C = P->C;
    const int logR = ilog2(R);
    // layout per prime: twr_f[R], twr_i[R], twc_f[C], twc_i[C], t4_f[NP], t4_i[NP]
    const size_t per = 2 * (size_t)R + 2 * (size_t)C + 2 * (size_t)NP;
    std::vector<uint2> host(per * kPrimes);
    std::vector<uint2> tmp;
    for (int i = 0; i < kPrimes; i++) {
        const uint32_t p = kP[i];
        const uint32_t g = generator(p);
        const uint32_t wN = powmod(g, (p - 1) / NP, p), wNi = invmod(wN, p);
        uint2 *base = host.data() + per * i;
        level_table(tmp, R, powmod(wN, C, p), p);
        std::copy(tmp.begin(), tmp.end(), base);
        level_table(tmp, R, powmod(wNi, C, p), p);
        std::copy(tmp.begin(), tmp.end(), base + R);
        level_table(tmp, C, powmod(wN, R, p), p);
        std::copy(tmp.begin(), tmp.end(), base + 2 * R);
        level_table(tmp, C, powmod(wNi, R, p), p);
        std::copy(tmp.begin(), tmp.end(), base + 2 * R + C);
        // four-step twiddles in storage order: position pos holds frequency k_r = bitrev(pos)
        const uint32_t scale = mulmod(invmod(NP % p, p), (uint32_t)((1ull << 32) % p), p);
        uint2 *t4f = base + 2 * R + 2 * C, *t4i = t4f + NP;
        for (uint32_t pos = 0; pos < R; pos++) {
            const uint32_t kr = bitrev(pos, logR);
            const uint32_t a1 = powmod(wN, kr, p), a1i = powmod(wNi, kr, p);
            uint32_t v = 1, vi = scale;
            for (uint32_t c = 0; c < C; c++) {
                t4f[pos * C + c] = shoup_pair(v, p);
                t4i[pos * C + c] = shoup_pair(vi, p);
                v = mulmod(v, a1, p);
                vi = mulmod(vi, a1i, p);
            }
        }
    }
    if (cudaMalloc((void **)&P->d_tables, host.size() * sizeof(uint2)) != cudaSuccess) return nullptr;
    if (cudaMemcpy(P->d_tables, host.data(), host.size() * sizeof(uint2), cudaMemcpyHostToDevice) != cudaSuccess)
        return nullptr;
    for (int i = 0; i < kPrimes; i++) {
        const uint2 *base = P->d_tables + per * i;
        P->tb.twr_f[i] = base;
        P->tb.twr_i[i] = base + R;
        P->tb.twc_f[i] = base + 2 * R;
        P->tb.twc_i[i] = base + 2 * R + C;
        P->tb.t4_f[i] = base + 2 * R + 2 * C;
        P->tb.t4_i[i] = base + 2 * R + 2 * C + NP;
    }
    g_plans[key] = P;
    return P;
}

// ---- exact host integers (64-bit limbs) -------------------------------------------------------

// N = k 2^n - 1 in nl limbs
std::vector<uint64_t> modulus(uint64_t k, uint64_t n, size_t nl) {
    std::vector<uint64_t> N(nl, 0);
    const u128 kk = (u128)k << (n % 64);
    N[n / 64] = (uint64_t)kk;
    if (n / 64 + 1 < nl) N[n / 64 + 1] = (uint64_t)(kk >> 64);
    for (size_t j = 0; j < nl; j++)
        if (N[j]--) break;
    return N;
}

bool geq(const std::vector<uint64_t> &a, const std::vector<uint64_t> &b) {
    for (size_t j = a.size(); j-- > 0;)
        if (a[j] != b[j]) return a[j] > b[j];
    return true;
}

void sub_in(std::vector<uint64_t> &a, const std::vector<uint64_t> &b) {
    uint64_t br = 0;
    for (size_t j = 0; j < a.size(); j++) {
        const u128 d = (u128)a[j] - b[j] - br;
        a[j] = (uint64_t)d;
        br = (uint64_t)(d >> 64) ? 1 : 0;
    }
}

// The sizes of a number of the engine for N = k 2^n - 1 and the modulus itself: host-only.
struct NumLayout {
    uint64_t k = 0, n = 0;
    uint32_t np = 0, W = 0, w = 0, NP = 0;
    size_t nlimbs = 0;
    std::vector<uint64_t> N;  // modulus, nlimbs limbs
    bool build(uint64_t k, uint64_t n);
};

}  // namespace kn

using namespace kn;

struct kn_engine : kn::NumLayout {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::shared_ptr<Plan> plan;
    Desc desc{};
    Desc *d_desc = nullptr;
    int2 *d_cols = nullptr, *d_rows = nullptr;
    int *d_test = nullptr;
    int *d_status = nullptr;
    uint32_t *d_res = nullptr, *d_res2 = nullptr;
    ulonglong2 *d_seg = nullptr;
    uint64_t *d_pw = nullptr;
    uint64_t *d_addend = nullptr;
    int64_t addend_c = 0;
    bool addend_ok = false;
    int err = 0;
};

namespace {

bool kok(kn_engine *e, cudaError_t c) {
    if (c != cudaSuccess && !e->err) e->err = (int)c;
    return c == cudaSuccess;
}

// x = sum words[j] 2^(w j) as nl limbs (words may be up to 64 bits wide)
void words_to_limbs(const uint64_t *words, uint32_t W, uint32_t w, std::vector<uint64_t> &l) {
    std::fill(l.begin(), l.end(), 0);
    for (uint32_t j = 0; j < W; j++) {
        const uint64_t bit = (uint64_t)w * j;
        const size_t li = bit / 64;
        const unsigned sh = bit % 64;
        u128 v = (u128)words[j] << sh;
        for (size_t t = li; v != 0 && t < l.size(); t++) {
            v += l[t];
            l[t] = (uint64_t)v;
            v >>= 64;
        }
    }
}

void limbs_to_words(const std::vector<uint64_t> &l, uint32_t W, uint32_t w, uint64_t *words) {
    const uint64_t M = (1ull << w) - 1;
    for (uint32_t j = 0; j < W; j++) {
        const uint64_t bit = (uint64_t)w * j;
        const size_t li = bit / 64;
        const unsigned sh = bit % 64;
        u128 v = li < l.size() ? (u128)l[li] : 0;
        if (li + 1 < l.size()) v |= (u128)l[li + 1] << 64;
        words[j] = (uint64_t)(v >> sh) & M;
    }
}

// v mod N for v of any size (limbs, little endian), using k 2^n == 1: v = T 2^n + L,
// T = q k + r -> v == L + q + r 2^n
void reduce_mod(const NumLayout *e, std::vector<uint64_t> v, std::vector<uint64_t> &out) {
    const uint64_t n = e->n, k = e->k;
    for (;;) {
        // T = v >> n
        const size_t s0 = n / 64;
        const unsigned sh = n % 64;
        std::vector<uint64_t> T;
        for (size_t j = s0; j < v.size(); j++) {
            u128 cur = v[j] >> sh;
            if (sh && j + 1 < v.size()) cur |= (u128)v[j + 1] << (64 - sh);
            T.push_back((uint64_t)cur);
        }
        while (!T.empty() && T.back() == 0) T.pop_back();
        if (T.empty() || (T.size() == 1 && T[0] < k)) break;  // v < k 2^n = N + 1
        // L = v mod 2^n
        v.resize(s0 + 1);
        v[s0] &= sh ? ((1ull << sh) - 1) : 0;
        if (!sh) v.resize(s0);
        // q = T / k, r = T mod k
        u128 rem = 0;
        for (size_t j = T.size(); j-- > 0;) {
            const u128 cur = (rem << 64) | T[j];
            T[j] = (uint64_t)(cur / k);
            rem = cur % k;
        }
        // v += q + r 2^n
        const size_t need = std::max(v.size(), T.size()) + (n + 64) / 64 + 2;
        v.resize(need, 0);
        u128 c = 0;
        for (size_t j = 0; j < v.size(); j++) {
            c += (u128)v[j] + (j < T.size() ? T[j] : 0);
            v[j] = (uint64_t)c;
            c >>= 64;
        }
        u128 add = (u128)(uint64_t)rem << sh;
        for (size_t j = s0; add != 0 && j < v.size(); j++) {
            add += v[j];
            v[j] = (uint64_t)add;
            add >>= 64;
        }
        while (v.size() > e->nlimbs && v.back() == 0) v.pop_back();
    }
    v.resize(e->nlimbs + 1, 0);
    std::vector<uint64_t> N = e->N;
    N.resize(e->nlimbs + 1, 0);
    while (geq(v, N)) sub_in(v, N);
    out.assign(v.begin(), v.begin() + e->nlimbs);
}

// Montgomery form x~ = x 2^n mod N of x in [0, N): x = q k + r -> x 2^n == q + r 2^n
void to_mont(const NumLayout *e, const uint64_t *limbs, std::vector<uint64_t> &out) {
    std::vector<uint64_t> q(limbs, limbs + e->nlimbs);
    u128 rem = 0;
    for (size_t j = q.size(); j-- > 0;) {
        const u128 cur = (rem << 64) | q[j];
        q[j] = (uint64_t)(cur / e->k);
        rem = cur % e->k;
    }
    q.resize(e->nlimbs + 2, 0);
    u128 add = (u128)(uint64_t)rem << (e->n % 64);
    for (size_t j = e->n / 64; add != 0 && j < q.size(); j++) {
        add += q[j];
        q[j] = (uint64_t)add;
        add >>= 64;
    }
    out.swap(q);
}

// A constant c as Montgomery words (a representative in [0, N)).
bool constant_words(const NumLayout *e, int64_t c, std::vector<uint64_t> &words) {
    std::vector<uint64_t> v(e->nlimbs, 0);
    if (c >= 0) {
        v[0] = (uint64_t)c;
    } else {
        v = e->N;
        std::vector<uint64_t> m(e->nlimbs, 0);
        m[0] = (uint64_t)(-c);
        sub_in(v, m);
    }
    std::vector<uint64_t> mont;
    to_mont(e, v.data(), mont);
    std::vector<uint64_t> red;
    reduce_mod(e, mont, red);  // keep the representative below N
    words.assign(e->W, 0);
    limbs_to_words(red, e->W, e->w, words.data());
    return true;
}

// Primes, word size and transform length for n: the fewest prime-points (primes x NP, NP the
// shortest power-of-2 length >= 2W), then the largest word w <= 50, subject to every convolution
// coefficient staying below the product of the primes in use (W (2^w - 1)^2 < p_0 ... p_(np-1))
// and W w leaving room for n + 2 log2 k + 8 bits.
void choose_sizes(uint64_t k, uint64_t n, uint32_t &np, uint32_t &w, uint32_t &W, uint32_t &NP) {
    int kb = 0;
    while (kb < 63 && (k >> kb) > 0) kb++;
    const uint64_t bits = n + 2 * (uint64_t)kb + 8;
    uint64_t best = 0;
    NP = 0;
    for (uint32_t q = 3; q <= (uint32_t)kPrimes; q++) {
        u128 prod = 1;
        for (uint32_t i = 0; i < q; i++) prod *= kP[i];
        for (uint32_t ww = 50; ww >= 24; ww--) {
            const uint64_t Wc = (bits + ww - 1) / ww;
            const u128 bound = (u128)Wc * (((u128)1 << ww) - 1) * (((u128)1 << ww) - 1);
            if (bound >= prod) continue;
            uint64_t len = 64;
            while (len < 2 * Wc) len <<= 1;
            const uint64_t cost = len * q;
            if (!best || cost < best) {
                best = cost;
                np = q;
                w = ww;
                W = (uint32_t)Wc;
                NP = (uint32_t)len;
            }
        }
    }
}

// The dynamic shared-memory limit is a per-kernel property of the device's context, shared by
// every engine and group of the process: raise it, never lower it, so a small engine created
// later cannot break a larger group's captured launches.
bool prepare_smem(int device, size_t col_smem, size_t row_smem) {
    static std::mutex mu;
    static size_t col_hw[64] = {}, row_hw[64] = {};
    if (device < 0 || device >= 64) return false;
    std::lock_guard<std::mutex> lock(mu);
    bool ok = true;
    if (col_smem > col_hw[device]) {
        ok = ok && cudaFuncSetAttribute(kn_col_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)col_smem) == cudaSuccess;
        ok = ok && cudaFuncSetAttribute(kn_col_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)col_smem) == cudaSuccess;
        if (ok) col_hw[device] = col_smem;
    }
    if (row_smem > row_hw[device]) {
        ok = ok && cudaFuncSetAttribute(kn_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem) == cudaSuccess;
        ok = ok && cudaFuncSetAttribute(kn_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)row_smem) == cudaSuccess;
        if (ok) row_hw[device] = row_smem;
    }
    return ok;
}

// x~ (W words of w bits) -> x = x~ 2^-n = x~ k (mod N) as canonical limbs
void from_mont(const NumLayout *e, const uint64_t *words, uint64_t *limbs) {
    std::vector<uint64_t> v((size_t)e->W * e->w / 64 + 3, 0);
    words_to_limbs(words, e->W, e->w, v);
    u128 c = 0;
    for (auto &l : v) {
        c += (u128)l * e->k;
        l = (uint64_t)c;
        c >>= 64;
    }
    v.push_back((uint64_t)c);
    std::vector<uint64_t> out;
    reduce_mod(e, v, out);
    std::copy(out.begin(), out.end(), limbs);
}

}  // namespace

bool kn::NumLayout::build(uint64_t kk, uint64_t nn) {
    if (!(kk & 1) || kk >= (1ull << 30) || nn < 8 || nn > (1ull << 26)) return false;
    k = kk;
    n = nn;
    choose_sizes(k, n, np, w, W, NP);
    if (!NP || NP > (1u << 20)) return false;
    nlimbs = (size_t)((n + 64 + 63) / 64);
    N = modulus(k, n, nlimbs);
    return true;
}

extern "C" {

int kn_layout(uint64_t k, uint64_t n, uint32_t *primes, uint32_t *w, uint32_t *W, uint32_t *NP) {
    NumLayout y;
    if (!y.build(k, n)) return -1;
    if (primes) *primes = y.np;
    if (w) *w = y.w;
    if (W) *W = y.W;
    if (NP) *NP = y.NP;
    return 0;
}

int kn_limbs_to_words(uint64_t k, uint64_t n, const uint64_t *limbs, uint64_t *words) {
    NumLayout y;
    if (!y.build(k, n)) return -1;
    std::vector<uint64_t> mont;
    to_mont(&y, limbs, mont);
    limbs_to_words(mont, y.W, y.w, words);
    return 0;
}

int kn_words_to_limbs(uint64_t k, uint64_t n, const uint64_t *words, uint64_t *limbs) {
    NumLayout y;
    if (!y.build(k, n)) return -1;
    from_mont(&y, words, limbs);
    return 0;
}

kn_engine *kn_engine_new(uint64_t k, uint64_t n, int device) {
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return nullptr;
    kn_engine *e = new (std::nothrow) kn_engine();
    if (!e) return nullptr;
    e->device = device;
    if (!e->build(k, n)) {
        delete e;
        return nullptr;
    }
    e->plan = get_plan(device, e->NP);
    if (!e->plan) {
        delete e;
        return nullptr;
    }
    const uint32_t R = e->plan->R, C = e->plan->C, NP = e->NP;
    bool ok = kok(e, cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) &&
              kok(e, cudaMalloc((void **)&e->d_desc, sizeof(Desc))) &&
              kok(e, cudaMalloc((void **)&e->d_res, (size_t)kPrimes * NP * 4)) &&
              kok(e, cudaMalloc((void **)&e->d_res2, (size_t)kPrimes * NP * 4)) &&
              kok(e, cudaMalloc((void **)&e->d_seg, (size_t)(NP / kG) * sizeof(ulonglong2))) &&
              kok(e, cudaMalloc((void **)&e->d_pw, (size_t)NP * 8)) &&
              kok(e, cudaMalloc((void **)&e->d_addend, (size_t)e->W * 8)) &&
              kok(e, cudaMalloc((void **)&e->d_status, sizeof(int))) &&
              kok(e, cudaMalloc((void **)&e->d_cols, (C / kG) * sizeof(int2))) &&
              kok(e, cudaMalloc((void **)&e->d_rows, R * sizeof(int2))) &&
              kok(e, cudaMalloc((void **)&e->d_test, sizeof(int)));
    if (ok) {
        std::vector<int2> cols(C / kG), rows(R);
        for (uint32_t g = 0; g < C / kG; g++) cols[g] = make_int2(0, (int)g);
        for (uint32_t r = 0; r < R; r++) rows[r] = make_int2(0, (int)r);
        const int zero = 0;
        ok = kok(e, cudaMemcpy(e->d_cols, cols.data(), cols.size() * sizeof(int2), cudaMemcpyHostToDevice)) &&
             kok(e, cudaMemcpy(e->d_rows, rows.data(), rows.size() * sizeof(int2), cudaMemcpyHostToDevice)) &&
             kok(e, cudaMemcpy(e->d_test, &zero, sizeof zero, cudaMemcpyHostToDevice)) &&
             kok(e, cudaMemcpy(e->d_status, &zero, sizeof zero, cudaMemcpyHostToDevice));
    }
    if (ok) ok = prepare_smem(device, col_smem_bytes(R), 2 * row_smem_bytes(C));
    if (!ok) {
        kn_engine_free(e);
        return nullptr;
    }
    Desc &d = e->desc;
    d.NP = NP;
    d.np = e->np;
    d.R = R;
    d.C = C;
    d.W = e->W;
    d.w = e->w;
    d.WN0 = (uint32_t)(n / e->w);
    d.BN0 = (uint32_t)(n % e->w);
    d.k = k;
    d.res = e->d_res;
    d.res2 = e->d_res2;
    d.seg = e->d_seg;
    d.pw = e->d_pw;
    d.status = e->d_status;
    d.tb = e->plan->tb;
    for (int i = 0; i < kPrimes; i++) {
        const uint32_t p = kP[i];
        uint32_t inv = 1;
        for (int t = 0; t < 5; t++) inv *= 2 - p * inv;  // p^-1 mod 2^32 by Newton steps
        d.pr[i].p = p;
        d.pr[i].pinv = (uint32_t)(0u - inv);
        d.pr[i].one = shoup_pair(1, p);
        d.pr[i].r32 = shoup_pair((uint32_t)((1ull << 32) % p), p);
    }
    d.crt.inv01 = shoup_pair(invmod(kP[0] % kP[1], kP[1]), kP[1]);
    d.crt.inv02 = shoup_pair(invmod(kP[0] % kP[2], kP[2]), kP[2]);
    d.crt.inv12 = shoup_pair(invmod(kP[1] % kP[2], kP[2]), kP[2]);
    d.crt.inv03 = shoup_pair(invmod(kP[0] % kP[3], kP[3]), kP[3]);
    d.crt.inv13 = shoup_pair(invmod(kP[1] % kP[3], kP[3]), kP[3]);
    d.crt.inv23 = shoup_pair(invmod(kP[2] % kP[3], kP[3]), kP[3]);
    // operands are kernel arguments: the descriptor is written once
    if (!kok(e, cudaMemcpy(e->d_desc, &d, sizeof d, cudaMemcpyHostToDevice))) {
        kn_engine_free(e);
        return nullptr;
    }
    return e;
}

void kn_engine_free(kn_engine *e) {
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    for (void *p : {(void *)e->d_desc, (void *)e->d_res, (void *)e->d_res2, (void *)e->d_seg, (void *)e->d_pw,
                    (void *)e->d_addend, (void *)e->d_status, (void *)e->d_cols, (void *)e->d_rows, (void *)e->d_test})
        if (p) cudaFree(p);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

uint32_t kn_num_words(const kn_engine *e) { return e ? e->W : 0; }
uint32_t kn_word_bits(const kn_engine *e) { return e ? e->w : 0; }
uint32_t kn_transform_len(const kn_engine *e) { return e ? e->NP : 0; }
size_t kn_limbs(const kn_engine *e) { return e ? e->nlimbs : 0; }

uint64_t *kn_num_alloc(kn_engine *e) {
    if (!e || e->err) return nullptr;
    cudaSetDevice(e->device);
    uint64_t *x = nullptr;
    if (!kok(e, cudaMalloc((void **)&x, (size_t)e->W * 8))) return nullptr;
    if (!kok(e, cudaMemsetAsync(x, 0, (size_t)e->W * 8, e->stream))) {
        cudaFree(x);
        return nullptr;
    }
    return x;
}

void kn_num_free(kn_engine *e, uint64_t *x) {
    if (!e || !x) return;
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    cudaFree(x);
}

int kn_set_limbs(kn_engine *e, uint64_t *x, const uint64_t *limbs) {
    if (!e || e->err) return -1;
    std::vector<uint64_t> mont;
    to_mont(e, limbs, mont);
    std::vector<uint64_t> words(e->W);
    limbs_to_words(mont, e->W, e->w, words.data());
    cudaSetDevice(e->device);
    if (!kok(e, cudaMemcpyAsync(x, words.data(), (size_t)e->W * 8, cudaMemcpyHostToDevice, e->stream))) return -1;
    return kok(e, cudaStreamSynchronize(e->stream)) ? 0 : -1;
}

int kn_get_limbs(kn_engine *e, const uint64_t *x, uint64_t *limbs) {
    if (!e || e->err) return -1;
    std::vector<uint64_t> words(e->W);
    cudaSetDevice(e->device);
    if (!kok(e, cudaMemcpyAsync(words.data(), x, (size_t)e->W * 8, cudaMemcpyDeviceToHost, e->stream)) ||
        !kok(e, cudaStreamSynchronize(e->stream)))
        return -1;
    int st = 0;
    if (!kok(e, cudaMemcpy(&st, e->d_status, sizeof st, cudaMemcpyDeviceToHost))) return -1;
    if (st) {
        e->err = -100 - st;
        return -1;
    }
    from_mont(e, words.data(), limbs);
    return 0;
}

static int run_product(kn_engine *e, uint64_t *x, const uint64_t *y, const uint64_t *addend) {
    const uint32_t R = e->plan->R, C = e->plan->C;
    const size_t col_smem = col_smem_bytes(R), row_smem = row_smem_bytes(C);
    const int ncols = (int)(C / kG), nrows = (int)R;
    kn_col_fwd<<<ncols, kColThreads, col_smem, e->stream>>>(e->d_desc, e->d_cols, ncols, 0, x);
    if (y) {
        kn_col_fwd<<<ncols, kColThreads, col_smem, e->stream>>>(e->d_desc, e->d_cols, ncols, 1, y);
        kn_rows<true><<<nrows, kRowThreads, 2 * row_smem, e->stream>>>(e->d_desc, e->d_rows, nrows);
    } else {
        kn_rows<false><<<nrows, kRowThreads, row_smem, e->stream>>>(e->d_desc, e->d_rows, nrows);
    }
    kn_col_inv<<<ncols, kColThreads, col_smem, e->stream>>>(e->d_desc, e->d_cols, ncols);
    kn_reduce<<<1, kReduceThreads, 0, e->stream>>>(e->d_desc, e->d_test, x, addend);
    return kok(e, cudaGetLastError()) ? 0 : -1;
}

int kn_square(kn_engine *e, uint64_t *x, uint64_t count) {
    if (!e || e->err) return -1;
    cudaSetDevice(e->device);
    for (uint64_t i = 0; i < count; i++)
        if (run_product(e, x, nullptr, nullptr)) return -1;
    return 0;
}

int kn_square_add(kn_engine *e, uint64_t *x, uint64_t count, int64_t c) {
    if (!e || e->err) return -1;
    cudaSetDevice(e->device);
    if (!e->addend_ok || e->addend_c != c) {
        std::vector<uint64_t> words;
        constant_words(e, c, words);
        if (!kok(e, cudaMemcpyAsync(e->d_addend, words.data(), (size_t)e->W * 8, cudaMemcpyHostToDevice, e->stream)) ||
            !kok(e, cudaStreamSynchronize(e->stream)))
            return -1;
        e->addend_c = c;
        e->addend_ok = true;
    }
    for (uint64_t i = 0; i < count; i++)
        if (run_product(e, x, nullptr, e->d_addend)) return -1;
    return 0;
}

int kn_mul(kn_engine *e, uint64_t *x, const uint64_t *y) {
    if (!e || e->err) return -1;
    cudaSetDevice(e->device);
    return run_product(e, x, y, nullptr);
}

int kn_copy(kn_engine *e, uint64_t *dst, const uint64_t *src) {
    if (!e || e->err) return -1;
    cudaSetDevice(e->device);
    if (dst == src) return 0;
    return kok(e, cudaMemcpyAsync(dst, src, (size_t)e->W * 8, cudaMemcpyDeviceToDevice, e->stream)) ? 0 : -1;
}

int kn_error(const kn_engine *e) { return e ? e->err : -1; }

int kn_sync(kn_engine *e) {
    if (!e) return -1;
    cudaSetDevice(e->device);
    kok(e, cudaStreamSynchronize(e->stream));
    return e->err;
}


// ---- groups: many tests squared by one launch set per squaring ---------------------------------

struct kn_group {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<kn_engine *> eng;
    std::vector<uint64_t *> xs;
    std::vector<Desc> h_desc;  // the device table's host copy, in work-list order
    std::vector<int> slot;     // member -> its index in the table
    Desc *d_desc = nullptr;
    int2 *d_cols = nullptr, *d_rows = nullptr;
    int *d_tests = nullptr;
    int ncols = 0, nrows = 0, ntests = 0;
    size_t col_smem = 0, row_smem = 0;
    int grid = 0;
    int threads = 128;  // block size of the transform kernels
    bool dirty = true;
    cudaGraphExec_t graph = nullptr;
    uint32_t graph_len = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int err = 0;
};

namespace {

bool gok(kn_group *g, cudaError_t c) {
    if (c != cudaSuccess && !g->err) g->err = (int)c;
    return c == cudaSuccess;
}

void group_free_lists(kn_group *g) {
    for (void *p : {(void *)g->d_desc, (void *)g->d_cols, (void *)g->d_rows, (void *)g->d_tests})
        if (p) cudaFree(p);
    g->d_desc = nullptr;
    g->d_cols = g->d_rows = nullptr;
    g->d_tests = nullptr;
    if (g->graph) cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
    g->graph_len = 0;
}

// descriptor table and work lists of the members, longest transforms first
bool group_build(kn_group *g) {
    if (!g->dirty) return true;
    group_free_lists(g);
    const int m = (int)g->eng.size();
    std::vector<int> order(m);
    for (int i = 0; i < m; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return g->eng[a]->NP > g->eng[b]->NP; });
    std::vector<Desc> descs(m);
    std::vector<int2> cols, rows;
    std::vector<int> tests(m);
    g->col_smem = g->row_smem = 0;
    for (int t = 0; t < m; t++) {
        kn_engine *e = g->eng[order[t]];
        descs[t] = e->desc;
        descs[t].x = g->xs[order[t]];
        descs[t].addend = nullptr;
        tests[t] = t;
        for (uint32_t c = 0; c < e->plan->C / kG; c++) cols.push_back(make_int2(t, (int)c));
        for (uint32_t r = 0; r < e->plan->R; r++) rows.push_back(make_int2(t, (int)r));
        g->col_smem = std::max(g->col_smem, col_smem_bytes(e->plan->R));
        g->row_smem = std::max(g->row_smem, row_smem_bytes(e->plan->C));
    }
    g->ncols = (int)cols.size();
    g->nrows = (int)rows.size();
    g->ntests = m;
    g->h_desc = descs;
    g->slot.assign(m, 0);
    for (int t = 0; t < m; t++) g->slot[order[t]] = t;
    bool ok = gok(g, cudaMalloc((void **)&g->d_desc, m * sizeof(Desc))) &&
              gok(g, cudaMalloc((void **)&g->d_cols, cols.size() * sizeof(int2))) &&
              gok(g, cudaMalloc((void **)&g->d_rows, rows.size() * sizeof(int2))) &&
              gok(g, cudaMalloc((void **)&g->d_tests, m * sizeof(int))) &&
              gok(g, cudaMemcpy(g->d_desc, descs.data(), m * sizeof(Desc), cudaMemcpyHostToDevice)) &&
              gok(g, cudaMemcpy(g->d_cols, cols.data(), cols.size() * sizeof(int2), cudaMemcpyHostToDevice)) &&
              gok(g, cudaMemcpy(g->d_rows, rows.data(), rows.size() * sizeof(int2), cudaMemcpyHostToDevice)) &&
              gok(g, cudaMemcpy(g->d_tests, tests.data(), m * sizeof(int), cudaMemcpyHostToDevice));
    if (ok) ok = prepare_smem(g->device, g->col_smem, 2 * g->row_smem);
    g->dirty = !ok;
    return ok;
}

void group_square_once(kn_group *g) {
    const int gc = std::min(g->ncols, g->grid), gr = std::min(g->nrows, g->grid);
    kn_col_fwd<<<gc, g->threads, g->col_smem, g->stream>>>(g->d_desc, g->d_cols, g->ncols, 0, nullptr);
    // a row item is 4 B units per register pass (B = 16 for the common C = 256): 64 threads
    kn_rows<false><<<std::min(g->nrows, 2 * g->grid), 64, g->row_smem, g->stream>>>(g->d_desc, g->d_rows, g->nrows);
    kn_col_inv<<<gc, g->threads, g->col_smem, g->stream>>>(g->d_desc, g->d_cols, g->ncols);
    kn_reduce<<<g->ntests, kReduceThreads, 0, g->stream>>>(g->d_desc, g->d_tests, nullptr, nullptr);
}

constexpr uint32_t kGroupChunk = 8;  // squarings per captured graph

}  // namespace

kn_group *kn_group_new(int device) {
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return nullptr;
    kn_group *g = new (std::nothrow) kn_group();
    if (!g) return nullptr;
    g->device = device;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    // 128-thread blocks, 16 per SM: on GB300 over 256 tests, 0.788 ms per squaring step against
    // 0.818 ms with 256 threads and 0.837 ms with 64
    g->threads = 128;
    g->grid = std::max(1, nsm) * 16;
    if (!gok(g, cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) || !gok(g, cudaEventCreate(&g->ev0)) ||
        !gok(g, cudaEventCreate(&g->ev1))) {
        kn_group_free(g);
        return nullptr;
    }
    return g;
}

void kn_group_free(kn_group *g) {
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    group_free_lists(g);
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
}

int kn_group_add(kn_group *g, kn_engine *e, uint64_t *x) {
    if (!g || !e || !x || g->err || e->device != g->device) return -1;
    for (kn_engine *o : g->eng)
        if (o == e) return -1;  // members own their engine's scratch
    kn_sync(e);
    g->eng.push_back(e);
    g->xs.push_back(x);
    g->dirty = true;
    return (int)g->eng.size() - 1;
}

namespace {

// the group's tables and its graph of kGroupChunk squarings, built if needed
bool group_prepare(kn_group *g) {
    if (!group_build(g)) return false;
    if (!g->graph) {
        cudaGraph_t graph = nullptr;
        if (!gok(g, cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal))) return false;
        for (uint32_t i = 0; i < kGroupChunk; i++) group_square_once(g);
        if (!gok(g, cudaStreamEndCapture(g->stream, &graph))) return false;
        const bool ok = gok(g, cudaGraphInstantiate(&g->graph, graph, 0));
        cudaGraphDestroy(graph);
        if (!ok) return false;
        g->graph_len = kGroupChunk;
    }
    return true;
}

// sticky device-side status of every member (a carry that did not settle)
void group_check_status(kn_group *g) {
    for (kn_engine *e : g->eng) {
        int st = 0;
        cudaMemcpy(&st, e->d_status, sizeof st, cudaMemcpyDeviceToHost);
        if (st) g->err = -100 - st;
    }
}

}  // namespace

int kn_groups_square(kn_group *const *gs, int ng, uint64_t count, float *gpu_ms) {
    if (!gs || ng < 1) return -1;
    for (int i = 0; i < ng; i++)
        if (!gs[i] || gs[i]->err || gs[i]->device != gs[0]->device) return -1;
    if (ng == 1) return kn_group_square(gs[0], count, gpu_ms);
    if (!count) return 0;
    kn_group *g0 = gs[0];
    cudaSetDevice(g0->device);
    std::vector<kn_group *> live;
    for (int i = 0; i < ng; i++) {
        if (gs[i]->eng.empty()) continue;
        if (!group_prepare(gs[i])) return -1;
        live.push_back(gs[i]);
    }
    if (live.empty()) return 0;
    // every stream starts after g0's start event, and g0's stream waits for all at the end
    bool ok = gok(g0, cudaEventRecord(g0->ev0, g0->stream));
    for (kn_group *g : live)
        if (g != g0) ok = ok && gok(g, cudaStreamWaitEvent(g->stream, g0->ev0, 0));
    uint64_t done = 0;
    for (; ok && done + kGroupChunk <= count; done += kGroupChunk)
        for (kn_group *g : live) ok = ok && gok(g, cudaGraphLaunch(g->graph, g->stream));
    for (; ok && done < count; done++)
        for (kn_group *g : live) group_square_once(g);
    for (kn_group *g : live)
        if (ok && g != g0)
            ok = gok(g, cudaEventRecord(g->ev1, g->stream)) && gok(g0, cudaStreamWaitEvent(g0->stream, g->ev1, 0));
    ok = ok && gok(g0, cudaEventRecord(g0->ev1, g0->stream)) && gok(g0, cudaGetLastError()) &&
         gok(g0, cudaStreamSynchronize(g0->stream));
    for (kn_group *g : live) {
        cudaStreamSynchronize(g->stream);
        group_check_status(g);
    }
    if (!ok) return -1;
    if (gpu_ms) cudaEventElapsedTime(gpu_ms, g0->ev0, g0->ev1);
    for (kn_group *g : live)
        if (g->err) return -1;
    return 0;
}

int kn_group_square(kn_group *g, uint64_t count, float *gpu_ms) {
    if (!g || g->err) return -1;
    if (g->eng.empty() || !count) return 0;
    cudaSetDevice(g->device);
    if (!group_prepare(g)) return -1;
    gok(g, cudaEventRecord(g->ev0, g->stream));
    uint64_t done = 0;
    for (; done + g->graph_len <= count; done += g->graph_len)
        if (!gok(g, cudaGraphLaunch(g->graph, g->stream))) return -1;
    for (; done < count; done++) group_square_once(g);
    gok(g, cudaEventRecord(g->ev1, g->stream));
    if (!gok(g, cudaGetLastError()) || !gok(g, cudaStreamSynchronize(g->stream))) return -1;
    if (gpu_ms) cudaEventElapsedTime(gpu_ms, g->ev0, g->ev1);
    group_check_status(g);
    return g->err ? -1 : 0;
}

int kn_group_mul(kn_group *g, const uint64_t *const *ys, float *gpu_ms) {
    if (!g || g->err || !ys) return -1;
    if (g->eng.empty()) return 0;
    cudaSetDevice(g->device);
    if (!group_build(g)) return -1;
    for (size_t i = 0; i < g->eng.size(); i++) g->h_desc[g->slot[i]].y = ys[i];
    if (!gok(g, cudaMemcpyAsync(g->d_desc, g->h_desc.data(), g->h_desc.size() * sizeof(Desc),
                                cudaMemcpyHostToDevice, g->stream)))
        return -1;
    const int gc = std::min(g->ncols, g->grid), gr = std::min(g->nrows, 2 * g->grid);
    gok(g, cudaEventRecord(g->ev0, g->stream));
    kn_col_fwd<<<gc, g->threads, g->col_smem, g->stream>>>(g->d_desc, g->d_cols, g->ncols, 0, nullptr);
    kn_col_fwd<<<gc, g->threads, g->col_smem, g->stream>>>(g->d_desc, g->d_cols, g->ncols, 1, nullptr);
    kn_rows<true><<<gr, 64, 2 * g->row_smem, g->stream>>>(g->d_desc, g->d_rows, g->nrows);
    kn_col_inv<<<gc, g->threads, g->col_smem, g->stream>>>(g->d_desc, g->d_cols, g->ncols);
    kn_reduce<<<g->ntests, kReduceThreads, 0, g->stream>>>(g->d_desc, g->d_tests, nullptr, nullptr);
    gok(g, cudaEventRecord(g->ev1, g->stream));
    if (!gok(g, cudaGetLastError()) || !gok(g, cudaStreamSynchronize(g->stream))) return -1;
    if (gpu_ms) cudaEventElapsedTime(gpu_ms, g->ev0, g->ev1);
    return 0;
}

int kn_group_error(const kn_group *g) { return g ? g->err : -1; }

}  // extern "C"
