// sm_103a kernels of one modular squaring / multiplication (see device.h for the data layout).
//
//   k_rows        row pass: forward row DIF of a row pair, real-split square (or product with a
//                 second operand), inverse row DIT.  Reference: src/fast2p.c:545-617 (pass 2),
//                 src/fast2p.c:514-543 (split formulas).
//   k_col_inverse column pass, first half: conj four-step twiddle, inverse column DIT, unweight
//                 and scale, round to nearest, track round-off, add constant digits, balanced
//                 carry within each 16-digit row segment, fold the top region.  Each segment's
//                 carry-out goes to the next segment's slot.  Reference: src/fast2p.c:376-451.
//   k_col_forward column pass, second half: absorb the carry-in (the segment's last digit is
//                 the sink, as src/fast2p.c:404-419), reweight, forward column DIF, twiddle.
//   k_col_digits  conj twiddle, inverse column DIT, unweight, round: the digits of a number.
// Every kernel walks a list of work items, so one launch serves one test or a whole batch of
// tests with different lengths.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "fft_device.cuh"
#include "kernels.h"

namespace kg {

__device__ __forceinline__ void split_pair(double2 &a, double2 &b, double2 w, bool mul, double2 ya,
                                           double2 yb) {
    // e = a + conj(b), o = -i (a - conj(b)); 4 V_k = e^2 + w o^2 + 2 i e o,
    // 4 V_{H-k} = conj(e^2 + w o^2) + 2 i conj(e o); products use e_x e_y + w o_x o_y and
    // e_x o_y + o_x e_y.
    const double er = a.x + b.x, ei = a.y - b.y;
    const double orr = a.y + b.y, oi = b.x - a.x;
    double Xr, Xi, Yr, Yi;
    if (!mul) {
        const double e2r = fma(er, er, -(ei * ei)), e2i = 2.0 * er * ei;
        const double o2r = fma(orr, orr, -(oi * oi)), o2i = 2.0 * orr * oi;
        Xr = fma(w.x, o2r, fma(-w.y, o2i, e2r));
        Xi = fma(w.x, o2i, fma(w.y, o2r, e2i));
        Yr = 2.0 * fma(er, orr, -(ei * oi));
        Yi = 2.0 * fma(er, oi, ei * orr);
    } else {
        const double fr = ya.x + yb.x, fi = ya.y - yb.y;
        const double gr = ya.y + yb.y, gi = yb.x - ya.x;
        const double pr = fma(orr, gr, -(oi * gi)), pi = fma(orr, gi, oi * gr);
        Xr = fma(w.x, pr, fma(-w.y, pi, fma(er, fr, -(ei * fi))));
        Xi = fma(w.x, pi, fma(w.y, pr, fma(er, fi, ei * fr)));
        Yr = fma(er, gr, -(ei * gi)) + fma(orr, fr, -(oi * fi));
        Yi = fma(er, gi, ei * gr) + fma(orr, fi, oi * fr);
    }
    a = make_double2(Xr - Yi, Xi + Yr);
    b = make_double2(Xr + Yi, Yr - Xi);
}

// Programmatic dependent launch: wait until the previous kernel of the stream has completed and
// its writes are visible, then let the next kernel's CTAs be scheduled while this one runs (they
// wait here in turn).  A kernel launched without the attribute passes through both at once.
// The next grid launches only after every CTA of this one has passed here, so its waiting CTAs
// never hold resources that CTAs of this grid still need.
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_leave() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// The work item's test descriptor, copied into shared memory.  An item reads the descriptor's
// fields (plans, table pointers, sizes) again at every stage, and from shared memory those
// reads stay off the texture path that the tables' own loads queue on.  Every thread of the
// block calls this after the previous item's last barrier; it ends with a barrier.
__device__ __forceinline__ const TestDesc &stage_desc(const TestDesc *tests, int t, TestDesc *s) {
    const int4 *src = reinterpret_cast<const int4 *>(tests + t);
    int4 *dst = reinterpret_cast<int4 *>(s);
    for (int i = threadIdx.x; i < (int)(sizeof(TestDesc) / 16); i += blockDim.x) dst[i] = __ldg(src + i);
    __syncthreads();
    return *s;
}

// One row pair of one test: forward row transforms, split square or product, inverse row
// transforms, written back in place.  Ends with a barrier after its last global write.
template <bool MUL>
__device__ __forceinline__ void rows_item(const TestDesc &T, int unit, double2 *x, const double2 *y,
                                          double2 *sm) {
    // shared memory: A = rows to transform forward, ls lanes interleaved (x row k_r, x row
    // R-k_r, and for a product the same rows of y); B = the split's output, 2 lanes, already in
    // the digit-reversed order the inverse transform wants
    constexpr int ls = MUL ? 4 : 2;
    const int C = T.C;
    double2 *A = sm, *B = sm + (size_t)ls * C;
    const int2 pr = T.pairs[unit];
    const bool self = pr.x == pr.y;
    const double2 *xa = x + (size_t)pr.x * C, *xb = x + (size_t)pr.y * C;
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        const int p = __ldg(&T.posc[c]) * ls;
        A[p + 0] = __ldcg(&xa[c]);
        A[p + 1] = __ldcg(&xb[c]);
        if (MUL) {
            A[p + 2] = __ldcg(&y[(size_t)pr.x * C + c]);
            A[p + 3] = __ldcg(&y[(size_t)pr.y * C + c]);
        }
    }
    __syncthreads();
    smem_fft<false>(A, T.rp, T.twr, ls, self ? (MUL ? 3 : 1) : ls);
    const double2 *swp = T.sw + (size_t)pr.x * C;
    const double2 zero = make_double2(0, 0);
    if (!self) {
        // U_k in row k_r pairs with U_{H-k} in row R-k_r, column C-1-k_c
        for (int kc = threadIdx.x; kc < C; kc += blockDim.x) {
            const int kb = C - 1 - kc;
            double2 a = A[kc * ls], b = A[kb * ls + 1];
            const double2 ya = MUL ? A[kc * ls + 2] : zero, yb = MUL ? A[kb * ls + 3] : zero;
            split_pair(a, b, __ldg(&swp[kc]), MUL, ya, yb);
            B[__ldg(&T.posc[kc]) * 2] = a;
            B[__ldg(&T.posc[kb]) * 2 + 1] = b;
        }
    } else {
        // rows 0 and R/2 pair with themselves: k_c with (C-k_c) mod C, resp. C-1-k_c
        for (int kc = threadIdx.x; kc < C; kc += blockDim.x) {
            const int kb = pr.x == 0 ? (C - kc) % C : C - 1 - kc;
            if (kb < kc) continue;
            double2 a = A[kc * ls], b = A[kb * ls];
            const double2 ya = MUL ? A[kc * ls + 2] : zero, yb = MUL ? A[kb * ls + 2] : zero;
            split_pair(a, b, __ldg(&swp[kc]), MUL, ya, yb);
            B[__ldg(&T.posc[kc]) * 2] = a;
            if (kb != kc) B[__ldg(&T.posc[kb]) * 2] = b;
        }
    }
    __syncthreads();
    smem_fft<true>(B, T.rp, T.twr, 2, self ? 1 : 2);
    double2 *oa = x + (size_t)pr.x * C, *ob = x + (size_t)pr.y * C;
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        oa[c] = B[c * 2];
        if (!self) ob[c] = B[c * 2 + 1];
    }
    __syncthreads();
}

template <bool MUL>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_rows(const TestDesc *__restrict__ tests,
                                                   const WorkItem *__restrict__ work, int nwork,
                                                   const int *nwork_dev, int step, double2 *xo,
                                                   const double2 *yo) {
    extern __shared__ double2 sm[];
    __shared__ TestDesc s_desc;
    pdl_enter();
    if (nwork_dev) nwork = *nwork_dev;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const WorkItem it = work[wi];
        if (step >= tests[it.test].count) continue;
        const TestDesc &T = stage_desc(tests, it.test, &s_desc);
        rows_item<MUL>(T, it.unit, xo ? xo : T.x, MUL ? (yo ? yo : T.y) : nullptr, sm);
    }
    pdl_leave();
}

// floor((hi) / k) for a signed 128-bit hi and 0 < k < 2^31, in 32-bit chunks
__device__ __forceinline__ __int128 floor_div_small(__int128 hi, unsigned long long k) {
    const bool neg = hi < 0;
    unsigned __int128 a = neg ? (unsigned __int128)(-hi) : (unsigned __int128)hi;
    unsigned __int128 q = 0;
    unsigned long long rem = 0;
#pragma unroll
    for (int c = 3; c >= 0; c--) {
        unsigned long long cur = (rem << 32) | (unsigned long long)((a >> (32 * c)) & 0xffffffffull);
        q |= (unsigned __int128)(cur / k) << (32 * c);
        rem = cur % k;
    }
    __int128 sq = (__int128)q;
    if (neg) sq = rem ? -sq - 1 : -sq;
    return sq;
}

// Fold of the top region held in dig[top_t..L-1] plus the carry cy at 2^{s_L}
// (reference src/ctx.c:345-375); returns the amount for digit 0.
__device__ long long fold_top(const TestDesc &T, long long *dig, long long cy) {
    const int L = T.L, t = T.top_t;
    __int128 H = (__int128)cy << T.top_shift;
    int pos = 0;
    for (int j = t; j < L; j++) {
        H += (__int128)dig[j] << pos;
        pos += T.bits[j];
    }
    const int m = T.top_m;
    const __int128 K = (__int128)T.k;
    __int128 lo = H & (((__int128)1 << m) - 1);
    __int128 hi = H >> m;
    __int128 q = floor_div_small(hi, T.k);
    __int128 top = lo + ((hi - q * K) << m);
    const __int128 span = K << m;
    if (2 * top >= span) {
        top -= span;
        q += 1;
    }
    for (int j = t; j + 1 < L; j++) {
        const int b = T.bits[j];
        __int128 qq = (top + ((__int128)1 << (b - 1))) >> b;
        dig[j] = (long long)(top - (qq << b));
        top = qq;
    }
    if (t < L) dig[L - 1] = (long long)top;
    return (long long)q;
}

__device__ __forceinline__ void block_max_err(unsigned long long v, unsigned long long *dst) {
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
        v = u > v ? u : v;
    }
    if ((threadIdx.x & 31) == 0 && v) atomicMax(dst, v);
}

// 1.5 * 2^52: for |v| < 2^51, fma(a, b, kMagic) rounds a*b to the nearest integer, which then
// sits in the low bits of the result's encoding.
constexpr double kMagic = 6755399441055744.0;
constexpr long long kMagicBits = 0x4338000000000000ll;

// The 2G digit widths of the row segment starting at word j0, packed four to a word, in one
// aligned load: j0 is a multiple of 2G (C is a multiple of G), and the table starts on a
// 256-byte boundary.  seg_width(w, i) unpacks width i.
template <int G>
struct SegWidths {
    unsigned w[2 * G / 4];
};

template <int G>
__device__ __forceinline__ SegWidths<G> load_segment_widths(const uint8_t *bits, int j0) {
    static_assert(G == 2 || G == 4 || G == 8, "column groups of 2, 4 or 8");
    SegWidths<G> s;
    if constexpr (G == 8) {
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(bits + j0));
        s.w[0] = v.x;
        s.w[1] = v.y;
        s.w[2] = v.z;
        s.w[3] = v.w;
    } else if constexpr (G == 4) {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(bits + j0));
        s.w[0] = v.x;
        s.w[1] = v.y;
    } else {
        s.w[0] = __ldg(reinterpret_cast<const unsigned *>(bits + j0));
    }
    return s;
}

template <int G>
__device__ __forceinline__ int seg_width(const SegWidths<G> &s, int i) {
    return (int)((s.w[i / 4] >> (8 * (i % 4))) & 0xffu);
}

// load the group's columns times conj(w_H^{c k_r}) into digit-reversed rows of the buffer
template <int G>
__device__ __forceinline__ void load_columns_conj(const TestDesc &T, const double2 *x, int g, double2 *sm) {
    const int C = T.C;
    for (int i = threadIdx.x; i < T.R * G; i += blockDim.x) {
        const int kr = i / G, l = i % G;
        const size_t e = (size_t)kr * C + g * G + l;
        sm[__ldg(&T.posr[kr]) * G + l] = cmulc(__ldcg(&x[e]), __ldg(&T.t4[e]));
    }
}

// One column group of one test, first half of the column pass: conj twiddle, inverse column
// transform, unweight and round, round-off, carry within each row segment (carry-out to the
// next segment's slot), top fold.  Ends with a barrier after its last global write.
template <bool ERR, int G>
__device__ __forceinline__ void col_inverse_item(const TestDesc &T, int g, int step, const double2 *x,
                                                 double2 *sm) {
    long long *smd = reinterpret_cast<long long *>(sm);
    const bool track = ERR && (step % T.err_every == 0);
    const int R = T.R, C = T.C;
    load_columns_conj<G>(T, x, g, sm);
    __syncthreads();
    smem_fft<true>(sm, T.cp, T.twc, G, G);
    // unweight, scale and round every value in parallel: one FMA with the magic constant
    // (two more when the round-off is tracked); the integer is read from the encoding
    unsigned long long emax = 0;
    for (int i = threadIdx.x; i < R * G; i += blockDim.x) {
        const int r = i / G, l = i % G;
        const int j = 2 * (r * C + g * G + l);
        const double2 z = sm[i];
        const double2 o = __ldg(reinterpret_cast<const double2 *>(T.osc + j));  // j is even
        const double o0 = o.x, o1 = o.y;
        const double t0 = fma(z.x, o0, kMagic), t1 = fma(z.y, o1, kMagic);
        const long long b0 = __double_as_longlong(t0), b1 = __double_as_longlong(t1);
        if (((b0 >> 52) != 0x433) | ((b1 >> 52) != 0x433)) {
            emax = 0x3FE0000000000000ull;  // |v| >= 2^51: report 0.5, the transform is too short
        } else if (track) {
            const unsigned long long e0 = __double_as_longlong(fabs(fma(z.x, o0, kMagic - t0)));
            const unsigned long long e1 = __double_as_longlong(fabs(fma(z.y, o1, kMagic - t1)));
            emax = max(emax, max(e0, e1));
        }
        reinterpret_cast<longlong2 *>(smd)[i] = make_longlong2(b0 - kMagicBits, b1 - kMagicBits);
    }
    __syncthreads();
    // balanced carry along each row segment (16 digits), constants added first; the carry-out
    // goes to the next segment's slot, the last segment's into the top fold
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const int j0 = 2 * (r * C + g * G);
        long long d[2 * G];
        const SegWidths<G> bw = load_segment_widths<G>(T.bits, j0);
        const longlong2 *row = reinterpret_cast<const longlong2 *>(smd) + G * r;
#pragma unroll
        for (int l = 0; l < G; l++) {
            const longlong2 p = row[l];
            d[2 * l] = p.x;
            d[2 * l + 1] = p.y;
        }
        long long cy = 0;
#pragma unroll
        for (int i = 0; i < 2 * G; i++) {
            long long v = d[i];
            for (int a = 0; a < T.nadd; a++)
                if (T.addj[a] == j0 + i) v += T.addv[a];
            v += cy;
            const int b = seg_width(bw, i);
            const long long q = (v + (1ll << (b - 1))) >> b;
            d[i] = v - (q << b);
            cy = q;
        }
        longlong2 *dst = reinterpret_cast<longlong2 *>(T.dig + j0);  // j0 is even
#pragma unroll
        for (int l = 0; l < G; l++) dst[l] = make_longlong2(d[2 * l], d[2 * l + 1]);
        if (g == T.NG - 1 && r == R - 1) {
            T.slot[0] = fold_top(T, T.dig, cy);  // this thread's own digits: visible
        } else {
            T.slot[g < T.NG - 1 ? (g + 1) * R + r : r + 1] = cy;
        }
    }
    block_max_err(emax, T.maxerr);  // every thread of the block reaches this
    __syncthreads();
}

template <bool ERR, int G>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_col_inverse(const TestDesc *__restrict__ tests,
                                                          const WorkItem *__restrict__ work,
                                                          int nwork, const int *nwork_dev,
                                                          int step, const double2 *xo) {
    extern __shared__ double2 sm[];
    __shared__ TestDesc s_desc;
    pdl_enter();
    if (nwork_dev) nwork = *nwork_dev;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const WorkItem it = work[wi];
        if (step >= tests[it.test].count) continue;
        const TestDesc &T = stage_desc(tests, it.test, &s_desc);
        col_inverse_item<ERR, G>(T, it.unit, step, xo ? xo : T.x, sm);
    }
    pdl_leave();
}

// One column group of one test, second half of the column pass: absorb the carry-in,
// reweight, forward column transform, twiddle.  Ends with a barrier after its last global write.
template <int G>
__device__ __forceinline__ void col_forward_item(const TestDesc &T, int g, double2 *x, bool use_slots,
                                                 double2 *sm) {
    const int R = T.R, C = T.C;
    // absorb the carry-in into the segment's first digits (the last digit takes any rest),
    // reweight, and place the row at its digit-reversed position
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const int j0 = 2 * (r * C + g * G);
        long long d[2 * G];
        const longlong2 *src = reinterpret_cast<const longlong2 *>(T.dig + j0);  // j0 is even
#pragma unroll
        for (int l = 0; l < G; l++) {
            const longlong2 p = __ldcg(src + l);
            d[2 * l] = p.x;
            d[2 * l + 1] = p.y;
        }
        long long cy = use_slots ? __ldcg(&T.slot[g * R + r]) : 0;
        const SegWidths<G> bw = load_segment_widths<G>(T.bits, j0);
#pragma unroll
        for (int i = 0; i < 2 * G - 1; i++) {
            if (cy) {
                const int b = seg_width(bw, i);
                const long long v = d[i] + cy;
                const long long q = (v + (1ll << (b - 1))) >> b;
                d[i] = v - (q << b);
                cy = q;
            }
        }
        d[2 * G - 1] += cy;
        double2 *row = sm + __ldg(&T.posr[r]) * G;
        const double2 *wv = reinterpret_cast<const double2 *>(T.w + j0);
#pragma unroll
        for (int l = 0; l < G; l++) {
            const double2 wl = __ldg(wv + l);
            row[l] = make_double2((double)d[2 * l] * wl.x, (double)d[2 * l + 1] * wl.y);
        }
    }
    __syncthreads();
    smem_fft<false>(sm, T.cp, T.twc, G, G);
    for (int i = threadIdx.x; i < R * G; i += blockDim.x) {
        const int kr = i / G, l = i % G;
        const size_t e = (size_t)kr * C + g * G + l;
        x[e] = cmul(sm[i], __ldg(&T.t4[e]));
    }
    __syncthreads();
}

template <int G>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_col_forward(const TestDesc *__restrict__ tests,
                                                          const WorkItem *__restrict__ work,
                                                          int nwork, const int *nwork_dev, int step,
                                                          double2 *xo, int use_slots) {
    extern __shared__ double2 sm[];
    __shared__ TestDesc s_desc;
    pdl_enter();
    if (nwork_dev) nwork = *nwork_dev;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const WorkItem it = work[wi];
        if (step >= tests[it.test].count) continue;
        const TestDesc &T = stage_desc(tests, it.test, &s_desc);
        col_forward_item<G>(T, it.unit, xo ? xo : T.x, use_slots != 0, sm);
    }
    pdl_leave();
}

// Waits until *ctr >= need, reading it with acquire semantics at GPU scope.  Gives up (returns
// false) when another CTA has raised *flag, or after `limit` SM cycles, raising *flag itself.
__device__ __noinline__ bool wait_count(const unsigned *ctr, unsigned need, unsigned *flag, long long limit) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
    if (v >= need) return true;
    const long long t0 = clock64();
    for (;;) {
        __nanosleep(128);
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
        if (v >= need) return true;
        if (*(volatile const unsigned *)flag) return false;
        if (clock64() - t0 > limit) {
            atomicOr(flag, 1u);
            return false;
        }
    }
}

// `nsteps` squarings of every test of the work lists in one persistent launch.
//
// The work is one queue, taken in order by atomically incrementing flow[kFlowNext]: for each
// step, every row pair, then every column group (inverse half), then every column group
// (forward half).  A CTA that takes an item first waits until the test's previous phase is
// complete: flow[kFlowDone + test] counts the test's finished items, and the phases of one test
// follow each other, so item counts alone say which phase is done.  Different tests overlap
// freely, so no CTA idles at the end of a phase or of a step, as it would at the end of a
// kernel launch.  Every wait is on items earlier in the queue, which CTAs already running hold,
// so each wait ends; one that runs out of time raises flow[kFlowTimeout] and every CTA returns.
template <int G>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_squarings(const TestDesc *__restrict__ tests,
                                                        const WorkItem *__restrict__ rows, int nrows,
                                                        const int *nrows_dev,
                                                        const WorkItem *__restrict__ cols, int ncols,
                                                        const int *ncols_dev, int step0, int nsteps,
                                                        unsigned *flow, long long wait_limit) {
    extern __shared__ double2 sm[];
    __shared__ TestDesc s_desc;
    __shared__ unsigned s_q;
    __shared__ int s_ok;
    const unsigned nr = (unsigned)(nrows_dev ? *nrows_dev : nrows);
    const unsigned nc = (unsigned)(ncols_dev ? *ncols_dev : ncols);
    const unsigned per_step = nr + 2 * nc;
    const unsigned total = per_step * (unsigned)nsteps;
    for (;;) {
        __syncthreads();  // every thread has read the previous item's s_q
        if (threadIdx.x == 0) {
            const unsigned q = atomicAdd(&flow[kFlowNext], 1u);
            int ok = 1;
            if (q < total) {
                const unsigned st = q / per_step, r = q % per_step;
                const WorkItem it = r < nr ? rows[r] : cols[(r - nr) % nc];
                const TestDesc &T = tests[it.test];
                unsigned need = st * (unsigned)(T.npairs + 2 * T.NG);
                if (r >= nr) need += (unsigned)T.npairs;
                if (r >= nr + nc) need += (unsigned)T.NG;
                ok = wait_count(&flow[kFlowDone + it.test], need, &flow[kFlowTimeout], wait_limit);
            }
            s_q = q;
            s_ok = ok;
        }
        __syncthreads();
        const unsigned q = s_q;
        if (q >= total || !s_ok) return;
        const unsigned st = q / per_step, r = q % per_step;
        const WorkItem it = r < nr ? rows[r] : cols[(r - nr) % nc];
        const TestDesc &T = stage_desc(tests, it.test, &s_desc);
        const int step = step0 + (int)st;
        if (step < T.count) {
            if (r < nr)
                rows_item<false>(T, it.unit, T.x, nullptr, sm);
            else if (r < nr + nc)
                col_inverse_item<true, G>(T, it.unit, step, T.x, sm);
            else
                col_forward_item<G>(T, it.unit, T.x, true, sm);
        }
        // each item ends with a barrier after its last global write: publish them, then count
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&flow[kFlowDone + it.test], 1u);
        }
    }
}

template <int G>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_col_digits(const TestDesc *__restrict__ tests,
                                                         const WorkItem *__restrict__ work,
                                                         int nwork, const double2 *xo, long long *digo) {
    extern __shared__ double2 sm[];
    __shared__ TestDesc s_desc;
    pdl_enter();
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const WorkItem it = work[wi];
        const TestDesc &T = stage_desc(tests, it.test, &s_desc);
        const double2 *x = xo ? xo : T.x;
        long long *dig = digo ? digo : T.dig;
        const int R = T.R, C = T.C, g = it.unit;
        load_columns_conj<G>(T, x, g, sm);
        __syncthreads();
        smem_fft<true>(sm, T.cp, T.twc, G, G);
        for (int i = threadIdx.x; i < R * G; i += blockDim.x) {
            const int r = i / G, l = i % G;
            const int j = 2 * (r * C + g * G + l);
            dig[j] = llrint(sm[i].x * T.idig[j]);
            dig[j + 1] = llrint(sm[i].y * T.idig[j + 1]);
        }
        __syncthreads();
    }
    pdl_leave();
}

// Zero test of a - b modulo N for two digit vectors of one test (the digits of two numbers, as
// k_col_digits leaves them): the Gerbicz check's comparison d == x0 * t^(2^B) and the tail's
// x == t, done where the numbers live.  The reference compares canonical limbs on the host
// (src/prp.c:291-296 and :470-474, via kite_get_limbs).
//
// The difference e = a - b is carried exactly as a whole number: the low digits (below top_t)
// are balanced in kEqualThreads chunks, each chunk's carry-out moving to the next chunk round
// by round until none is left; the top region (digits top_t..L-1 with the carry out of the low
// digits) is folded by k*2^n == 1 and re-centred (fold_top), and the fold's amount for digit 0
// rippled in the same way.  Afterwards every low digit is balanced and the top region lies in
// [-k 2^m/2, k 2^m/2), so |e| < N and e == 0 (mod N) exactly when every digit is zero.
// *flag = 1 (equal), 0 (not equal), or 2 when the carry did not settle within its bounds (the
// caller then compares on the host).  a is overwritten; one CTA per test.
constexpr int kEqualThreads = 512;

__device__ __forceinline__ long long ripple(long long *e, const uint8_t *bits, int j0, int j1, long long c) {
    for (int j = j0; j < j1 && c; j++) {
        const int b = bits[j];
        const long long v = e[j] + c;
        c = (v + (1ll << (b - 1))) >> b;
        e[j] = v - (c << b);
    }
    return c;
}

__global__ void __launch_bounds__(kEqualThreads) k_equal_mod_n(const TestDesc *__restrict__ tests, int test,
                                                               long long *__restrict__ a,
                                                               const long long *__restrict__ b, int *flag) {
    __shared__ long long s_out[kEqualThreads];  // carry out of chunk i, not yet moved on
    __shared__ long long s_in0;                  // carry into chunk 0 (from the fold)
    __shared__ long long s_top;                  // carry out of the low digits into the top region
    __shared__ int s_more;
    const TestDesc &T = tests[test];
    const int L = T.L, t = T.top_t, tid = threadIdx.x, nt = blockDim.x;
    for (int j = tid; j < L; j += nt) a[j] -= b[j];
    // chunks of the low digits [0, t): nch chunks of cs digits (the last one may be shorter)
    const int cs = (t + nt - 1) / nt, nch = (t + cs - 1) / cs;
    const int j0 = min(t, tid * cs), j1 = min(t, j0 + cs);
    if (tid == 0) {
        s_in0 = 0;
        s_top = 0;
    }
    __syncthreads();
    // every chunk balanced on its own, from no carry
    long long c = 0;
    if (tid < nch) {
        for (int j = j0; j < j1; j++) {
            const int bw = T.bits[j];
            const long long v = a[j] + c;
            c = (v + (1ll << (bw - 1))) >> bw;
            a[j] = v - (c << bw);
        }
        s_out[tid] = c;
    }
    int settled = 0;
    for (int pass = 0; pass < 64; pass++) {
        // move the carries on until every chunk has absorbed its carry-in; a carry advances at
        // least one chunk per round, so nch + 1 rounds always suffice
        int quiet = 0;
        for (int round = 0; round <= nch + 1; round++) {
            __syncthreads();
            const long long cin = tid == 0 ? s_in0 : (tid < nch ? s_out[tid - 1] : 0);
            const long long to_top = s_out[nch - 1];
            __syncthreads();
            if (tid == 0) {
                s_in0 = 0;
                s_top += to_top;
            }
            long long r = 0;
            if (tid < nch) {
                r = ripple(a, T.bits, j0, j1, cin);
                s_out[tid] = r;
            }
            if (!__syncthreads_or(r != 0)) {
                quiet = 1;
                break;
            }
        }
        if (!quiet) break;  // not settled within the bound: undetermined
        // fold the top region (always once, again whenever a carry reached it)
        if (tid == 0) {
            const long long add = s_top;
            s_top = 0;
            s_more = 0;
            if (pass == 0 || add) {
                long long q;
                if (t < L) {
                    a[t] += add;
                    q = fold_top(T, a, 0);
                } else {
                    q = fold_top(T, a, add);
                }
                s_in0 = q;
                s_more = q != 0;
            }
        }
        __syncthreads();
        if (!s_more) {
            settled = 1;
            break;
        }
    }
    int nonzero = 0;
    for (int j = tid; j < L; j += nt) nonzero |= a[j] != 0;
    nonzero = __syncthreads_or(nonzero);
    if (tid == 0) *flag = settled ? (nonzero ? 0 : 1) : 2;
}

// x op= y element-wise over n complex values: 0 copy, 1 add, 2 sub
__global__ void k_elementwise(double2 *x, const double2 *y, size_t n, int op) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double2 b = y[i];
        if (op == 0) {
            x[i] = b;
        } else {
            const double2 a = x[i];
            x[i] = op == 1 ? cadd(a, b) : csub(a, b);
        }
    }
}

// ---- host launch wrappers --------------------------------------------------------------------

static int set_smem(const void *fn, size_t bytes) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess
               ? 0
               : -1;
}

// The limit is a property of each kernel in the device's context, shared by every engine and
// batch of the process, so it only ever grows: lowering it for a small length would make later
// launches (or captured graphs) of a longer length fail.
int kernels_prepare(size_t row_smem, size_t col_smem) {
    static std::mutex mu;
    static size_t row_hw[kMaxDevices] = {}, col_hw[kMaxDevices] = {}, sq_hw[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -1;
    std::lock_guard<std::mutex> lock(mu);
    int rc = 0;
    if (row_smem > row_hw[dev]) {
        rc |= set_smem((const void *)k_rows<false>, row_smem);
        rc |= set_smem((const void *)k_rows<true>, row_smem);
        if (!rc) row_hw[dev] = row_smem;
    }
    if (col_smem > col_hw[dev]) {
        rc |= set_smem((const void *)k_col_inverse<false, 2>, col_smem);
        rc |= set_smem((const void *)k_col_inverse<true, 2>, col_smem);
        rc |= set_smem((const void *)k_col_inverse<false, 4>, col_smem);
        rc |= set_smem((const void *)k_col_inverse<true, 4>, col_smem);
        rc |= set_smem((const void *)k_col_inverse<false, 8>, col_smem);
        rc |= set_smem((const void *)k_col_inverse<true, 8>, col_smem);
        rc |= set_smem((const void *)k_col_forward<2>, col_smem);
        rc |= set_smem((const void *)k_col_forward<4>, col_smem);
        rc |= set_smem((const void *)k_col_forward<8>, col_smem);
        rc |= set_smem((const void *)k_col_digits<2>, col_smem);
        rc |= set_smem((const void *)k_col_digits<4>, col_smem);
        rc |= set_smem((const void *)k_col_digits<8>, col_smem);
        if (!rc) col_hw[dev] = col_smem;
    }
    const size_t sq_smem = squarings_smem(row_smem, col_smem);
    if (sq_smem > sq_hw[dev]) {
        int r2 = set_smem((const void *)k_squarings<2>, sq_smem);
        r2 |= set_smem((const void *)k_squarings<4>, sq_smem);
        r2 |= set_smem((const void *)k_squarings<8>, sq_smem);
        if (!r2) sq_hw[dev] = sq_smem;
        rc |= r2;
    }
    return rc;
}

// Pass kernels launch with programmatic stream serialization (each enters through pdl_enter),
// so in a stream or graph the next pass's CTAs are scheduled while the previous pass drains.
// KITE_GB300_PDL=0 launches them plainly.
static bool pdl_enabled() {
    static const bool on = [] {
        const char *t = getenv("KITE_GB300_PDL");
        return !t || atoi(t) != 0;
    }();
    return on;
}

template <typename... Params, typename... Args>
static void launch_pass(void (*k)(Params...), int grid, int block, size_t smem, cudaStream_t st, Args... args) {
    if (!pdl_enabled()) {
        k<<<grid, block, smem, st>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, static_cast<Params>(args)...);
}

void launch_rows(const LaunchSet &s, bool mul, double2 *x, const double2 *y, int step) {
    const size_t smem = s.row_smem_per_lane * (mul ? 6 : 4);
    if (mul)
        launch_pass(k_rows<true>, s.grid_rows, s.threads, smem, s.stream, s.tests, s.rows, s.nrows, s.nrows_dev, step, x, y);
    else
        launch_pass(k_rows<false>, s.grid_rows, s.threads, smem, s.stream, s.tests, s.rows, s.nrows, s.nrows_dev, step, x, y);
}

template <int G>
static void col_inverse_g(const LaunchSet &s, bool err, const double2 *x, int step) {
    if (err)
        launch_pass(k_col_inverse<true, G>, s.grid_cols, s.threads, s.col_smem, s.stream, s.tests, s.cols, s.ncols, s.ncols_dev, step, x);
    else
        launch_pass(k_col_inverse<false, G>, s.grid_cols, s.threads, s.col_smem, s.stream, s.tests, s.cols, s.ncols, s.ncols_dev, step, x);
}

void launch_col_inverse(const LaunchSet &s, bool err, const double2 *x, int step) {
    switch (s.G) {
    case 2: col_inverse_g<2>(s, err, x, step); break;
    case 4: col_inverse_g<4>(s, err, x, step); break;
    default: col_inverse_g<8>(s, err, x, step); break;
    }
}

void launch_col_forward(const LaunchSet &s, double2 *x, bool use_slots, int step) {
    const int u = use_slots ? 1 : 0;
    switch (s.G) {
    case 2: launch_pass(k_col_forward<2>, s.grid_cols, s.threads, s.col_smem, s.stream, s.tests, s.cols, s.ncols, s.ncols_dev, step, x, u); break;
    case 4: launch_pass(k_col_forward<4>, s.grid_cols, s.threads, s.col_smem, s.stream, s.tests, s.cols, s.ncols, s.ncols_dev, step, x, u); break;
    default: launch_pass(k_col_forward<8>, s.grid_cols, s.threads, s.col_smem, s.stream, s.tests, s.cols, s.ncols, s.ncols_dev, step, x, u); break;
    }
}

// shared memory of k_squarings: a row pair squared (4 lanes of the longest row; row_smem is
// sized for the 6 lanes of a product) or a column group
size_t squarings_smem(size_t row_smem, size_t col_smem) { return std::max(row_smem / 6 * 4, col_smem); }

template <int G>
static int squarings_per_sm(const LaunchSet &s) {
    int per_sm = 0;
    const size_t smem = squarings_smem(s.row_smem_per_lane * 6, s.col_smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_squarings<G>, s.threads, smem) != cudaSuccess)
        return 0;
    return per_sm;
}

int squarings_grid(const LaunchSet &s, int nsm) {
    switch (s.G) {
    case 2: return squarings_per_sm<2>(s) * nsm;
    case 4: return squarings_per_sm<4>(s) * nsm;
    default: return squarings_per_sm<8>(s) * nsm;
    }
}

int launch_squarings(const LaunchSet &s, unsigned *flow, int step0, int nsteps, int grid, long long wait_limit) {
    if (grid < 1) return -1;
    const size_t smem = squarings_smem(s.row_smem_per_lane * 6, s.col_smem);
#define KG_SQ_ARGS s.tests, s.rows, s.nrows, s.nrows_dev, s.cols, s.ncols, s.ncols_dev, step0, nsteps, flow, wait_limit
    switch (s.G) {
    case 2: k_squarings<2><<<grid, s.threads, smem, s.stream>>>(KG_SQ_ARGS); break;
    case 4: k_squarings<4><<<grid, s.threads, smem, s.stream>>>(KG_SQ_ARGS); break;
    default: k_squarings<8><<<grid, s.threads, smem, s.stream>>>(KG_SQ_ARGS); break;
    }
#undef KG_SQ_ARGS
    return 0;
}

void launch_col_digits(const LaunchSet &s, const double2 *x, long long *dig) {
    switch (s.G) {
    case 2: launch_pass(k_col_digits<2>, s.grid_cols, s.threads, s.col_smem, s.stream, s.tests, s.cols, s.ncols, x, dig); break;
    case 4: launch_pass(k_col_digits<4>, s.grid_cols, s.threads, s.col_smem, s.stream, s.tests, s.cols, s.ncols, x, dig); break;
    default: launch_pass(k_col_digits<8>, s.grid_cols, s.threads, s.col_smem, s.stream, s.tests, s.cols, s.ncols, x, dig); break;
    }
}

void launch_equal(cudaStream_t st, const TestDesc *tests, int test, long long *a, const long long *b, int *flag) {
    k_equal_mod_n<<<1, kEqualThreads, 0, st>>>(tests, test, a, b, flag);
}

void launch_elementwise(cudaStream_t st, double2 *x, const double2 *y, size_t n, int op) {
    int grid = (int)((n + 255) / 256);
    if (grid > 4096) grid = 4096;
    k_elementwise<<<grid, 256, 0, st>>>(x, y, n, op);
}

// Dependent DFMA chains: 8 independent chains per thread so the pipe, not latency, limits.
__global__ void k_fp64_probe(double *out, int iters) {
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const double m = 0.999999999, c = 1e-12;
    for (int i = 0; i < iters; i++) {
        a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
        a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
    const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s > 1e300) out[0] = s;
}

// The probe's variants for kc_fp64_probe_rate: CH independent chains per thread of one FP64
// opcode (0 DFMA, 1 DMUL, 2 DADD).
template <int CH, int OP>
__global__ void k_fp64_probe_var(double *out, int iters) {
    double a[CH];
#pragma unroll
    for (int c = 0; c < CH; c++) a[c] = threadIdx.x * 1e-9 + c;
    const double m = 0.999999999, k = 1e-12;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < CH; c++) a[c] = OP == 0 ? fma(a[c], m, k) : OP == 1 ? a[c] * m : a[c] + k;
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < CH; c++) s += a[c];
    if (s > 1e300) out[0] = s;
}

int launch_fp64_probe_var(cudaStream_t st, int grid, int block, int iters, int chains, int op, double *out) {
#define KG_PROBE(CH, OP) k_fp64_probe_var<CH, OP><<<grid, block, 0, st>>>(out, iters)
    if (op < 0 || op > 2) return -1;
    switch (chains * 4 + op) {
    case 4 * 4 + 0: KG_PROBE(4, 0); break;
    case 8 * 4 + 0: KG_PROBE(8, 0); break;
    case 16 * 4 + 0: KG_PROBE(16, 0); break;
    case 8 * 4 + 1: KG_PROBE(8, 1); break;
    case 8 * 4 + 2: KG_PROBE(8, 2); break;
    default: return -1;
    }
#undef KG_PROBE
    return 0;
}

void launch_fp64_probe(cudaStream_t st, int grid, int block, int iters, double *out) {
    k_fp64_probe<<<grid, block, 0, st>>>(out, iters);
}

}  // namespace kg
