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

template <bool MUL>
__global__ void __launch_bounds__(kThreads) k_rows(const TestDesc *__restrict__ tests,
                                                   const WorkItem *__restrict__ work, int nwork,
                                                   const int *nwork_dev, int step, double2 *xo,
                                                   const double2 *yo) {
    extern __shared__ double2 sm[];
    constexpr int ls = MUL ? 4 : 2;
    if (nwork_dev) nwork = *nwork_dev;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const WorkItem it = work[wi];
        const TestDesc &T = tests[it.test];
        if (step >= T.count) continue;
        double2 *x = xo ? xo : T.x;
        const double2 *y = MUL ? (yo ? yo : T.y) : nullptr;
        const int C = T.C;
        const int2 pr = T.pairs[it.unit];
        const double2 *xa = x + (size_t)pr.x * C, *xb = x + (size_t)pr.y * C;
        for (int c = threadIdx.x; c < C; c += blockDim.x) {
            sm[c * ls + 0] = xa[c];
            sm[c * ls + 1] = xb[c];
            if (MUL) {
                sm[c * ls + 2] = y[(size_t)pr.x * C + c];
                sm[c * ls + 3] = y[(size_t)pr.y * C + c];
            }
        }
        __syncthreads();
        smem_fft<false>(sm, T.rp, T.twr, ls, ls);
        const double2 *swp = T.sw + (size_t)pr.x * C;
        const double2 zero = make_double2(0, 0);
        if (pr.x != pr.y) {
            for (int q = threadIdx.x; q < C; q += blockDim.x) {
                const int qb = T.part1[q];
                double2 a = sm[q * ls], b = sm[qb * ls + 1];
                double2 ya = MUL ? sm[q * ls + 2] : zero, yb = MUL ? sm[qb * ls + 3] : zero;
                split_pair(a, b, swp[q], MUL, ya, yb);
                sm[q * ls] = a;
                sm[qb * ls + 1] = b;
            }
        } else {
            const int *part = pr.x == T.prow0 ? T.part0 : T.part1;
            for (int q = threadIdx.x; q < C; q += blockDim.x) {
                const int qb = part[q];
                if (qb < q) continue;
                double2 a = sm[q * ls], b = sm[qb * ls];
                double2 ya = MUL ? sm[q * ls + 2] : zero, yb = MUL ? sm[qb * ls + 2] : zero;
                split_pair(a, b, swp[q], MUL, ya, yb);
                sm[q * ls] = a;
                if (qb != q) sm[qb * ls] = b;
            }
        }
        __syncthreads();
        smem_fft<true>(sm, T.rp, T.twr, ls, 2);
        double2 *oa = x + (size_t)pr.x * C, *ob = x + (size_t)pr.y * C;
        for (int c = threadIdx.x; c < C; c += blockDim.x) {
            oa[c] = sm[c * ls + 0];
            if (pr.x != pr.y) ob[c] = sm[c * ls + 1];
        }
        __syncthreads();
    }
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

template <bool ERR>
__global__ void __launch_bounds__(kThreads) k_col_inverse(const TestDesc *__restrict__ tests,
                                                          const WorkItem *__restrict__ work,
                                                          int nwork, const int *nwork_dev,
                                                          int step, const double2 *xo) {
    extern __shared__ double2 sm[];
    constexpr int G = kGroup;
    if (nwork_dev) nwork = *nwork_dev;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const WorkItem it = work[wi];
        const TestDesc &T = tests[it.test];
        if (step >= T.count) continue;
        const bool track = ERR && (step % T.err_every == 0);
        const double2 *x = xo ? xo : T.x;
        const int R = T.R, C = T.C, g = it.unit;
        for (int i = threadIdx.x; i < R * G; i += blockDim.x) {
            const int p = i / G, c = g * G + i % G;
            sm[i] = cmulc(x[(size_t)p * C + c], T.t4[(size_t)p * C + c]);
        }
        __syncthreads();
        smem_fft<true>(sm, T.cp, T.twc, G, G);
        unsigned long long emax = 0;
        for (int r = threadIdx.x; r < R; r += blockDim.x) {
            const int j0 = 2 * (r * C + g * G);
            long long d[2 * G];
            long long cy = 0;
#pragma unroll
            for (int i = 0; i < 2 * G; i++) {
                const int j = j0 + i;
                const double2 z = sm[r * G + i / 2];
                const double v = ((i & 1) ? z.y : z.x) * T.osc[j];
                const double rv = rint(v);
                if (ERR && track) {
                    const unsigned long long e = (unsigned long long)__double_as_longlong(fabs(v - rv));
                    emax = e > emax ? e : emax;
                }
                long long xi = (long long)rv;
                for (int a = 0; a < T.nadd; a++)
                    if (T.addj[a] == j) xi += T.addv[a];
                xi += cy;
                const int b = T.bits[j];
                const long long q = (xi + (1ll << (b - 1))) >> b;
                d[i] = xi - (q << b);
                cy = q;
            }
#pragma unroll
            for (int i = 0; i < 2 * G; i++) T.dig[j0 + i] = d[i];
            if (g == T.NG - 1 && r == R - 1) {
                T.slot[0] = fold_top(T, T.dig, cy);  // this thread's own digits: visible
            } else {
                T.slot[g < T.NG - 1 ? (g + 1) * R + r : r + 1] = cy;
            }
        }
        if (ERR && track) block_max_err(emax, T.maxerr);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreads) k_col_forward(const TestDesc *__restrict__ tests,
                                                          const WorkItem *__restrict__ work,
                                                          int nwork, const int *nwork_dev, int step,
                                                          double2 *xo, int use_slots) {
    extern __shared__ double2 sm[];
    constexpr int G = kGroup;
    if (nwork_dev) nwork = *nwork_dev;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const WorkItem it = work[wi];
        const TestDesc &T = tests[it.test];
        if (step >= T.count) continue;
        double2 *x = xo ? xo : T.x;
        const int R = T.R, C = T.C, g = it.unit;
        for (int r = threadIdx.x; r < R; r += blockDim.x) {
            const int j0 = 2 * (r * C + g * G);
            long long d[2 * G];
#pragma unroll
            for (int i = 0; i < 2 * G; i++) d[i] = T.dig[j0 + i];
            long long cy = use_slots ? T.slot[g * R + r] : 0;
#pragma unroll
            for (int i = 0; i < 2 * G - 1; i++) {
                if (cy) {
                    const int b = T.bits[j0 + i];
                    const long long v = d[i] + cy;
                    const long long q = (v + (1ll << (b - 1))) >> b;
                    d[i] = v - (q << b);
                    cy = q;
                }
            }
            d[2 * G - 1] += cy;
#pragma unroll
            for (int l = 0; l < G; l++)
                sm[r * G + l] = make_double2((double)d[2 * l] * T.w[j0 + 2 * l],
                                             (double)d[2 * l + 1] * T.w[j0 + 2 * l + 1]);
        }
        __syncthreads();
        smem_fft<false>(sm, T.cp, T.twc, G, G);
        for (int i = threadIdx.x; i < R * G; i += blockDim.x) {
            const int p = i / G, c = g * G + i % G;
            x[(size_t)p * C + c] = cmul(sm[i], T.t4[(size_t)p * C + c]);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kThreads) k_col_digits(const TestDesc *__restrict__ tests,
                                                         const WorkItem *__restrict__ work,
                                                         int nwork, const double2 *xo) {
    extern __shared__ double2 sm[];
    constexpr int G = kGroup;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const WorkItem it = work[wi];
        const TestDesc &T = tests[it.test];
        const double2 *x = xo ? xo : T.x;
        const int R = T.R, C = T.C, g = it.unit;
        for (int i = threadIdx.x; i < R * G; i += blockDim.x) {
            const int p = i / G, c = g * G + i % G;
            sm[i] = cmulc(x[(size_t)p * C + c], T.t4[(size_t)p * C + c]);
        }
        __syncthreads();
        smem_fft<true>(sm, T.cp, T.twc, G, G);
        for (int i = threadIdx.x; i < R * G; i += blockDim.x) {
            const int r = i / G, l = i % G;
            const int j = 2 * (r * C + g * G + l);
            T.dig[j] = llrint(sm[i].x * T.idig[j]);
            T.dig[j + 1] = llrint(sm[i].y * T.idig[j + 1]);
        }
        __syncthreads();
    }
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

int kernels_prepare(size_t row_smem, size_t col_smem) {
    int rc = 0;
    rc |= set_smem((const void *)k_rows<false>, row_smem);
    rc |= set_smem((const void *)k_rows<true>, row_smem);
    rc |= set_smem((const void *)k_col_inverse<false>, col_smem);
    rc |= set_smem((const void *)k_col_inverse<true>, col_smem);
    rc |= set_smem((const void *)k_col_forward, col_smem);
    rc |= set_smem((const void *)k_col_digits, col_smem);
    return rc;
}

void launch_rows(const LaunchSet &s, bool mul, double2 *x, const double2 *y, int step) {
    const size_t smem = s.row_smem_per_lane * (mul ? 4 : 2);
    if (mul)
        k_rows<true><<<s.grid_rows, kThreads, smem, s.stream>>>(s.tests, s.rows, s.nrows, s.nrows_dev, step, x, y);
    else
        k_rows<false><<<s.grid_rows, kThreads, smem, s.stream>>>(s.tests, s.rows, s.nrows, s.nrows_dev, step, x, y);
}

void launch_col_inverse(const LaunchSet &s, bool err, const double2 *x, int step) {
    if (err)
        k_col_inverse<true><<<s.grid_cols, kThreads, s.col_smem, s.stream>>>(s.tests, s.cols, s.ncols, s.ncols_dev, step, x);
    else
        k_col_inverse<false><<<s.grid_cols, kThreads, s.col_smem, s.stream>>>(s.tests, s.cols, s.ncols, s.ncols_dev, step, x);
}

void launch_col_forward(const LaunchSet &s, double2 *x, bool use_slots, int step) {
    k_col_forward<<<s.grid_cols, kThreads, s.col_smem, s.stream>>>(s.tests, s.cols, s.ncols, s.ncols_dev, step, x,
                                                                   use_slots ? 1 : 0);
}

void launch_col_digits(const LaunchSet &s, const double2 *x) {
    k_col_digits<<<s.grid_cols, kThreads, s.col_smem, s.stream>>>(s.tests, s.cols, s.ncols, x);
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

void launch_fp64_probe(cudaStream_t st, int grid, int block, int iters, double *out) {
    k_fp64_probe<<<grid, block, 0, st>>>(out, iters);
}

}  // namespace kg
