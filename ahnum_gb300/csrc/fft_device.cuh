// Device building blocks: complex helpers, radix-2/3/4/5/7/8 butterflies and the in-place
// shared-memory mixed-radix transform used by the row and column kernels.
#pragma once

#include <cuda_runtime.h>

#include "device.h"

namespace kg {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
// a * w
__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
    return make_double2(fma(a.x, w.x, -(a.y * w.y)), fma(a.x, w.y, a.y * w.x));
}
// a * conj(w)
__device__ __forceinline__ double2 cmulc(double2 a, double2 w) {
    return make_double2(fma(a.x, w.x, a.y * w.y), fma(a.y, w.x, -(a.x * w.y)));
}

// cos(2 pi r / P), sin(2 pi r / P) for the odd radices
template <int P>
__device__ __forceinline__ double cos2pi(int r);
template <int P>
__device__ __forceinline__ double sin2pi(int r);

template <>
__device__ __forceinline__ double cos2pi<3>(int r) { return -0.5; }
template <>
__device__ __forceinline__ double sin2pi<3>(int r) { return r == 1 ? 0.86602540378443864676 : -0.86602540378443864676; }
template <>
__device__ __forceinline__ double cos2pi<5>(int r) {
    return (r == 1 || r == 4) ? 0.30901699437494742410 : -0.80901699437494742410;
}
template <>
__device__ __forceinline__ double sin2pi<5>(int r) {
    switch (r) {
    case 1: return 0.95105651629515357212;
    case 2: return 0.58778525229247312917;
    case 3: return -0.58778525229247312917;
    default: return -0.95105651629515357212;
    }
}
template <>
__device__ __forceinline__ double cos2pi<7>(int r) {
    switch (r) {
    case 1: case 6: return 0.62348980185873353053;
    case 2: case 5: return -0.22252093395631440429;
    default: return -0.90096886790241912624;
    }
}
template <>
__device__ __forceinline__ double sin2pi<7>(int r) {
    switch (r) {
    case 1: return 0.78183148246802980871;
    case 2: return 0.97492791218182360702;
    case 3: return 0.43388373911755812048;
    case 4: return -0.43388373911755812048;
    case 5: return -0.97492791218182360702;
    default: return -0.78183148246802980871;
    }
}

// Length-P DFT in registers; forward uses exp(-2 pi i/P), INV exp(+2 pi i/P), unnormalised.
template <int P, bool INV>
struct Dft;

template <bool INV>
struct Dft<2, INV> {
    static __device__ __forceinline__ void run(double2 *x) {
        double2 a = x[0], b = x[1];
        x[0] = cadd(a, b);
        x[1] = csub(a, b);
    }
};

template <bool INV>
struct Dft<4, INV> {
    static __device__ __forceinline__ void run(double2 *x) {
        double2 a = cadd(x[0], x[2]), b = csub(x[0], x[2]);
        double2 c = cadd(x[1], x[3]), d = csub(x[1], x[3]);
        double2 f = INV ? make_double2(-d.y, d.x) : make_double2(d.y, -d.x);  // d * (+-i)
        x[0] = cadd(a, c);
        x[2] = csub(a, c);
        x[1] = cadd(b, f);
        x[3] = csub(b, f);
    }
};

template <bool INV>
struct Dft<8, INV> {
    static __device__ __forceinline__ void run(double2 *x) {
        double2 e[4] = {x[0], x[2], x[4], x[6]};
        double2 o[4] = {x[1], x[3], x[5], x[7]};
        Dft<4, INV>::run(e);
        Dft<4, INV>::run(o);
        const double h = 0.70710678118654752440;
        double2 t1, t2, t3;
        if (!INV) {
            t1 = make_double2((o[1].x + o[1].y) * h, (o[1].y - o[1].x) * h);
            t2 = make_double2(o[2].y, -o[2].x);
            t3 = make_double2((o[3].y - o[3].x) * h, -(o[3].x + o[3].y) * h);
        } else {
            t1 = make_double2((o[1].x - o[1].y) * h, (o[1].x + o[1].y) * h);
            t2 = make_double2(-o[2].y, o[2].x);
            t3 = make_double2(-(o[3].x + o[3].y) * h, (o[3].x - o[3].y) * h);
        }
        x[0] = cadd(e[0], o[0]);
        x[4] = csub(e[0], o[0]);
        x[1] = cadd(e[1], t1);
        x[5] = csub(e[1], t1);
        x[2] = cadd(e[2], t2);
        x[6] = csub(e[2], t2);
        x[3] = cadd(e[3], t3);
        x[7] = csub(e[3], t3);
    }
};

// odd P: pair x_m with x_{P-m}; y_j = A_j -+ i Z_j, y_{P-j} = A_j +- i Z_j
template <int P, bool INV>
struct DftOdd {
    static __device__ __forceinline__ void run(double2 *x) {
        constexpr int h = (P - 1) / 2;
        double2 a[h], b[h];
#pragma unroll
        for (int m = 1; m <= h; m++) {
            a[m - 1] = cadd(x[m], x[P - m]);
            b[m - 1] = csub(x[m], x[P - m]);
        }
        double2 y[P];
        y[0] = x[0];
#pragma unroll
        for (int m = 0; m < h; m++) y[0] = cadd(y[0], a[m]);
#pragma unroll
        for (int j = 1; j <= h; j++) {
            double2 A = x[0];
            double2 Z = make_double2(sin2pi<P>(j % P) * b[0].x, sin2pi<P>(j % P) * b[0].y);
#pragma unroll
            for (int m = 1; m <= h; m++) {
                const double c = cos2pi<P>((j * m) % P);
                A.x = fma(c, a[m - 1].x, A.x);
                A.y = fma(c, a[m - 1].y, A.y);
                if (m > 1) {
                    const double s = sin2pi<P>((j * m) % P);
                    Z.x = fma(s, b[m - 1].x, Z.x);
                    Z.y = fma(s, b[m - 1].y, Z.y);
                }
            }
            if (!INV) {
                y[j] = make_double2(A.x + Z.y, A.y - Z.x);
                y[P - j] = make_double2(A.x - Z.y, A.y + Z.x);
            } else {
                y[j] = make_double2(A.x - Z.y, A.y + Z.x);
                y[P - j] = make_double2(A.x + Z.y, A.y - Z.x);
            }
        }
#pragma unroll
        for (int t = 0; t < P; t++) x[t] = y[t];
    }
};
template <bool INV>
struct Dft<3, INV> : DftOdd<3, INV> {};
template <bool INV>
struct Dft<5, INV> : DftOdd<5, INV> {};
template <bool INV>
struct Dft<7, INV> : DftOdd<7, INV> {};

// One stage of the in-place transform over `nl` interleaved sequences; element e of sequence l
// is at buf[e * ls + l].  Forward (DIF): butterfly, then output twiddles w_{P*span}^{t*j}.
// Inverse (DIT): conjugate input twiddles, then the inverse butterfly.
template <int P, bool INV>
__device__ __forceinline__ void fft_stage(double2 *__restrict__ buf, int n, int span, int ls, int nl,
                                          const double2 *__restrict__ tw) {
    const int total = (n / P) * nl;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int l = i % nl;
        const int bf = i / nl;
        const int j = bf % span;
        const int blk = bf / span;
        const int base = (blk * P * span + j) * ls + l;
        const int stride = span * ls;
        double2 x[P];
#pragma unroll
        for (int t = 0; t < P; t++) x[t] = buf[base + t * stride];
        if (!INV) {
            Dft<P, false>::run(x);
            if (j) {
#pragma unroll
                for (int t = 1; t < P; t++) x[t] = cmul(x[t], __ldg(&tw[t * span + j]));
            }
        } else {
            if (j) {
#pragma unroll
                for (int t = 1; t < P; t++) x[t] = cmulc(x[t], __ldg(&tw[t * span + j]));
            }
            Dft<P, true>::run(x);
        }
#pragma unroll
        for (int t = 0; t < P; t++) buf[base + t * stride] = x[t];
    }
}

template <bool INV>
__device__ __forceinline__ void fft_stage_dispatch(int p, double2 *buf, int n, int span, int ls, int nl,
                                                   const double2 *tw) {
    switch (p) {
    case 2: fft_stage<2, INV>(buf, n, span, ls, nl, tw); break;
    case 3: fft_stage<3, INV>(buf, n, span, ls, nl, tw); break;
    case 4: fft_stage<4, INV>(buf, n, span, ls, nl, tw); break;
    case 5: fft_stage<5, INV>(buf, n, span, ls, nl, tw); break;
    case 7: fft_stage<7, INV>(buf, n, span, ls, nl, tw); break;
    case 8: fft_stage<8, INV>(buf, n, span, ls, nl, tw); break;
    default: break;
    }
}

// Whole transform; the caller synchronises before (data loaded) and this returns after a
// final barrier.
template <bool INV>
__device__ __forceinline__ void smem_fft(double2 *buf, const FftPlan &pl, const double2 *tw, int ls, int nl) {
    if (!INV) {
        for (int st = 0; st < pl.nst; st++) {
            fft_stage_dispatch<false>(pl.rad[st], buf, pl.n, pl.span[st], ls, nl, tw + pl.off[st]);
            __syncthreads();
        }
    } else {
        for (int st = pl.nst - 1; st >= 0; st--) {
            fft_stage_dispatch<true>(pl.rad[st], buf, pl.n, pl.span[st], ls, nl, tw + pl.off[st]);
            __syncthreads();
        }
    }
}

}  // namespace kg
