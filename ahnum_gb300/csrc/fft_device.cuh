// Device building blocks: complex helpers, radix butterflies and the in-place shared-memory
// mixed-radix transform used by the row and column kernels.
//
// Every transform here is decimation in time (twiddles on the inputs of each butterfly).  The
// caller places element i at position pos(i) (the digit-reversed order of the plan), then the
// stages run from the last plan stage (span 1, no twiddles) to the first; the output is in
// natural order.  The forward transform uses exp(-2 pi i/n) and the inverse its conjugate;
// both are unnormalised.
//
// GB300's FP64 pipe is the bottleneck of the whole path, so the radix-2 and radix-4 stages use
// tangent-form twiddles: w_t = c_t (1 + i tau_t), x_t * (1 + i tau_t) costs 2 FMAs and the real
// factors c_t are folded into the butterfly, whose adds become FMAs.  A radix-4 butterfly with its
// three twiddles is 22 FP64 instructions instead of 28.  The odd radices (3, 5, 7) use plain
// complex twiddles.
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
// c * z + a (real c)
__device__ __forceinline__ double2 cfma(double c, double2 z, double2 a) {
    return make_double2(fma(c, z.x, a.x), fma(c, z.y, a.y));
}
// x * (1 + i tau)
__device__ __forceinline__ double2 tan_rot(double2 x, double tau) {
    return make_double2(fma(-tau, x.y, x.x), fma(tau, x.x, x.y));
}

// cos(2 pi r / P), sin(2 pi r / P) for the odd radices
template <int P>
__device__ __forceinline__ double cos2pi(int r);
template <int P>
__device__ __forceinline__ double sin2pi(int r);

template <>
__device__ __forceinline__ double cos2pi<3>(int) { return -0.5; }
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

// Radix-2 DIT butterfly, twiddle record {tau1, c1}: w1 = c1 (1 + i tau1) (conj for INV).
template <bool INV>
__device__ __forceinline__ void dit2_tan(double2 *x, const double2 *rec) {
    const double2 r = __ldg(rec);
    const double2 z1 = tan_rot(x[1], INV ? -r.x : r.x);
    const double2 x0 = x[0];
    x[0] = cfma(r.y, z1, x0);
    x[1] = cfma(-r.y, z1, x0);
}

// Radix-4 DIT butterfly, twiddle record {tau1, tau2}, {tau3, c1}, {c2, rho = c3/c1}:
//   y0 = a + c1 e', y2 = a - c1 e', y1 = b -+ i c1 f', y3 = b +- i c1 f'
// with z_t = x_t (1 + i tau_t), a = x0 + c2 z2, b = x0 - c2 z2, e' = z1 + rho z3, f' = z1 - rho z3.
template <bool INV>
__device__ __forceinline__ void dit4_tan(double2 *x, const double2 *rec) {
    const double2 r0 = __ldg(rec), r1 = __ldg(rec + 1), r2 = __ldg(rec + 2);
    const double s = INV ? -1.0 : 1.0;
    const double2 z1 = tan_rot(x[1], s * r0.x);
    const double2 z2 = tan_rot(x[2], s * r0.y);
    const double2 z3 = tan_rot(x[3], s * r1.x);
    const double c1 = r1.y, c2 = r2.x, rho = r2.y;
    const double2 a = cfma(c2, z2, x[0]);
    const double2 b = cfma(-c2, z2, x[0]);
    const double2 e = cfma(rho, z3, z1);
    const double2 f = cfma(-rho, z3, z1);
    x[0] = cfma(c1, e, a);
    x[2] = cfma(-c1, e, a);
    if (!INV) {
        x[1] = make_double2(fma(c1, f.y, b.x), fma(-c1, f.x, b.y));
        x[3] = make_double2(fma(-c1, f.y, b.x), fma(c1, f.x, b.y));
    } else {
        x[1] = make_double2(fma(-c1, f.y, b.x), fma(c1, f.x, b.y));
        x[3] = make_double2(fma(c1, f.y, b.x), fma(-c1, f.x, b.y));
    }
}

// One DIT stage over `nl` interleaved sequences: element e of sequence l at buf[e * ls + l].
// Twiddle records of this stage: (P-1) double2 per j.
template <int P, bool INV>
__device__ __forceinline__ void dit_stage(double2 *__restrict__ buf, int n, int span, int ls, int nl,
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
        // span 1 (every j = 0) takes the plain butterfly; other stages take the twiddled one for
        // every j, j = 0 included with its unit record, so no warp runs both code paths
        if (span == 1) {
            Dft<P, INV>::run(x);
        } else if (P == 4) {
            dit4_tan<INV>(x, tw + j * 3);
        } else if (P == 2) {
            dit2_tan<INV>(x, tw + j);
        } else {
#pragma unroll
            for (int t = 1; t < P; t++) {
                const double2 w = __ldg(&tw[j * (P - 1) + t - 1]);
                x[t] = INV ? cmulc(x[t], w) : cmul(x[t], w);
            }
            Dft<P, INV>::run(x);
        }
#pragma unroll
        for (int t = 0; t < P; t++) buf[base + t * stride] = x[t];
    }
}

template <bool INV>
__device__ __forceinline__ void dit_stage_dispatch(int p, double2 *buf, int n, int span, int ls, int nl,
                                                   const double2 *tw) {
    switch (p) {
    case 2: dit_stage<2, INV>(buf, n, span, ls, nl, tw); break;
    case 3: dit_stage<3, INV>(buf, n, span, ls, nl, tw); break;
    case 4: dit_stage<4, INV>(buf, n, span, ls, nl, tw); break;
    case 5: dit_stage<5, INV>(buf, n, span, ls, nl, tw); break;
    case 7: dit_stage<7, INV>(buf, n, span, ls, nl, tw); break;
    default: break;
    }
}

// Whole transform on data already placed in digit-reversed order (buf[pos(i)] = x_i); the
// caller synchronises before, and this returns after a final barrier with natural order.
template <bool INV>
__device__ __forceinline__ void smem_fft(double2 *buf, const FftPlan &pl, const double2 *tw, int ls, int nl) {
    for (int st = pl.nst - 1; st >= 0; st--) {
        dit_stage_dispatch<INV>(pl.rad[st], buf, pl.n, pl.span[st], ls, nl, tw + pl.off[st]);
        __syncthreads();
    }
}

}  // namespace kg
