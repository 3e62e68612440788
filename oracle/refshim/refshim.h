/* Forced include for building the reference's portable C backends with gcc on Linux.
 *
 * The reference calls Apple libm's __cospi/__sinpi (cos(pi*x), sin(pi*x)).  glibc has no
 * such functions, so these stand-ins reduce the argument exactly before calling cos/sin:
 * x mod 2 is exact in binary floating point, and the reflections below (2-r, 1-r, 0.5-r)
 * are exact for r in the ranges where they are used.  Only the final multiply by pi and the
 * libm call round.  A plain cos(M_PI*x) loses accuracy for x near 2 and measurably raises
 * the round-off of long transforms.
 *
 * Test infrastructure only: nothing in the product links this.
 */
#ifndef KITE_REFSHIM_H
#define KITE_REFSHIM_H
#include <math.h>

static inline double refshim_cospi_0_half(double r) { /* r in [0, 0.5] */
    return r > 0.25 ? sin(M_PI * (0.5 - r)) : cos(M_PI * r);
}
static inline double refshim_sinpi_0_half(double r) { /* r in [0, 0.5] */
    return r > 0.25 ? cos(M_PI * (0.5 - r)) : sin(M_PI * r);
}
static inline double __cospi(double x) {
    double r = fmod(fabs(x), 2.0);          /* cos is even */
    if (r > 1.0) r = 2.0 - r;               /* cos(pi(2-r)) = cos(pi r) */
    if (r > 0.5) return -refshim_cospi_0_half(1.0 - r);
    return refshim_cospi_0_half(r);
}
static inline double __sinpi(double x) {
    double s = x < 0 ? -1.0 : 1.0;          /* sin is odd */
    double r = fmod(fabs(x), 2.0);
    if (r > 1.0) { r -= 1.0; s = -s; }      /* sin(pi(r+1)) = -sin(pi r) */
    if (r > 0.5) r = 1.0 - r;               /* sin(pi(1-r)) = sin(pi r) */
    return s * refshim_sinpi_0_half(r);
}
#endif
