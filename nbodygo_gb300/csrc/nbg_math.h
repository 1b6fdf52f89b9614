/*
 * nbg_math.h - project-owned FP64 elementary functions for collision resolution.
 *
 * The elastic-collision formulas (reference: cmd/body/collisioncalc.go:104-160)
 * call acos, atan2, sin, cos, asin and tan.  Go's math package, glibc and CUDA
 * each round these differently in the last bits, so a GPU kernel calling
 * CUDA's functions could never reproduce a CPU result bit for bit.  Both the
 * CPU oracle and every GPU kernel therefore call the functions below, which use
 * only +, -, *, /, sqrt, fabs, copysign and rint - all correctly rounded and
 * identical on x86-64, aarch64 and sm_103a provided no multiply-add contraction
 * happens (host: -ffp-contract=off; device: --fmad=false).
 *
 * Methods (all published; constants derived by gen_math_constants.py):
 *  - sin/cos/tan: additive argument reduction by pi/2 with a three-part
 *    constant (Cody & Waite, 1980), then Taylor polynomials of sin and cos on
 *    [-pi/4, pi/4] (terms to x^21 / x^22; truncation error < 2^-80).  cos adds
 *    the rounding error of 1 - x^2/2 back (Kahan-style compensation).
 *  - atan: reflection atan(x) = pi/2 - atan(1/x) for x > 1, then the identity
 *    atan(t) = pi/6 + atan((t*sqrt3 - 1)/(t + sqrt3)) for t > tan(pi/12), then
 *    the Taylor series of atan on |u| <= tan(pi/12) (terms to u^29).
 *  - atan2: C99 / Go special cases, then atan of the smaller/larger ratio
 *    with pi/2 and pi corrections carried as hi+lo pairs.
 *  - asin(x) = atan2(x, sqrt((1-x)(1+x))), acos(x) = atan2(sqrt((1-x)(1+x)), x).
 *
 * Accuracy: a few ulps against glibc over the arguments the collision code
 * produces (tests/test_math.py measures it).  Arguments beyond |x| ~ 1.6e6 are
 * reduced with growing error (the collision code only passes angles in
 * [-2*pi, 2*pi]); the result is still identical on every platform.
 */
#ifndef NBG_MATH_H
#define NBG_MATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define NBG_FN __host__ __device__ static inline
#else
#define NBG_FN static inline
#endif

#define NBG_DBL_MAX 0x1.fffffffffffffp+1023

#define NBG_PIO2_1 0x1.921fb54400000p+0
#define NBG_PIO2_2 0x1.0b4611a600000p-34
#define NBG_PIO2_3 0x1.3198a2e037073p-69
#define NBG_TWO_OVER_PI 0x1.45f306dc9c883p-1
#define NBG_PIO2_HI 0x1.921fb54442d18p+0
#define NBG_PIO2_LO 0x1.1a62633145c07p-54
#define NBG_PI_HI 0x1.921fb54442d18p+1
#define NBG_PI_LO 0x1.1a62633145c07p-53
#define NBG_PIO6_HI 0x1.0c152382d7366p-1
#define NBG_PIO6_LO (-0x1.ee6913347c2a6p-55)
#define NBG_PIO4_HI 0x1.921fb54442d18p-1
#define NBG_PI3O4_HI 0x1.2d97c7f3321d2p+1
#define NBG_SQRT3 0x1.bb67ae8584caap+0
#define NBG_TAN_PI_12 0x1.126145e9ecd56p-2

NBG_FN int nbg_signbit(double x)
{
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return (int)(u >> 63);
}

NBG_FN double nbg_nan(void)
{
    uint64_t u = 0x7ff8000000000001ull;
    double d;
    memcpy(&d, &u, sizeof d);
    return d;
}

NBG_FN int nbg_isinf(double x) { return fabs(x) > NBG_DBL_MAX; }
NBG_FN int nbg_isfinite(double x) { return fabs(x) <= NBG_DBL_MAX; }

/* sin(r) for |r| <= ~pi/4: r + r^3 * P(r^2), Taylor coefficients 1/(2k+1)!. */
NBG_FN double nbg_sin_poly(double r)
{
    double z = r * r;
    double p = 0x1.71b8ef6dcf572p-66;
    p = -0x1.2f49b46814157p-57 + z * p;
    p = 0x1.952c77030ad4ap-49 + z * p;
    p = -0x1.ae7f3e733b81fp-41 + z * p;
    p = 0x1.6124613a86d09p-33 + z * p;
    p = -0x1.ae64567f544e4p-26 + z * p;
    p = 0x1.71de3a556c734p-19 + z * p;
    p = -0x1.a01a01a01a01ap-13 + z * p;
    p = 0x1.1111111111111p-7 + z * p;
    p = -0x1.5555555555555p-3 + z * p;
    return r + (r * z) * p;
}

/* cos(r) for |r| <= ~pi/4: 1 - r^2/2 + r^4 * Q(r^2), Taylor coefficients. */
NBG_FN double nbg_cos_poly(double r)
{
    double z = r * r;
    double q = -0x1.0ce396db7f853p-70;
    q = 0x1.e542ba4020225p-62 + z * q;
    q = -0x1.6827863b97d97p-53 + z * q;
    q = 0x1.ae7f3e733b81fp-45 + z * q;
    q = -0x1.93974a8c07c9dp-37 + z * q;
    q = 0x1.1eed8eff8d898p-29 + z * q;
    q = -0x1.27e4fb7789f5cp-22 + z * q;
    q = 0x1.a01a01a01a01ap-16 + z * q;
    q = -0x1.6c16c16c16c17p-10 + z * q;
    q = 0x1.5555555555555p-5 + z * q;
    double hz = 0.5 * z;
    double w = 1.0 - hz;
    return w + (((1.0 - w) - hz) + (z * z) * q);
}

/* x = k*pi/2 + r with |r| <= ~pi/4; *quadrant = k mod 4. */
NBG_FN double nbg_reduce_pio2(double x, int *quadrant)
{
    if (fabs(x) <= NBG_PIO4_HI) {
        *quadrant = 0;
        return x;
    }
    double k = rint(x * NBG_TWO_OVER_PI);
    double r = ((x - k * NBG_PIO2_1) - k * NBG_PIO2_2) - k * NBG_PIO2_3;
    long long ki = fabs(k) < 0x1p62 ? (long long)k : 0;
    *quadrant = (int)(ki & 3);
    return r;
}

NBG_FN double nbg_sin(double x)
{
    if (x == 0.0) return x; /* keeps the sign of zero */
    if (!nbg_isfinite(x)) return nbg_nan();
    int q;
    double r = nbg_reduce_pio2(x, &q);
    switch (q) {
    case 0: return nbg_sin_poly(r);
    case 1: return nbg_cos_poly(r);
    case 2: return -nbg_sin_poly(r);
    default: return -nbg_cos_poly(r);
    }
}

NBG_FN double nbg_cos(double x)
{
    if (!nbg_isfinite(x)) return nbg_nan();
    int q;
    double r = nbg_reduce_pio2(x, &q);
    switch (q) {
    case 0: return nbg_cos_poly(r);
    case 1: return -nbg_sin_poly(r);
    case 2: return -nbg_cos_poly(r);
    default: return nbg_sin_poly(r);
    }
}

NBG_FN double nbg_tan(double x)
{
    if (x == 0.0) return x;
    if (!nbg_isfinite(x)) return nbg_nan();
    int q;
    double r = nbg_reduce_pio2(x, &q);
    double s = nbg_sin_poly(r);
    double c = nbg_cos_poly(r);
    return (q & 1) ? -c / s : s / c;
}

/* atan(u) for |u| <= tan(pi/12): u + u^3 * P(u^2), coefficients (-1)^k/(2k+1). */
NBG_FN double nbg_atan_poly(double u)
{
    double z = u * u;
    double p = 0x1.1a7b9611a7b96p-5;
    p = -0x1.2f684bda12f68p-5 + z * p;
    p = 0x1.47ae147ae147bp-5 + z * p;
    p = -0x1.642c8590b2164p-5 + z * p;
    p = 0x1.8618618618618p-5 + z * p;
    p = -0x1.af286bca1af28p-5 + z * p;
    p = 0x1.e1e1e1e1e1e1ep-5 + z * p;
    p = -0x1.1111111111111p-4 + z * p;
    p = 0x1.3b13b13b13b14p-4 + z * p;
    p = -0x1.745d1745d1746p-4 + z * p;
    p = 0x1.c71c71c71c71cp-4 + z * p;
    p = -0x1.2492492492492p-3 + z * p;
    p = 0x1.999999999999ap-3 + z * p;
    p = -0x1.5555555555555p-2 + z * p;
    return u + (u * z) * p;
}

/* atan(t) for 0 <= t <= 1. */
NBG_FN double nbg_atan01(double t)
{
    if (t > NBG_TAN_PI_12) {
        double u = (t * NBG_SQRT3 - 1.0) / (t + NBG_SQRT3);
        return NBG_PIO6_HI + (nbg_atan_poly(u) + NBG_PIO6_LO);
    }
    return nbg_atan_poly(t);
}

NBG_FN double nbg_atan(double x)
{
    if (x != x) return x + x;
    double ax = fabs(x);
    double r;
    if (ax > 1.0)
        r = NBG_PIO2_HI - (nbg_atan01(1.0 / ax) - NBG_PIO2_LO);
    else
        r = nbg_atan01(ax);
    return copysign(r, x);
}

NBG_FN double nbg_atan2(double y, double x)
{
    if (x != x || y != y) return x + y;
    if (y == 0.0) {
        if (x > 0.0 || (x == 0.0 && !nbg_signbit(x))) return y;
        return copysign(NBG_PI_HI, y);
    }
    if (x == 0.0) return copysign(NBG_PIO2_HI, y);
    if (nbg_isinf(x)) {
        if (x > 0.0) return nbg_isinf(y) ? copysign(NBG_PIO4_HI, y) : copysign(0.0, y);
        return nbg_isinf(y) ? copysign(NBG_PI3O4_HI, y) : copysign(NBG_PI_HI, y);
    }
    if (nbg_isinf(y)) return copysign(NBG_PIO2_HI, y);
    double ax = fabs(x), ay = fabs(y), r;
    if (ay <= ax)
        r = nbg_atan01(ay / ax);
    else
        r = NBG_PIO2_HI - (nbg_atan01(ax / ay) - NBG_PIO2_LO);
    if (x < 0.0) r = NBG_PI_HI - (r - NBG_PI_LO);
    return copysign(r, y);
}

NBG_FN double nbg_asin(double x)
{
    if (x != x) return x + x;
    if (fabs(x) > 1.0) return nbg_nan();
    return nbg_atan2(x, sqrt((1.0 - x) * (1.0 + x)));
}

NBG_FN double nbg_acos(double x)
{
    if (x != x) return x + x;
    if (fabs(x) > 1.0) return nbg_nan();
    return nbg_atan2(sqrt((1.0 - x) * (1.0 + x)), x);
}

/* Go's math.Min: NaN if either is NaN, -0 beats +0. */
NBG_FN double nbg_go_min(double x, double y)
{
    if (x != x || y != y) return nbg_nan();
    if (x == 0.0 && y == 0.0) return nbg_signbit(x) ? x : y;
    return x < y ? x : y;
}

/* Go's math.Max: NaN if either is NaN, +0 beats -0. */
NBG_FN double nbg_go_max(double x, double y)
{
    if (x != x || y != y) return nbg_nan();
    if (x == 0.0 && y == 0.0) return nbg_signbit(x) ? y : x;
    return x > y ? x : y;
}

#endif /* NBG_MATH_H */
