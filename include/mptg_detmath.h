/*
 * mptg_detmath.h - deterministic FP64 elementary functions (sin, cos, acos)
 * compiled identically for the host (C/C++, -ffp-contract=off) and the
 * device (CUDA, explicit round-to-nearest intrinsics, so no FMA contraction).
 *
 * Why: the planner's validity booleans (link-arm forward kinematics) and the
 * SO(3)/SE(3) distances depend on sin/cos/acos.  glibc and CUDA's libdevice
 * are not guaranteed to round these identically, so a device kernel and a CPU
 * checker that each call "their" sin would disagree on rare inputs.  Both sides
 * call the functions below instead, built only from +, -, *, /, sqrt and rint
 * (all correctly rounded in IEEE-754 on both machines), so results are
 * bit-identical everywhere.
 *
 * Methods (written from the mathematics, no library constants):
 *  - sin/cos: Cody & Waite additive argument reduction by pi/2 split into three
 *    parts (W. J. Cody, W. Waite, "Software Manual for the Elementary
 *    Functions", 1980), then the Taylor series of sin and cos on |r| <= pi/4
 *    truncated after the r^19 / r^18 terms (truncation error < 1e-21).
 *    Coefficients are (-1)^n/(2n+1)! and (-1)^n/(2n)!, rounded to double.
 *  - acos: acos(x) = pi/2 - asin(x) for |x| <= 1/2 and
 *    acos(x) = 2 asin(sqrt((1-x)/2)) for |x| > 1/2; asin(z), |z| <= 1/2, by
 *    its Maclaurin series with coefficients (2n)!/(4^n (n!)^2 (2n+1)),
 *    27 terms (truncation error < 1e-19 relative).
 * Accuracy against correctly-rounded results is a few ulp; the unit tests
 * measure it against glibc/numpy.  Argument reduction is exact for
 * |x| < 2^20 * pi/2, which covers every angle the planner forms (|x| <= 10 pi).
 */
#ifndef MPTG_DETMATH_H
#define MPTG_DETMATH_H

#if defined(__CUDACC__)
#define MPTG_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#define MPTG_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define MPTG_DADD(a, b) __dadd_rn((a), (b))
#define MPTG_DSUB(a, b) __dsub_rn((a), (b))
#define MPTG_DMUL(a, b) __dmul_rn((a), (b))
#define MPTG_DDIV(a, b) __ddiv_rn((a), (b))
#define MPTG_DSQRT(a) __dsqrt_rn(a)
#define MPTG_DRINT(a) rint(a)
#else
#define MPTG_DADD(a, b) ((a) + (b))
#define MPTG_DSUB(a, b) ((a) - (b))
#define MPTG_DMUL(a, b) ((a) * (b))
#define MPTG_DDIV(a, b) ((a) / (b))
#define MPTG_DSQRT(a) sqrt(a)
#define MPTG_DRINT(a) rint(a)
#endif

#define MPTG_PI 0x1.921fb54442d18p+1
#define MPTG_TWO_PI 0x1.921fb54442d18p+2
#define MPTG_PI_2 0x1.921fb54442d18p+0
#define MPTG_2_OVER_PI 0x1.45f306dc9c883p-1
/* pi/2 = PIO2_1 + PIO2_2 + PIO2_3, the first two with 33 significant bits so
 * that k*PIO2_1 and k*PIO2_2 are exact for |k| < 2^20. */
#define MPTG_PIO2_1 0x1.921fb54400000p+0
#define MPTG_PIO2_2 0x1.0b4611a600000p-34
#define MPTG_PIO2_3 0x1.3198a2e037073p-69

/* sin(r), cos(r) for |r| <= pi/4 (Taylor series, Horner in z = r^2). */
MPTG_HD double mptg_sin_kernel(double r) {
    double z = MPTG_DMUL(r, r);
    double p = -0x1.2f49b46814157p-57;              /* -1/19! */
    p = MPTG_DADD(MPTG_DMUL(p, z), 0x1.952c77030ad4ap-49);   /* 1/17! */
    p = MPTG_DADD(MPTG_DMUL(p, z), -0x1.ae7f3e733b81fp-41);  /* -1/15! */
    p = MPTG_DADD(MPTG_DMUL(p, z), 0x1.6124613a86d09p-33);   /* 1/13! */
    p = MPTG_DADD(MPTG_DMUL(p, z), -0x1.ae64567f544e4p-26);  /* -1/11! */
    p = MPTG_DADD(MPTG_DMUL(p, z), 0x1.71de3a556c734p-19);   /* 1/9! */
    p = MPTG_DADD(MPTG_DMUL(p, z), -0x1.a01a01a01a01ap-13);  /* -1/7! */
    p = MPTG_DADD(MPTG_DMUL(p, z), 0x1.1111111111111p-7);    /* 1/5! */
    p = MPTG_DADD(MPTG_DMUL(p, z), -0x1.5555555555555p-3);   /* -1/3! */
    return MPTG_DADD(r, MPTG_DMUL(MPTG_DMUL(r, z), p));
}

MPTG_HD double mptg_cos_kernel(double r) {
    double z = MPTG_DMUL(r, r);
    double p = -0x1.6827863b97d97p-53;              /* -1/18! */
    p = MPTG_DADD(MPTG_DMUL(p, z), 0x1.ae7f3e733b81fp-45);   /* 1/16! */
    p = MPTG_DADD(MPTG_DMUL(p, z), -0x1.93974a8c07c9dp-37);  /* -1/14! */
    p = MPTG_DADD(MPTG_DMUL(p, z), 0x1.1eed8eff8d898p-29);   /* 1/12! */
    p = MPTG_DADD(MPTG_DMUL(p, z), -0x1.27e4fb7789f5cp-22);  /* -1/10! */
    p = MPTG_DADD(MPTG_DMUL(p, z), 0x1.a01a01a01a01ap-16);   /* 1/8! */
    p = MPTG_DADD(MPTG_DMUL(p, z), -0x1.6c16c16c16c17p-10);  /* -1/6! */
    p = MPTG_DADD(MPTG_DMUL(p, z), 0x1.5555555555555p-5);    /* 1/4! */
    p = MPTG_DADD(MPTG_DMUL(p, z), -0x1.0000000000000p-1);   /* -1/2! */
    return MPTG_DADD(1.0, MPTG_DMUL(z, p));
}

/* sin and cos of x; exact reduction for |x| < 2^20 * pi/2. */
MPTG_HD void mptg_sincos(double x, double* s, double* c) {
    double k = MPTG_DRINT(MPTG_DMUL(x, MPTG_2_OVER_PI));
    double r = MPTG_DSUB(x, MPTG_DMUL(k, MPTG_PIO2_1));
    r = MPTG_DSUB(r, MPTG_DMUL(k, MPTG_PIO2_2));
    r = MPTG_DSUB(r, MPTG_DMUL(k, MPTG_PIO2_3));
    double sr = mptg_sin_kernel(r);
    double cr = mptg_cos_kernel(r);
    long long q = (long long)k;
    int quad = (int)(q & 3);
    switch (quad) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
    }
}

/* asin(z) for |z| <= 1/2 by its Maclaurin series (27 terms). */
MPTG_HD double mptg_asin_series(double z) {
    double w = MPTG_DMUL(z, z);
    double p = 0x1.018f963c229bfp-9;                           /* n=27 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.1052bc5fa960ap-9);     /* 26 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.208d3570ae5a6p-9);     /* 25 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.3275586c5f2f0p-9);     /* 24 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.464c0950f7d47p-9);     /* 23 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.5c5f56efaaaabp-9);     /* 22 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.750de64d7d05fp-9);     /* 21 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.90cb77f60c7cep-9);     /* 20 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.b026f57b13b14p-9);     /* 19 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.d3d2a8e0dd67dp-9);     /* 18 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.fcaf8fb6db6dbp-9);     /* 17 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.15ee9d45d1746p-8);     /* 16 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.31683bdef7bdfp-8);     /* 15 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.51ba308d3dcb1p-8);     /* 14 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.782dda12f684cp-8);     /* 13 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.a6863d70a3d71p-8);     /* 12 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.df3bd37a6f4dfp-8);     /* 11 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.12ef3cf3cf3cfp-7);     /* 10 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.3fde50d79435ep-7);     /* 9 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.7a87878787878p-7);     /* 8 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.c99999999999ap-7);     /* 7 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.1c4ec4ec4ec4fp-6);     /* 6 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.6e8ba2e8ba2e9p-6);     /* 5 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.f1c71c71c71c7p-6);     /* 4 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.6db6db6db6db7p-5);     /* 3 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.3333333333333p-4);     /* 2 */
    p = MPTG_DADD(MPTG_DMUL(p, w), 0x1.5555555555555p-3);     /* 1 */
    return MPTG_DADD(z, MPTG_DMUL(MPTG_DMUL(z, w), p));
}

/* acos(x) for x in [-1, 1]; NaN propagates, |x| > 1 returns NaN. */
MPTG_HD double mptg_acos(double x) {
    double a = x < 0 ? -x : x;
    double r;
    if (!(a <= 1.0)) return MPTG_DSUB(x, x) / MPTG_DSUB(x, x); /* NaN */
    if (a <= 0.5) {
        r = MPTG_DSUB(MPTG_PI_2, mptg_asin_series(a));
    } else {
        double z = MPTG_DSQRT(MPTG_DMUL(MPTG_DSUB(1.0, a), 0.5));
        r = MPTG_DMUL(2.0, mptg_asin_series(z));
    }
    return x < 0 ? MPTG_DSUB(MPTG_PI, r) : r;
}

MPTG_HD double mptg_sin(double x) { double s, c; mptg_sincos(x, &s, &c); return s; }
MPTG_HD double mptg_cos(double x) { double s, c; mptg_sincos(x, &s, &c); return c; }

#endif /* MPTG_DETMATH_H */
