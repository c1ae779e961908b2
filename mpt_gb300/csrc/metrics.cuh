// metrics.cuh - metric spaces on the device.
//
// Two versions of every distance:
//  * dist64: the exact definition in FP64 with explicit round-to-nearest
//    intrinsics (no FMA contraction), evaluated in the same operation order
//    as the reference formulas so results are bit-identical to a CPU that
//    evaluates the same expressions with -ffp-contract=off.
//    L2  : sqrt of the left-to-right sum of squared differences
//          (src/mpt/lp_space.hpp, nigh LPSpace<_, D, 2>; test/lp_space_test.cpp:39-50)
//    L1  : left-to-right sum of |differences|
//    SO2 : left-to-right sum of min(d, 2pi - d), d = |a - b|
//          (nigh SO2LPSpace<_, D, 1>; test/so2_space_test.cpp:39-65)
//    SO3 : acos(min(1, |a.b|)), a.b summed x, y, z, w
//          (nigh SO3Space; test/so3_space_test.cpp:39-56)
//    SE3 : w0 * SO3 + w1 * L2(translation)
//          (SE3Space = Cartesian<Scaled<SO3,w0>, Scaled<L2,w1>>; test/se3_space_test.cpp:45-89)
//  * dist32: an FP32 approximation for the bulk sweep, with an a-priori
//    absolute error bound err32() used to decide which candidates must be
//    re-ranked in FP64 (see kd-tree search).
#pragma once
#include "common.cuh"

#define U32 5.9604645e-8f  // 2^-24, unit roundoff of FP32
#define PI_F 3.14159265358979323846f
#define TWO_PI_F 6.28318530717958647692f

// SO(3)/SE(3) FP32 angle error bound (radians): input rounding of the unit
// quaternion components (4u per chord), asinf rounding, and the difference
// between the chord form and acos(|dot|) for states whose squared norm is
// within 1e-12 of one (at most sqrt(2e-12) = 1.5e-6).
#define MPTG_SO3_ERR32 1.0e-5f
// inserted/queried quaternions must satisfy | |q|^2 - 1 | <= this
#define MPTG_QUAT_NORM_TOL 1.0e-12

__device__ __forceinline__ double so2_dist1_64(double a, double b) {
    double d = fabs(__dsub_rn(a, b));
    if (d > MPTG_TWO_PI) d = fmod(d, MPTG_TWO_PI);
    return d > MPTG_PI ? __dsub_rn(MPTG_TWO_PI, d) : d;
}

__device__ __forceinline__ double quat_dot64(const double* a, const double* b) {
    double s = __dmul_rn(a[0], b[0]);
    s = __dadd_rn(s, __dmul_rn(a[1], b[1]));
    s = __dadd_rn(s, __dmul_rn(a[2], b[2]));
    s = __dadd_rn(s, __dmul_rn(a[3], b[3]));
    return s;
}

__device__ __forceinline__ double so3_dist64(const double* a, const double* b) {
    double d = fabs(quat_dot64(a, b));
    if (d > 1.0) d = 1.0;
    return mptg_acos(d);
}

__device__ __forceinline__ double l2_dist64(const double* a, const double* b, int D) {
    double s = 0.0;
    for (int i = 0; i < D; ++i) {
        double d = __dsub_rn(a[i], b[i]);
        s = __dadd_rn(s, __dmul_rn(d, d));
    }
    return __dsqrt_rn(s);
}

// exact FP64 distance; a, b point at D doubles
__device__ __forceinline__ double dist64(int metric, int D, double w0, double w1, const double* a,
                                         const double* b) {
    switch (metric) {
    case MPTG_METRIC_L2: return l2_dist64(a, b, D);
    case MPTG_METRIC_L1: {
        double r = 0.0;
        for (int i = 0; i < D; ++i) r = __dadd_rn(r, fabs(__dsub_rn(a[i], b[i])));
        return r;
    }
    case MPTG_METRIC_SO2: {
        double r = 0.0;
        for (int i = 0; i < D; ++i) r = __dadd_rn(r, so2_dist1_64(a[i], b[i]));
        return r;
    }
    case MPTG_METRIC_SO3: return so3_dist64(a, b);
    case MPTG_METRIC_SE3:
        return __dadd_rn(__dmul_rn(w0, so3_dist64(a, b)), __dmul_rn(w1, l2_dist64(a + 4, b + 4, 3)));
    }
    return __longlong_as_double(0x7ff8000000000000ll);
}

// ---- interpolation (exact FP64, mirrors the reference expressions) ----
// fmod(x, 2pi) is x itself when |x| < 2pi (fmod is exact), which skips the
// library's reduction loop in the common case
__device__ __forceinline__ double fmod_2pi(double x) { return fabs(x) < MPTG_TWO_PI ? x : fmod(x, MPTG_TWO_PI); }
__device__ __forceinline__ double so2_ccw64(double a, double b) {
    double d = fmod_2pi(__dsub_rn(b, a));
    if (d < 0) d = __dadd_rn(d, MPTG_TWO_PI);
    return d;
}
__device__ __forceinline__ double so2_bound64(double v) {
    v = fmod_2pi(v);
    if (v < -MPTG_PI) v = __dadd_rn(v, MPTG_TWO_PI);
    else if (v >= MPTG_PI) v = __dsub_rn(v, MPTG_TWO_PI);
    return v;
}
__device__ __forceinline__ double so2_interp64(double a, double b, double t) {
    // src/mpt/so2_space.hpp:44-65
    double ccw = so2_ccw64(a, b);
    if (ccw < MPTG_PI) return so2_bound64(__dadd_rn(a, __dmul_rn(ccw, t)));
    double cw = __dsub_rn(MPTG_TWO_PI, ccw);
    return so2_bound64(__dsub_rn(a, __dmul_rn(cw, t)));
}
__device__ __forceinline__ void so3_interp64(const double* a, const double* b, double t, double* q) {
    // src/mpt/so3_space.hpp:44-83
    double d = quat_dot64(a, b);
    double ad = fabs(d);
    double s0, s1;
    if (d >= 1.0 - 2.220446049250313e-16) {
        s0 = __dsub_rn(1.0, t);
        s1 = t;
    } else {
        double theta = mptg_acos(ad);
        double sinTheta = mptg_sin(theta);
        s0 = __ddiv_rn(mptg_sin(__dmul_rn(__dsub_rn(1.0, t), theta)), sinTheta);
        s1 = __ddiv_rn(mptg_sin(__dmul_rn(t, theta)), sinTheta);
    }
    if (d < 0) s1 = -s1;
    for (int i = 0; i < 4; ++i) q[i] = __dadd_rn(__dmul_rn(s0, a[i]), __dmul_rn(s1, b[i]));
}
__device__ __forceinline__ void interp64(int metric, int D, const double* a, const double* b, double t,
                                         double* q) {
    switch (metric) {
    case MPTG_METRIC_L2:
    case MPTG_METRIC_L1:
        // src/mpt/lp_space.hpp:44-54: (b - a) * t + a
        for (int i = 0; i < D; ++i) q[i] = __dadd_rn(__dmul_rn(__dsub_rn(b[i], a[i]), t), a[i]);
        break;
    case MPTG_METRIC_SO2:
        for (int i = 0; i < D; ++i) q[i] = so2_interp64(a[i], b[i], t);
        break;
    case MPTG_METRIC_SO3: so3_interp64(a, b, t, q); break;
    case MPTG_METRIC_SE3:
        so3_interp64(a, b, t, q);
        for (int i = 4; i < 7; ++i) q[i] = __dadd_rn(__dmul_rn(__dsub_rn(b[i], a[i]), t), a[i]);
        break;
    }
}

// ---- FP32 sweep distances ---------------------------------------------
// q, p: DMAX floats (entries >= D are zero for Lp/SO2 so they add nothing)
template <int MK, int DMAX>
__device__ __forceinline__ float dist32(const float* q, const float* p, float w0, float w1) {
    if constexpr (MK == MPTG_METRIC_L2) {
        float s = 0.f;
#pragma unroll
        for (int d = 0; d < DMAX; ++d) { float t = q[d] - p[d]; s = fmaf(t, t, s); }
        return sqrtf(s);
    } else if constexpr (MK == MPTG_METRIC_L1) {
        float s = 0.f;
#pragma unroll
        for (int d = 0; d < DMAX; ++d) s += fabsf(q[d] - p[d]);
        return s;
    } else if constexpr (MK == MPTG_METRIC_SO2) {
        float s = 0.f;
#pragma unroll
        for (int d = 0; d < DMAX; ++d) {
            float t = fabsf(q[d] - p[d]);
            s += fminf(t, TWO_PI_F - t);
        }
        return s;
    } else {  // SO3 (DMAX 4) / SE3 (DMAX 8, translation in 4..6)
        float dot = q[0] * p[0] + q[1] * p[1] + q[2] * p[2] + q[3] * p[3];
        float sg = dot < 0.f ? -1.f : 1.f;
        float c2 = 0.f;
#pragma unroll
        for (int d = 0; d < 4; ++d) { float t = q[d] - sg * p[d]; c2 = fmaf(t, t, c2); }
        float ang = 2.f * asinf(fminf(1.f, 0.5f * sqrtf(c2)));
        if constexpr (MK == MPTG_METRIC_SO3) {
            return ang;
        } else {
            float s = 0.f;
#pragma unroll
            for (int d = 4; d < 7; ++d) { float t = q[d] - p[d]; s = fmaf(t, t, s); }
            return w0 * ang + w1 * sqrtf(s);
        }
    }
}

// Absolute bound on |dist32 - dist64| for any stored point, given the largest
// coordinate magnitude M over the tree and the query (Lp / translation part).
// Lp: input rounding to FP32 moves each coordinate by <= u*M, so the distance
// moves by <= 2u*M*sqrt(D) (L2) or 2u*M*D (L1); the FP32 evaluation adds a
// relative error <= (D+3)u on a distance <= 2M*sqrt(D) (L2) / 2M*D (L1).
// SO2: each wrapped term carries <= 8u*pi, the sum adds D*u*D*pi.
// A factor 2 of slack is applied on top.
template <int MK>
__device__ __forceinline__ float err32(int D, float M, float w0, float w1) {
    float fd = (float)D;
    if (MK == MPTG_METRIC_L2) return 2.f * U32 * M * sqrtf(fd) * (2.f + 2.f * (fd + 3.f)) + 1e-30f;
    if (MK == MPTG_METRIC_L1) return 2.f * U32 * M * fd * (2.f + 2.f * (fd + 3.f)) + 1e-30f;
    if (MK == MPTG_METRIC_SO2) return 2.f * U32 * PI_F * fd * (8.f + fd);
    if (MK == MPTG_METRIC_SO3) return MPTG_SO3_ERR32;
    // SE3: rotation bound plus a 3-D L2 bound
    return w0 * MPTG_SO3_ERR32 + w1 * (2.f * U32 * M * 1.7320508f * (2.f + 2.f * 6.f)) + 1e-30f;
}
