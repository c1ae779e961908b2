// grid.cuh - exact occupancy-grid validity (demo/png_2d_scenario.hpp:104-110)
// and the DMV step count of grid edges (discrete_motion_validator.hpp:78),
// shared by the batched validity kernels (scene.cu) and the persistent block
// planner (bplan.cu).  FP32 filters with a-priori error margins decide almost
// every case; the rest is recomputed in FP64 with round-to-nearest intrinsics.
#pragma once
#include "metrics.cuh"
#include "scene.cuh"

enum { VF_INVALID = 0, VF_VALID = 1, VF_UNSURE = 2 };

__device__ __forceinline__ bool grid_valid64(const SceneView& s, const double* q) {
    double vx = __dadd_rn(q[0], 0.5), vy = __dadd_rn(q[1], 0.5);
    if (!(vx > -1.0 && vx < (double)s.width && vy > -1.0 && vy < (double)s.height)) return false;
    int x = __double2int_rz(vx), y = __double2int_rz(vy);
    return __ldg(&s.grid[(size_t)s.width * y + x]) == 0;
}

// grid: cell = (int)(x + 0.5) per axis; e bounds |v32 - v64| for v = x + 0.5
__device__ __forceinline__ int grid_valid32(const SceneView& s, float x, float y, float e) {
    float vx = x + 0.5f, vy = y + 0.5f;
    // every decision boundary (integers, -1 and the grid size) must be farther than e
    float fx = vx - floorf(vx), fy = vy - floorf(vy);
    if (fx <= e || fx >= 1.f - e || fy <= e || fy >= 1.f - e) return VF_UNSURE;
    if (!(vx > -1.f && vx < (float)s.width && vy > -1.f && vy < (float)s.height)) return VF_INVALID;
    int xi = (int)vx, yi = (int)vy;
    return __ldg(&s.grid[(size_t)s.width * yi + xi]) == 0 ? VF_VALID : VF_INVALID;
}

// exact decision for a grid state given in FP64 (FP32 filter first)
__device__ __forceinline__ bool grid_valid_f(const SceneView& s, const double* q) {
    float x = __double2float_rn(q[0]), y = __double2float_rn(q[1]);
    float e = 4.f * U32 * (fabsf(x) + fabsf(y) + 1.f);
    int r = (x == x && y == y && fabsf(x) < 1e7f && fabsf(y) < 1e7f) ? grid_valid32(s, x, y, e) : VF_UNSURE;
    if (r != VF_UNSURE) return r == VF_VALID;
    return grid_valid64(s, q);
}

// grid edge step count ceil(|a - b| * inv) (the L2 metric, dist64) with an
// FP32 filter: FP64 only when the FP32 value lies within its error bound of
// an integer
__device__ __forceinline__ long long grid_edge_steps(const double* A, const double* B, double inv,
                                                    bool* used64 = nullptr) {
    float dx = __double2float_rn(A[0]) - __double2float_rn(B[0]);
    float dy = __double2float_rn(A[1]) - __double2float_rn(B[1]);
    float m32 = sqrtf(dx * dx + dy * dy);
    float M = fmaxf(fmaxf(fabsf((float)A[0]), fabsf((float)A[1])), fmaxf(fabsf((float)B[0]), fabsf((float)B[1])));
    float err = 16.f * U32 * (M + m32) + 1e-30f;
    if (m32 == m32) {
        float x = m32 * (float)inv;
        float e = err * (float)inv + 4.f * U32 * x;
        float lo = ceilf(x - e), hi = ceilf(x + e);
        if (lo == hi && x < 1e7f) return (long long)lo;
    }
    if (used64) *used64 = true;
    double sd = ceil(__dmul_rn(l2_dist64(A, B, 2), inv));
    if (!(sd >= 0.0) || sd > (double)MPTG_MAX_EDGE_SAMPLES) return -1;
    return (long long)sd;
}

