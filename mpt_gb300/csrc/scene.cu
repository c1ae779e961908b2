// scene.cu - batched state validity and discretised motion validity.
//
// Replaces, batched on the device:
//   Scenario::valid(q)   src/mpt/impl/prrt/prrt.hpp:439, modelled by
//     demo/png_2d_scenario.hpp:104-110            (occupancy grid)
//     demo/link_manipulator_scenario.hpp:99-116   (planar link arm)
//     demo/se3_rigid_body_scenario.hpp:282-312    (rigid mesh, see mesh.cu)
//   Scenario::link(a, b) through DiscreteMotionValidator
//     src/mpt/discrete_motion_validator.hpp:71-130
//
// The DMV result is the AND of valid() over the fixed sample set
// {b} U {interpolate(a, b, i/steps) : 1 <= i < steps}, so evaluation order
// does not change it.  Grid edges: a thread per edge checks b and the step
// count, then a warp per surviving edge takes 32 samples per round in a
// coarse-to-fine spread (lane j of round r tests sample j*R + r).  Planar-arm
// edges: a warp (up to 8 warps for small batches) per edge decides one sample
// at a time with the lanes split over the (link, obstacle) pairs, so it leaves
// soon after the first colliding link of the first colliding sample.
//
// Exactness: every boolean equals the FP64 definition.  Values are first
// computed in FP32 with an a-priori error margin; a decision whose FP32 value
// lies inside the margin of its boundary is recomputed in FP64 with explicit
// round-to-nearest intrinsics (no FMA contraction) and the deterministic
// sin/cos of mptg_detmath.h, the same expressions the CPU checker evaluates.
#include "metrics.cuh"
#include "scene.cuh"
#include "grid.cuh"
#include <algorithm>
#include <vector>

// ------------------------------------------------------------------ arm
__device__ __forceinline__ double dist_point_segment_sq64(double px, double py, double ax, double ay, double bx,
                                                          double by) {
    // demo/shape_hierarchy.hpp:259-270
    double vx = __dsub_rn(bx, ax), vy = __dsub_rn(by, ay);
    double wx = __dsub_rn(px, ax), wy = __dsub_rn(py, ay);
    double c1 = __dadd_rn(__dmul_rn(vx, wx), __dmul_rn(vy, wy));
    if (c1 <= 0) return __dadd_rn(__dmul_rn(wx, wx), __dmul_rn(wy, wy));
    double c2 = __dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy));
    if (c2 <= c1) {
        double ex = __dsub_rn(px, bx), ey = __dsub_rn(py, by);
        return __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
    }
    double f = __ddiv_rn(c1, c2);
    double ex = __dadd_rn(__dsub_rn(ax, px), __dmul_rn(vx, f));
    double ey = __dadd_rn(__dsub_rn(ay, py), __dmul_rn(vy, f));
    return __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
}

__device__ __forceinline__ double orient2d64(double ax, double ay, double bx, double by, double cx, double cy) {
    return __dsub_rn(__dmul_rn(__dsub_rn(bx, ax), __dsub_rn(cy, ay)), __dmul_rn(__dsub_rn(by, ay), __dsub_rn(cx, ax)));
}

__device__ __forceinline__ bool on_seg_box64(double ax, double ay, double bx, double by, double px, double py) {
    return fmin(ax, bx) <= px && px <= fmax(ax, bx) && fmin(ay, by) <= py && py <= fmax(ay, by);
}

// closed segments [a,b], [c,d] touch or cross
__device__ __forceinline__ bool segs_intersect64(double ax, double ay, double bx, double by, double cx, double cy,
                                                 double dx, double dy) {
    double o1 = orient2d64(ax, ay, bx, by, cx, cy);
    double o2 = orient2d64(ax, ay, bx, by, dx, dy);
    double o3 = orient2d64(cx, cy, dx, dy, ax, ay);
    double o4 = orient2d64(cx, cy, dx, dy, bx, by);
    if (((o1 > 0 && o2 < 0) || (o1 < 0 && o2 > 0)) && ((o3 > 0 && o4 < 0) || (o3 < 0 && o4 > 0))) return true;
    if (o1 == 0 && on_seg_box64(ax, ay, bx, by, cx, cy)) return true;
    if (o2 == 0 && on_seg_box64(ax, ay, bx, by, dx, dy)) return true;
    if (o3 == 0 && on_seg_box64(cx, cy, dx, dy, ax, ay)) return true;
    if (o4 == 0 && on_seg_box64(cx, cy, dx, dy, bx, by)) return true;
    return false;
}

// FP64 forward kinematics: joint positions x[0..n], y[0..n]
__device__ __forceinline__ void arm_fk64(const SceneView& s, const double* q, double* x, double* y) {
    double fx = 0.0, fy = 0.0, angle = 0.0;
    x[0] = 0.0; y[0] = 0.0;
    for (int i = 0; i < s.nlinks; ++i) {
        angle = __dadd_rn(angle, q[i]);
        double sn, cs;
        mptg_sincos(angle, &sn, &cs);
        double L = s.link_len64[i];
        fx = __dadd_rn(fx, __dmul_rn(L, cs));
        fy = __dadd_rn(fy, __dmul_rn(L, sn));
        x[i + 1] = fx; y[i + 1] = fy;
    }
}

// demo/link_manipulator_scenario.hpp:99-116 plus non-adjacent self-intersection
__device__ bool arm_valid64(const SceneView& s, const double* q) {
    double x[MPTG_MAX_DIM + 1], y[MPTG_MAX_DIM + 1];
    arm_fk64(s, q, x, y);
    for (int i = 0; i < s.nlinks; ++i) {
        for (int k = 0; k < s.ndiscs; ++k) {
            const double* dk = s.discs64 + 3 * k;
            double rr = __dmul_rn(__dadd_rn(dk[2], s.robot_radius), __dadd_rn(dk[2], s.robot_radius));
            if (!(dist_point_segment_sq64(dk[0], dk[1], x[i], y[i], x[i + 1], y[i + 1]) > rr)) return false;
        }
    }
    if (s.self_collision) {
        for (int i = 0; i < s.nlinks; ++i)
            for (int j = i + 2; j < s.nlinks; ++j)
                if (segs_intersect64(x[i], y[i], x[i + 1], y[i + 1], x[j], y[j], x[j + 1], y[j + 1])) return false;
    }
    return true;
}

// ------------------------------------------------------------------ FP32 filters
// Each filter returns VF_INVALID or VF_VALID (grid.cuh) when the FP32
// evaluation decides the state with certainty (every FP32 quantity lies
// farther from its decision boundary than an a-priori bound on its error),
// else VF_UNSURE, and the caller re-evaluates the state in FP64.

__device__ __forceinline__ float dpseg2_32(float px, float py, float ax, float ay, float bx, float by) {
    float vx = bx - ax, vy = by - ay, wx = px - ax, wy = py - ay;
    float c1 = vx * wx + vy * wy;
    if (c1 <= 0.f) return wx * wx + wy * wy;
    float c2 = vx * vx + vy * vy;
    if (c2 <= c1) { float ex = px - bx, ey = py - by; return ex * ex + ey * ey; }
    float f = c1 / c2;
    float ex = ax - px + vx * f, ey = ay - py + vy * f;
    return ex * ex + ey * ey;
}

// Scenario::valid for grid states, thread per state
__global__ void __launch_bounds__(256) k_grid_states(SceneView s, const double* __restrict__ q, int n,
                                                     uint8_t* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double st[2] = {q[(size_t)i * 2], q[(size_t)i * 2 + 1]};
    out[i] = grid_valid_f(s, st) ? 1 : 0;
}

// grid phase A, thread per edge: the end state (checked first, as the DMV
// does), then the step count; edges with interior samples go to the work list
__global__ void __launch_bounds__(256) k_grid_edges_a(SceneView s, const double* __restrict__ a,
                                                      const double* __restrict__ b, int n, double inv,
                                                      uint8_t* __restrict__ out, int* __restrict__ work,
                                                      int* __restrict__ wsteps, int* __restrict__ wcount,
                                                      unsigned long long* __restrict__ nsamp) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const double A[2] = {a[(size_t)e * 2], a[(size_t)e * 2 + 1]};
    const double B[2] = {b[(size_t)e * 2], b[(size_t)e * 2 + 1]};
    if (nsamp) atomicAdd(nsamp, 1ull);
    if (!grid_valid_f(s, B)) { out[e] = 0; return; }
    long long steps = grid_edge_steps(A, B, inv);
    if (steps < 0) { out[e] = 0; return; }
    out[e] = 1;
    if (steps >= 2) {
        int k = atomicAdd(wcount, 1);
        work[k] = e;
        wsteps[k] = (int)steps;
    }
}

// grid phase B, warp per surviving edge: interior samples i*delta,
// 1 <= i < steps, coarse-to-fine (lane j of round r takes sample 1 + j*R + r),
// FP32 filter per sample with the exact FP64 sample as fallback; ballot early exit
__global__ void __launch_bounds__(256) k_grid_edges_b(SceneView s, const double* __restrict__ a,
                                                      const double* __restrict__ b, const int* __restrict__ work,
                                                      const int* __restrict__ wsteps, const int* __restrict__ wcount,
                                                      uint8_t* __restrict__ out, unsigned long long* __restrict__ nsamp) {
    const int lane = threadIdx.x & 31;
    const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (w >= *wcount) return;
    const int e = work[w];
    const int steps = wsteps[w];
    const double A[2] = {a[(size_t)e * 2], a[(size_t)e * 2 + 1]};
    const double B[2] = {b[(size_t)e * 2], b[(size_t)e * 2 + 1]};
    float a32[2], dir32[2];
    for (int d = 0; d < 2; ++d) {
        a32[d] = __double2float_rn(A[d]);
        dir32[d] = __double2float_rn(__dsub_rn(B[d], A[d]));
    }
    const float eps = 8.f * U32 * (fabsf(a32[0]) + fabsf(a32[1]) + fabsf(dir32[0]) + fabsf(dir32[1]) + 1.f);
    const int M = steps - 1;
    const int R = (M + 31) / 32;
    const double delta = __ddiv_rn(1.0, (double)steps);
    bool ok = true;
    unsigned long long cnt = 0;
    for (int r = 0; ok && r < R; ++r) {
        int k = 1 + lane * R + r;
        bool v = true;
        if (k <= M) {
            ++cnt;
            float t = (float)k / (float)steps;
            int res = grid_valid32(s, fmaf(dir32[0], t, a32[0]), fmaf(dir32[1], t, a32[1]), eps);
            if (res == VF_UNSURE) {
                double qs[2];
                interp64(MPTG_METRIC_L2, 2, A, B, __dmul_rn((double)k, delta), qs);
                v = grid_valid64(s, qs);
            } else {
                v = res == VF_VALID;
            }
        }
        if (__any_sync(0xffffffffu, !v)) ok = false;
    }
    if (nsamp) {
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
        if (!ok) out[e] = 0;
        if (nsamp) atomicAdd(nsamp, cnt);
    }
}

// ------------------------------------------------------------------ planar arm, warp per state
// One warp decides one arm state at a time.  Lane j < nlinks owns joint j
// (its cumulative angle and sincos); every lane then runs the same FMA chain
// over the shuffled sines and cosines, and lane m keeps joint position m.
// The (link, disc) pairs are split over the lanes link by link (lane l takes
// discs l, l+32, ...), the self pairs (i, j >= i+2) likewise, and the warp
// stops at the first link with a certain collision.  Pairs the FP32 filter
// cannot decide are re-tested in FP64 on a warp-parallel forward kinematics
// that reproduces arm_fk64 operation for operation, so the result is exactly
// arm_valid64's: the state is invalid iff some pair collides in FP64.

#define FULL_MASK 0xffffffffu
#define ARM_SELF_SLOTS 4  // (16-2)(16-1)/2 = 105 self pairs at most: 4 per lane

struct ArmLane {
    float L32;       // link length of joint `lane`
    double L64;
    int sij[ARM_SELF_SLOTS];  // self pairs lane + 32 c: i | j << 8
    int nself;
};

__device__ __forceinline__ ArmLane arm_lane(const SceneView& s, int lane) {
    ArmLane al;
    al.L32 = lane < s.nlinks ? __ldg(&s.link32[lane]) : 0.f;
    al.L64 = lane < s.nlinks ? __ldg(&s.link_len64[lane]) : 0.0;
    const int nl = s.nlinks;
    al.nself = nl >= 3 ? (nl - 2) * (nl - 1) / 2 : 0;
#pragma unroll
    for (int c = 0; c < ARM_SELF_SLOTS; ++c) {
        int p = lane + 32 * c, i = 0, j = 2;
        if (p < al.nself) {
            for (i = 0; i < nl; ++i) {
                int cnt = nl - 2 - i;
                if (p < cnt) { j = i + 2 + p; break; }
                p -= cnt;
            }
        } else {
            i = 0;
            j = 2;
        }
        al.sij[c] = i | (j << 8);
    }
    return al;
}

__device__ __forceinline__ float warp_max_f(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(FULL_MASK, v, o));
    return v;
}

// FP32 test of link [a,b] against disc k, every point within dd of its FP64
// position (per coordinate)
__device__ __forceinline__ int arm_disc32(const SceneView& s, int k, float ax, float ay, float bx, float by,
                                          float dd) {
    const float4 d = __ldg(&s.discs32[k]);  // 1 KB per scene: L1-resident
    float d2 = dpseg2_32(d.x, d.y, ax, ay, bx, by);
    // the distance moves by <= dd, so d^2 by <= 2*d*dd + dd^2
    float m = 3.f * sqrtf(fmaxf(d2, d.z)) * dd + dd * dd + 8.f * U32 * (d2 + d.z);
    return d2 <= d.z - m ? VF_INVALID : (d2 > d.z + m ? VF_VALID : VF_UNSURE);
}

// Margin of one FP32 orientation v x w (v, w differences of joint positions,
// nv, nw their FP32 L1 norms).  Each coordinate of a joint position is within
// delta/2 of the FP64 one, so each coordinate of v and w is within delta, and
//   |V x W - v x w| <= delta*(|v|_1 + |w|_1) + 2*delta^2;
// the FP32 evaluation (two differences, two products, a difference) and the
// FP64 one round by less than 8u(|v|_1 + 2delta)(|w|_1 + 2delta).  The margin
// doubles both, which also covers the rounding of the norms and of itself.
__device__ __forceinline__ float orient_margin32(float nv, float nw, float delta) {
    return 2.f * delta * (nv + nw) + 4.f * delta * delta + 16.f * U32 * (nv + 2.f * delta) * (nw + 2.f * delta) +
           1e-30f;
}

// FP32 test of links [a,b] and [c,d] (segs_intersect64 in FP64)
__device__ __forceinline__ int arm_self32(float ax, float ay, float bx, float by, float cx, float cy, float dx,
                                          float dy, float delta) {
    const float nab = fabsf(bx - ax) + fabsf(by - ay), ncd = fabsf(dx - cx) + fabsf(dy - cy);
    const float nac = fabsf(cx - ax) + fabsf(cy - ay), nad = fabsf(dx - ax) + fabsf(dy - ay);
    const float nbc = fabsf(bx - cx) + fabsf(by - cy);
    const float o1 = (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
    const float o2 = (bx - ax) * (dy - ay) - (by - ay) * (dx - ax);
    const float o3 = (dx - cx) * (ay - cy) - (dy - cy) * (ax - cx);
    const float o4 = (dx - cx) * (by - cy) - (dy - cy) * (bx - cx);
    const bool s1 = fabsf(o1) > orient_margin32(nab, nac, delta), s2 = fabsf(o2) > orient_margin32(nab, nad, delta);
    const bool s3 = fabsf(o3) > orient_margin32(ncd, nac, delta), s4 = fabsf(o4) > orient_margin32(ncd, nbc, delta);
    const bool c12 = s1 && s2, c34 = s3 && s4;
    // every FP64 orientation has the FP32 sign and none is 0
    if (c12 && c34) return ((o1 > 0) != (o2 > 0) && (o3 > 0) != (o4 > 0)) ? VF_INVALID : VF_VALID;
    // Bounding boxes apart by more than 2*delta stay apart in FP64, so none of
    // segs_intersect64's collinear cases can fire; then one certain same-sign
    // pair of orientations rules out its proper crossing.
    const float g = 2.f * delta;
    const bool apart = fmaxf(ax, bx) + g < fminf(cx, dx) || fmaxf(cx, dx) + g < fminf(ax, bx) ||
                       fmaxf(ay, by) + g < fminf(cy, dy) || fmaxf(cy, dy) + g < fminf(ay, by);
    return (apart && ((c12 && (o1 > 0) == (o2 > 0)) || (c34 && (o3 > 0) == (o4 > 0)))) ? VF_VALID : VF_UNSURE;
}

// The exact FP64 joint angle of lane `lane` for one sample: b itself (t < 0)
// or so2 interpolate(a, b, t), the DMV's sample expression.
struct ArmSample {
    double a, b, t;
};

// arm_fk64 across the warp: lane m receives joint position m (x64, y64); q64
// holds joint `lane`'s angle on lanes < nlinks
__device__ __noinline__ void arm_fk64_warp(const SceneView& s, const ArmLane& al, int lane, double q64,
                                              double& x64, double& y64) {
    const int nl = s.nlinks;
    double angle = 0.0;
    for (int i = 0; i < nl; ++i) {
        double qi = __shfl_sync(FULL_MASK, q64, i);
        if (i <= lane) angle = __dadd_rn(angle, qi);
    }
    double sn = 0.0, cs = 0.0;
    if (lane < nl) mptg_sincos(angle, &sn, &cs);
    double fx = 0.0, fy = 0.0;
    x64 = 0.0;
    y64 = 0.0;
    for (int i = 0; i < nl; ++i) {
        double Li = __shfl_sync(FULL_MASK, al.L64, i);
        fx = __dadd_rn(fx, __dmul_rn(Li, __shfl_sync(FULL_MASK, cs, i)));
        fy = __dadd_rn(fy, __dmul_rn(Li, __shfl_sync(FULL_MASK, sn, i)));
        if (lane == i + 1) { x64 = fx; y64 = fy; }
    }
}

// FP64 joint positions of a sample (the rare path, out of line)
__device__ __noinline__ void arm_sample_fk64(const SceneView& s, const ArmLane& al, int lane, const ArmSample& smp,
                                             double& x64, double& y64) {
    double q64 = 0.0;
    if (lane < s.nlinks) q64 = smp.t < 0.0 ? smp.b : so2_interp64(smp.a, smp.b, smp.t);
    arm_fk64_warp(s, al, lane, q64, x64, y64);
}

// One arm state, warp-uniform result.  q32: joint `lane`'s FP32 angle, within
// ea of the exact one; smp: how to get joint `lane`'s exact FP64 angle (only
// when some pair needs FP64).  force64 sends every pair to FP64 (inputs
// outside the range of the FP32 error bound).
__device__ __forceinline__ bool arm_state_warp(const SceneView& s, const ArmLane& al, int lane, float q32, float ea,
                                               bool force64, const ArmSample& smp) {
    const int nl = s.nlinks;
    // FP32 forward kinematics.  Error bound against the FP64 kinematics
    // (arm_fk64 on the exact angles), with u = 2^-24 and joint angles within
    // ea of the exact ones, |q32| <= 2pi (the callers send larger inputs to
    // FP64):
    //  * cumulative angle: |ang| <= pi before each add, so |ang + q| <= 3pi and
    //    the add rounds by <= 3u*pi; the wrap subtracts TWO_PI_F exactly
    //    (Sterbenz) and TWO_PI_F is within u*pi of 2pi; after i joints the
    //    angle is within i*(ea + 4u*pi) of the exact one (mod 2pi);
    //  * sincosf is within 2 ulp (<= 4u) of sin/cos of its argument;
    //  * each FMA position step adds <= u*reach (rounding) + u*L (FP32 link).
    // So every joint position is within
    //   R*(nlinks*(ea + 5u*pi) + 5u) + nlinks*u*R  <=  delta / 2.
    float ang = 0.f;
    for (int i = 0; i < nl; ++i) {
        float qi = __shfl_sync(FULL_MASK, q32, i);
        if (i <= lane) {
            ang += qi;
            if (ang > PI_F) ang -= TWO_PI_F;
            else if (ang < -PI_F) ang += TWO_PI_F;
        }
    }
    float sn, cs;
    sincosf(ang, &sn, &cs);
    float xm = 0.f, ym = 0.f;
    {
        float x = 0.f, y = 0.f;
        for (int i = 0; i < nl; ++i) {
            float Li = __shfl_sync(FULL_MASK, al.L32, i);
            x = fmaf(Li, __shfl_sync(FULL_MASK, cs, i), x);
            y = fmaf(Li, __shfl_sync(FULL_MASK, sn, i), y);
            if (lane == i + 1) { xm = x; ym = y; }
        }
    }
    const float R = s.arm_reach;
    const float delta = 2.f * R * ((float)nl * (ea + 5.f * U32 * PI_F) + (float)(nl + 5) * U32) + 1e-30f;
    // the disc test's FP32 evaluation (coordinates of magnitude <= arm_span)
    // rounds like a further perturbation of the points by <= 8u*arm_span
    const float dd = delta + 8.f * U32 * s.arm_span;
    const int C = (s.ndiscs + 31) >> 5;
    const bool self = s.self_collision && al.nself > 0;
    // The FP32 tests of all pairs first, with a vote on certain collisions
    // every second link and one on undecided pairs at the end: the tests are
    // independent, so the scheduler overlaps them, and the result does not
    // depend on the order (the state is invalid iff some pair collides in
    // FP64; an FP32 INVALID is a certain FP64 collision).
    bool inv = false, uns = force64 && (lane < s.ndiscs || (self && lane < al.nself));
    if (!force64) {
#pragma unroll 2
        for (int i = 0; i < nl; ++i) {
            const float ax = __shfl_sync(FULL_MASK, xm, i), ay = __shfl_sync(FULL_MASK, ym, i);
            const float bx = __shfl_sync(FULL_MASK, xm, i + 1), by = __shfl_sync(FULL_MASK, ym, i + 1);
            for (int c = 0; c < C; ++c) {
                const int k = lane + 32 * c;
                if (k < s.ndiscs) {
                    const int r = arm_disc32(s, k, ax, ay, bx, by, dd);
                    inv |= r == VF_INVALID;
                    uns |= r == VF_UNSURE;
                }
            }
            // colliding states leave early, every second link
            if ((i & 1) && __any_sync(FULL_MASK, inv)) return false;
        }
        if (self) {
#pragma unroll
            for (int c = 0; c < ARM_SELF_SLOTS; ++c) {
                if (32 * c >= al.nself) break;
                const int i = al.sij[c] & 0xff, j = al.sij[c] >> 8;
                const float ax = __shfl_sync(FULL_MASK, xm, i), ay = __shfl_sync(FULL_MASK, ym, i);
                const float bx = __shfl_sync(FULL_MASK, xm, i + 1), by = __shfl_sync(FULL_MASK, ym, i + 1);
                const float cx = __shfl_sync(FULL_MASK, xm, j), cy = __shfl_sync(FULL_MASK, ym, j);
                const float dx = __shfl_sync(FULL_MASK, xm, j + 1), dy = __shfl_sync(FULL_MASK, ym, j + 1);
                if (lane + 32 * c < al.nself) {
                    const int r = arm_self32(ax, ay, bx, by, cx, cy, dx, dy, delta);
                    inv |= r == VF_INVALID;
                    uns |= r == VF_UNSURE;
                }
            }
        }
    }
    if (__any_sync(FULL_MASK, inv)) return false;
    if (!__any_sync(FULL_MASK, uns)) return true;
    // the rare path: FP64 kinematics once, then the undecided pairs in FP64
    double x64 = 0.0, y64 = 0.0;
    arm_sample_fk64(s, al, lane, smp, x64, y64);
    bool hit = false;
    for (int i = 0; i < nl; ++i) {
        const float ax = __shfl_sync(FULL_MASK, xm, i), ay = __shfl_sync(FULL_MASK, ym, i);
        const float bx = __shfl_sync(FULL_MASK, xm, i + 1), by = __shfl_sync(FULL_MASK, ym, i + 1);
        const double pax = __shfl_sync(FULL_MASK, x64, i), pay = __shfl_sync(FULL_MASK, y64, i);
        const double pbx = __shfl_sync(FULL_MASK, x64, i + 1), pby = __shfl_sync(FULL_MASK, y64, i + 1);
        for (int c = 0; c < C; ++c) {
            const int k = lane + 32 * c;
            if (k < s.ndiscs && (force64 || arm_disc32(s, k, ax, ay, bx, by, dd) == VF_UNSURE)) {
                const double* dk = s.discs64 + 3 * k;
                double rr = __dmul_rn(__dadd_rn(dk[2], s.robot_radius), __dadd_rn(dk[2], s.robot_radius));
                hit |= !(dist_point_segment_sq64(dk[0], dk[1], pax, pay, pbx, pby) > rr);
            }
        }
    }
    if (self) {
#pragma unroll
        for (int c = 0; c < ARM_SELF_SLOTS; ++c) {
            if (32 * c >= al.nself) break;
            const int i = al.sij[c] & 0xff, j = al.sij[c] >> 8;
            const float ax = __shfl_sync(FULL_MASK, xm, i), ay = __shfl_sync(FULL_MASK, ym, i);
            const float bx = __shfl_sync(FULL_MASK, xm, i + 1), by = __shfl_sync(FULL_MASK, ym, i + 1);
            const float cx = __shfl_sync(FULL_MASK, xm, j), cy = __shfl_sync(FULL_MASK, ym, j);
            const float dx = __shfl_sync(FULL_MASK, xm, j + 1), dy = __shfl_sync(FULL_MASK, ym, j + 1);
            const double pax = __shfl_sync(FULL_MASK, x64, i), pay = __shfl_sync(FULL_MASK, y64, i);
            const double pbx = __shfl_sync(FULL_MASK, x64, i + 1), pby = __shfl_sync(FULL_MASK, y64, i + 1);
            const double pcx = __shfl_sync(FULL_MASK, x64, j), pcy = __shfl_sync(FULL_MASK, y64, j);
            const double pdx = __shfl_sync(FULL_MASK, x64, j + 1), pdy = __shfl_sync(FULL_MASK, y64, j + 1);
            if (lane + 32 * c < al.nself &&
                (force64 || arm_self32(ax, ay, bx, by, cx, cy, dx, dy, delta) == VF_UNSURE))
                hit |= segs_intersect64(pax, pay, pbx, pby, pcx, pcy, pdx, pdy);
        }
    }
    return !__any_sync(FULL_MASK, hit);
}

// a state given in FP64, joint `lane` in qd; the FP32 angles are within
// 2u|q| + u*pi of it (rounding, plus the wrap); non-finite or huge angles go
// to FP64 pair by pair
__device__ __forceinline__ bool arm_state_exact(const SceneView& s, const ArmLane& al, int lane, double qd) {
    const float q32 = __double2float_rn(qd);
    const bool fin = lane >= s.nlinks || fabsf(q32) <= 4.f;  // false for NaN
    const float mx = warp_max_f(lane < s.nlinks && fin ? fabsf(q32) : 0.f);
    const bool force64 = !__all_sync(FULL_MASK, fin);
    return arm_state_warp(s, al, lane, q32, 2.f * U32 * mx + U32 * PI_F, force64, ArmSample{0.0, qd, -1.0});
}

// Scenario::valid for planar-arm states, warp per state
__global__ void __launch_bounds__(256) k_arm_states(SceneView s, const double* __restrict__ q, int n,
                                                    uint8_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int e = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (e >= n) return;
    const ArmLane al = arm_lane(s, lane);
    const double qd = lane < s.D ? q[(size_t)e * s.D + lane] : 0.0;
    const bool ok = arm_state_exact(s, al, lane, qd);
    if (lane == 0) out[e] = ok ? 1 : 0;
}

// one warp's share of edge e (see k_arm_edges); false iff it met an invalid
// sample or the step count is out of range
__device__ __forceinline__ bool arm_edge_warp(const SceneView& s, const double* __restrict__ a,
                                              const double* __restrict__ b, int e, double inv, int resolution,
                                              int lane, int g, int G, volatile int* dead, unsigned long long& cnt) {
    const int D = s.D;
    const ArmLane al = arm_lane(s, lane);
    const double Ad = lane < D ? a[(size_t)e * D + lane] : 0.0;
    const double Bd = lane < D ? b[(size_t)e * D + lane] : 0.0;
    bool ok = true;
    if (g == 0) {
        cnt = 1;
        ok = arm_state_exact(s, al, lane, Bd);
    }
    long long steps = 0;
    if (ok) {
        // ceil(m(a, b) * inv): m = max wrapped joint difference (resolution 1)
        // or the SO(2)^n distance, summed in joint order as dist64 does
        const double dd = lane < D ? so2_dist1_64(Ad, Bd) : 0.0;
        double m = 0.0;
        if (resolution == 1) {
            m = dd;
            for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(FULL_MASK, m, o));
        } else {
            for (int i = 0; i < D; ++i) m = __dadd_rn(m, __shfl_sync(FULL_MASK, dd, i));
        }
        const double sd = ceil(__dmul_rn(m, inv));
        if (!(sd >= 0.0) || sd > (double)MPTG_MAX_EDGE_SAMPLES) ok = false;
        else steps = (long long)sd;
    }
    if (ok && steps >= 2) {
        const float a32 = __double2float_rn(Ad);
        float dir32 = 0.f;
        if (lane < D) {
            // signed shortest-arc offset of interpolate (src/mpt/so2_space.hpp:44-65)
            double ccw = so2_ccw64(Ad, Bd);
            dir32 = __double2float_rn(ccw < MPTG_PI ? ccw : -__dsub_rn(MPTG_TWO_PI, ccw));
        }
        // q32 = fma(dir32, t, a32) is within u(|a| + 2|dir| + |q|) <= u(2|a| + 3|dir|)
        // of the exact sample (FP32 rounding of a, dir and t, then the FMA)
        const bool fin = lane >= D || (fabsf(a32) <= 3.1416f && fabsf(dir32) <= 3.1416f);
        const bool force64 = !__all_sync(FULL_MASK, fin);
        const float ea = warp_max_f(lane < D && fin ? 4.f * U32 * (fabsf(a32) + fabsf(dir32)) : 0.f);
        const int M = (int)steps - 1;
        const int R = (M + 31) / 32;
        const double delta = __ddiv_rn(1.0, (double)steps);
        for (int r = 0; ok && r < R; ++r) {
            for (int j = g; ok && j < 32; j += G) {
                const int k = 1 + j * R + r;
                if (k > M) continue;
                // another warp of the edge met an invalid sample (lane 0's read, warp-uniform)
                if (dead && __shfl_sync(FULL_MASK, *dead, 0)) return true;
                ++cnt;
                const float t = (float)k / (float)steps;
                const float q32 = fmaf(dir32, t, a32);
                ok = arm_state_warp(s, al, lane, q32, ea, force64, ArmSample{Ad, Bd, __dmul_rn((double)k, delta)});
            }
        }
    }
    return ok;
}

// DMV link for planar-arm edges, 2^lg warps per edge (lg <= 3; 1 for large
// batches, more when the batch is too small to fill the GPU): the end state
// (warp 0), then the step count (edge_steps' FP64 value, lane per joint), then
// the interior samples i*delta in the coarse-to-fine order of k_grid_edges_b,
// dealt round-robin to the edge's warps.  The edge is valid iff no warp finds
// an invalid sample, whatever the order; a warp that finds one raises the
// edge's shared flag and the others stop at their next sample.
__global__ void __launch_bounds__(256, 4) k_arm_edges(SceneView s, const double* __restrict__ a,
                                                   const double* __restrict__ b, int n, double inv, int resolution,
                                                   uint8_t* __restrict__ out, unsigned long long* __restrict__ nsamp,
                                                   int lg) {
    __shared__ int dead[8];  // per edge of the block
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lg > 0) {
        if (threadIdx.x < 8) dead[threadIdx.x] = 0;
        __syncthreads();
    }
    const int G = 1 << lg, g = w & (G - 1), slot = w >> lg;
    const int e = (int)(((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5) >> lg);
    bool ok = true;
    unsigned long long cnt = 0;
    if (e < n) {
        ok = arm_edge_warp(s, a, b, e, inv, resolution, lane, g, G, lg > 0 ? &dead[slot] : nullptr, cnt);
        if (!ok && lg > 0 && lane == 0) atomicExch(&dead[slot], 1);
    }
    if (lg > 0) {
        __syncthreads();
        ok = dead[slot] == 0;
    }
    if (e < n && lane == 0) {
        if (g == 0) out[e] = ok ? 1 : 0;
        if (nsamp) atomicAdd(nsamp, cnt);
    }
}

// ------------------------------------------------------------------ host

void scratch_free(EdgeScratch* s) {
    void* ptrs[] = {s->work, s->wsteps, s->wcount, s->mwork, s->nwork, s->samples, s->sample_edge, s->sample_ok,
                    s->counts, s->offs, s->okb};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s->hbuf) cudaFreeHost(s->hbuf);
    *s = EdgeScratch();
}

static void scene_free(mptg_scene* s) {
    void* ptrs[] = {s->grid, s->link_len64, s->discs64, s->discs32, s->link32};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    scratch_free(&s->scratch);
    mesh_scene_free(s);
    delete s;
}

SceneView scene_view(const mptg_scene* s) {
    SceneView v;
    memset(&v, 0, sizeof(v));
    v.kind = s->kind; v.metric = s->metric; v.D = s->D; v.w0 = s->w0; v.w1 = s->w1;
    v.grid = s->grid; v.width = s->width; v.height = s->height;
    v.nlinks = s->nlinks; v.link_len64 = s->link_len64; v.ndiscs = s->ndiscs; v.discs64 = s->discs64;
    v.robot_radius = s->robot_radius; v.self_collision = s->self_collision;
    v.discs32 = s->discs32; v.link32 = s->link32; v.arm_reach = s->arm_reach; v.arm_span = s->arm_span;
    mesh_fill_view(s, &v);
    return v;
}

// FP32 copies for the filters: discs as (cx, cy, (r + robot_radius)^2) with
// the square taken in FP64 as the exact test does
static cudaError_t scene_make_f32(mptg_scene* s, const mptg_scene_desc* d) {
    std::vector<float4> dc(d->ndiscs > 0 ? d->ndiscs : 1);
    for (int k = 0; k < d->ndiscs; ++k) {
        double r = d->discs[3 * k + 2] + d->robot_radius;
        dc[k] = make_float4((float)d->discs[3 * k], (float)d->discs[3 * k + 1], (float)(r * r), 0.f);
    }
    std::vector<float> ll(d->nlinks);
    double reach = 0;
    for (int i = 0; i < d->nlinks; ++i) { ll[i] = (float)d->link_len[i]; reach += fabs(d->link_len[i]); }
    s->arm_reach = (float)(reach * (1.0 + 1e-6)) + 1e-6f;
    double cmax = 0;
    for (int k = 0; k < d->ndiscs; ++k) cmax = std::max(cmax, fabs(d->discs[3 * k]) + fabs(d->discs[3 * k + 1]));
    s->arm_span = (float)((2.0 * reach + cmax) * (1.0 + 1e-6)) + 1e-6f;
    cudaError_t e = cudaMalloc((void**)&s->discs32, dc.size() * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemcpy(s->discs32, dc.data(), dc.size() * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->link32, ll.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(s->link32, ll.data(), ll.size() * sizeof(float), cudaMemcpyHostToDevice);
    return e;
}

static mptg_status scene_reserve(mptg_ctx* ctx, EdgeScratch* x, size_t n, cudaStream_t s) {
    if (!x->wcount) MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&x->wcount, sizeof(int)));
    if (n <= x->work_cap) return MPTG_OK;
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    cudaFree(x->work);
    cudaFree(x->wsteps);
    x->work = x->wsteps = nullptr;
    x->work_cap = 0;
    size_t cap = n + n / 2 + 1024;
    MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&x->work, cap * sizeof(int)));
    MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&x->wsteps, cap * sizeof(int)));
    x->work_cap = cap;
    return MPTG_OK;
}

mptg_status scene_edges_dev(mptg_scene* sc, const double* da, const double* db, int n, double step, int resolution,
                            uint8_t* dout, cudaStream_t s, unsigned long long* nsamp, EdgeScratch* scr) {
    if (n <= 0) return MPTG_OK;
    EdgeScratch* x = scr ? scr : &sc->scratch;
    if (sc->kind == MPTG_SCENE_RIGID_MESH)
        return mesh_edges_dev(sc, da, db, n, step, resolution, dout, s, nsamp, x);
    if (sc->kind == MPTG_SCENE_PLANAR_ARM) {
        // up to 8 warps per edge while the batch has fewer than 16 warps per SM
        int lg = 0;
        while (lg < 3 && ((size_t)n << lg) < (size_t)sc->ctx->sms * 16) ++lg;
        k_arm_edges<<<mptg_blocks(((size_t)n * 32) << lg, 256), 256, 0, s>>>(scene_view(sc), da, db, n, 1.0 / step,
                                                                            resolution, dout, nsamp, lg);
        MPTG_LAUNCHED(sc->ctx);
        return MPTG_OK;
    }
    mptg_status st = scene_reserve(sc->ctx, x, (size_t)n, s);
    if (st) return st;
    SceneView v = scene_view(sc);
    MPTG_CUDA_TRY(sc->ctx, cudaMemsetAsync(x->wcount, 0, sizeof(int), s));
    k_grid_edges_a<<<mptg_blocks(n, 128), 128, 0, s>>>(v, da, db, n, 1.0 / step, dout, x->work, x->wsteps,
                                                       x->wcount, nsamp);
    // one warp per edge that survived phase A (surplus warps exit at once)
    k_grid_edges_b<<<mptg_blocks((size_t)n * 32, 256), 256, 0, s>>>(v, da, db, x->work, x->wsteps, x->wcount, dout,
                                                                    nsamp);
    sc->ctx->launches += 2;
    return MPTG_OK;
}

mptg_status scene_states_dev(mptg_scene* sc, const double* dq, int n, uint8_t* dout, cudaStream_t s,
                             EdgeScratch* scr) {
    if (n <= 0) return MPTG_OK;
    if (sc->kind == MPTG_SCENE_RIGID_MESH) return mesh_states_dev(sc, dq, n, dout, s, scr ? scr : &sc->scratch);
    SceneView v = scene_view(sc);
    if (sc->kind == MPTG_SCENE_PLANAR_ARM)
        k_arm_states<<<mptg_blocks((size_t)n * 32, 256), 256, 0, s>>>(v, dq, n, dout);
    else
        k_grid_states<<<mptg_blocks(n, 256), 256, 0, s>>>(v, dq, n, dout);
    MPTG_LAUNCHED(sc->ctx);
    return MPTG_OK;
}

extern "C" {

mptg_status mptg_scene_create(mptg_ctx* ctx, const mptg_scene_desc* d, mptg_scene** out) {
    if (!ctx || !d || !out) return MPTG_ERR_INVALID_ARG;
    *out = nullptr;
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    mptg_scene* s = new mptg_scene();
    s->ctx = ctx;
    s->kind = d->kind;
    cudaError_t e = cudaSuccess;
    switch (d->kind) {
    case MPTG_SCENE_GRID: {
        if (!d->grid || d->width <= 0 || d->height <= 0) {
            delete s;
            return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "grid scene needs cells and a positive size");
        }
        s->metric = MPTG_METRIC_L2; s->D = 2;
        s->width = d->width; s->height = d->height;
        size_t bytes = (size_t)d->width * d->height;
        e = cudaMalloc((void**)&s->grid, bytes);
        if (e == cudaSuccess) e = cudaMemcpy(s->grid, d->grid, bytes, cudaMemcpyHostToDevice);
        break;
    }
    case MPTG_SCENE_PLANAR_ARM: {
        if (d->nlinks < 1 || d->nlinks > MPTG_MAX_DIM || !d->link_len || d->ndiscs < 0 || (d->ndiscs && !d->discs)) {
            delete s;
            return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "planar arm needs 1..16 links and a disc list");
        }
        s->metric = MPTG_METRIC_SO2; s->D = d->nlinks;
        s->nlinks = d->nlinks; s->ndiscs = d->ndiscs;
        s->robot_radius = d->robot_radius; s->self_collision = d->self_collision;
        e = cudaMalloc((void**)&s->link_len64, d->nlinks * sizeof(double));
        if (e == cudaSuccess) e = cudaMemcpy(s->link_len64, d->link_len, d->nlinks * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc((void**)&s->discs64, (d->ndiscs * 3 + 1) * sizeof(double));
        if (e == cudaSuccess && d->ndiscs)
            e = cudaMemcpy(s->discs64, d->discs, d->ndiscs * 3 * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = scene_make_f32(s, d);
        break;
    }
    case MPTG_SCENE_RIGID_MESH: {
        s->metric = MPTG_METRIC_SE3; s->D = 7;
        s->w0 = d->w_rot > 0 ? d->w_rot : 1.0;
        s->w1 = d->w_pos > 0 ? d->w_pos : 1.0;
        mptg_status st = mesh_scene_create(ctx, d, s);
        if (st != MPTG_OK) {
            scene_free(s);
            return st;
        }
        break;
    }
    default:
        delete s;
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "unknown scene kind %d", d->kind);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        scene_free(s);
        return mptg_fail(ctx, MPTG_ERR_OOM, "scene allocation failed: %s", cudaGetErrorString(e));
    }
    *out = s;
    return MPTG_OK;
}

mptg_status mptg_scene_destroy(mptg_scene* s) {
    if (!s) return MPTG_ERR_INVALID_ARG;
    cudaDeviceSynchronize();
    scene_free(s);
    return MPTG_OK;
}

mptg_status mptg_scene_space(mptg_scene* s, int* dim, int* metric, double weights[2]) {
    if (!s) return MPTG_ERR_INVALID_ARG;
    if (dim) *dim = s->D;
    if (metric) *metric = s->metric;
    if (weights) { weights[0] = s->w0; weights[1] = s->w1; }
    return MPTG_OK;
}

mptg_status mptg_valid_states(mptg_scene* sc, const double* q, size_t n, uint8_t* out, void* stream) {
    if (!sc) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = sc->ctx;
    if (n == 0) return MPTG_OK;
    if (!q || !out) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "null buffer");
    if (n > (size_t)INT32_MAX) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "too many states");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf bq, bo;
    mptg_status st;
    if ((st = mptg_stage_in(ctx, q, n * sc->D * sizeof(double), s, &bq))) return st;
    if ((st = mptg_stage_out_alloc(ctx, out, n, s, &bo))) return st;
    if ((st = scene_states_dev(sc, (const double*)bq.dptr, (int)n, (uint8_t*)bo.dptr, s))) return st;
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    return mptg_stage_finish(ctx, s, &bo, 1, &bq, 1);
}

mptg_status mptg_valid_edges(mptg_scene* sc, const double* a, const double* b, size_t n, double step, int resolution,
                             uint8_t* out, void* stream) {
    if (!sc) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = sc->ctx;
    if (n == 0) return MPTG_OK;
    if (!a || !b || !out) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "null buffer");
    if (!(step > 0)) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "step must be positive");
    if (resolution != 0 && resolution != 1) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "resolution must be 0 or 1");
    if (resolution == 1 && sc->metric != MPTG_METRIC_SO2)
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "joint-step resolution needs an SO2 scene");
    if (n > (size_t)INT32_MAX / 32) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "too many edges");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf ba, bb, bo;
    mptg_status st;
    size_t sb = n * sc->D * sizeof(double);
    if ((st = mptg_stage_in(ctx, a, sb, s, &ba))) return st;
    if ((st = mptg_stage_in(ctx, b, sb, s, &bb))) return st;
    if ((st = mptg_stage_out_alloc(ctx, out, n, s, &bo))) return st;
    if ((st = scene_edges_dev(sc, (const double*)ba.dptr, (const double*)bb.dptr, (int)n, step, resolution,
                              (uint8_t*)bo.dptr, s, nullptr)))
        return st;
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    DevBuf ins[2] = {ba, bb};
    return mptg_stage_finish(ctx, s, &bo, 1, ins, 2);
}

}  // extern "C"
