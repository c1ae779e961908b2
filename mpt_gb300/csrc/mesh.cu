// mesh.cu - rigid-body (SE(3)) mesh-vs-mesh validity.
//
// Replaces fcl::collide(robot BVHModel<OBBRSS>, T(q), environment, I) in
// demo/se3_rigid_body_scenario.hpp:282-312: a state is valid iff no triangle
// of the robot placed at T(q) = Translation(p) * Rotation(quaternion)
// intersects an environment triangle.
//
// Exactness: the result is the OR, over all (robot, environment) triangle
// pairs, of an FP64 triangle-triangle test (T. Moller, "A Fast
// Triangle-Triangle Intersection Test", JGT 1997, no epsilon snapping) on
// robot vertices transformed in FP64 in a fixed operation order.  Every cull
// in front of it is conservative (FP32 boxes rounded outward and grown by a
// margin far above FP32 rounding), so it can only skip pairs that cannot
// intersect, and the boolean equals the CPU checker's.
//
// Per batch of states:
//  k_mesh_sphere  (thread per state) robot bounding sphere at p vs the
//                 environment AABB tree: no box within reach -> valid
//  k_mesh_detail  (block per remaining state, thread per robot leaf) the
//                 robot leaf's world AABB (its robot-frame box rotated by
//                 |R|) against the environment tree; triangle pairs of
//                 overlapping leaves go to the FP64 test; the block stops
//                 at the first intersection
// Both trees are built once per scene on the host (top-down median split on
// the longest axis, leaves of <= 8 triangles).
#include <algorithm>
#include <numeric>

#include "metrics.cuh"
#include "scene.cuh"

#define MESH_LEAF 8
#define MESH_MARGIN 1e-3f  // box growth, >> FP32 rounding of scene coordinates (|x| <= 1e3)
#define MESH_STACK 64

struct BvhNode {  // 32 bytes
    float lo[3];
    int a;        // internal: left child; leaf: first triangle
    float hi[3];
    int b;        // internal: right child; leaf: -(count)
};

struct MeshData {
    // environment (world frame), triangles in leaf order
    double* env_tris = nullptr;   // [nenv][9]
    float* env_boxes = nullptr;   // [nenv][6] lo.xyz, hi.xyz, outward-rounded plus margin
    BvhNode* env_nodes = nullptr;
    int nenv = 0, nenv_nodes = 0;
    // robot (robot frame), triangles in leaf order
    double* robot_tris = nullptr;  // [nrobot][9]
    BvhNode* robot_leaves = nullptr;  // robot leaves only (AABBs in the robot frame)
    int nrobot = 0, nrleaves = 0;
    double robot_radius = 0.0;     // max |vertex| in the robot frame
    // FP32 copies for the certified pre-tests (round to nearest of the FP64 data)
    float* env_tris32 = nullptr;    // [nenv][9]
    float* robot_tris32 = nullptr;  // [nrobot][9]
    float env_max = 0.f;            // >= max |coordinate| of the environment
    float robot_l1 = 0.f;           // >= max |x|+|y|+|z| of a robot vertex
};

// ------------------------------------------------------------------ host BVH build

namespace {

struct Box { double lo[3], hi[3]; };

Box tri_box(const double* t) {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = std::min(std::min(t[d], t[3 + d]), t[6 + d]);
        b.hi[d] = std::max(std::max(t[d], t[3 + d]), t[6 + d]);
    }
    return b;
}

// outward FP32 rounding plus a margin
void store_box(BvhNode& n, const Box& b) {
    for (int d = 0; d < 3; ++d) {
        n.lo[d] = std::nextafter((float)b.lo[d], -INFINITY) - MESH_MARGIN;
        n.hi[d] = std::nextafter((float)b.hi[d], INFINITY) + MESH_MARGIN;
    }
}

int build_rec(const std::vector<double>& tris, std::vector<int>& idx, int start, int count,
              std::vector<BvhNode>& nodes, std::vector<int>* leaves) {
    int id = (int)nodes.size();
    nodes.push_back(BvhNode());
    Box b;
    for (int d = 0; d < 3; ++d) { b.lo[d] = INFINITY; b.hi[d] = -INFINITY; }
    for (int i = 0; i < count; ++i) {
        Box t = tri_box(&tris[9 * (size_t)idx[start + i]]);
        for (int d = 0; d < 3; ++d) { b.lo[d] = std::min(b.lo[d], t.lo[d]); b.hi[d] = std::max(b.hi[d], t.hi[d]); }
    }
    store_box(nodes[id], b);
    if (count <= MESH_LEAF) {
        nodes[id].a = start;
        nodes[id].b = -count;
        if (leaves) leaves->push_back(id);
        return id;
    }
    int ax = 0;
    for (int d = 1; d < 3; ++d)
        if (b.hi[d] - b.lo[d] > b.hi[ax] - b.lo[ax]) ax = d;
    auto cen = [&](int t) { const double* p = &tris[9 * (size_t)t]; return p[ax] + p[3 + ax] + p[6 + ax]; };
    int mid = count / 2;
    std::nth_element(idx.begin() + start, idx.begin() + start + mid, idx.begin() + start + count,
                     [&](int x, int y) { double cx = cen(x), cy = cen(y); return cx < cy || (cx == cy && x < y); });
    int l = build_rec(tris, idx, start, mid, nodes, leaves);
    int r = build_rec(tris, idx, start + mid, count - mid, nodes, leaves);
    nodes[id].a = l;
    nodes[id].b = r;
    return id;
}

}  // namespace

// ------------------------------------------------------------------ device helpers


// Entry k (row-major) of the rotation matrix of the unit quaternion
// (x, y, z, w), with the CPU checker's expressions (oracle.c quat_to_mat):
// products p1 = (2a) b and p2 = (2c) d of quaternion components (t_a = 2a
// first, then t_a b), the diagonal 1 - (p1 + p2), the rest p1 + p2 or
// p1 - p2 (= p1 + (-p2) exactly).  One instruction sequence for every k, so
// that nine lanes compute the nine entries together; the operand indices
// a, b, c, d into (x, y, z, w) are packed two bits per k.
__device__ __forceinline__ double quat_entry64(const double* q, int k) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    auto pick = [&](unsigned table) {
        const unsigned i = (table >> (2 * k)) & 3u;
        return i == 0 ? x : i == 1 ? y : i == 2 ? z : w;
    };
    const double p1 = __dmul_rn(__dmul_rn(2.0, pick(0xa865u)), pick(0x4401u));
    const double p2 = __dmul_rn(__dmul_rn(2.0, pick(0x1129au)), pick(0x1fefeu));
    const double sum = __dadd_rn(p1, (0x62u >> k) & 1u ? -p2 : p2);
    return (0x111u >> k) & 1u ? __dsub_rn(1.0, sum) : sum;
}

__device__ __forceinline__ void xform64(const double* R, const double* p, const double* v, double* o) {
    o[0] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(R[0], v[0]), __dmul_rn(R[1], v[1])), __dmul_rn(R[2], v[2])), p[0]);
    o[1] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(R[3], v[0]), __dmul_rn(R[4], v[1])), __dmul_rn(R[5], v[2])), p[1]);
    o[2] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(R[6], v[0]), __dmul_rn(R[7], v[1])), __dmul_rn(R[8], v[2])), p[2]);
}

__device__ __forceinline__ void sub3d(const double* a, const double* b, double* c) {
    c[0] = __dsub_rn(a[0], b[0]); c[1] = __dsub_rn(a[1], b[1]); c[2] = __dsub_rn(a[2], b[2]);
}
__device__ __forceinline__ void cross3d(const double* a, const double* b, double* c) {
    c[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
    c[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
    c[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
}
__device__ __forceinline__ double dot3d(const double* a, const double* b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}
__device__ __forceinline__ double orient2d_m(double ax, double ay, double bx, double by, double cx, double cy) {
    return __dsub_rn(__dmul_rn(__dsub_rn(bx, ax), __dsub_rn(cy, ay)), __dmul_rn(__dsub_rn(by, ay), __dsub_rn(cx, ax)));
}
__device__ __forceinline__ bool on_box2(double ax, double ay, double bx, double by, double px, double py) {
    return fmin(ax, bx) <= px && px <= fmax(ax, bx) && fmin(ay, by) <= py && py <= fmax(ay, by);
}
__device__ bool seg2_intersect(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy) {
    double o1 = orient2d_m(ax, ay, bx, by, cx, cy), o2 = orient2d_m(ax, ay, bx, by, dx, dy);
    double o3 = orient2d_m(cx, cy, dx, dy, ax, ay), o4 = orient2d_m(cx, cy, dx, dy, bx, by);
    if (((o1 > 0 && o2 < 0) || (o1 < 0 && o2 > 0)) && ((o3 > 0 && o4 < 0) || (o3 < 0 && o4 > 0))) return true;
    if (o1 == 0 && on_box2(ax, ay, bx, by, cx, cy)) return true;
    if (o2 == 0 && on_box2(ax, ay, bx, by, dx, dy)) return true;
    if (o3 == 0 && on_box2(cx, cy, dx, dy, ax, ay)) return true;
    if (o4 == 0 && on_box2(cx, cy, dx, dy, bx, by)) return true;
    return false;
}
__device__ bool point_in_tri2(double px, double py, const double* t) {
    double d1 = orient2d_m(t[0], t[1], t[2], t[3], px, py);
    double d2 = orient2d_m(t[2], t[3], t[4], t[5], px, py);
    double d3 = orient2d_m(t[4], t[5], t[0], t[1], px, py);
    bool neg = d1 < 0 || d2 < 0 || d3 < 0, pos = d1 > 0 || d2 > 0 || d3 > 0;
    return !(neg && pos);
}
__device__ bool coplanar_tt(const double* n, const double* V0, const double* V1, const double* V2, const double* U0,
                            const double* U1, const double* U2) {
    double a0 = fabs(n[0]), a1 = fabs(n[1]), a2 = fabs(n[2]);
    int i0, i1;
    if (a0 > a1) { if (a0 > a2) { i0 = 1; i1 = 2; } else { i0 = 0; i1 = 1; } }
    else { if (a2 > a1) { i0 = 0; i1 = 1; } else { i0 = 0; i1 = 2; } }
    double v[6] = {V0[i0], V0[i1], V1[i0], V1[i1], V2[i0], V2[i1]};
    double u[6] = {U0[i0], U0[i1], U1[i0], U1[i1], U2[i0], U2[i1]};
    for (int e = 0; e < 3; ++e) {
        int e1 = (e + 1) % 3;
        for (int f = 0; f < 3; ++f) {
            int f1 = (f + 1) % 3;
            if (seg2_intersect(v[2 * e], v[2 * e + 1], v[2 * e1], v[2 * e1 + 1], u[2 * f], u[2 * f + 1], u[2 * f1],
                               u[2 * f1 + 1]))
                return true;
        }
    }
    if (point_in_tri2(v[0], v[1], u)) return true;
    if (point_in_tri2(u[0], u[1], v)) return true;
    return false;
}
__device__ __forceinline__ double lerp_isect(double VVa, double VVb, double Da, double Db) {
    // VVa + (VVb - VVa) * Da / (Da - Db), evaluated left to right as the checker does
    return __dadd_rn(VVa, __ddiv_rn(__dmul_rn(__dsub_rn(VVb, VVa), Da), __dsub_rn(Da, Db)));
}
__device__ bool tri_interval(double VV0, double VV1, double VV2, double D0, double D1, double D2, double D0D1,
                             double D0D2, double* i0, double* i1) {
    if (D0D1 > 0) { *i0 = lerp_isect(VV2, VV0, D2, D0); *i1 = lerp_isect(VV2, VV1, D2, D1); }
    else if (D0D2 > 0) { *i0 = lerp_isect(VV1, VV0, D1, D0); *i1 = lerp_isect(VV1, VV2, D1, D2); }
    else if (__dmul_rn(D1, D2) > 0 || D0 != 0) { *i0 = lerp_isect(VV0, VV1, D0, D1); *i1 = lerp_isect(VV0, VV2, D0, D2); }
    else if (D1 != 0) { *i0 = lerp_isect(VV1, VV0, D1, D0); *i1 = lerp_isect(VV1, VV2, D1, D2); }
    else if (D2 != 0) { *i0 = lerp_isect(VV2, VV0, D2, D0); *i1 = lerp_isect(VV2, VV1, D2, D1); }
    else return true;
    return false;
}

// Moller's test in FP64 (same expressions as the CPU checker)
__device__ bool tri_tri64(const double* t1, const double* t2) {
    const double *V0 = t1, *V1 = t1 + 3, *V2 = t1 + 6;
    const double *U0 = t2, *U1 = t2 + 3, *U2 = t2 + 6;
    double E1[3], E2[3], N1[3], N2[3], Dv[3];
    sub3d(V1, V0, E1); sub3d(V2, V0, E2); cross3d(E1, E2, N1);
    double d1 = -dot3d(N1, V0);
    double du0 = __dadd_rn(dot3d(N1, U0), d1), du1 = __dadd_rn(dot3d(N1, U1), d1), du2 = __dadd_rn(dot3d(N1, U2), d1);
    double du0du1 = __dmul_rn(du0, du1), du0du2 = __dmul_rn(du0, du2);
    if (du0du1 > 0 && du0du2 > 0) return false;
    sub3d(U1, U0, E1); sub3d(U2, U0, E2); cross3d(E1, E2, N2);
    double d2 = -dot3d(N2, U0);
    double dv0 = __dadd_rn(dot3d(N2, V0), d2), dv1 = __dadd_rn(dot3d(N2, V1), d2), dv2 = __dadd_rn(dot3d(N2, V2), d2);
    double dv0dv1 = __dmul_rn(dv0, dv1), dv0dv2 = __dmul_rn(dv0, dv2);
    if (dv0dv1 > 0 && dv0dv2 > 0) return false;
    cross3d(N1, N2, Dv);
    double mx = fabs(Dv[0]);
    int index = 0;
    double bb = fabs(Dv[1]), cc = fabs(Dv[2]);
    if (bb > mx) { mx = bb; index = 1; }
    if (cc > mx) index = 2;
    double a0, a1, b0, b1;
    if (tri_interval(V0[index], V1[index], V2[index], dv0, dv1, dv2, dv0dv1, dv0dv2, &a0, &a1))
        return coplanar_tt(N1, V0, V1, V2, U0, U1, U2);
    if (tri_interval(U0[index], U1[index], U2[index], du0, du1, du2, du0du1, du0du2, &b0, &b1))
        return coplanar_tt(N1, V0, V1, V2, U0, U1, U2);
    if (a0 > a1) { double t = a0; a0 = a1; a1 = t; }
    if (b0 > b1) { double t = b0; b0 = b1; b1 = t; }
    return !(a1 < b0 || b1 < a0);
}

__device__ __forceinline__ bool box_overlap(const float* lo, const float* hi, const BvhNode& n) {
    return !(n.lo[0] > hi[0] || n.hi[0] < lo[0] || n.lo[1] > hi[1] || n.hi[1] < lo[1] || n.lo[2] > hi[2] ||
             n.hi[2] < lo[2]);
}

struct MeshView {
    const double* env_tris;
    const float* env_boxes;
    const BvhNode* env_nodes;
    const double* robot_tris;
    const BvhNode* robot_leaves;
    const float* env_tris32;
    const float* robot_tris32;
    int nenv, nrleaves;
    float reach;  // robot bounding radius + margin
    float env_max, robot_l1;
};

// robot bounding sphere (center p, radius reach) against the environment tree
__global__ void k_mesh_sphere(MeshView m, const double* __restrict__ q, int n, int D, uint8_t* __restrict__ out,
                              int* __restrict__ work, int* __restrict__ nwork) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* s = q + (size_t)i * D;
    float p[3] = {(float)s[4], (float)s[5], (float)s[6]};
    bool bad = !(s[4] == s[4] && s[5] == s[5] && s[6] == s[6] && s[0] == s[0] && s[1] == s[1] && s[2] == s[2] &&
                 s[3] == s[3]);
    float r = m.reach + 1e-3f * (1.f + fabsf(p[0]) + fabsf(p[1]) + fabsf(p[2]));
    float lo[3] = {p[0] - r, p[1] - r, p[2] - r}, hi[3] = {p[0] + r, p[1] + r, p[2] + r};
    bool near = false;
    if (!bad && m.nenv > 0) {
        int stack[MESH_STACK];
        int sp = 0;
        stack[sp++] = 0;
        while (sp && !near) {
            BvhNode nd = m.env_nodes[stack[--sp]];
            if (!box_overlap(lo, hi, nd)) continue;
            // sphere-box distance (the box test above is the sphere's bounding cube)
            float d2 = 0.f;
            for (int d = 0; d < 3; ++d) {
                float o = fmaxf(fmaxf(nd.lo[d] - p[d], p[d] - nd.hi[d]), 0.f);
                d2 = fmaf(o, o, d2);
            }
            if (d2 > r * r) continue;
            if (nd.b < 0) { near = true; break; }
            if (sp + 2 <= MESH_STACK) { stack[sp++] = nd.a; stack[sp++] = nd.b; }
            else near = true;  // cannot happen for trees of depth < 62; stay conservative
        }
    }
    if (bad) {
        out[i] = 0;
    } else if (!near) {
        out[i] = 1;
    } else {
        out[i] = 0;  // decided by k_mesh_detail
        work[atomicAdd(nwork, 1)] = i;
    }
}

// block per state, thread per robot leaf
// The FP64 decision of one (robot, environment) triangle pair: the robot
// triangle transformed by (R, P) in the CPU checker's operation order, then
// Moller's test.  Kept out of line: it is the rare path.
__device__ __noinline__ bool pair_hits64(const double* R, const double* P, const double* lt, const double* et) {
    double wt[9];
    xform64(R, P, lt, wt);
    xform64(R, P, lt + 3, wt + 3);
    xform64(R, P, lt + 6, wt + 6);
    return tri_tri64(wt, et);
}

#include "tri32.cuh"

#define MESH_DETAIL_THREADS 128
#define MESH_CAND 512   // environment leaves within the robot's bounding sphere
#define MESH_FRONT 512  // breadth-first frontier of that sweep
#define MESH_QUEUE 512  // (robot leaf, environment leaf) pairs per round
static_assert(MESH_LEAF == 8, "k_mesh_detail spreads 8 x 8 triangle pairs per leaf pair");

// The robot triangle `lt` (robot frame, FP32) placed at (R32, P32) in FP32.
__device__ __forceinline__ void robot_tri32(const float* R32, const float* P32, const float* lt, float* V) {
#pragma unroll
    for (int vtx = 0; vtx < 3; ++vtx)
#pragma unroll
        for (int r = 0; r < 3; ++r)
            V[3 * vtx + r] = fmaf(R32[3 * r], lt[3 * vtx],
                                  fmaf(R32[3 * r + 1], lt[3 * vtx + 1], fmaf(R32[3 * r + 2], lt[3 * vtx + 2], P32[r])));
}

// One (robot triangle ri, environment triangle ei) pair: the world box of the
// FP32 robot triangle (grown by a margin far above the transform's error)
// against the environment triangle's box, then the certified FP32 verdicts
// (a separating plane, or a certain crossing), and only then the FP64 test.
__device__ __forceinline__ bool pair_hits(const MeshView& m, const double* R, const double* P, const float* R32,
                                          const float* P32, float eps, float X, int ri, int ei) {
    float V[9];
    robot_tri32(R32, P32, m.robot_tris32 + 9 * (size_t)ri, V);
    const float* eb = m.env_boxes + 6 * (size_t)ei;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float lo = fminf(V[d], fminf(V[3 + d], V[6 + d])), hi = fmaxf(V[d], fmaxf(V[3 + d], V[6 + d]));
        float mg = MESH_MARGIN * (1.f + fabsf(lo) + fabsf(hi));
        if (lo - mg > eb[3 + d] || hi + mg < eb[d]) return false;
    }
    float U[9];
    const float* et = m.env_tris32 + 9 * (size_t)ei;
#pragma unroll
    for (int k = 0; k < 9; ++k) U[k] = et[k];
    const int v32 = tri_pair32(V, U, eps, X);
    if (v32 != 0) return v32 > 0;
    return pair_hits64(R, P, m.robot_tris + 9 * (size_t)ri, m.env_tris + 9 * (size_t)ei);
}

__device__ __forceinline__ bool sphere_box(const float* p, float r, const BvhNode& nd) {
    float d2 = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float o = fmaxf(fmaxf(nd.lo[d] - p[d], p[d] - nd.hi[d]), 0.f);
        d2 = fmaf(o, o, d2);
    }
    return d2 <= r * r;
}

// world AABB of robot leaf rl at (R32, P32): center R c + p, half |R| h, grown
__device__ __forceinline__ void robot_leaf_box(const BvhNode& rl, const float* R32, const float* P32, float* lo,
                                               float* hi) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float cw = P32[r], hw = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float rv = R32[3 * r + k];
            cw = fmaf(rv, 0.5f * (rl.lo[k] + rl.hi[k]), cw);
            hw = fmaf(fabsf(rv), 0.5f * (rl.hi[k] - rl.lo[k]), hw);
        }
        float mg = MESH_MARGIN * (1.f + fabsf(cw) + hw);
        lo[r] = cw - hw - mg;
        hi[r] = cw + hw + mg;
    }
}

// Block per state that the sphere test could not clear.
//  1. The block sweeps the environment tree breadth first for the leaves whose
//     boxes meet the robot's bounding sphere (candidates, in shared memory).
//  2. Thread t takes robot leaf t (of each chunk of 128) and queues the
//     (robot leaf, candidate) pairs whose boxes overlap.
//  3. The 64 triangle pairs of every queued leaf pair are spread over the
//     whole block: triangle box test, certified FP32 separating planes, FP64.
// The block stops at the first intersection.  More candidates than fit
// (MESH_CAND / MESH_FRONT) fall back to a per-thread depth-first walk.
//
// For the interior samples of a batch of edges (sample_edge != nullptr), a
// block first reads its edge's result in edge_out and skips the sample when
// another sample has already made the edge invalid (the edge result is the
// AND of its samples, so the skipped sample's own result cannot matter), and
// a colliding sample clears edge_out at once.  Blocks take the work items in
// the scattered order w * MESH_PERM mod nwork, so the samples of one edge are
// spread over the launch and most samples after an edge's first collision
// are skipped.
#define MESH_PERM 1000003ull  // prime; the identity order when it divides nwork
__global__ void __launch_bounds__(MESH_DETAIL_THREADS, 8) k_mesh_detail(MeshView m, const double* __restrict__ q, int D,
                                                                      const int* __restrict__ work,
                                                                      const int* __restrict__ nwork,
                                                                      uint8_t* __restrict__ out,
                                                                      const int* __restrict__ sample_edge,
                                                                      uint8_t* __restrict__ edge_out) {
    __shared__ double R[9];
    __shared__ double P[3];
    __shared__ float R32[9], P32[3];
    __shared__ float eps_s, X_s;
    __shared__ int front[2][MESH_FRONT];
    __shared__ int nfront[2];
    __shared__ int cand[MESH_CAND];
    __shared__ float cbox[6][MESH_CAND];
    __shared__ int ncand, overflow, nq;
    __shared__ int qra[MESH_QUEUE], qrc[MESH_QUEUE], qea[MESH_QUEUE], qec[MESH_QUEUE];
    __shared__ volatile int hit;
    const int w = blockIdx.x;
    const int nw = *nwork;
    if (w >= nw) return;
    const int i = work[(unsigned long long)nw % MESH_PERM ? (int)(((unsigned long long)w * MESH_PERM) % nw) : w];
    const int tid = threadIdx.x;
    __shared__ int dead;
    const double* s = q + (size_t)i * D;
    // one read of the edge's result for the whole block (other blocks may
    // clear it at any time, so per-thread reads could disagree)
    if (tid == 0) dead = sample_edge && __ldcg(&edge_out[sample_edge[i]]) == 0;
    __syncthreads();
    if (dead) {  // block-uniform
        if (tid == 0) out[i] = 0;
        return;
    }
    // the pose: lanes 0-8 the rotation entries, lanes 9-11 the position (an
    // FP64 instruction costs the FP64 pipe the same for one active lane as
    // for 32, so the entries are computed side by side, not by one thread)
    if (tid < 12) {
        double v;
        if (tid < 9) {
            v = quat_entry64(s, tid);
            R[tid] = v;
        } else {
            v = s[4 + tid - 9];
            P[tid - 9] = v;
        }
        const float f = (float)v;
        if (tid < 9) R32[tid] = f;
        else P32[tid - 9] = f;
    }
    __syncwarp();
    if (tid == 0) {
        float pm = 0.f;
        for (int k = 0; k < 3; ++k) pm = fmaxf(pm, fabsf(P32[k]));
        pm = pm * (1.f + 2.f * U32);
        // FP32 world vertex fma(R, v, P) against xform64: <= u(5|v|_1 + 4|P|);
        // FP32 environment coordinates: <= u |x|
        eps_s = fmaxf(6.f * U32 * (m.robot_l1 + pm), U32 * m.env_max) * 1.01f;
        X_s = fmaxf(m.env_max, m.robot_l1 + pm);
        front[0][0] = 0;
        nfront[0] = m.nenv > 0 ? 1 : 0;
        nfront[1] = 0;
        ncand = 0;
        overflow = 0;
        nq = 0;
        hit = 0;
    }
    __syncthreads();
    const float eps = eps_s, X = X_s;
    // 1. candidates: environment leaves within the bounding sphere (center p,
    //    radius reach plus a margin far above FP32 rounding)
    {
        const float pc[3] = {P32[0], P32[1], P32[2]};
        const float rad = m.reach + 1e-3f * (1.f + fabsf(pc[0]) + fabsf(pc[1]) + fabsf(pc[2]));
        int cur = 0;
        for (int level = 0; level < 2 * MESH_STACK; ++level) {
            const int nf = min(nfront[cur], MESH_FRONT);
            if (nf == 0) break;
            for (int k = tid; k < nf; k += MESH_DETAIL_THREADS) {
                const int node = front[cur][k];
                const BvhNode nd = m.env_nodes[node];
                if (!sphere_box(pc, rad, nd)) continue;
                if (nd.b < 0) {
                    const int c = atomicAdd(&ncand, 1);
                    if (c < MESH_CAND) {
                        cand[c] = node;
                        cbox[0][c] = nd.lo[0]; cbox[1][c] = nd.lo[1]; cbox[2][c] = nd.lo[2];
                        cbox[3][c] = nd.hi[0]; cbox[4][c] = nd.hi[1]; cbox[5][c] = nd.hi[2];
                    } else {
                        overflow = 1;
                    }
                } else {
                    const int f = atomicAdd(&nfront[cur ^ 1], 2);
                    if (f + 2 <= MESH_FRONT) { front[cur ^ 1][f] = nd.a; front[cur ^ 1][f + 1] = nd.b; }
                    else overflow = 1;
                }
            }
            __syncthreads();
            if (tid == 0) nfront[cur] = 0;
            cur ^= 1;
            __syncthreads();
        }
        if (tid == 0 && nfront[cur] != 0) overflow = 1;
        __syncthreads();
    }
    if (overflow) {
        // per-thread depth-first walk with each robot leaf's world box
        for (int leaf = tid; leaf < m.nrleaves && !hit; leaf += MESH_DETAIL_THREADS) {
            const BvhNode rl = m.robot_leaves[leaf];
            float lo[3], hi[3];
            robot_leaf_box(rl, R32, P32, lo, hi);
            int stack[MESH_STACK];
            int sp = 0;
            stack[sp++] = 0;
            while (sp && !hit) {
                BvhNode nd = m.env_nodes[stack[--sp]];
                if (!box_overlap(lo, hi, nd)) continue;
                if (nd.b >= 0) {
                    if (sp + 2 <= MESH_STACK) { stack[sp++] = nd.a; stack[sp++] = nd.b; }
                    continue;
                }
                for (int e = nd.a; e < nd.a - nd.b && !hit; ++e)
                    for (int rt = 0; rt < -rl.b; ++rt)
                        if (pair_hits(m, R, P, R32, P32, eps, X, rl.a + rt, e)) { hit = 1; break; }
            }
        }
        __syncthreads();
        if (tid == 0) out[i] = hit ? 0 : 1;
        return;
    }
    const int nc = min(ncand, MESH_CAND);
    for (int base = 0; base < m.nrleaves && !hit; base += MESH_DETAIL_THREADS) {
        // 2. this thread's robot leaf against the candidates
        const int leaf = base + tid;
        float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f};
        int ra = 0, rc = 0, c_next = nc;
        if (leaf < m.nrleaves) {
            const BvhNode rl = m.robot_leaves[leaf];
            robot_leaf_box(rl, R32, P32, lo, hi);
            ra = rl.a;
            rc = -rl.b;
            c_next = 0;
        }
        for (;;) {
            while (c_next < nc) {
                const bool ov = !(cbox[0][c_next] > hi[0] || cbox[3][c_next] < lo[0] || cbox[1][c_next] > hi[1] ||
                                  cbox[4][c_next] < lo[1] || cbox[2][c_next] > hi[2] || cbox[5][c_next] < lo[2]);
                if (ov) {
                    const int slot = atomicAdd(&nq, 1);
                    if (slot >= MESH_QUEUE) break;  // queue full: retry this candidate next round
                    const BvhNode el = m.env_nodes[cand[c_next]];
                    qra[slot] = ra;
                    qrc[slot] = rc;
                    qea[slot] = el.a;
                    qec[slot] = -el.b;
                }
                ++c_next;
            }
            const bool more = c_next < nc;
            __syncthreads();
            // 3. triangle pairs of the queued leaf pairs, spread over the block
            const int npairs = min(nq, MESH_QUEUE);
            for (int j = tid; j < npairs * 64 && !hit; j += MESH_DETAIL_THREADS) {
                const int e = j >> 6, rt = (j >> 3) & 7, et = j & 7;
                if (rt >= qrc[e] || et >= qec[e]) continue;
                if (pair_hits(m, R, P, R32, P32, eps, X, qra[e] + rt, qea[e] + et)) hit = 1;
            }
            __syncthreads();
            if (tid == 0) nq = 0;
            if (!__syncthreads_or(more) || hit) break;
        }
    }
    __syncthreads();
    if (tid == 0) {
        out[i] = hit ? 0 : 1;
        if (hit && sample_edge) edge_out[sample_edge[i]] = 0;
    }
}

// ------------------------------------------------------------------ edges
// after the end states were checked (okb): the number of interior samples
// (steps - 1) of every edge whose end state is valid; the edge result starts
// as the end state's
__global__ void k_mesh_edge_counts(int metric, int D, double w0, double w1, const double* __restrict__ a,
                                   const double* __restrict__ b, int n, double inv, const uint8_t* __restrict__ okb,
                                   int* __restrict__ counts, uint8_t* __restrict__ out) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    int c = 0;
    uint8_t ok = okb[e];
    if (ok) {
        double m = dist64(metric, D, w0, w1, a + (size_t)e * D, b + (size_t)e * D);
        double sd = ceil(__dmul_rn(m, inv));
        if (!(sd >= 0.0) || sd > (double)MPTG_MAX_EDGE_SAMPLES) ok = 0;  // NaN or absurdly long: invalid
        else if (sd >= 2.0) c = (int)sd - 1;
    }
    counts[e] = c;
    out[e] = ok;
}

// exclusive scan of counts (negative = 0) over n <= 2^20 edges: 1024 threads,
// each scans a contiguous chunk
__global__ void __launch_bounds__(1024) k_mesh_scan(const int* __restrict__ counts, int n, int* __restrict__ offs,
                                                    int* __restrict__ total) {
    __shared__ long long s[1024];
    int t = threadIdx.x;
    int chunk = (n + 1023) / 1024;
    int lo = t * chunk, hi = min(n, lo + chunk);
    long long sum = 0;
    for (int e = lo; e < hi; ++e) sum += counts[e] > 0 ? counts[e] : 0;
    s[t] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        long long v = t >= o ? s[t - o] : 0;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    long long run = t ? s[t - 1] : 0;
    for (int e = lo; e < hi; ++e) {
        offs[e] = (int)run;
        run += counts[e] > 0 ? counts[e] : 0;
    }
    if (t == 1023) *total = (int)s[1023];
}

__global__ void k_mesh_edge_samples(int metric, int D, const double* __restrict__ a, const double* __restrict__ b,
                                    int n, const int* __restrict__ counts, const int* __restrict__ offs,
                                    double* __restrict__ samples, int* __restrict__ sample_edge) {
    int e = blockIdx.x;
    if (e >= n) return;
    int c = counts[e];  // interior samples i = 1 .. c of steps = c + 1
    if (c <= 0) return;
    const double* A = a + (size_t)e * D;
    const double* B = b + (size_t)e * D;
    double delta = __ddiv_rn(1.0, (double)(c + 1));
    for (int k = threadIdx.x; k < c; k += blockDim.x) {
        double* o = samples + (size_t)(offs[e] + k) * D;
        double A2[MPTG_MAX_DIM], B2[MPTG_MAX_DIM], qv[MPTG_MAX_DIM];
        for (int d = 0; d < D; ++d) { A2[d] = A[d]; B2[d] = B[d]; }
        interp64(metric, D, A2, B2, __dmul_rn((double)(k + 1), delta), qv);
        for (int d = 0; d < D; ++d) o[d] = qv[d];
        sample_edge[offs[e] + k] = e;
    }
}


__global__ void k_mesh_add_count(unsigned long long* __restrict__ c, unsigned long long v) { *c += v; }

__global__ void k_mesh_edge_reduce(const uint8_t* __restrict__ ok, const int* __restrict__ sample_edge, int total,
                                   uint8_t* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < total && !ok[k]) out[sample_edge[k]] = 0;
}

// ------------------------------------------------------------------ host

static MeshView mesh_view(const MeshData* md) {
    MeshView v;
    v.env_tris = md->env_tris; v.env_boxes = md->env_boxes; v.env_nodes = md->env_nodes;
    v.robot_tris = md->robot_tris; v.robot_leaves = md->robot_leaves;
    v.env_tris32 = md->env_tris32; v.robot_tris32 = md->robot_tris32;
    v.nenv = md->nenv; v.nrleaves = md->nrleaves;
    v.reach = (float)md->robot_radius * (1.f + 1e-5f) + MESH_MARGIN;
    v.env_max = md->env_max; v.robot_l1 = md->robot_l1;
    return v;
}

mptg_status mesh_scene_create(mptg_ctx* ctx, const mptg_scene_desc* d, mptg_scene* s) {
    if (d->nrobot < 1 || !d->robot_tris || d->nenv < 0 || (d->nenv && !d->env_tris) || d->nenv > (1 << 28) ||
        d->nrobot > (1 << 24))
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "rigid mesh scene needs robot triangles and an environment");
    MeshData* md = new MeshData();
    s->mesh = md;
    // environment tree
    std::vector<double> env(d->env_tris, d->env_tris + 9 * (size_t)d->nenv);
    std::vector<int> eidx(d->nenv);
    std::iota(eidx.begin(), eidx.end(), 0);
    std::vector<BvhNode> enodes;
    if (d->nenv) build_rec(env, eidx, 0, (int)d->nenv, enodes, nullptr);
    std::vector<double> env_sorted(env.size());
    for (size_t i = 0; i < eidx.size(); ++i)
        std::copy(&env[9 * (size_t)eidx[i]], &env[9 * (size_t)eidx[i]] + 9, &env_sorted[9 * i]);
    std::vector<float> env_boxes(6 * (size_t)d->nenv + 6);
    for (size_t i = 0; i < (size_t)d->nenv; ++i) {
        Box b = tri_box(&env_sorted[9 * i]);
        for (int k = 0; k < 3; ++k) {
            env_boxes[6 * i + k] = std::nextafter((float)b.lo[k], -INFINITY) - MESH_MARGIN;
            env_boxes[6 * i + 3 + k] = std::nextafter((float)b.hi[k], INFINITY) + MESH_MARGIN;
        }
    }
    // robot tree (only its leaves are used on the device)
    std::vector<double> rob(d->robot_tris, d->robot_tris + 9 * (size_t)d->nrobot);
    std::vector<int> ridx(d->nrobot);
    std::iota(ridx.begin(), ridx.end(), 0);
    std::vector<BvhNode> rnodes;
    std::vector<int> rleaf_ids;
    build_rec(rob, ridx, 0, (int)d->nrobot, rnodes, &rleaf_ids);
    std::vector<double> rob_sorted(rob.size());
    for (size_t i = 0; i < ridx.size(); ++i)
        std::copy(&rob[9 * (size_t)ridx[i]], &rob[9 * (size_t)ridx[i]] + 9, &rob_sorted[9 * i]);
    std::vector<BvhNode> rleaves;
    for (int id : rleaf_ids) rleaves.push_back(rnodes[id]);
    double rad = 0.0;
    for (size_t v = 0; v < rob.size() / 3; ++v) {
        double x = rob[3 * v], y = rob[3 * v + 1], z = rob[3 * v + 2];
        rad = std::max(rad, std::sqrt(x * x + y * y + z * z));
    }
    md->robot_radius = rad;
    std::vector<float> env32(env_sorted.size()), rob32(rob_sorted.size());
    double emax = 0.0, rl1 = 0.0;
    for (size_t i = 0; i < env_sorted.size(); ++i) {
        env32[i] = (float)env_sorted[i];
        emax = std::max(emax, std::fabs(env_sorted[i]));
    }
    for (size_t i = 0; i < rob_sorted.size(); ++i) rob32[i] = (float)rob_sorted[i];
    for (size_t v = 0; v < rob_sorted.size() / 3; ++v)
        rl1 = std::max(rl1, std::fabs(rob_sorted[3 * v]) + std::fabs(rob_sorted[3 * v + 1]) +
                                std::fabs(rob_sorted[3 * v + 2]));
    md->env_max = (float)(emax * (1.0 + 1e-6)) + 1e-6f;
    md->robot_l1 = (float)(rl1 * (1.0 + 1e-6)) + 1e-6f;
    md->nenv = (int)d->nenv;
    md->nenv_nodes = (int)enodes.size();
    md->nrobot = (int)d->nrobot;
    md->nrleaves = (int)rleaves.size();
    cudaError_t e = cudaSuccess;
    auto up = [&](void** dst, const void* src, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(dst, bytes ? bytes : 16);
        if (e == cudaSuccess && bytes) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    };
    up((void**)&md->env_tris, env_sorted.data(), env_sorted.size() * sizeof(double));
    up((void**)&md->env_boxes, env_boxes.data(), env_boxes.size() * sizeof(float));
    up((void**)&md->env_nodes, enodes.data(), enodes.size() * sizeof(BvhNode));
    up((void**)&md->robot_tris, rob_sorted.data(), rob_sorted.size() * sizeof(double));
    up((void**)&md->robot_leaves, rleaves.data(), rleaves.size() * sizeof(BvhNode));
    up((void**)&md->env_tris32, env32.data(), env32.size() * sizeof(float));
    up((void**)&md->robot_tris32, rob32.data(), rob32.size() * sizeof(float));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return mptg_fail(ctx, MPTG_ERR_OOM, "mesh scene allocation failed: %s", cudaGetErrorString(e));
    }
    return MPTG_OK;
}

void mesh_scene_free(mptg_scene* s) {
    MeshData* md = s->mesh;
    if (!md) return;
    void* ptrs[] = {md->env_tris, md->env_boxes, md->env_nodes, md->robot_tris, md->robot_leaves, md->env_tris32,
                    md->robot_tris32};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete md;
    s->mesh = nullptr;
}

void mesh_fill_view(const mptg_scene*, SceneView*) {}

static mptg_status grow(mptg_ctx* ctx, void** p, size_t* cap, size_t need, size_t elem, cudaStream_t s) {
    if (need <= *cap) return MPTG_OK;
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (*p) cudaFree(*p);
    *p = nullptr;
    size_t n = need + need / 2 + 1024;
    MPTG_CUDA_TRY(ctx, cudaMalloc(p, n * elem));
    *cap = n;
    return MPTG_OK;
}

static mptg_status mesh_scratch_init(mptg_ctx* ctx, EdgeScratch* x) {
    if (!x->nwork) MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&x->nwork, sizeof(int)));
    if (!x->hbuf) MPTG_CUDA_TRY(ctx, cudaMallocHost((void**)&x->hbuf, 4 * sizeof(int)));
    return MPTG_OK;
}

mptg_status mesh_states_dev(mptg_scene* sc, const double* dq, int n, uint8_t* dout, cudaStream_t s, EdgeScratch* x,
                            const int* sample_edge, uint8_t* edge_out) {
    mptg_ctx* ctx = sc->ctx;
    MeshData* md = sc->mesh;
    if (n <= 0) return MPTG_OK;
    mptg_status st = mesh_scratch_init(ctx, x);
    if (st) return st;
    size_t cap = x->mwork_cap;
    if ((st = grow(ctx, (void**)&x->mwork, &cap, (size_t)n, sizeof(int), s))) return st;
    x->mwork_cap = cap;
    MeshView v = mesh_view(md);
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(x->nwork, 0, sizeof(int), s));
    k_mesh_sphere<<<mptg_blocks(n, 128), 128, 0, s>>>(v, dq, n, sc->D, dout, x->mwork, x->nwork);
    MPTG_LAUNCHED(ctx);
    if (n <= 16384) {
        // small batches: one block per state, the blocks past the device-side
        // count leave at once, and no host round trip is needed
        k_mesh_detail<<<n, MESH_DETAIL_THREADS, 0, s>>>(v, dq, sc->D, x->mwork, x->nwork, dout, sample_edge,
                                                        edge_out);
        MPTG_LAUNCHED(ctx);
        MPTG_CUDA_TRY(ctx, cudaGetLastError());
        return MPTG_OK;
    }
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(x->hbuf, x->nwork, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    int nw = x->hbuf[0];
    if (nw > 0) {
        // one block per state that the sphere test could not clear
        k_mesh_detail<<<nw, MESH_DETAIL_THREADS, 0, s>>>(v, dq, sc->D, x->mwork, x->nwork, dout, sample_edge,
                                                         edge_out);
        MPTG_LAUNCHED(ctx);
    }
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    return MPTG_OK;
}

mptg_status mesh_edges_dev(mptg_scene* sc, const double* da, const double* db, int n, double step, int resolution,
                           uint8_t* dout, cudaStream_t s, unsigned long long* nsamp, EdgeScratch* x) {
    mptg_ctx* ctx = sc->ctx;
    if (n <= 0) return MPTG_OK;
    if (resolution != 0) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "rigid mesh edges use the space metric");
    if (n > (1 << 20)) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "at most 2^20 mesh edges per call");
    mptg_status st = mesh_scratch_init(ctx, x);
    if (st) return st;
    size_t cap = x->edge_cap, cap2 = x->edge_cap, cap3 = x->edge_cap;
    if ((st = grow(ctx, (void**)&x->counts, &cap, (size_t)n + 1, sizeof(int), s))) return st;
    if ((st = grow(ctx, (void**)&x->offs, &cap2, (size_t)n + 1, sizeof(int), s))) return st;
    if ((st = grow(ctx, (void**)&x->okb, &cap3, (size_t)n + 1, 1, s))) return st;
    x->edge_cap = std::min(cap, std::min(cap2, cap3));
    // phase A: every edge's end state first (the DMV checks `to` before any
    // interior sample); only edges whose end state is valid expand further
    if ((st = mesh_states_dev(sc, db, n, x->okb, s, x))) return st;
    if (nsamp) {
        k_mesh_add_count<<<1, 1, 0, s>>>(nsamp, (unsigned long long)n);
        MPTG_LAUNCHED(ctx);
    }
    k_mesh_edge_counts<<<mptg_blocks(n, 128), 128, 0, s>>>(sc->metric, sc->D, sc->w0, sc->w1, da, db, n, 1.0 / step,
                                                           x->okb, x->counts, dout);
    k_mesh_scan<<<1, 1024, 0, s>>>(x->counts, n, x->offs, x->offs + n);
    ctx->launches += 2;
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(x->hbuf + 1, x->offs + n, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    int total = x->hbuf[1];
    if (total > 0) {
        cap = x->sample_cap;
        cap2 = x->sample_cap;
        cap3 = x->sample_cap;
        if ((st = grow(ctx, (void**)&x->samples, &cap, (size_t)total, sc->D * sizeof(double), s))) return st;
        if ((st = grow(ctx, (void**)&x->sample_edge, &cap2, (size_t)total, sizeof(int), s))) return st;
        if ((st = grow(ctx, (void**)&x->sample_ok, &cap3, (size_t)total, 1, s))) return st;
        x->sample_cap = std::min(cap, std::min(cap2, cap3));
        k_mesh_edge_samples<<<n, 64, 0, s>>>(sc->metric, sc->D, da, db, n, x->counts, x->offs, x->samples,
                                             x->sample_edge);
        MPTG_LAUNCHED(ctx);
        st = mesh_states_dev(sc, x->samples, total, x->sample_ok, s, x, x->sample_edge, dout);
        if (st) return st;
        k_mesh_edge_reduce<<<mptg_blocks(total, 256), 256, 0, s>>>(x->sample_ok, x->sample_edge, total, dout);
        MPTG_LAUNCHED(ctx);
        if (nsamp) {
            k_mesh_add_count<<<1, 1, 0, s>>>(nsamp, (unsigned long long)total);
            MPTG_LAUNCHED(ctx);
        }
    }
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    return MPTG_OK;
}
