/*
 * oracle.c - CPU restatement of MPT's planner hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * test and bench.py's CPU-baseline leg load it; the mpt_gb300 product never
 * does.  Compiled with -O2 -ffp-contract=off so every FP64 expression rounds
 * exactly as written (the device code uses explicit __dadd_rn/__dmul_rn).
 *
 * Reference files restated here (paths inside the MPT project):
 *   src/mpt/lp_space.hpp:44-54          L_p interpolate
 *   src/mpt/so2_space.hpp:44-65         SO(2) interpolate (ccwDist/bound from nigh)
 *   src/mpt/so3_space.hpp:44-83         SO(3) slerp with the d >= 1-eps fallback
 *   src/mpt/cartesian_space.hpp:43-68   element-wise interpolate
 *   src/mpt/scaled_space.hpp:44-52      scaled interpolate
 *   src/mpt/discrete_motion_validator.hpp:71-130   DMV (bisection ring queue)
 *   demo/png_2d_scenario.hpp:104-110    grid valid()
 *   demo/link_manipulator_scenario.hpp:99-116 + demo/shape_hierarchy.hpp:228-270
 *                                       planar-arm valid()
 *   demo/se3_rigid_body_scenario.hpp:282-312  rigid-body valid() (fcl::collide)
 * Distances are nigh's (not vendored); their formulas are pinned by
 * test/lp_space_test.cpp, so2_space_test.cpp, so3_space_test.cpp,
 * se3_space_test.cpp and scaled_space_test.cpp (see tests/test_oracle_kats.py).
 */
#include "oracle.h"
#include "../include/mptg_detmath.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TWO_PI MPTG_TWO_PI
#define PI MPTG_PI

/* ------------------------------------------------------------------ */
/* SO(2) helpers (nigh so2::ccwDist / so2::bound).  The reference KATs in
 * test/so2_space_test.cpp:73-83 (exact ==) admit this choice: ccwDist is the
 * counter-clockwise angle from a to b reduced into [0, 2pi) with fmod, bound
 * reduces into [-pi, pi) with fmod plus one correction. */
double orc_so2_ccw(double a, double b) {
    double d = fmod(b - a, TWO_PI);
    if (d < 0) d += TWO_PI;
    return d;
}

double orc_so2_bound(double v) {
    v = fmod(v, TWO_PI);
    if (v < -PI) v += TWO_PI;
    else if (v >= PI) v -= TWO_PI;
    return v;
}

/* wrapped |a-b| for one joint: min(d, 2pi - d) with d = |a-b| reduced. */
static double so2_dist1(double a, double b) {
    double d = fabs(a - b);
    if (d > TWO_PI) d = fmod(d, TWO_PI);
    return d > PI ? TWO_PI - d : d;
}

static double quat_dot(const double* a, const double* b) {
    /* coefficient order (x, y, z, w) as so3_space.hpp:52-55 sums it */
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
}

static double so3_dist(const double* a, const double* b) {
    double d = fabs(quat_dot(a, b));
    if (d > 1.0) d = 1.0;
    return mptg_acos(d);
}

static double l2_dist(const double* a, const double* b, int dim) {
    double s = 0;
    for (int i = 0; i < dim; ++i) { double d = a[i] - b[i]; s += d * d; }
    return sqrt(s);
}

double orc_distance(const orc_space* s, const double* a, const double* b) {
    switch (s->metric) {
    case ORC_L2: return l2_dist(a, b, s->dim);
    case ORC_L1: { double r = 0; for (int i = 0; i < s->dim; ++i) r += fabs(a[i] - b[i]); return r; }
    case ORC_SO2: { double r = 0; for (int i = 0; i < s->dim; ++i) r += so2_dist1(a[i], b[i]); return r; }
    case ORC_SO3: return so3_dist(a, b);
    case ORC_SE3: return s->w[0] * so3_dist(a, b) + s->w[1] * l2_dist(a + 4, b + 4, 3);
    }
    return NAN;
}

/* lp_space.hpp:44-54: q_i = (b_i - a_i) * t + a_i */
static void lp_interp(const double* a, const double* b, double t, double* q, int dim) {
    for (int i = 0; i < dim; ++i) q[i] = (b[i] - a[i]) * t + a[i];
}

/* so3_space.hpp:44-83 */
static void so3_interp(const double* a, const double* b, double t, double* q) {
    double d = quat_dot(a, b);
    double ad = fabs(d);
    double s0, s1;
    if (d >= 1.0 - DBL_EPSILON) {
        s0 = 1.0 - t;
        s1 = t;
    } else {
        double theta = mptg_acos(ad);
        double sinTheta = mptg_sin(theta);
        s0 = mptg_sin((1.0 - t) * theta) / sinTheta;
        s1 = mptg_sin(t * theta) / sinTheta;
    }
    if (d < 0) s1 = -s1;
    for (int i = 0; i < 4; ++i) q[i] = s0 * a[i] + s1 * b[i];
}

void orc_interpolate(const orc_space* s, const double* a, const double* b, double t, double* q) {
    switch (s->metric) {
    case ORC_L2: case ORC_L1: lp_interp(a, b, t, q, s->dim); break;
    case ORC_SO2: /* so2_space.hpp:44-65 */
        for (int i = 0; i < s->dim; ++i) {
            double ccw = orc_so2_ccw(a[i], b[i]);
            if (ccw < PI) q[i] = orc_so2_bound(a[i] + ccw * t);
            else { double cw = 2 * PI - ccw; q[i] = orc_so2_bound(a[i] - cw * t); }
        }
        break;
    case ORC_SO3: so3_interp(a, b, t, q); break;
    case ORC_SE3: /* cartesian_space.hpp:43-68, element 0 = SO3, element 1 = L2 */
        so3_interp(a, b, t, q);
        lp_interp(a + 4, b + 4, t, q + 4, 3);
        break;
    }
}

/* ------------------------------------------------------------------ */
/* Brute-force exact NN */
static int nthreads_or_default(int n) { return n > 0 ? n : 1; }

void orc_nn_brute(const orc_space* s, const double* pts, int64_t n, const double* q,
                  int64_t nq, int32_t* idx, double* dist, int nthreads) {
    int D = s->dim;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads_or_default(nthreads))
    for (int64_t i = 0; i < nq; ++i) {
        double best = INFINITY; int32_t bi = -1;
        for (int64_t j = 0; j < n; ++j) {
            double d = orc_distance(s, q + i * D, pts + j * D);
            if (d < best || (bi < 0 && d == best)) { best = d; bi = (int32_t)j; }
        }
        idx[i] = bi; dist[i] = best;
    }
}

void orc_knn_brute(const orc_space* s, const double* pts, int64_t n, const double* q,
                   int64_t nq, int k, int32_t* idx, double* dist, int nthreads) {
    int D = s->dim;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads_or_default(nthreads))
    for (int64_t i = 0; i < nq; ++i) {
        int32_t* bi = idx + i * k; double* bd = dist + i * k;
        int cnt = 0;
        for (int64_t j = 0; j < n; ++j) {
            double d = orc_distance(s, q + i * D, pts + j * D);
            if (d != d) continue;
            if (cnt == k && !(d < bd[k - 1])) continue; /* equal distance: lower index already kept */
            int p = cnt < k ? cnt++ : k - 1;
            while (p > 0 && bd[p - 1] > d) { bd[p] = bd[p - 1]; bi[p] = bi[p - 1]; --p; }
            bd[p] = d; bi[p] = (int32_t)j;
        }
        for (int p = cnt; p < k; ++p) { bd[p] = INFINITY; bi[p] = -1; }
    }
}

/* ------------------------------------------------------------------ */
/* CPU kd-tree (baseline NN).  Sliding-midpoint splits on the widest axis of
 * the cell's points, buckets of at most leaf_size points, near-child-first
 * depth-first search with a cell lower bound.  Exact FP64 results, lowest
 * index on ties. */
typedef struct {
    int dim;              /* split dim, -1 = leaf */
    double split;
    int32_t child;        /* internal: left child (right = child + 1); leaf: start in perm */
    int32_t count;        /* leaf: number of points */
} kd_node;

typedef struct {
    orc_space s;
    const double* pts;
    int64_t n;
    int32_t* perm;
    kd_node* nodes;
    double* lo;           /* per-node cell bounds, dim doubles each */
    double* hi;
    int64_t nnodes, cap;
    int leaf;
} kd_tree;

static int64_t kd_alloc(kd_tree* t, int64_t cnt) {
    if (t->nnodes + cnt > t->cap) {
        int64_t nc = t->cap * 2 + cnt + 16;
        t->nodes = (kd_node*)realloc(t->nodes, nc * sizeof(kd_node));
        t->lo = (double*)realloc(t->lo, nc * t->s.dim * sizeof(double));
        t->hi = (double*)realloc(t->hi, nc * t->s.dim * sizeof(double));
        t->cap = nc;
    }
    int64_t r = t->nnodes; t->nnodes += cnt; return r;
}

static void kd_build_rec(kd_tree* t, int64_t node, int64_t start, int64_t count, int depth) {
    int D = t->s.dim;
    if (count <= t->leaf || depth > 200) {
        t->nodes[node].dim = -1; t->nodes[node].child = (int32_t)start; t->nodes[node].count = (int32_t)count;
        return;
    }
    /* widest dimension of the points */
    int bd = 0; double bext = -1, bmin = 0, bmax = 0;
    for (int d = 0; d < D; ++d) {
        double mn = INFINITY, mx = -INFINITY;
        for (int64_t i = 0; i < count; ++i) {
            double v = t->pts[(int64_t)t->perm[start + i] * D + d];
            if (v < mn) mn = v;
            if (v > mx) mx = v;
        }
        if (mx - mn > bext) { bext = mx - mn; bd = d; bmin = mn; bmax = mx; }
    }
    if (!(bext > 0)) {
        t->nodes[node].dim = -1; t->nodes[node].child = (int32_t)start; t->nodes[node].count = (int32_t)count;
        return;
    }
    double split = 0.5 * (bmin + bmax);
    if (!(split > bmin)) split = bmax;
    int64_t i = start, j = start + count - 1;
    while (i <= j) {
        double v = t->pts[(int64_t)t->perm[i] * D + bd];
        if (v < split) ++i;
        else { int32_t tmp = t->perm[i]; t->perm[i] = t->perm[j]; t->perm[j] = tmp; --j; }
    }
    int64_t nl = i - start;
    int64_t c = kd_alloc(t, 2);
    /* kd_alloc may move arrays: index, never hold pointers */
    t->nodes[node].dim = bd; t->nodes[node].split = split; t->nodes[node].child = (int32_t)c; t->nodes[node].count = 0;
    for (int d = 0; d < D; ++d) {
        t->lo[c * D + d] = t->lo[node * D + d]; t->hi[c * D + d] = t->hi[node * D + d];
        t->lo[(c + 1) * D + d] = t->lo[node * D + d]; t->hi[(c + 1) * D + d] = t->hi[node * D + d];
    }
    t->hi[c * D + bd] = split;
    t->lo[(c + 1) * D + bd] = split;
    kd_build_rec(t, c, start, nl, depth + 1);
    kd_build_rec(t, c + 1, start + nl, count - nl, depth + 1);
}

void* orc_kd_build(const orc_space* s, const double* pts, int64_t n, int leaf_size) {
    kd_tree* t = (kd_tree*)calloc(1, sizeof(kd_tree));
    t->s = *s; t->pts = pts; t->n = n; t->leaf = leaf_size > 0 ? leaf_size : 8;
    t->perm = (int32_t*)malloc((n > 0 ? n : 1) * sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) t->perm[i] = (int32_t)i;
    int64_t root = kd_alloc(t, 1);
    int D = s->dim;
    for (int d = 0; d < D; ++d) {
        double lo = -INFINITY, hi = INFINITY;
        if (s->metric == ORC_SO2) { lo = -PI; hi = PI; }
        t->lo[root * D + d] = lo; t->hi[root * D + d] = hi;
    }
    kd_build_rec(t, root, 0, n, 0);
    return t;
}

/* distance from point q to the box [lo, hi] under the metric: a lower bound
 * of the distance to every point inside the box. */
static double kd_box_lb(const kd_tree* t, const double* q, const double* lo, const double* hi) {
    int D = t->s.dim;
    switch (t->s.metric) {
    case ORC_L2: case ORC_L1: {
        double acc = 0;
        for (int d = 0; d < D; ++d) {
            double o = 0;
            if (q[d] < lo[d]) o = lo[d] - q[d]; else if (q[d] > hi[d]) o = q[d] - hi[d];
            acc += t->s.metric == ORC_L2 ? o * o : o;
        }
        return t->s.metric == ORC_L2 ? sqrt(acc) : acc;
    }
    case ORC_SO2: {
        double acc = 0;
        for (int d = 0; d < D; ++d) {
            if (q[d] >= lo[d] && q[d] <= hi[d]) continue;
            double a = so2_dist1(q[d], lo[d]), b = so2_dist1(q[d], hi[d]);
            acc += a < b ? a : b;
        }
        return acc;
    }
    case ORC_SO3: case ORC_SE3: {
        /* rotation part: chord distance from +-q to the box bounds the angle */
        double cp = 0, cm = 0;
        for (int d = 0; d < 4; ++d) {
            double o = 0, v = q[d];
            if (v < lo[d]) o = lo[d] - v; else if (v > hi[d]) o = v - hi[d];
            cp += o * o;
            o = 0; v = -q[d];
            if (v < lo[d]) o = lo[d] - v; else if (v > hi[d]) o = v - hi[d];
            cm += o * o;
        }
        double c2 = cp < cm ? cp : cm;
        double x = 1.0 - 0.5 * c2;
        if (x < 0) x = 0;
        double rot = x >= 1.0 ? 0.0 : mptg_acos(x);
        if (t->s.metric == ORC_SO3) return rot;
        double acc = 0;
        for (int d = 4; d < 7; ++d) {
            double o = 0;
            if (q[d] < lo[d]) o = lo[d] - q[d]; else if (q[d] > hi[d]) o = q[d] - hi[d];
            acc += o * o;
        }
        return t->s.w[0] * rot + t->s.w[1] * sqrt(acc);
    }
    }
    return 0;
}

typedef struct { double best; int32_t idx; int64_t evals; } kd_result;

static void kd_search(const kd_tree* t, int64_t node, const double* q, kd_result* r) {
    int D = t->s.dim;
    const kd_node* nd = &t->nodes[node];
    if (nd->dim < 0) {
        for (int32_t i = 0; i < nd->count; ++i) {
            int32_t p = t->perm[nd->child + i];
            double d = orc_distance(&t->s, q, t->pts + (int64_t)p * D);
            r->evals++;
            if (d < r->best || (d == r->best && p < r->idx)) { r->best = d; r->idx = p; }
        }
        return;
    }
    int64_t c = nd->child;
    int64_t nearc = q[nd->dim] < nd->split ? c : c + 1;
    int64_t farc = nearc == c ? c + 1 : c;
    kd_search(t, nearc, q, r);
    double lb = kd_box_lb(t, q, t->lo + farc * D, t->hi + farc * D);
    /* a relative slack makes the bound robust to its own rounding */
    if (lb * (1.0 - 1e-12) - 1e-300 <= r->best) kd_search(t, farc, q, r);
}

void orc_kd_nearest(void* tree, const double* q, int64_t nq, int32_t* idx, double* dist,
                    int nthreads, int64_t* dist_evals) {
    kd_tree* t = (kd_tree*)tree;
    int D = t->s.dim;
    int64_t total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+:total) num_threads(nthreads_or_default(nthreads))
    for (int64_t i = 0; i < nq; ++i) {
        kd_result r = {INFINITY, INT32_MAX, 0};
        if (t->n > 0) kd_search(t, 0, q + i * D, &r);
        idx[i] = t->n > 0 ? r.idx : -1; dist[i] = r.best;
        total += r.evals;
    }
    if (dist_evals) *dist_evals = total;
}

void orc_kd_free(void* tree) {
    kd_tree* t = (kd_tree*)tree;
    if (!t) return;
    free(t->perm); free(t->nodes); free(t->lo); free(t->hi); free(t);
}

/* ------------------------------------------------------------------ */
/* Scenario validity */

/* demo/png_2d_scenario.hpp:104-110: round-half-up via (int)(x + 0.5).  The
 * reference does no bounds check; here a cell index outside the grid is an
 * obstacle (the reference would read out of bounds there). */
static int grid_valid(const orc_scene* sc, const double* q) {
    double vx = q[0] + 0.5, vy = q[1] + 0.5;
    if (!(vx > -1.0 && vx < (double)sc->width && vy > -1.0 && vy < (double)sc->height)) return 0;
    int x = (int)vx, y = (int)vy;
    return sc->grid[(int64_t)sc->width * y + x] == 0;
}

/* demo/shape_hierarchy.hpp:259-270 */
static double dist_point_segment_sq(double px, double py, double ax, double ay, double bx, double by) {
    double vx = bx - ax, vy = by - ay;
    double wx = px - ax, wy = py - ay;
    double c1 = vx * wx + vy * wy;
    if (c1 <= 0) return wx * wx + wy * wy;
    double c2 = vx * vx + vy * vy;
    if (c2 <= c1) { double ex = px - bx, ey = py - by; return ex * ex + ey * ey; }
    double f = c1 / c2;
    double ex = ax - px + vx * f, ey = ay - py + vy * f;
    return ex * ex + ey * ey;
}

static double orient2d(double ax, double ay, double bx, double by, double cx, double cy) {
    return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}

static int on_segment_box(double ax, double ay, double bx, double by, double px, double py) {
    return fmin(ax, bx) <= px && px <= fmax(ax, bx) && fmin(ay, by) <= py && py <= fmax(ay, by);
}

/* closed-segment intersection (touching counts) with FP64 orientation signs */
static int segments_intersect(const double* p, const double* q) {
    double ax = p[0], ay = p[1], bx = p[2], by = p[3];
    double cx = q[0], cy = q[1], dx = q[2], dy = q[3];
    double o1 = orient2d(ax, ay, bx, by, cx, cy);
    double o2 = orient2d(ax, ay, bx, by, dx, dy);
    double o3 = orient2d(cx, cy, dx, dy, ax, ay);
    double o4 = orient2d(cx, cy, dx, dy, bx, by);
    if (((o1 > 0 && o2 < 0) || (o1 < 0 && o2 > 0)) && ((o3 > 0 && o4 < 0) || (o3 < 0 && o4 > 0)))
        return 1;
    if (o1 == 0 && on_segment_box(ax, ay, bx, by, cx, cy)) return 1;
    if (o2 == 0 && on_segment_box(ax, ay, bx, by, dx, dy)) return 1;
    if (o3 == 0 && on_segment_box(cx, cy, dx, dy, ax, ay)) return 1;
    if (o4 == 0 && on_segment_box(cx, cy, dx, dy, bx, by)) return 1;
    return 0;
}

/* demo/link_manipulator_scenario.hpp:99-116 (forward kinematics by cumulative
 * angles; link-vs-disc via squared point-segment distance against
 * (r + robotRadius)^2) plus the non-adjacent link self-intersection test that
 * the planar-arm workload adds.  sin/cos are the deterministic mptg_sincos. */
#define ORC_MAX_LINKS 64
static int arm_valid(const orc_scene* sc, const double* q) {
    double seg[ORC_MAX_LINKS][4];
    double fx = 0, fy = 0, angle = 0;
    int nl = sc->nlinks;
    for (int i = 0; i < nl; ++i) {
        angle += q[i];
        double s, c;
        mptg_sincos(angle, &s, &c);
        double tx = fx + sc->link_len[i] * c;
        double ty = fy + sc->link_len[i] * s;
        for (int k = 0; k < sc->ndiscs; ++k) {
            const double* dk = sc->discs + 3 * k;
            double rr = (dk[2] + sc->robot_radius) * (dk[2] + sc->robot_radius);
            if (!(dist_point_segment_sq(dk[0], dk[1], fx, fy, tx, ty) > rr)) return 0;
        }
        seg[i][0] = fx; seg[i][1] = fy; seg[i][2] = tx; seg[i][3] = ty;
        fx = tx; fy = ty;
    }
    if (sc->self_collision) {
        for (int i = 0; i < nl; ++i)
            for (int j = i + 2; j < nl; ++j)
                if (segments_intersect(seg[i], seg[j])) return 0;
    }
    return 1;
}

/* ---- rigid mesh (SE3) ---- */

/* Rotation of v by unit quaternion (x, y, z, w) through the rotation matrix
 * R = I + 2 [ -(yy+zz), xy-wz, xz+wy ; xy+wz, -(xx+zz), yz-wx ; xz-wy, yz+wx, -(xx+yy) ],
 * then translation: the transform Translation(p) * Quaternion(q) of
 * demo/se3_rigid_body_scenario.hpp:282-285. */
static void quat_to_mat(const double* q, double* R) {
    double x = q[0], y = q[1], z = q[2], w = q[3];
    double tx = 2 * x, ty = 2 * y, tz = 2 * z;
    double twx = tx * w, twy = ty * w, twz = tz * w;
    double txx = tx * x, txy = ty * x, txz = tz * x;
    double tyy = ty * y, tyz = tz * y, tzz = tz * z;
    R[0] = 1 - (tyy + tzz); R[1] = txy - twz; R[2] = txz + twy;
    R[3] = txy + twz; R[4] = 1 - (txx + tzz); R[5] = tyz - twx;
    R[6] = txz - twy; R[7] = tyz + twx; R[8] = 1 - (txx + tyy);
}

static void xform(const double* R, const double* p, const double* v, double* o) {
    o[0] = R[0] * v[0] + R[1] * v[1] + R[2] * v[2] + p[0];
    o[1] = R[3] * v[0] + R[4] * v[1] + R[5] * v[2] + p[1];
    o[2] = R[6] * v[0] + R[7] * v[1] + R[8] * v[2] + p[2];
}

static void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void sub3(const double* a, const double* b, double* c) { c[0] = a[0] - b[0]; c[1] = a[1] - b[1]; c[2] = a[2] - b[2]; }

/* 2-D helpers for the coplanar case of Moller's test */
static int edge_edge_2d(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy) {
    double p[4] = {ax, ay, bx, by}, q[4] = {cx, cy, dx, dy};
    return segments_intersect(p, q);
}
static int point_in_tri_2d(double px, double py, const double* t) {
    double d1 = orient2d(t[0], t[1], t[2], t[3], px, py);
    double d2 = orient2d(t[2], t[3], t[4], t[5], px, py);
    double d3 = orient2d(t[4], t[5], t[0], t[1], px, py);
    int neg = d1 < 0 || d2 < 0 || d3 < 0, pos = d1 > 0 || d2 > 0 || d3 > 0;
    return !(neg && pos);
}
static int coplanar_tri_tri(const double* n, const double* V0, const double* V1, const double* V2,
                            const double* U0, const double* U1, const double* U2) {
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
            if (edge_edge_2d(v[2 * e], v[2 * e + 1], v[2 * e1], v[2 * e1 + 1],
                             u[2 * f], u[2 * f + 1], u[2 * f1], u[2 * f1 + 1])) return 1;
        }
    }
    if (point_in_tri_2d(v[0], v[1], u)) return 1;
    if (point_in_tri_2d(u[0], u[1], v)) return 1;
    return 0;
}

/* interval of a triangle on the intersection line (Moller 1997, the
 * "compute intervals" step); returns 1 when the triangles are coplanar. */
static int tri_interval(double VV0, double VV1, double VV2, double D0, double D1, double D2,
                        double D0D1, double D0D2, double* i0, double* i1) {
    if (D0D1 > 0) {
        *i0 = VV2 + (VV0 - VV2) * D2 / (D2 - D0); *i1 = VV2 + (VV1 - VV2) * D2 / (D2 - D1);
    } else if (D0D2 > 0) {
        *i0 = VV1 + (VV0 - VV1) * D1 / (D1 - D0); *i1 = VV1 + (VV2 - VV1) * D1 / (D1 - D2);
    } else if (D1 * D2 > 0 || D0 != 0) {
        *i0 = VV0 + (VV1 - VV0) * D0 / (D0 - D1); *i1 = VV0 + (VV2 - VV0) * D0 / (D0 - D2);
    } else if (D1 != 0) {
        *i0 = VV1 + (VV0 - VV1) * D1 / (D1 - D0); *i1 = VV1 + (VV2 - VV1) * D1 / (D1 - D2);
    } else if (D2 != 0) {
        *i0 = VV2 + (VV0 - VV2) * D2 / (D2 - D0); *i1 = VV2 + (VV1 - VV2) * D2 / (D2 - D1);
    } else {
        return 1;
    }
    return 0;
}

/* Triangle-triangle intersection after T. Moller, "A Fast Triangle-Triangle
 * Intersection Test", J. Graphics Tools 2(2), 1997, without epsilon snapping:
 * FP64 plane-side tests, interval overlap on the line of intersection, and
 * a 2-D edge/containment test for coplanar pairs.  Touching counts. */
int orc_tri_tri(const double* t1, const double* t2) {
    const double *V0 = t1, *V1 = t1 + 3, *V2 = t1 + 6;
    const double *U0 = t2, *U1 = t2 + 3, *U2 = t2 + 6;
    double E1[3], E2[3], N1[3], N2[3], D[3];
    sub3(V1, V0, E1); sub3(V2, V0, E2); cross3(E1, E2, N1);
    double d1 = -dot3(N1, V0);
    double du0 = dot3(N1, U0) + d1, du1 = dot3(N1, U1) + d1, du2 = dot3(N1, U2) + d1;
    double du0du1 = du0 * du1, du0du2 = du0 * du2;
    if (du0du1 > 0 && du0du2 > 0) return 0;
    sub3(U1, U0, E1); sub3(U2, U0, E2); cross3(E1, E2, N2);
    double d2 = -dot3(N2, U0);
    double dv0 = dot3(N2, V0) + d2, dv1 = dot3(N2, V1) + d2, dv2 = dot3(N2, V2) + d2;
    double dv0dv1 = dv0 * dv1, dv0dv2 = dv0 * dv2;
    if (dv0dv1 > 0 && dv0dv2 > 0) return 0;
    cross3(N1, N2, D);
    double mx = fabs(D[0]); int index = 0;
    double bb = fabs(D[1]), cc = fabs(D[2]);
    if (bb > mx) { mx = bb; index = 1; }
    if (cc > mx) { index = 2; }
    double vp0 = V0[index], vp1 = V1[index], vp2 = V2[index];
    double up0 = U0[index], up1 = U1[index], up2 = U2[index];
    double a0, a1, b0, b1;
    if (tri_interval(vp0, vp1, vp2, dv0, dv1, dv2, dv0dv1, dv0dv2, &a0, &a1))
        return coplanar_tri_tri(N1, V0, V1, V2, U0, U1, U2);
    if (tri_interval(up0, up1, up2, du0, du1, du2, du0du1, du0du2, &b0, &b1))
        return coplanar_tri_tri(N1, V0, V1, V2, U0, U1, U2);
    if (a0 > a1) { double t = a0; a0 = a1; a1 = t; }
    if (b0 > b1) { double t = b0; b0 = b1; b1 = t; }
    return !(a1 < b0 || b1 < a0);
}

/* Environment acceleration for the oracle: a static AABB tree over the
 * environment triangles, built once per scene pointer.  Any intersecting pair
 * has overlapping closed AABBs, so the result equals the OR of orc_tri_tri
 * over all pairs. */
typedef struct { double lo[3], hi[3]; int32_t left, right, start, count; } aabb_node;
typedef struct { const double* tris; int64_t n; int32_t* perm; aabb_node* nodes; int64_t nn; } env_bvh;

static void tri_box(const double* t, double* lo, double* hi) {
    for (int d = 0; d < 3; ++d) {
        lo[d] = fmin(fmin(t[d], t[3 + d]), t[6 + d]);
        hi[d] = fmax(fmax(t[d], t[3 + d]), t[6 + d]);
    }
}

static int32_t bvh_build_rec(env_bvh* b, int64_t start, int64_t count) {
    int32_t id = (int32_t)b->nn++;
    aabb_node* nd = &b->nodes[id];
    for (int d = 0; d < 3; ++d) { nd->lo[d] = INFINITY; nd->hi[d] = -INFINITY; }
    for (int64_t i = 0; i < count; ++i) {
        double lo[3], hi[3];
        tri_box(b->tris + 9 * (int64_t)b->perm[start + i], lo, hi);
        for (int d = 0; d < 3; ++d) { nd->lo[d] = fmin(nd->lo[d], lo[d]); nd->hi[d] = fmax(nd->hi[d], hi[d]); }
    }
    if (count <= 8) { nd->left = nd->right = -1; nd->start = (int32_t)start; nd->count = (int32_t)count; return id; }
    int ax = 0; double ext = -1;
    for (int d = 0; d < 3; ++d) if (nd->hi[d] - nd->lo[d] > ext) { ext = nd->hi[d] - nd->lo[d]; ax = d; }
    double mid = 0.5 * (nd->lo[ax] + nd->hi[ax]);
    int64_t i = start, j = start + count - 1;
    while (i <= j) {
        const double* t = b->tris + 9 * (int64_t)b->perm[i];
        double c = (t[ax] + t[3 + ax] + t[6 + ax]) / 3.0;
        if (c < mid) ++i; else { int32_t tmp = b->perm[i]; b->perm[i] = b->perm[j]; b->perm[j] = tmp; --j; }
    }
    int64_t nl = i - start;
    if (nl == 0 || nl == count) nl = count / 2;
    nd->start = -1; nd->count = 0;
    int32_t l = bvh_build_rec(b, start, nl);
    int32_t r = bvh_build_rec(b, start + nl, count - nl);
    b->nodes[id].left = l; b->nodes[id].right = r;
    return id;
}

static env_bvh* g_bvh = NULL;
static const double* g_bvh_key = NULL;
static int64_t g_bvh_n = -1;

static env_bvh* get_env_bvh(const orc_scene* sc) {
    if (g_bvh && g_bvh_key == sc->env_tris && g_bvh_n == sc->nenv) return g_bvh;
    if (g_bvh) { free(g_bvh->perm); free(g_bvh->nodes); free(g_bvh); }
    env_bvh* b = (env_bvh*)calloc(1, sizeof(env_bvh));
    b->tris = sc->env_tris; b->n = sc->nenv;
    b->perm = (int32_t*)malloc((sc->nenv + 1) * sizeof(int32_t));
    for (int64_t i = 0; i < sc->nenv; ++i) b->perm[i] = (int32_t)i;
    b->nodes = (aabb_node*)malloc((2 * sc->nenv + 2) * sizeof(aabb_node));
    if (sc->nenv > 0) bvh_build_rec(b, 0, sc->nenv);
    g_bvh = b; g_bvh_key = sc->env_tris; g_bvh_n = sc->nenv;
    return b;
}

static int bvh_hit(const env_bvh* b, const double* tri, const double* lo, const double* hi) {
    int32_t stack[128]; int sp = 0;
    if (b->n == 0) return 0;
    stack[sp++] = 0;
    while (sp) {
        const aabb_node* nd = &b->nodes[stack[--sp]];
        if (nd->lo[0] > hi[0] || nd->hi[0] < lo[0] || nd->lo[1] > hi[1] || nd->hi[1] < lo[1] ||
            nd->lo[2] > hi[2] || nd->hi[2] < lo[2]) continue;
        if (nd->left < 0) {
            for (int32_t i = 0; i < nd->count; ++i) {
                const double* e = b->tris + 9 * (int64_t)b->perm[nd->start + i];
                double elo[3], ehi[3];
                tri_box(e, elo, ehi);
                if (elo[0] > hi[0] || ehi[0] < lo[0] || elo[1] > hi[1] || ehi[1] < lo[1] ||
                    elo[2] > hi[2] || ehi[2] < lo[2]) continue;
                if (orc_tri_tri(tri, e)) return 1;
            }
        } else {
            if (sp + 2 > 128) return 1; /* cannot happen for trees of depth < 64 */
            stack[sp++] = nd->left; stack[sp++] = nd->right;
        }
    }
    return 0;
}

/* demo/se3_rigid_body_scenario.hpp:282-312: valid iff the robot mesh placed at
 * T(q) does not intersect the environment mesh. */
static int mesh_valid(const orc_scene* sc, const double* q) {
    env_bvh* b = g_bvh;
    double R[9];
    quat_to_mat(q, R);
    for (int64_t i = 0; i < sc->nrobot; ++i) {
        const double* t = sc->robot_tris + 9 * i;
        double w[9], lo[3], hi[3];
        xform(R, q + 4, t, w); xform(R, q + 4, t + 3, w + 3); xform(R, q + 4, t + 6, w + 6);
        tri_box(w, lo, hi);
        if (bvh_hit(b, w, lo, hi)) return 0;
    }
    return 1;
}

static int state_valid(const orc_scene* sc, const double* q) {
    switch (sc->kind) {
    case 0: return grid_valid(sc, q);
    case 1: return arm_valid(sc, q);
    case 2: return mesh_valid(sc, q);
    }
    return 0;
}

int orc_state_valid(const orc_scene* sc, const double* q) {
    if (sc->kind == 2) get_env_bvh(sc);
    return state_valid(sc, q);
}

void orc_valid_states(const orc_scene* sc, const orc_space* sp, const double* q, int64_t n,
                      uint8_t* out, int nthreads) {
    int D = sp->dim;
    if (sc->kind == 2) get_env_bvh(sc);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads_or_default(nthreads))
    for (int64_t i = 0; i < n; ++i) out[i] = (uint8_t)state_valid(sc, q + i * D);
}

static double step_measure(const orc_space* sp, int resolution, const double* a, const double* b) {
    if (resolution == 1) {
        double m = 0;
        for (int i = 0; i < sp->dim; ++i) { double d = so2_dist1(a[i], b[i]); if (d > m) m = d; }
        return m;
    }
    return orc_distance(sp, a, b);
}

/* discrete_motion_validator.hpp:71-130.  Checks `to`, then the samples
 * interpolate(from, to, i * (1/steps)) for i in [1, steps-1] in bisection
 * order through a 256-entry ring queue, switching to a sequential scan of a
 * range when the queue is full.  Returns the validity and counts samples. */
#define DMV_QUEUE 256
static int dmv_edge(const orc_scene* sc, const orc_space* sp, const double* from, const double* to,
                    double invStep, int resolution, int64_t* nsamples) {
    double q[16];
    int64_t cnt = 1;
    int ok = 1;
    if (!state_valid(sc, to)) { ok = 0; goto done; }
    {
        double steps_d = ceil(step_measure(sp, resolution, from, to) * invStep);
        size_t steps = (size_t)steps_d;
        if (steps < 2) goto done;
        double delta = 1.0 / (double)steps;
        size_t qmin[DMV_QUEUE], qmax[DMV_QUEUE];
        qmin[0] = 1; qmax[0] = steps - 1;
        size_t qs = 0, qe = 1;
        while (qs != qe) {
            size_t mn = qmin[qs % DMV_QUEUE], mx = qmax[qs % DMV_QUEUE];
            ++qs;
            if (mn == mx) {
                orc_interpolate(sp, from, to, (double)mn * delta, q); ++cnt;
                if (!state_valid(sc, q)) { ok = 0; goto done; }
            } else if (qe + 2 < qs + DMV_QUEUE) {
                size_t mid = (mn + mx) / 2;
                orc_interpolate(sp, from, to, (double)mid * delta, q); ++cnt;
                if (!state_valid(sc, q)) { ok = 0; goto done; }
                if (mn < mid) { qmin[qe % DMV_QUEUE] = mn; qmax[qe % DMV_QUEUE] = mid - 1; ++qe; }
                if (mid < mx) { qmin[qe % DMV_QUEUE] = mid + 1; qmax[qe % DMV_QUEUE] = mx; ++qe; }
            } else {
                for (size_t i = mn; i <= mx; ++i) {
                    orc_interpolate(sp, from, to, (double)i * delta, q); ++cnt;
                    if (!state_valid(sc, q)) { ok = 0; goto done; }
                }
            }
        }
    }
done:
    if (nsamples) *nsamples = cnt;
    return ok;
}

void orc_valid_edges(const orc_scene* sc, const orc_space* sp, const double* a, const double* b,
                     int64_t n, double step, int resolution, uint8_t* out, int64_t* samples,
                     int nthreads) {
    int D = sp->dim;
    double inv = 1.0 / step;
    int64_t total = 0;
    if (sc->kind == 2) get_env_bvh(sc);
#pragma omp parallel for schedule(dynamic, 16) reduction(+:total) num_threads(nthreads_or_default(nthreads))
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        out[i] = (uint8_t)dmv_edge(sc, sp, a + i * D, b + i * D, inv, resolution, &c);
        total += c;
    }
    if (samples) *samples = total;
}

/* ------------------------------------------------------------------ */
/* Wavefront planner, restated for the checker.
 *
 * The reference's worker loop (src/mpt/impl/prrt/prrt.hpp:358-452) run as the
 * GPU planner runs it: wavefronts of W samples drawn from Philox4x32-10
 * (Salmon, Moraes, Dror, Shaw, SC'11: round function and constants as
 * published) addressed by (sample, wavefront, block); every sample of a
 * wavefront sees the tree as it stood before the wavefront; accepted samples
 * are appended in sample order.  Per sample: goal with probability goal_bias
 * until the first solution (:363-389), nearest (exact, lowest id), skip when
 * d == 0 (:425), steer to range (:430-434), valid + link through the DMV
 * (:439-442), GoalState test (:443-445), insert with parent (:447). */
static void orc_philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

double orc_uniform(uint64_t seed, uint32_t i, uint32_t w, uint32_t j) {
    uint32_t c[4] = {i, w, j >> 1, 0x6d707467u};
    orc_philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    uint32_t a = (j & 1) ? c[2] : c[0], b = (j & 1) ? c[3] : c[1];
    uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return (double)m * (1.0 / 9007199254740992.0);
}

/* goal_index: the one sample of this wavefront that is the goal (the lowest
 * index whose bias draw hits), or -1 */
static void plan_sample(const orc_space* sp, const orc_plan_params* pp, const double* lo, const double* hi,
                        const double* goal, int goal_index, uint32_t i, uint32_t w, double* q) {
    int D = sp->dim;
    if (goal && (int)i == goal_index) {
        for (int d = 0; d < D; ++d) q[d] = goal[d];
        return;
    }
    if (sp->metric == ORC_SO3 || sp->metric == ORC_SE3) {
        /* Shoemake uniform rotation (src/mpt/impl/uniform_sampler_so3.hpp:55-68) */
        double a = orc_uniform(pp->seed, i, w, 0);
        double b = TWO_PI * orc_uniform(pp->seed, i, w, 1);
        double c = TWO_PI * orc_uniform(pp->seed, i, w, 2);
        double s1 = sqrt(1.0 - a), s2 = sqrt(a), sb, cb, sc, cc;
        mptg_sincos(b, &sb, &cb);
        mptg_sincos(c, &sc, &cc);
        q[0] = s1 * sb; q[1] = s1 * cb; q[2] = s2 * sc; q[3] = s2 * cc;
        for (int d = 4; d < D; ++d) q[d] = lo[d] + (hi[d] - lo[d]) * orc_uniform(pp->seed, i, w, (uint32_t)(d - 1));
    } else if (sp->metric == ORC_SO2) {
        for (int d = 0; d < D; ++d) q[d] = -PI + TWO_PI * orc_uniform(pp->seed, i, w, (uint32_t)d);
    } else {
        for (int d = 0; d < D; ++d) q[d] = lo[d] + (hi[d] - lo[d]) * orc_uniform(pp->seed, i, w, (uint32_t)d);
    }
}

/* Sample i of wavefront w of the planners' sample stream, without goal bias
 * (plan_sample); lets the reference's one-sample-at-a-time planners be fed
 * the same states in the same order. */
void orc_sample_state(const orc_space* sp, const orc_plan_params* pp, const double* lo, const double* hi,
                      uint32_t i, uint32_t w, double* q) {
    plan_sample(sp, pp, lo, hi, NULL, -1, i, w, q);
}

/* Nearest-neighbour search of the replays: 0 the brute-force scan (the
 * definition), 1 the exact kd-tree above built over the tree's states once
 * per wavefront -- the same (distance, lowest id) answer -- or 2 the kd-tree
 * up to 7 dimensions and the scan above (where a per-wavefront kd-tree does
 * not pay), for CPU timing runs of the planner. */
static int g_plan_kd = 0;
void orc_set_plan_nn(int mode) { g_plan_kd = mode; }

/* One wavefront's candidates (prrt.hpp:411-442): sample i, its nearest tree
 * node par[i] among the first n states, the steered new state nw[i] and
 * ok[i] = valid(new) && link(near, new), all against the tree as it stood
 * before the wavefront. */
static void plan_wave(const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp, const double* lo,
                      const double* hi, const double* goal, int goal_index, int w, double range, double inv,
                      const double* states, int64_t n, double* nw, int32_t* par, uint8_t* ok, int nthreads) {
    const int D = sp->dim, W = pp->wavefront;
    const int use_kd = g_plan_kd == 1 || (g_plan_kd == 2 && D <= 7);
    kd_tree* kd = (use_kd && n > 0) ? (kd_tree*)orc_kd_build(sp, states, n, 8) : NULL;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads_or_default(nthreads))
    for (int i = 0; i < W; ++i) {
        double s[16], a[16];
        plan_sample(sp, pp, lo, hi, goal, goal_index, (uint32_t)i, (uint32_t)w, s);
        double best = INFINITY;
        int32_t bi = -1;
        if (kd) {
            kd_result r = {INFINITY, INT32_MAX, 0};
            kd_search(kd, 0, s, &r);
            if (r.idx != INT32_MAX) { best = r.best; bi = r.idx; }
        } else {
            for (int64_t j = 0; j < n; ++j) {
                double dj = orc_distance(sp, s, states + j * D);
                if (dj < best || (bi < 0 && dj == best)) { best = dj; bi = (int32_t)j; }
            }
        }
        ok[i] = 0;
        if (bi < 0 || best == 0.0 || best != best) continue;
        for (int d = 0; d < D; ++d) a[d] = states[(int64_t)bi * D + d];
        double* q = nw + (size_t)i * D;
        if (best > range) orc_interpolate(sp, a, s, range / best, q);
        else for (int d = 0; d < D; ++d) q[d] = s[d];
        par[i] = bi;
        ok[i] = (uint8_t)dmv_edge(sc, sp, a, q, inv, pp->resolution, NULL);
    }
    if (kd) orc_kd_free(kd);
}

int64_t orc_plan(const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp, const double* lo,
                 const double* hi, const double* start, const double* goal, int max_waves, int stop_when_solved,
                 double* states, int32_t* parents, int32_t* goals, int64_t* ngoals, int nthreads) {
    int D = sp->dim;
    int W = pp->wavefront;
    double range = pp->range > 0 ? pp->range : INFINITY;
    double inv = 1.0 / pp->edge_step;
    int64_t n = 1, ng = 0;
    for (int d = 0; d < D; ++d) states[d] = start[d];
    parents[0] = -1;
    if (sc->kind == 2) get_env_bvh(sc);
    double* nw = (double*)malloc((size_t)W * D * sizeof(double));
    int32_t* par = (int32_t*)malloc((size_t)W * sizeof(int32_t));
    uint8_t* ok = (uint8_t*)malloc((size_t)W);
    for (int w = 0; w < max_waves; ++w) {
        if (stop_when_solved && ng > 0) break;
        if (n >= pp->max_nodes) break;
        /* at most one goal sample per wavefront: the lowest index whose bias
         * draw hits (the reference draws goal samples on one worker only) */
        int goal_index = -1;
        if (goal && ng == 0 && pp->goal_bias > 0)
            for (int i = 0; i < W; ++i)
                if (orc_uniform(pp->seed, (uint32_t)i, (uint32_t)w, 16) < pp->goal_bias) { goal_index = i; break; }
        plan_wave(sc, sp, pp, lo, hi, goal, goal_index, w, range, inv, states, n, nw, par, ok, nthreads);
        for (int i = 0; i < W && n < pp->max_nodes; ++i) {
            if (!ok[i]) continue;
            for (int d = 0; d < D; ++d) states[n * D + d] = nw[(size_t)i * D + d];
            parents[n] = par[i];
            if (goal && orc_distance(sp, nw + (size_t)i * D, goal) <= pp->goal_radius) goals[ng++] = (int32_t)n;
            ++n;
        }
    }
    free(nw); free(par); free(ok);
    *ngoals = ng;
    return n;
}

/* ------------------------------------------------------------------ */
/* Wavefront PRRT*: the worker's addSample of
 * src/mpt/impl/prrt_star/prrt_star.hpp:505-657 with the neighbourhood of
 * src/mpt/impl/rrg_rewire_neighbors.hpp:47-66, restated for wavefronts.
 * Per wavefront, against the tree as it stood before it:
 *  1. the PRRT candidates (plan_wave), accepted in sample order up to the
 *     node budget;
 *  2. k = ceil(f e (1 + 1/dim) ln(n0 + 1)) (at most 64 and n0) nearest old
 *     nodes of each new state, sorted by (distance, id);
 *  3. choose parent: the key of a neighbour is (cost + d, d, id); near keeps
 *     (cost[near] + d(near, new), d(near, new), near); the parent is the
 *     smallest key among near and the neighbours whose key is below near's
 *     and whose link(neighbour, new) is valid;
 *  4. insert the new nodes (ids n0 + a in acceptance order) with that parent;
 *  5. rewire: every neighbour whose key is above the chosen parent's (the
 *     ones the reference's sorted loop did not reach) with
 *     cost(new) + d < cost(neighbour) and a valid link(new, neighbour)
 *     proposes the new node as its parent; each neighbour takes the proposal
 *     with the smallest (cost, new id);
 *  6. every cost is recomputed from the edge lengths by pointer jumping:
 *     s <- elen, a <- parent; ceil(log2(n + 1)) rounds of
 *     s[x] <- s[x] + s[a[x]], a[x] <- a[a[x]] (for a[x] >= 0).
 * Costs are therefore sums in pointer-jumping order, the definition the GPU
 * planner computes bit for bit. */
static int star_key_less(double c1, double d1, int32_t i1, double c2, double d2, int32_t i2) {
    if (c1 != c2) return c1 < c2;
    if (d1 != d2) return d1 < d2;
    return i1 < i2;
}

static void star_costs(const int32_t* parents, const double* elen, int64_t n, double* costs) {
    double* s = (double*)malloc((size_t)n * sizeof(double));
    double* s2 = (double*)malloc((size_t)n * sizeof(double));
    int32_t* a = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    int32_t* a2 = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    for (int64_t x = 0; x < n; ++x) { s[x] = elen[x]; a[x] = parents[x]; }
    int rounds = 0;
    while (((int64_t)1 << rounds) < n + 1) ++rounds;
    for (int r = 0; r < rounds; ++r) {
        for (int64_t x = 0; x < n; ++x) {
            if (a[x] >= 0) { s2[x] = s[x] + s[a[x]]; a2[x] = a[a[x]]; }
            else { s2[x] = s[x]; a2[x] = -1; }
        }
        double* ts = s; s = s2; s2 = ts;
        int32_t* ta = a; a = a2; a2 = ta;
    }
    for (int64_t x = 0; x < n; ++x) costs[x] = s[x];
    free(s); free(s2); free(a); free(a2);
}

int64_t orc_plan_star(const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp, const double* lo,
                      const double* hi, const double* start, const double* goal, int max_waves,
                      double rewire_factor, double* states, int32_t* parents, double* costs, int32_t* goals,
                      int64_t* ngoals, int64_t* rewires, int nthreads) {
    const int D = sp->dim, W = pp->wavefront;
    const double range = pp->range > 0 ? pp->range : INFINITY;
    const double inv = 1.0 / pp->edge_step;
    int64_t n = 1, ng = 0, nrw = 0;
    for (int d = 0; d < D; ++d) states[d] = start[d];
    parents[0] = -1;
    costs[0] = 0.0;
    if (sc->kind == 2) get_env_bvh(sc);
    double* elen = (double*)malloc((size_t)pp->max_nodes * sizeof(double));
    elen[0] = 0.0;
    double* nw = (double*)malloc((size_t)W * D * sizeof(double));
    int32_t* par = (int32_t*)malloc((size_t)W * sizeof(int32_t));
    uint8_t* ok = (uint8_t*)malloc((size_t)W);
    int32_t* acc = (int32_t*)malloc((size_t)W * sizeof(int32_t));
    double* qa = (double*)malloc((size_t)W * D * sizeof(double));
    int32_t* ki = (int32_t*)malloc((size_t)W * 64 * sizeof(int32_t));
    double* kd = (double*)malloc((size_t)W * 64 * sizeof(double));
    int32_t* cpar = (int32_t*)malloc((size_t)W * sizeof(int32_t));
    double* ccost = (double*)malloc((size_t)W * sizeof(double));
    double* celen = (double*)malloc((size_t)W * sizeof(double));
    uint8_t* rok = (uint8_t*)malloc((size_t)W * 64);
    double* bestc = (double*)malloc((size_t)pp->max_nodes * sizeof(double));
    int32_t* besta = (int32_t*)malloc((size_t)pp->max_nodes * sizeof(int32_t));
    for (int w = 0; w < max_waves; ++w) {
        if (n >= pp->max_nodes) break;
        int goal_index = -1;
        if (goal && ng == 0 && pp->goal_bias > 0)
            for (int i = 0; i < W; ++i)
                if (orc_uniform(pp->seed, (uint32_t)i, (uint32_t)w, 16) < pp->goal_bias) { goal_index = i; break; }
        plan_wave(sc, sp, pp, lo, hi, goal, goal_index, w, range, inv, states, n, nw, par, ok, nthreads);
        int A = 0;
        for (int i = 0; i < W && n + A < pp->max_nodes; ++i)
            if (ok[i]) acc[A++] = i;
        if (A == 0) continue;
        const int64_t n0 = n;
        int k = (int)ceil(rewire_factor * 2.718281828459045 * (1.0 + 1.0 / D) * log((double)n0 + 1.0));
        if (k > 64) k = 64;
        if (k > n0) k = (int)n0;
        if (k < 1) k = 1;
        for (int a = 0; a < A; ++a)
            for (int d = 0; d < D; ++d) qa[(size_t)a * D + d] = nw[(size_t)acc[a] * D + d];
        orc_knn_brute(sp, states, n0, qa, A, k, ki, kd, nthreads);
        /* 3. choose parent */
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads_or_default(nthreads))
        for (int a = 0; a < A; ++a) {
            const double* q = qa + (size_t)a * D;
            const int32_t near = par[acc[a]];
            const double dn = orc_distance(sp, states + (int64_t)near * D, q);
            const double cn = costs[near] + dn;
            int32_t bp = near;
            double bc = cn, bd = dn;
            for (int j = 0; j < k; ++j) {
                const int32_t nb = ki[a * k + j];
                if (nb < 0 || nb == near) continue;
                const double dj = kd[a * k + j], cj = costs[nb] + dj;
                if (!star_key_less(cj, dj, nb, cn, dn, near)) continue;
                if (!star_key_less(cj, dj, nb, bc, bd, bp)) continue;
                if (dmv_edge(sc, sp, states + (int64_t)nb * D, q, inv, pp->resolution, NULL)) {
                    bp = nb; bc = cj; bd = dj;
                }
            }
            cpar[a] = bp; ccost[a] = bc; celen[a] = bd;
        }
        /* 4. insert */
        for (int a = 0; a < A; ++a) {
            for (int d = 0; d < D; ++d) states[(n0 + a) * D + d] = qa[(size_t)a * D + d];
            parents[n0 + a] = cpar[a];
            elen[n0 + a] = celen[a];
            if (goal && orc_distance(sp, qa + (size_t)a * D, goal) <= pp->goal_radius) goals[ng++] = (int32_t)(n0 + a);
        }
        n = n0 + A;
        /* 5. rewire proposals (old costs), then the best proposal per neighbour */
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads_or_default(nthreads))
        for (int a = 0; a < A; ++a) {
            const double* q = qa + (size_t)a * D;
            for (int j = 0; j < k; ++j) {
                const int32_t nb = ki[a * k + j];
                rok[a * k + j] = 0;
                if (nb < 0) continue;
                const double dj = kd[a * k + j], cj = costs[nb] + dj;
                if (!star_key_less(ccost[a], celen[a], cpar[a], cj, dj, nb)) continue;  /* reached by step 3 */
                const double nc = ccost[a] + dj;
                if (!(nc < costs[nb])) continue;
                rok[a * k + j] = (uint8_t)dmv_edge(sc, sp, q, states + (int64_t)nb * D, inv, pp->resolution, NULL);
            }
        }
        for (int a = 0; a < A; ++a)
            for (int j = 0; j < k; ++j)
                if (rok[a * k + j]) { bestc[ki[a * k + j]] = INFINITY; besta[ki[a * k + j]] = -1; }
        for (int a = 0; a < A; ++a)
            for (int j = 0; j < k; ++j) {
                if (!rok[a * k + j]) continue;
                const int32_t nb = ki[a * k + j];
                const double nc = ccost[a] + kd[a * k + j];
                if (besta[nb] < 0 || nc < bestc[nb] || (nc == bestc[nb] && a < besta[nb])) { bestc[nb] = nc; besta[nb] = a; }
            }
        for (int a = 0; a < A; ++a)
            for (int j = 0; j < k; ++j) {
                const int32_t nb = ki[a * k + j];
                if (!rok[a * k + j] || besta[nb] != a) continue;
                parents[nb] = (int32_t)(n0 + a);
                elen[nb] = kd[a * k + j];
                besta[nb] = -2;  /* applied */
                ++nrw;
            }
        /* 6. costs */
        star_costs(parents, elen, n, costs);
    }
    free(elen); free(nw); free(par); free(ok); free(acc); free(qa); free(ki); free(kd);
    free(cpar); free(ccost); free(celen); free(rok); free(bestc); free(besta);
    *ngoals = ng;
    *rewires = nrw;
    return n;
}

/* ------------------------------------------------------------------ */
/* PPRM roadmap: the worker's addSample of src/mpt/impl/pprm/pprm.hpp:298-339
 * applied one sample at a time, in the sample order of the wavefront
 * planner's stream (no goal samples):
 *   valid(q) (:299-300); k = ceil((e + e/dim) ln(n + 1)) (:302-303, kRRG_ of
 *   :145; at most 64 and n) nearest of the n nodes by (distance, id); skip
 *   when the nearest is closer than DBL_EPSILON (:306-308); goal flag from the
 *   caller or GoalState(radius) (:312-316); for each neighbour in order, an
 *   edge (q, nbr, d) when link(q, nbr) is valid (:325-334) and a union of the
 *   components (:341-363, whose flags OR together); solved once a union
 *   leaves a component holding a start and a goal (:332-333, component.hpp
 *   isSolution).  The roadmap is then a pure function of the sample
 *   sequence, which is what the wavefront GPU planner reproduces. */
static int32_t uf_root(int32_t* uf, int32_t x) {
    while (uf[x] != x) { uf[x] = uf[uf[x]]; x = uf[x]; }
    return x;
}

int orc_prm_k(int64_t n, int dim) {
    if (n <= 0) return 0;
    const double e = 2.718281828459045, kRRG = e + e / dim;
    double kd = ceil(kRRG * log((double)n + 1.0));
    int k = kd > 64.0 ? 64 : (int)kd;
    if (k > n) k = (int)n;
    return k < 1 ? 1 : k;
}

typedef struct {
    const orc_scene* sc; const orc_space* sp; const orc_plan_params* pp; const double* goal;
    double* states; uint8_t* flags; int32_t* uf; uint8_t* cflag; int64_t n;
    int32_t* efrom; int32_t* eto; double* edist; int64_t ne, ecap;
    int64_t* stats; double* kd; int32_t* ki;
} prm_state;

static int32_t prm_add(prm_state* P, const double* q, int flag) {
    const int D = P->sp->dim;
    P->stats[1]++;
    if (!state_valid(P->sc, q)) return -1;
    P->stats[2]++;
    const int64_t n = P->n;
    const int k = orc_prm_k(n, D);
    int cnt = 0;
    for (int64_t j = 0; j < n; ++j) {
        double dj = orc_distance(P->sp, q, P->states + j * D);
        if (!(dj == dj)) continue;
        if (cnt == k) {
            if (!(dj < P->kd[k - 1])) continue; /* ids ascend: a tie keeps the earlier id */
            cnt--;
        }
        int pos = cnt;
        while (pos > 0 && P->kd[pos - 1] > dj) { P->kd[pos] = P->kd[pos - 1]; P->ki[pos] = P->ki[pos - 1]; --pos; }
        P->kd[pos] = dj;
        P->ki[pos] = (int32_t)j;
        cnt++;
    }
    if (cnt > 0 && P->kd[0] < DBL_EPSILON) { P->stats[3]++; return -1; }
    if (n >= P->pp->max_nodes) return -1;
    int isgoal = (flag & 2) || (P->goal && orc_distance(P->sp, q, P->goal) <= P->pp->goal_radius);
    uint8_t f = (uint8_t)(flag | (isgoal ? 2 : 0));
    for (int d = 0; d < D; ++d) P->states[n * D + d] = q[d];
    P->flags[n] = f;
    P->uf[n] = (int32_t)n;
    P->cflag[n] = f;
    P->n = n + 1;
    if (isgoal) P->stats[6]++;
    const double inv = 1.0 / P->pp->edge_step;
    for (int t = 0; t < cnt; ++t) {
        const int32_t nb = P->ki[t];
        P->stats[4]++;
        if (!dmv_edge(P->sc, P->sp, q, P->states + (int64_t)nb * D, inv, P->pp->resolution, NULL)) continue;
        if (P->ne < P->ecap) {
            P->efrom[P->ne] = (int32_t)n; P->eto[P->ne] = nb; P->edist[P->ne] = P->kd[t];
        }
        P->ne++;
        int32_t a = uf_root(P->uf, (int32_t)n), b = uf_root(P->uf, nb);
        if (a != b) {
            if (a > b) { int32_t x = a; a = b; b = x; }
            P->uf[b] = a;
            P->cflag[a] |= P->cflag[b];
        }
        if (P->cflag[a] == 3) P->stats[7] = 1;
    }
    return (int32_t)n;
}

static int edge_cmp(const void* x, const void* y) {
    const int64_t* a = (const int64_t*)x; const int64_t* b = (const int64_t*)y;
    return a[0] < b[0] ? -1 : (a[0] > b[0] ? 1 : 0);
}

/* Dijkstra from the start nodes (distance 0, in id order) to the first goal
 * node settled; heap order (distance, id); adjacency in (from, to) edge order,
 * each edge listed at both ends; a node's predecessor changes only on a strict
 * improvement.  Returns the path length (0 when no goal is reachable). */
int64_t orc_prm_dijkstra(int64_t n, const uint8_t* flags, int64_t ne, const int32_t* efrom, const int32_t* eto,
                         const double* edist, int32_t* path, double* cost) {
    int64_t* key = (int64_t*)malloc((size_t)(ne > 0 ? ne : 1) * 2 * sizeof(int64_t));
    for (int64_t e = 0; e < ne; ++e) { key[2 * e] = ((int64_t)efrom[e] << 32) | (uint32_t)eto[e]; key[2 * e + 1] = e; }
    qsort(key, (size_t)ne, 2 * sizeof(int64_t), edge_cmp);
    int64_t* deg = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    for (int64_t e = 0; e < ne; ++e) { deg[efrom[e] + 1]++; deg[eto[e] + 1]++; }
    for (int64_t v = 0; v < n; ++v) deg[v + 1] += deg[v];
    int64_t* fill = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    memcpy(fill, deg, (size_t)n * sizeof(int64_t));
    int32_t* adj = (int32_t*)malloc((size_t)(2 * ne > 0 ? 2 * ne : 1) * sizeof(int32_t));
    double* adjw = (double*)malloc((size_t)(2 * ne > 0 ? 2 * ne : 1) * sizeof(double));
    for (int64_t s = 0; s < ne; ++s) {
        int64_t e = key[2 * s + 1];
        int32_t a = efrom[e], b = eto[e];
        adj[fill[a]] = b; adjw[fill[a]++] = edist[e];
        adj[fill[b]] = a; adjw[fill[b]++] = edist[e];
    }
    double* dist = (double*)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
    int32_t* pred = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    uint8_t* done = (uint8_t*)calloc((size_t)n + 1, 1);
    /* binary heap of (dist, id), lazy deletion */
    int64_t hcap = 2 * ne + n + 1, hn = 0;
    double* hd = (double*)malloc((size_t)hcap * sizeof(double));
    int32_t* hi = (int32_t*)malloc((size_t)hcap * sizeof(int32_t));
#define HLESS(i, j) (hd[i] < hd[j] || (hd[i] == hd[j] && hi[i] < hi[j]))
#define HSWAP(i, j) do { double td = hd[i]; hd[i] = hd[j]; hd[j] = td; int32_t ti = hi[i]; hi[i] = hi[j]; hi[j] = ti; } while (0)
    for (int64_t v = 0; v < n; ++v) { dist[v] = INFINITY; pred[v] = -1; }
    for (int64_t v = 0; v < n; ++v)
        if (flags[v] & 1) {
            dist[v] = 0.0;
            int64_t c = hn++; hd[c] = 0.0; hi[c] = (int32_t)v;
            while (c > 0 && HLESS(c, (c - 1) / 2)) { HSWAP(c, (c - 1) / 2); c = (c - 1) / 2; }
        }
    int32_t found = -1;
    while (hn > 0) {
        double du = hd[0]; int32_t u = hi[0];
        hn--; hd[0] = hd[hn]; hi[0] = hi[hn];
        for (int64_t c = 0;;) {
            int64_t l = 2 * c + 1, r = l + 1, m = c;
            if (l < hn && HLESS(l, m)) m = l;
            if (r < hn && HLESS(r, m)) m = r;
            if (m == c) break;
            HSWAP(c, m); c = m;
        }
        if (done[u] || du != dist[u]) continue;
        done[u] = 1;
        if (flags[u] & 2) { found = u; break; }
        for (int64_t t = deg[u]; t < deg[u + 1]; ++t) {
            int32_t v = adj[t];
            double nd = du + adjw[t];
            if (nd < dist[v]) {
                dist[v] = nd; pred[v] = u;
                int64_t c = hn++; hd[c] = nd; hi[c] = v;
                while (c > 0 && HLESS(c, (c - 1) / 2)) { HSWAP(c, (c - 1) / 2); c = (c - 1) / 2; }
            }
        }
    }
#undef HLESS
#undef HSWAP
    int64_t len = 0;
    *cost = INFINITY;
    if (found >= 0) {
        *cost = dist[found];
        for (int32_t v = found; v >= 0; v = pred[v]) len++;
        if (path) {
            int64_t i = len;
            for (int32_t v = found; v >= 0; v = pred[v]) path[--i] = v;
        }
    }
    free(key); free(deg); free(fill); free(adj); free(adjw); free(dist); free(pred); free(done); free(hd); free(hi);
    return len;
}

int64_t orc_prm(const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp, const double* lo,
                const double* hi, const double* goal, const double* starts, int nstarts, const double* goals,
                int ngoals, int max_waves, int stop_when_solved, double* states, uint8_t* flags, int64_t* ne,
                int32_t* efrom, int32_t* eto, double* edist, int64_t ecap, int64_t* stats) {
    const int D = sp->dim, W = pp->wavefront;
    if (sc->kind == 2) get_env_bvh(sc);
    prm_state P;
    memset(&P, 0, sizeof(P));
    P.sc = sc; P.sp = sp; P.pp = pp; P.goal = goal;
    P.states = states; P.flags = flags;
    P.uf = (int32_t*)malloc((size_t)pp->max_nodes * sizeof(int32_t));
    P.cflag = (uint8_t*)malloc((size_t)pp->max_nodes);
    P.efrom = efrom; P.eto = eto; P.edist = edist; P.ecap = ecap;
    P.stats = stats;
    P.kd = (double*)malloc(64 * sizeof(double));
    P.ki = (int32_t*)malloc(64 * sizeof(int32_t));
    for (int i = 0; i < 8; ++i) stats[i] = 0;
    for (int i = 0; i < nstarts; ++i) prm_add(&P, starts + (size_t)i * D, 1);
    for (int i = 0; i < ngoals; ++i) prm_add(&P, goals + (size_t)i * D, 2);
    double* q = (double*)malloc((size_t)D * sizeof(double));
    for (int w = 0; w < max_waves; ++w) {
        if (stop_when_solved && stats[7]) break;
        if (P.n >= pp->max_nodes) break;
        for (int i = 0; i < W; ++i) {
            plan_sample(sp, pp, lo, hi, NULL, -1, (uint32_t)i, (uint32_t)w, q);
            prm_add(&P, q, 0);
        }
        stats[0]++;
    }
    stats[5] = P.ne;
    *ne = P.ne;
    free(q); free(P.uf); free(P.cflag); free(P.kd); free(P.ki);
    return P.n;
}
