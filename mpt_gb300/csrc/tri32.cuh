// tri32.cuh - certified FP32 verdicts on triangle pairs, shared by the mesh
// kernels (mesh.cu) and a host test against the oracle's FP64 Moller test
// (tests/cpp/tri32_check.cpp).  Every verdict is one the FP64 test
// (tri_tri64 in mesh.cu, orc_tri_tri in the oracle) is certain to share.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define MPTG_HD __host__ __device__ __forceinline__
#else
#define MPTG_HD inline
#endif
#ifndef U32
#define U32 5.9604645e-8f  // 2^-24, unit roundoff of FP32
#endif

// True when the plane of triangle U certainly separates the points V0..V2:
// every d_i = n.(V_i - U0), n = (U1 - U0) x (U2 - U0), lies beyond its error
// bound with one sign.  The FP32 coordinates are within eps (per coordinate)
// of the FP64 coordinates tri_tri64 uses, and X bounds every |coordinate|.
// Bound (2-norms bounded by the computed L1 norms): the differences move by
// a = 4 eps + u|.| (perturbation plus rounding), the normal by
// nu = |e1| a2 + |e2| a1 + a1 a2 + 4u|e1||e2| (perturbation plus the cross
// product's rounding), each d by |n| w + |w| nu + 2 nu w + 3u|n||w| (the dot
// product's rounding), plus the FP64 test's own rounding (far below
// 1e-13 (|e1||e2| + |n|)(X + 1)).  Then every FP64 distance in tri_tri64 has
// the FP32 sign and none is 0, so the test returns false at this plane.
// The three signed distances d[i] = n.(V_i - U0) and their common bound E.
MPTG_HD float plane_dists32(const float* U, const float* V, float eps, float X, float* dv, float* nout = nullptr,
                            float* nuout = nullptr) {
    const float e1x = U[3] - U[0], e1y = U[4] - U[1], e1z = U[5] - U[2];
    const float e2x = U[6] - U[0], e2y = U[7] - U[1], e2z = U[8] - U[2];
    const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    const float l1 = fabsf(e1x) + fabsf(e1y) + fabsf(e1z), l2 = fabsf(e2x) + fabsf(e2y) + fabsf(e2z);
    const float ln = fabsf(nx) + fabsf(ny) + fabsf(nz);
    const float a1 = 4.f * eps + U32 * l1, a2 = 4.f * eps + U32 * l2;
    const float nu = l1 * a2 + l2 * a1 + a1 * a2 + 4.f * U32 * l1 * l2;
    float lw = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float wx = V[3 * i] - U[0], wy = V[3 * i + 1] - U[1], wz = V[3 * i + 2] - U[2];
        dv[i] = fmaf(nx, wx, fmaf(ny, wy, nz * wz));
        lw = fmaxf(lw, fabsf(wx) + fabsf(wy) + fabsf(wz));
    }
    const float w = 4.f * eps + U32 * lw;
    if (nout) {
        nout[0] = nx;
        nout[1] = ny;
        nout[2] = nz;
        // the FP64 normal's own rounding on top of nu
        *nuout = nu + 1e-13f * l1 * l2;
    }
    return ((ln + nu) * w + (lw + w) * nu + nu * w + 3.f * U32 * ln * lw +
            1e-13f * (l1 * l2 + ln) * (X + 1.f)) * 1.01f + 1e-30f;
}

MPTG_HD bool plane_separates32(const float* U, const float* V, float eps, float X) {
    float d[3];
    const float E = plane_dists32(U, V, eps, X, d);
    return fminf(d[0], fminf(d[1], d[2])) > E || fmaxf(d[0], fmaxf(d[1], d[2])) < -E;
}

// orient3d(p, q, a, b) = (q - p) . ((a - p) x (b - p)) in FP32, and in *err a
// bound on its distance from the exact value at the FP64 coordinates (every
// FP32 coordinate within eps of its FP64 counterpart).  Each difference is
// off by at most dl = 2 eps + u max|.| per component (2-norm <= 2 dl); with
// L1 norms la, lb, lc (grown by 3 dl to cover the exact vectors) the
// perturbation moves the determinant by <= 2dl(lb lc + la lc + la lb) +
// 4dl^2(la + lb + lc) + 8dl^3, and the FP32 cross and dot products round by
// <= 5u la lb lc (6u taken).
MPTG_HD float orient3d32(const float* p, const float* q, const float* a, const float* b, float eps,
                                            float* err) {
    const float ax = q[0] - p[0], ay = q[1] - p[1], az = q[2] - p[2];
    const float bx = a[0] - p[0], by = a[1] - p[1], bz = a[2] - p[2];
    const float cx = b[0] - p[0], cy = b[1] - p[1], cz = b[2] - p[2];
    const float x = by * cz - bz * cy, y = bz * cx - bx * cz, z = bx * cy - by * cx;
    const float det = fmaf(ax, x, fmaf(ay, y, az * z));
    float la = fabsf(ax) + fabsf(ay) + fabsf(az), lb = fabsf(bx) + fabsf(by) + fabsf(bz);
    float lc = fabsf(cx) + fabsf(cy) + fabsf(cz);
    const float dl = 2.f * eps + U32 * fmaxf(la, fmaxf(lb, lc));
    la += 3.f * dl;
    lb += 3.f * dl;
    lc += 3.f * dl;
    *err = (2.f * dl * (lb * lc + la * lc + la * lb) + 4.f * dl * dl * (la + lb + lc) + 8.f * dl * dl * dl +
            6.f * U32 * la * lb * lc) * 1.01f + 1e-30f;
    return det;
}

// The segment PQ, whose ends lie strictly on opposite sides of triangle T's
// plane, passes through T's interior: the three orientations of PQ against
// T's edges are certainly nonzero and of one sign.
MPTG_HD bool pierces32(const float* P, const float* Q, const float* T, float eps) {
    float e0, e1, e2;
    const float s0 = orient3d32(P, Q, T, T + 3, eps, &e0);
    const float s1 = orient3d32(P, Q, T + 3, T + 6, eps, &e1);
    const float s2 = orient3d32(P, Q, T + 6, T, eps, &e2);
    return (s0 > e0 && s1 > e1 && s2 > e2) || (s0 < -e0 && s1 < -e1 && s2 < -e2);
}

// The interval that tri_interval computes along one coordinate axis for a
// triangle whose vertex coordinates on that axis are c[0..2] and whose
// distances d[0..2] to the other triangle's plane all lie beyond their bound
// E with certain signs: the points where the two edges from the lone vertex
// cross the plane, c_a + (c_b - c_a) d_a / (d_a - d_b).  [*lo, *hi] holds
// the FP64 endpoints: each FP32 endpoint is within
//   eps (coordinates) + |c_b - c_a| E / (S - 2E) (the ratio, S = |d_a| + |d_b|:
//   its gradient has L1 norm 1 / S, and S stays above S - 2E over the
//   perturbation) + 4u (|c_a| + |c_b - c_a|) (FP32 rounding)
// of the FP64 one, whose own rounding is far below 1e-13 (X + 1).
MPTG_HD void interval32(float c0, float c1, float c2, const float* d, float E, float eps, float X, float* lo,
                        float* hi) {
    const bool p0 = d[0] > 0.f, p1 = d[1] > 0.f, p2 = d[2] > 0.f;
    float ca, cb0, cb1, da, db0, db1;
    if (p0 == p1) { ca = c2; da = d[2]; cb0 = c0; db0 = d[0]; cb1 = c1; db1 = d[1]; }
    else if (p0 == p2) { ca = c1; da = d[1]; cb0 = c0; db0 = d[0]; cb1 = c2; db1 = d[2]; }
    else { ca = c0; da = d[0]; cb0 = c1; db0 = d[1]; cb1 = c2; db1 = d[2]; }
    float l = INFINITY, h = -INFINITY;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const float cb = j ? cb1 : cb0, db = j ? db1 : db0;
        const float dc = cb - ca;
        const float S = fabsf(da) + fabsf(db);
        const float t = fmaf(dc, da / (da - db), ca);
        const float et = (eps + (fabsf(dc) + 2.f * eps) * E / (S - 2.f * E) + 4.f * U32 * (fabsf(ca) + fabsf(dc)) +
                          1e-13f * (X + 1.f)) * 1.01f;
        l = fminf(l, t - et);
        h = fmaxf(h, t + et);
    }
    *lo = l;
    *hi = h;
}

// True when the two triangles' intervals on the planes' common line are
// certainly apart on every axis that tri_tri64 may project them onto: it
// takes the axis of the largest |component| of D = N1 x N2 in FP64, and the
// FP32 D is within eD of it per component, so every axis whose FP32
// |component| comes within 2 eD of the largest is checked.  All six plane
// distances must already lie beyond their bounds (certain signs).
MPTG_HD bool intervals_apart32(const float* V, const float* U, const float* dv, float Ev, const float* du, float Eu,
                               const float* nv, float nuv, const float* nu_, float nuu, float eps, float X) {
    const float D[3] = {nv[1] * nu_[2] - nv[2] * nu_[1], nv[2] * nu_[0] - nv[0] * nu_[2],
                        nv[0] * nu_[1] - nv[1] * nu_[0]};
    const float lv = fabsf(nv[0]) + fabsf(nv[1]) + fabsf(nv[2]), lu = fabsf(nu_[0]) + fabsf(nu_[1]) + fabsf(nu_[2]);
    // per component: 2 (|dv| |u| + |v| |du| + |dv| |du|) perturbation, 4u |v| |u| FP32 rounding,
    // 1e-13 |v| |u| for FP64's own cross product
    const float eD = (2.f * (nuv * lu + lv * nuu + nuv * nuu) + (4.f * U32 + 1e-13f) * lv * lu) * 1.01f;
    const float m = fmaxf(fabsf(D[0]), fmaxf(fabsf(D[1]), fabsf(D[2])));
    if (!(m >= 0.f)) return false;  // NaN: no verdict
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (!(fabsf(D[k]) >= m - 2.f * eD)) continue;
        float alo, ahi, blo, bhi;
        interval32(V[k], V[3 + k], V[6 + k], dv, Ev, eps, X, &alo, &ahi);
        interval32(U[k], U[3 + k], U[6 + k], du, Eu, eps, X, &blo, &bhi);
        if (!(ahi < blo || bhi < alo)) return false;
    }
    return true;
}

// FP32 verdict on a triangle pair that Moller's FP64 test (tri_tri64) is
// certain to share: -1 = separated (a plane separates the other triangle's
// vertices, or both straddle the other's plane and their intervals on the
// planes' common line are certainly apart: intervals_apart32), 1 =
// intersecting, 0 = undecided.
// Intersecting: every vertex of each triangle lies beyond its bound on a
// definite side of the other's plane, both triangles straddle the other's
// plane, and an edge of one crossing the other's plane certainly passes
// through the other's interior.  Then the FP64 coordinates describe
// triangles that cross along a segment of length far above FP64 rounding:
// the FP64 test sees the same signs, takes a non-degenerate interval branch,
// and finds the two intervals on the planes' common line overlapping.
MPTG_HD int tri_pair32(const float* V, const float* U, float eps, float X) {
    float dv[3], du[3], nU[3], nV[3], nuU, nuV;
    const float Ev = plane_dists32(U, V, eps, X, dv, nU, &nuU);  // V's vertices against U's plane
    if (fminf(dv[0], fminf(dv[1], dv[2])) > Ev || fmaxf(dv[0], fmaxf(dv[1], dv[2])) < -Ev) return -1;
    const float Eu = plane_dists32(V, U, eps, X, du, nV, &nuV);  // U's vertices against V's plane
    if (fminf(du[0], fminf(du[1], du[2])) > Eu || fmaxf(du[0], fmaxf(du[1], du[2])) < -Eu) return -1;
#pragma unroll
    for (int i = 0; i < 3; ++i)
        if (!(fabsf(dv[i]) > Ev) || !(fabsf(du[i]) > Eu)) return 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int j = i == 2 ? 0 : i + 1;
        if ((dv[i] > 0.f) != (dv[j] > 0.f) && pierces32(V + 3 * i, V + 3 * j, U, eps)) return 1;
        if ((du[i] > 0.f) != (du[j] > 0.f) && pierces32(U + 3 * i, U + 3 * j, V, eps)) return 1;
    }
    return intervals_apart32(V, U, dv, Ev, du, Eu, nV, nuV, nU, nuU, eps, X) ? -1 : 0;
}

