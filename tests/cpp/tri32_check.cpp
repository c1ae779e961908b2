// Host check of the certified FP32 triangle-pair verdicts (mpt_gb300/csrc/
// tri32.cuh) against the oracle's FP64 Moller test (orc_tri_tri).  Two
// families:
//  * random pairs at three scales, many of them touching, sharing a vertex
//    within 1e-9 or offset by 1e-7, with FP32 coordinates rounded from the
//    FP64 ones (eps = u max|x|);
//  * pairs as k_mesh_detail meets them: a robot triangle (robot frame, within
//    the unit ball) placed by a random rotation at a position up to 20 away,
//    in FP64 (R v + p) and in FP32 (fma(R32, v32, p32)), against a box-face
//    triangle (axis-aligned, a 1/7 grid cell) within 1e-6 .. 0.05 of it, with
//    the kernel's eps = max(6u(robot_l1 + |p|), u env_max).
// Every "separated" verdict must be a pair the FP64 test rejects and every
// "crossing" verdict one it accepts.  The undecided share (the pairs left to
// FP64 on the GPU) is printed.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../mpt_gb300/csrc/tri32.cuh"
extern "C" {
#include "../../oracle/oracle.h"
}

struct Tally {
    long pairs = 0, hits = 0, cross = 0, sep = 0, wrong = 0;
    void add(int r, int m) {
        ++pairs;
        hits += m;
        if (r == 1) { ++cross; wrong += !m; }
        if (r == -1) { ++sep; wrong += m; }
    }
    void print(const char* name) const {
        std::printf("%s: pairs %ld intersecting %ld certified-crossing %ld certified-separated %ld undecided %ld "
                    "wrong %ld\n", name, pairs, hits, cross, sep, pairs - cross - sep, wrong);
    }
};

static void random_pairs(long pairs, Tally& t) {
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    for (long it = 0; it < pairs; ++it) {
        double t1[9], t2[9];
        const double c[3] = {20 * u(rng) - 10, 20 * u(rng) - 10, 20 * u(rng) - 10};
        const double sc = it % 3 == 0 ? 1.0 : (it % 3 == 1 ? 0.3 : 0.05);
        for (int k = 0; k < 9; ++k) t1[k] = c[k % 3] + sc * (2 * u(rng) - 1);
        const double off = (it & 4) ? 1e-7 * (2 * u(rng) - 1) : 0.3 * sc * (2 * u(rng) - 1);
        for (int k = 0; k < 9; ++k) t2[k] = c[k % 3] + sc * (2 * u(rng) - 1) + off;
        if (it % 11 == 0)
            for (int k = 0; k < 3; ++k) t2[k] = t1[3 + k] + 1e-9 * (2 * u(rng) - 1);
        float V[9], U[9], X = 0.f;
        for (int k = 0; k < 9; ++k) {
            V[k] = (float)t1[k];
            U[k] = (float)t2[k];
            X = std::fmax(X, std::fmax(std::fabs(V[k]), std::fabs(U[k])));
        }
        t.add(tri_pair32(V, U, U32 * X * 1.01f, X), orc_tri_tri(t1, t2));
    }
}

static void mesh_pairs(long pairs, Tally& t) {
    std::mt19937_64 rng(11);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    const double cell = 1.0 / 7.0;
    for (long it = 0; it < pairs; ++it) {
        // rotation (the kernel's quaternion-to-matrix expressions) and position
        double q[4], qn = 0;
        for (int k = 0; k < 4; ++k) { q[k] = 2 * u(rng) - 1; qn += q[k] * q[k]; }
        qn = std::sqrt(qn);
        for (int k = 0; k < 4; ++k) q[k] /= qn;
        const double x = q[0], y = q[1], z = q[2], w = q[3];
        const double tx = 2 * x, ty = 2 * y, tz = 2 * z;
        const double twx = tx * w, twy = ty * w, twz = tz * w, txx = tx * x, txy = ty * x, txz = tz * x;
        const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
        const double R[9] = {1 - (tyy + tzz), txy - twz, txz + twy, txy + twz, 1 - (txx + tzz),
                             tyz - twx, txz - twy, tyz + twx, 1 - (txx + tyy)};
        const double P[3] = {20 * u(rng), 20 * u(rng), 20 * u(rng)};
        float R32[9], P32[3], pm = 0.f;
        for (int k = 0; k < 9; ++k) R32[k] = (float)R[k];
        for (int k = 0; k < 3; ++k) { P32[k] = (float)P[k]; pm = std::fmax(pm, std::fabs(P32[k])); }
        pm *= 1.f + 2.f * U32;
        // robot triangle near the unit sphere, side about 0.1, in FP32 robot coordinates
        double dir[3], dn = 0;
        for (int k = 0; k < 3; ++k) { dir[k] = 2 * u(rng) - 1; dn += dir[k] * dir[k]; }
        dn = std::sqrt(dn);
        const double rad = 0.5 + 0.45 * u(rng);
        float lt[9];
        double rl1 = 0;
        for (int v = 0; v < 3; ++v) {
            double l1 = 0;
            for (int k = 0; k < 3; ++k) {
                lt[3 * v + k] = (float)(rad * dir[k] / dn + 0.1 * (2 * u(rng) - 1));
                l1 += std::fabs((double)lt[3 * v + k]);
            }
            rl1 = std::fmax(rl1, l1);
        }
        double t1[9];
        float V[9];
        for (int v = 0; v < 3; ++v)
            for (int r = 0; r < 3; ++r) {
                t1[3 * v + r] = ((R[3 * r] * lt[3 * v] + R[3 * r + 1] * lt[3 * v + 1]) + R[3 * r + 2] * lt[3 * v + 2]) +
                                P[r];
                V[3 * v + r] = std::fmaf(R32[3 * r], lt[3 * v],
                                         std::fmaf(R32[3 * r + 1], lt[3 * v + 1],
                                                   std::fmaf(R32[3 * r + 2], lt[3 * v + 2], P32[r])));
            }
        // box-face triangle: plane ax = (a robot vertex's coordinate + offset), a grid cell around the
        // robot triangle's centroid
        const int ax = (int)(u(rng) * 3) % 3, a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
        const int vi = (int)(u(rng) * 3) % 3;
        const double off = (it & 1) ? 1e-6 * (2 * u(rng) - 1) : 0.05 * (2 * u(rng) - 1);
        const double plane = (double)(float)(t1[3 * vi + ax] + off);
        const double c1 = (t1[a1] + t1[3 + a1] + t1[6 + a1]) / 3, c2 = (t1[a2] + t1[3 + a2] + t1[6 + a2]) / 3;
        const double g1 = (std::floor(c1 / cell + (u(rng) - 0.5)) ) * cell, g2 = (std::floor(c2 / cell + (u(rng) - 0.5))) * cell;
        double t2[9];
        const double corner[3][2] = {{0, 0}, {1, 0}, {(it & 2) ? 1.0 : 0.0, 1}};
        for (int v = 0; v < 3; ++v) {
            t2[3 * v + ax] = plane;
            t2[3 * v + a1] = (double)(float)(g1 + corner[v][0] * cell);
            t2[3 * v + a2] = (double)(float)(g2 + corner[v][1] * cell);
        }
        float U[9], env_max = 0.f;
        for (int k = 0; k < 9; ++k) { U[k] = (float)t2[k]; env_max = std::fmax(env_max, std::fabs(U[k])); }
        const float robot_l1 = (float)rl1 * (1.f + 1e-6f) + 1e-6f;
        const float eps = std::fmax(6.f * U32 * (robot_l1 + pm), U32 * env_max) * 1.01f;
        const float X = std::fmax(env_max, robot_l1 + pm);
        t.add(tri_pair32(V, U, eps, X), orc_tri_tri(t1, t2));
    }
}

int main(int argc, char** argv) {
    const long pairs = argc > 1 ? std::atol(argv[1]) : 400000;
    Tally a, b;
    random_pairs(pairs, a);
    mesh_pairs(pairs, b);
    a.print("random");
    b.print("mesh");
    return a.wrong != 0 || b.wrong != 0 || a.cross == 0 || a.sep == 0 || b.sep == 0;
}
