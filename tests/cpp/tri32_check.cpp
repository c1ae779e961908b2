// Host check of the certified FP32 triangle-pair verdicts (mpt_gb300/csrc/
// tri32.cuh) against the oracle's FP64 Moller test (orc_tri_tri): random
// triangle pairs at three scales, many of them touching, sharing a vertex
// within 1e-9 or offset by 1e-7, with FP32 coordinates rounded from the FP64
// ones (eps = u max|x|).  Every "separated" verdict must be a pair the FP64
// test rejects and every "crossing" verdict one it accepts.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../../mpt_gb300/csrc/tri32.cuh"
extern "C" {
#include "../../oracle/oracle.h"
}

int main(int argc, char** argv) {
    const long pairs = argc > 1 ? std::atol(argv[1]) : 400000;
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    long hits = 0, cross = 0, sep = 0, wrong = 0;
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
        const int r = tri_pair32(V, U, U32 * X * 1.01f, X);
        const int m = orc_tri_tri(t1, t2);
        hits += m;
        if (r == 1) { ++cross; wrong += !m; }
        if (r == -1) { ++sep; wrong += m; }
    }
    std::printf("pairs %ld intersecting %ld certified-crossing %ld certified-separated %ld wrong %ld\n", pairs, hits,
                cross, sep, wrong);
    return wrong != 0 || cross == 0 || sep == 0;
}
