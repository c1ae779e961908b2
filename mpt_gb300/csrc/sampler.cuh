// sampler.cuh - the uniform state sampler of the wavefront planners: sample i
// of wavefront w is a pure function of (seed, i, w), drawn from the Philox
// stream of philox.cuh, so the CPU restatement replays every sample exactly.
#pragma once
#include "common.cuh"
#include "philox.cuh"

// Uniform state over the space: Shoemake's rotation then a box for SO(3) and
// SE(3) (src/mpt/impl/uniform_sampler_so3.hpp:55-68), U[-pi, pi) per joint for
// SO(2)^n (src/mpt/impl/uniform_sampler_so2.hpp:57-64), else the box
// [lo, hi) (src/mpt/uniform_box_sampler.hpp:60-68).
__device__ __forceinline__ void sample_uniform_state(int metric, int D, uint64_t seed, uint32_t i, uint32_t wave,
                                                     const double* __restrict__ lo, const double* __restrict__ hi,
                                                     double* __restrict__ q) {
    if (metric == MPTG_METRIC_SO3 || metric == MPTG_METRIC_SE3) {
        double a = phx_uniform(seed, i, wave, 0);
        double b = __dmul_rn(MPTG_TWO_PI, phx_uniform(seed, i, wave, 1));
        double c = __dmul_rn(MPTG_TWO_PI, phx_uniform(seed, i, wave, 2));
        double s1 = __dsqrt_rn(__dsub_rn(1.0, a)), s2 = __dsqrt_rn(a);
        double sb, cb, sc, cc;
        mptg_sincos(b, &sb, &cb);
        mptg_sincos(c, &sc, &cc);
        q[0] = __dmul_rn(s1, sb); q[1] = __dmul_rn(s1, cb); q[2] = __dmul_rn(s2, sc); q[3] = __dmul_rn(s2, cc);
        for (int d = 4; d < D; ++d) {
            double u = phx_uniform(seed, i, wave, (uint32_t)(d - 1));
            q[d] = __dadd_rn(lo[d], __dmul_rn(__dsub_rn(hi[d], lo[d]), u));
        }
    } else if (metric == MPTG_METRIC_SO2) {
        for (int d = 0; d < D; ++d)
            q[d] = __dadd_rn(-MPTG_PI, __dmul_rn(MPTG_TWO_PI, phx_uniform(seed, i, wave, (uint32_t)d)));
    } else {
        for (int d = 0; d < D; ++d) {
            double u = phx_uniform(seed, i, wave, (uint32_t)d);
            q[d] = __dadd_rn(lo[d], __dmul_rn(__dsub_rn(hi[d], lo[d]), u));
        }
    }
}
