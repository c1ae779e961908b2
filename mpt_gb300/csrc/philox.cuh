// philox.cuh - Philox4x32-10 counter-based generator (J. K. Salmon, M. A.
// Moraes, R. O. Dror, D. E. Shaw, "Parallel random numbers: as easy as 1, 2,
// 3", SC'11), written from the published round function and constants, for
// host and device.  Replaces the per-worker MT19937 streams of
// src/mpt/mersenne_twister.hpp with a stream addressed by (sample, wavefront,
// block): every planner sample is reproducible from the seed alone, which is
// what lets the CPU checker replay a wavefront exactly.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define PHX_HD __host__ __device__ __forceinline__
#else
#define PHX_HD static inline
#endif

PHX_HD void phx_mulhilo(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

// 10 rounds of Philox4x32 on counter c with key k (in place)
PHX_HD void phx_4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        phx_mulhilo(M0, c[0], &hi0, &lo0);
        phx_mulhilo(M1, c[2], &hi1, &lo1);
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        uint32_t n3 = lo0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += W0;
        k1 += W1;
    }
}

// 53-bit uniform double in [0, 1) from two 32-bit words (exact in FP64)
PHX_HD double phx_u01(uint32_t a, uint32_t b) {
    uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return (double)m * (1.0 / 9007199254740992.0);
}

// uniform number j (0 <= j < 32) of sample i in wavefront w
PHX_HD double phx_uniform(uint64_t seed, uint32_t i, uint32_t w, uint32_t j) {
    uint32_t c[4] = {i, w, j >> 1, 0x6d707467u};
    phx_4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return (j & 1) ? phx_u01(c[2], c[3]) : phx_u01(c[0], c[1]);
}
