// surrogate.cu - learned collision surrogate: an MLP trained on the GPU by
// this project's own forward/backward kernels.
//
// No counterpart in the reference (a GB300 addition): the network only orders
// and culls candidate edges; an edge still enters the tree only after the
// exact check (scene.cu / mesh.cu) accepts it.
//
// Network: in (<= 16, SE(3) states use 7) -> 256 -> 256 -> 256 -> 256 -> 1,
// SiLU after each hidden layer, logit out (1 = in collision).  BF16 weights and
// activations, FP32 accumulation; FP32 master weights, Adam, BCE-with-logits.
//   layer 0 (in -> 256) and the output layer (256 -> 1): CUDA cores
//   layers 1-3 (256 -> 256), forward, input-gradient and weight-gradient
//   products: k_sg_umma, a tcgen05 GEMM -- operand tiles moved by TMA
//   (128-byte swizzle) through a 4-stage mbarrier ring, one thread issuing
//   128 x 256 x 16 UMMAs into a TMEM accumulator, the epilogue reading TMEM
//   with tcgen05.ld and fusing bias + SiLU (forward), SiLU' (backward), the
//   split-K sums (weight gradients), or, when scoring, the output layer
// The scoring path stores no FP32 pre-activations and no transposes: only the
// BF16 activations the next layer reads, and the logits.
#include <cuda_bf16.h>

#include "metrics.cuh"
#include "philox.cuh"
#include "umma.cuh"

#include <mutex>

#define SG_W 256
#define SG_MAXIN 16
#define SG_TM 128                                 // rows per CTA (UMMA M)
#define SG_BK 64                                  // K per pipeline stage: one 128-byte swizzle row
#define SG_STAGES 4
#define SG_A_BYTES (SG_TM * SG_BK * 2)            // 16 KB
#define SG_B_BYTES (SG_W * SG_BK * 2)             // 32 KB: all 256 outputs (UMMA N = 256)
#define SG_STAGE_BYTES (SG_A_BYTES + SG_B_BYTES)
#define SG_SMEM (SG_STAGES * SG_STAGE_BYTES + 1024 + 256)
#define SG_TIMEOUT_NS 2000000000ull               // a GEMM takes microseconds; 2 s means something is wrong

typedef __nv_bfloat16 bf16;

struct mptg_surrogate {
    mptg_ctx* ctx = nullptr;
    int in = 7;
    double scale[SG_MAXIN], shift[SG_MAXIN];
    size_t nparam = 0;
    float* P = nullptr;   // FP32 master parameters
    float* G = nullptr;   // gradients
    float* Mo = nullptr;  // Adam first moment
    float* Vo = nullptr;  // Adam second moment
    // BF16 copies of the hidden weights: [l][out][in] and transposed [l][in][out]
    bf16* Wb = nullptr;
    bf16* WTb = nullptr;
    int step = 0;
    // activations for a batch of capacity cap
    size_t cap = 0;
    bf16* X = nullptr;            // [cap][16]
    float* Z = nullptr;           // [4][cap][256] pre-activations
    bf16* H = nullptr;            // [4][cap][256]
    bf16* HT = nullptr;           // [4][256][cap]
    bf16* dZ = nullptr;           // [cap][256] current layer
    bf16* dZT = nullptr;          // [256][cap]
    float* dH = nullptr;          // [cap][256] (output-layer backprop)
    float* zout = nullptr;        // [cap]
    float* dzout = nullptr;       // [cap]
    float* loss = nullptr;        // [1]
    double* dstates = nullptr;    // staging for host inputs [cap][in]
    uint8_t* dlabels = nullptr;
    float* dlogits = nullptr;
    int* err = nullptr;           // device error word: a tcgen05 GEMM wait ran out (1 load, 2 MMA, 3 epilogue)
    double* dnorm = nullptr;      // scale [16], shift [16] on the device (the fused scorer)
    CUtensorMap wmap;             // the three hidden layers' BF16 weights, [768][256] (the fused scorer)
    bool wmap_ok = false;
    // held by a planner from scoring until its stream has consumed the logits,
    // since the activation buffers above are shared
    std::mutex mu;
};

std::mutex* mptg_surrogate_mutex(mptg_surrogate* s) { return &s->mu; }

// parameter layout (floats)
struct SgLayout {
    size_t W0, b0, W[4], b[4], w4, b4, total;
};
static SgLayout sg_layout(int in) {
    SgLayout L;
    size_t o = 0;
    L.W0 = o; o += (size_t)SG_W * in;
    L.b0 = o; o += SG_W;
    for (int l = 1; l <= 3; ++l) { L.W[l] = o; o += (size_t)SG_W * SG_W; L.b[l] = o; o += SG_W; }
    L.w4 = o; o += SG_W;
    L.b4 = o; o += 1;
    L.total = o;
    return L;
}

// sigmoid(z) = (1 + tanh(z / 2)) / 2 with the hardware tanh (tanh.approx.f32,
// relative error about 2^-11): one MUFU operation instead of an exponential
// and a division.  The activations it feeds are rounded to BF16 (2^-8), so
// the approximation is below their rounding; training and scoring use the
// same function.
__device__ __forceinline__ float sg_tanh(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sg_sigmoid(float z) { return fmaf(0.5f, sg_tanh(0.5f * z), 0.5f); }
__device__ __forceinline__ float sg_silu(float z) {
    const float h = 0.5f * z;
    return fmaf(h, sg_tanh(h), h);  // z sigmoid(z) = z/2 + (z/2) tanh(z/2)
}
__device__ __forceinline__ float sg_dsilu(float z) {
    float s = sg_sigmoid(z);
    return s * (1.f + z * (1.f - s));
}

// ------------------------------------------------------------------ tensor-core GEMM
// C[m][n] = sum_k A[m][k] * B[n][k] for the 128 rows m of tile blockIdx.y and
// all 256 n, over the K range of split blockIdx.z (kblocks * 64 elements).
// A and B are K-major BF16 ([rows][ld]) read through TMA tensor maps.
enum { EPI_FWD = 0, EPI_BWD = 1, EPI_GRAD = 2, EPI_SCORE = 3, EPI_SCORE_OUT = 4 };

struct EpiArgs {
    // forward: z = acc + bias; Z[m][n] = z; H[m][n] = silu(z) (bf16), HT[n][m]
    // scoring: H only; scoring output: zout[m] = sum_n silu(z) w4[n] + b4
    const float* bias;
    float* Z;
    bf16* H;
    bf16* HT;
    int ldt;  // leading dimension of the transposed outputs (= M)
    // backward: dz = acc * silu'(Zin[m][n]); dZ[m][n], dZT[n][m]
    const float* Zin;
    bf16* dZ;
    bf16* dZT;
    // gradient: G[m][n] += acc
    float* G;
    int ldc;
    const float* w4;
    const float* b4;
    float* zout;
};

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// The fused epilogue of 16 accumulator columns c .. c+15 of row m (v = the
// FP32 sums), per EPI; `out` accumulates the scoring output layer.
// bias and w4 are ep.bias and ep.w4, or copies of them in shared memory.
template <int EPI>
__device__ __forceinline__ void sg_epilogue16(const EpiArgs& ep, const float* bias, const float* w4, size_t m, int c,
                                              const float (&v)[16], float& out) {
    if (EPI == EPI_GRAD) {
#pragma unroll
        for (int j = 0; j < 16; ++j) atomicAdd(&ep.G[m * ep.ldc + c + j], v[j]);
    } else if (EPI == EPI_BWD) {
        const float4* zi = reinterpret_cast<const float4*>(ep.Zin + m * SG_W + c);
        float zin[16];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float4 t = zi[j];
            zin[4 * j] = t.x; zin[4 * j + 1] = t.y; zin[4 * j + 2] = t.z; zin[4 * j + 3] = t.w;
        }
        uint32_t pk[8];
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
            float a = v[j] * sg_dsilu(zin[j]), b = v[j + 1] * sg_dsilu(zin[j + 1]);
            pk[j / 2] = pack_bf16x2(a, b);
            __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&pk[j / 2]);
            ep.dZT[(size_t)(c + j) * ep.ldt + m] = h.x;
            ep.dZT[(size_t)(c + j + 1) * ep.ldt + m] = h.y;
        }
        uint4* o = reinterpret_cast<uint4*>(ep.dZ + m * SG_W + c);
        o[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        o[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    } else {
        float z[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) z[j] = v[j] + bias[c + j];
        if (EPI == EPI_FWD) {
            float4* zo = reinterpret_cast<float4*>(ep.Z + m * SG_W + c);
#pragma unroll
            for (int j = 0; j < 4; ++j) zo[j] = make_float4(z[4 * j], z[4 * j + 1], z[4 * j + 2], z[4 * j + 3]);
        }
        if (EPI == EPI_SCORE_OUT) {
#pragma unroll
            for (int j = 0; j < 16; ++j)
                out = fmaf(__bfloat162float(__float2bfloat16_rn(sg_silu(z[j]))),
                           __bfloat162float(__float2bfloat16_rn(w4[c + j])), out);
        } else {
            uint32_t pk[8];
#pragma unroll
            for (int j = 0; j < 16; j += 2) pk[j / 2] = pack_bf16x2(sg_silu(z[j]), sg_silu(z[j + 1]));
            uint4* o = reinterpret_cast<uint4*>(ep.H + m * SG_W + c);
            o[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            o[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            if (EPI == EPI_FWD) {
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&pk[j]);
                    ep.HT[(size_t)(c + 2 * j) * ep.ldt + m] = h.x;
                    ep.HT[(size_t)(c + 2 * j + 1) * ep.ldt + m] = h.y;
                }
            }
        }
    }
}

// Warp roles: warp 0 lane 0 issues the TMA loads, warp 1 lane 0 the UMMAs;
// then all four warps run the epilogue, warp w on TMEM lanes (= tile rows)
// 32w .. 32w + 31.  Every wait is bounded (SG_TIMEOUT_NS); a wait that runs
// out sets *err, drains the loads already issued, frees TMEM and returns.
template <int EPI>
__global__ void __launch_bounds__(128, 1) k_sg_umma(const __grid_constant__ CUtensorMap ta,
                                                    const __grid_constant__ CUtensorMap tb, int kblocks, EpiArgs ep,
                                                    int* __restrict__ err) {
    extern __shared__ uint8_t sg_smem_raw[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t raw = umma::smem_u32(sg_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;  // the 128-byte swizzle needs 1024-byte aligned tiles
    uint8_t* smem = sg_smem_raw + (base - raw);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + SG_STAGES * SG_STAGE_BYTES);
    uint64_t* empty = full + SG_STAGES;
    uint64_t* accf = empty + SG_STAGES;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(accf + 1);
    int* counts = reinterpret_cast<int*>(tslot + 1);  // [0] stages loaded, [1] stages consumed
    const int m0 = blockIdx.y * SG_TM;
    const int k0 = blockIdx.z * kblocks * SG_BK;
    if (tid == 0) {
        for (int s = 0; s < SG_STAGES; ++s) {
            umma::mbar_init(&full[s], 1);
            umma::mbar_init(&empty[s], 1);
        }
        umma::mbar_init(accf, 1);
        counts[0] = counts[1] = 0;
        umma::fence_mbar_init();
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, SG_W);  // 256 FP32 columns x 128 lanes: the 128 x 256 accumulator
        umma::tmem_relinquish();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint64_t deadline = umma::globaltimer_ns() + SG_TIMEOUT_NS;

    if (warp == 0) {
        if (lane == 0) {
            int kb = 0;
            for (; kb < kblocks; ++kb) {
                const int s = kb % SG_STAGES;
                if (kb >= SG_STAGES && !umma::mbar_wait(&empty[s], ((kb / SG_STAGES) - 1) & 1, deadline)) {
                    atomicExch(err, 1);
                    break;
                }
                uint8_t* sa = smem + s * SG_STAGE_BYTES;
                umma::mbar_arrive_expect_tx(&full[s], SG_STAGE_BYTES);
                umma::tma_load_2d(sa, &ta, &full[s], k0 + kb * SG_BK, m0);
                umma::tma_load_2d(sa + SG_A_BYTES, &tb, &full[s], k0 + kb * SG_BK, 0);
            }
            counts[0] = kb;
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = umma::idesc_bf16_f32(SG_TM, SG_W);
            int kb = 0;
            for (; kb < kblocks; ++kb) {
                const int s = kb % SG_STAGES;
                if (!umma::mbar_wait(&full[s], (kb / SG_STAGES) & 1, deadline)) {
                    atomicExch(err, 2);
                    break;
                }
                umma::fence_after_sync();
                const uint32_t sa = base + s * SG_STAGE_BYTES, sb = sa + SG_A_BYTES;
#pragma unroll
                for (int k = 0; k < SG_BK / 16; ++k)
                    umma::mma_bf16(tmem, umma::sdesc_k128(sa + 32 * k), umma::sdesc_k128(sb + 32 * k), idesc,
                                   (kb | k) != 0);
                umma::mma_commit(&empty[s]);  // the stage is free once these UMMAs have read it
            }
            counts[1] = kb;
            umma::mma_commit(accf);  // the accumulator is ready once every UMMA has completed
        }
        __syncwarp();
    }
    const bool ok = umma::mbar_wait(accf, 0, deadline + SG_TIMEOUT_NS);
    umma::fence_after_sync();
    if (!ok) {
        if (tid == 0) atomicExch(err, 3);
    } else {
        const int row = warp * 32 + lane;
        const size_t m = (size_t)(m0 + row);
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        float out = 0.f;
#pragma unroll 1
        for (int c = 0; c < SG_W; c += 16) {
            float v[16];
            umma::tmem_ld16(trow + c, v);
            sg_epilogue16<EPI>(ep, ep.bias, ep.w4, m, c, v, out);
        }
        if (EPI == EPI_SCORE_OUT) ep.zout[m] = out + __ldg(ep.b4);
    }
    umma::fence_before_sync();
    __syncthreads();
    // loads issued but never consumed (a wait ran out) must land before the
    // shared memory they write is released
    if (tid == 0 && counts[1] < counts[0]) {
        const uint64_t drain = umma::globaltimer_ns() + SG_TIMEOUT_NS;
        for (int kb = counts[1]; kb < counts[0]; ++kb)
            umma::mbar_wait(&full[kb % SG_STAGES], (kb / SG_STAGES) & 1, drain);
    }
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, SG_W);
}

// ------------------------------------------------------------------ persistent GEMM (K = 256)
// C = A B^T with B the 256 x 256 weights, for every 128-row tile of A, by one
// CTA per SM that loops over tiles (tile = blockIdx.x + i * gridDim.x):
//   warp 0   TMA: the weights once (four 64-wide K slices, 128 KB, resident),
//            then each tile's four A slices through a 4-stage ring
//   warp 1   UMMA: per tile, 4 x 4 MMAs 128 x 256 x 16 into one of two TMEM
//            accumulators (2 x 256 columns), then a commit to its `full` barrier
//   warps 2-17 epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (the rows
//            its lane group may access) and the 64 columns of quarter
//            (w - 2) / 4, runs the fused per-row work of sg_epilogue16 on
//            them, then arrives on the accumulator's `empty` barrier
// so the epilogue of one tile overlaps the loads and UMMAs of the next.  The
// epilogue is the long part of a tile (a sigmoid per element against 16 UMMAs
// per tile), so four warps share each lane group and each SM sub-partition
// holds four of them to hide their latencies.  The bias and output weights
// are read from shared memory.  The scoring output layer's dot product is
// summed per quarter; the quarter-0 warp adds the other three quarters'
// partial sums (in quarter order, so every run gives the same bits) once a
// `ready` barrier says they are written, and only then arrives on `empty`, so
// the next tile on that accumulator cannot overwrite the partial sums early.
// All waits are bounded as in k_sg_umma.
#define SGP_EPI_WARPS 16
#define SGP_THREADS (64 + 32 * SGP_EPI_WARPS)
#define SGP_B_BYTES (4 * SG_W * SG_BK * 2)   // 128 KB of resident weights
#define SGP_F_BYTES ((2 * SG_W + 2 * 4 * SG_TM) * 4)  // bias, w4, partial sums [2][4][128]
#define SGP_SMEM (SGP_B_BYTES + SG_STAGES * SG_A_BYTES + SGP_F_BYTES + 1024 + 256)

template <int EPI>
__global__ void __launch_bounds__(SGP_THREADS, 1) k_sg_umma_p(const __grid_constant__ CUtensorMap ta,
                                                              const __grid_constant__ CUtensorMap tb, int ntiles,
                                                              EpiArgs ep, int* __restrict__ err) {
    extern __shared__ uint8_t sg_smem_raw[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t raw = umma::smem_u32(sg_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t* smem = sg_smem_raw + (base - raw);
    uint8_t* sB = smem;                     // [4][256][64] bf16, swizzled
    uint8_t* sA = smem + SGP_B_BYTES;       // [stage][128][64] bf16, swizzled
    float* sbias = reinterpret_cast<float*>(sA + SG_STAGES * SG_A_BYTES);
    float* sw4 = sbias + SG_W;
    float* spart = sw4 + SG_W;              // [acc][quarter][row] output-layer partial sums
    uint64_t* bfull = reinterpret_cast<uint64_t*>(spart + 2 * 4 * SG_TM);
    uint64_t* afull = bfull + 1;
    uint64_t* aempty = afull + SG_STAGES;
    uint64_t* accfull = aempty + SG_STAGES;
    uint64_t* accempty = accfull + 2;
    uint64_t* pready = accempty + 2;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(pready + 2);
    int* counts = reinterpret_cast<int*>(tslot + 1);  // [0] A slices loaded, [1] consumed, [2] weights loaded
    const int my_tiles = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (tid == 0) {
        umma::mbar_init(bfull, 1);
        for (int s = 0; s < SG_STAGES; ++s) {
            umma::mbar_init(&afull[s], 1);
            umma::mbar_init(&aempty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            umma::mbar_init(&accfull[a], 1);
            umma::mbar_init(&accempty[a], 32 * SGP_EPI_WARPS);
            umma::mbar_init(&pready[a], 32 * (SGP_EPI_WARPS - 4));
        }
        counts[0] = counts[1] = counts[2] = 0;
        umma::fence_mbar_init();
    }
    for (int i = tid; i < SG_W; i += SGP_THREADS) {
        sbias[i] = ep.bias ? __ldg(&ep.bias[i]) : 0.f;
        sw4[i] = ep.w4 ? __ldg(&ep.w4[i]) : 0.f;
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, 2 * SG_W);
        umma::tmem_relinquish();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint64_t deadline = umma::globaltimer_ns() + SG_TIMEOUT_NS;

    if (warp == 0) {
        if (lane == 0 && my_tiles > 0) {
            umma::mbar_arrive_expect_tx(bfull, SGP_B_BYTES);
            for (int kb = 0; kb < 4; ++kb) umma::tma_load_2d(sB + kb * (SG_W * SG_BK * 2), &tb, bfull, kb * SG_BK, 0);
            counts[2] = 1;
            int g = 0;
            bool ok = true;
            for (int i = 0; ok && i < my_tiles; ++i) {
                const int m0 = ((int)blockIdx.x + i * (int)gridDim.x) * SG_TM;
                for (int kb = 0; kb < 4; ++kb, ++g) {
                    const int s = g % SG_STAGES;
                    if (g >= SG_STAGES && !umma::mbar_wait(&aempty[s], ((g / SG_STAGES) - 1) & 1, deadline)) {
                        atomicExch(err, 1);
                        ok = false;
                        break;
                    }
                    umma::mbar_arrive_expect_tx(&afull[s], SG_A_BYTES);
                    umma::tma_load_2d(sA + s * SG_A_BYTES, &ta, &afull[s], kb * SG_BK, m0);
                }
            }
            counts[0] = g;
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0 && my_tiles > 0) {
            constexpr uint32_t idesc = umma::idesc_bf16_f32(SG_TM, SG_W);
            bool ok = umma::mbar_wait(bfull, 0, deadline);
            if (!ok) atomicExch(err, 2);
            umma::fence_after_sync();
            int g = 0;
            for (int i = 0; ok && i < my_tiles; ++i) {
                const int acc = i & 1;
                if (i >= 2 && !umma::mbar_wait(&accempty[acc], ((i >> 1) - 1) & 1, deadline)) {
                    atomicExch(err, 2);
                    ok = false;
                    break;
                }
                umma::fence_after_sync();
                const uint32_t d = tmem + (uint32_t)(acc * SG_W);
                for (int kb = 0; kb < 4; ++kb, ++g) {
                    const int s = g % SG_STAGES;
                    if (!umma::mbar_wait(&afull[s], (g / SG_STAGES) & 1, deadline)) {
                        atomicExch(err, 2);
                        ok = false;
                        break;
                    }
                    umma::fence_after_sync();
                    const uint32_t a0 = base + SGP_B_BYTES + s * SG_A_BYTES;
                    const uint32_t b0 = base + kb * (SG_W * SG_BK * 2);
#pragma unroll
                    for (int k = 0; k < SG_BK / 16; ++k)
                        umma::mma_bf16(d, umma::sdesc_k128(a0 + 32 * k), umma::sdesc_k128(b0 + 32 * k), idesc,
                                       (kb | k) != 0);
                    umma::mma_commit(&aempty[s]);
                }
                if (ok) umma::mma_commit(&accfull[acc]);
            }
            counts[1] = g;
        }
        __syncwarp();
    } else {
        // epilogue warps: lane group (warp % 4), column quarter (warp - 2) / 4
        const int grp = warp & 3, qtr = (warp - 2) >> 2, row = grp * 32 + lane;
        const uint32_t lane_off = (uint32_t)(grp * 32) << 16;
        for (int i = 0; i < my_tiles; ++i) {
            const int acc = i & 1;
            const bool ok = umma::mbar_wait(&accfull[acc], (i >> 1) & 1, deadline);
            __syncwarp();
            if (!ok) {
                if (lane == 0) atomicExch(err, 3);
                break;
            }
            umma::fence_after_sync();
            const size_t m = (size_t)(((int)blockIdx.x + i * (int)gridDim.x) * SG_TM + row);
            const uint32_t trow = tmem + lane_off + (uint32_t)(acc * SG_W);
            float out = 0.f;
#pragma unroll
            for (int c = 64 * qtr; c < 64 * qtr + 64; c += 16) {
                float v[16];
                umma::tmem_ld16(trow + c, v);
                sg_epilogue16<EPI>(ep, sbias, sw4, m, c, v, out);
            }
            if (EPI == EPI_SCORE_OUT) {
                float* part = spart + acc * 4 * SG_TM;
                if (qtr) {
                    part[qtr * SG_TM + row] = out;
                    umma::mbar_arrive(&pready[acc]);  // release: the partial sum is written
                } else {
                    const bool got = umma::mbar_wait(&pready[acc], (i >> 1) & 1, deadline);
                    if (got) {
                        out += part[SG_TM + row];
                        out += part[2 * SG_TM + row];
                        out += part[3 * SG_TM + row];
                        ep.zout[m] = out + __ldg(ep.b4);
                    } else if (lane == 0) {
                        atomicExch(err, 3);
                    }
                }
            }
            umma::fence_before_sync();
            umma::mbar_arrive(&accempty[acc]);
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    // loads issued but never consumed (a wait ran out) must land before the
    // shared memory they write is released
    if (tid == 0) {
        const uint64_t drain = umma::globaltimer_ns() + SG_TIMEOUT_NS;
        if (counts[2] && counts[1] == 0) umma::mbar_wait(bfull, 0, drain);
        for (int g = counts[1]; g < counts[0]; ++g) umma::mbar_wait(&afull[g % SG_STAGES], (g / SG_STAGES) & 1, drain);
    }
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 2 * SG_W);
}

// ------------------------------------------------------------------ fused scorer
// Logits of n states by the whole MLP in one persistent launch, the
// activations never leaving the SM.  Each CTA loops over 128-row tiles; two
// CTAs share an SM, so one's tensor-core phase runs while the other's
// CUDA-core phase does.  Per tile:
//   layer 0  the epilogue warps normalise their row's state and compute its
//            columns of SiLU(W0 x + b0) on CUDA cores (k_sg_inputs and
//            k_sg_layer0's arithmetic), written as BF16 into the A tile in
//            shared memory in the layout TMA's 128-byte swizzle gives (16-byte
//            chunk c of row r of a 64-wide K slice at chunk c ^ (r % 8));
//   layers 1-3  warp 1 issues the 16 UMMAs 128 x 256 x 16 of the layer (A from
//            that tile, B the layer's weights) into the TMEM accumulator; the
//            epilogue warps read it back and write SiLU(acc + bias) as the next
//            layer's A tile over the one just consumed, or, after layer 3, the
//            output layer's dot product (a chain per 64-column quarter, the
//            quarters added in order);
// while warp 0 streams the three layers' weights (128 KB each) from L2
// through a TMA ring of 64-wide K slices.  HBM traffic is the states in and
// the logits out.  The arithmetic equals k_sg_inputs + k_sg_layer0 + three
// k_sg_umma_p launches (the same UMMA sequence and epilogue steps), so the
// logits are the same bits.  Barriers: a_ready (the epilogue threads: A
// written and the accumulator read), acc_full (commit of a layer's UMMAs),
// w_full / w_empty per ring stage, pready (the output layer's partial sums);
// every wait is bounded as in k_sg_umma.
#define SGF_EPI 8                                   // epilogue warps: two per TMEM lane group
#define SGF_PARTS (SGF_EPI / 4)                     // column parts per row
#define SGF_PCOLS (SG_W / SGF_PARTS)                // columns per part (128)
#define SGF_STAGES 1                                // weight ring stages (one 32 KB slice)
#define SGF_CTAS 2                                  // CTAs per SM
#define SGF_THREADS (64 + 32 * SGF_EPI)
#define SGF_A_BYTES (SG_TM * SG_W * 2)              // 64 KB: the A tile, 4 K slices of 16 KB
#define SGF_WSTAGE (SG_W * SG_BK * 2)               // 32 KB: one 64-wide K slice of a layer's weights
// W0 (BF16-rounded, [k][n] for k < in), b0, b1-b3, w4, quarter sums [4][128]
#define SGF_F_FLOATS(in) ((in) * SG_W + 5 * SG_W + 4 * SG_TM)
#define SGF_SMEM(in) (SGF_A_BYTES + SGF_STAGES * SGF_WSTAGE + SGF_F_FLOATS(in) * 4 + 1024 + 256)

struct FusedArgs {
    const double* states;  // [n][in]
    int n, in;
    const double* norm;    // scale [16], shift [16]
    const float* W0;       // [256][in] FP32 master
    const float* b0;
    const float* b1;
    const float* b2;
    const float* b3;
    const float* w4;
    const float* b4;
    float* out;            // [n] logits
};

// the BF16 pair (a, b) as one 32-bit word, low half a
__device__ __forceinline__ uint32_t sgf_pack(float a, float b) { return pack_bf16x2(a, b); }

// 64 BF16 values of row r (K slice kb) into the swizzled A tile
__device__ __forceinline__ void sgf_store_row(uint8_t* sA, int r, int kb, const uint32_t (&pk)[32]) {
    uint8_t* row = sA + (size_t)kb * (SG_TM * SG_BK * 2) + (size_t)r * 128;
#pragma unroll
    for (int c = 0; c < 8; ++c)
        *reinterpret_cast<uint4*>(row + ((c ^ (r & 7)) << 4)) =
            make_uint4(pk[4 * c], pk[4 * c + 1], pk[4 * c + 2], pk[4 * c + 3]);
}

__global__ void __launch_bounds__(SGF_THREADS, SGF_CTAS) k_sg_score_fused(const __grid_constant__ CUtensorMap tw,
                                                                        int ntiles, FusedArgs fa,
                                                                        int* __restrict__ err) {
    extern __shared__ uint8_t sg_smem_raw[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t raw = umma::smem_u32(sg_smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t* smem = sg_smem_raw + (base - raw);
    uint8_t* sA = smem;                                  // [4][128][64] bf16, swizzled
    uint8_t* sW = smem + SGF_A_BYTES;                    // [stage][256][64] bf16, swizzled
    float* sW0 = reinterpret_cast<float*>(sW + SGF_STAGES * SGF_WSTAGE);  // [k][256], k < in
    float* sb0 = sW0 + fa.in * SG_W;
    float* sb = sb0 + SG_W;                              // [3][256] b1, b2, b3
    float* sw4 = sb + 3 * SG_W;
    float* spart = sw4 + SG_W;                           // [4][128] quarter sums
    uint64_t* a_ready = reinterpret_cast<uint64_t*>(spart + 4 * SG_TM);
    uint64_t* acc_full = a_ready + 1;
    uint64_t* pready = acc_full + 1;
    uint64_t* w_full = pready + 1;
    uint64_t* w_empty = w_full + SGF_STAGES;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(w_empty + SGF_STAGES);
    int* counts = reinterpret_cast<int*>(tslot + 1);    // [0] weight slices loaded, [1] consumed
    const int my_tiles = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int nslices = my_tiles * 3 * 4;
    if (tid == 0) {
        umma::mbar_init(a_ready, 32 * SGF_EPI);
        umma::mbar_init(acc_full, 1);
        umma::mbar_init(pready, 32 * (SGF_EPI - 4));
        for (int s = 0; s < SGF_STAGES; ++s) {
            umma::mbar_init(&w_full[s], 1);
            umma::mbar_init(&w_empty[s], 1);
        }
        counts[0] = counts[1] = 0;
        umma::fence_mbar_init();
    }
    for (int i = tid; i < SG_W; i += SGF_THREADS) {
        for (int k = 0; k < fa.in; ++k)
            sW0[k * SG_W + i] = __bfloat162float(__float2bfloat16_rn(__ldg(&fa.W0[i * fa.in + k])));
        sb0[i] = __ldg(&fa.b0[i]);
        sb[i] = __ldg(&fa.b1[i]);
        sb[SG_W + i] = __ldg(&fa.b2[i]);
        sb[2 * SG_W + i] = __ldg(&fa.b3[i]);
        sw4[i] = __ldg(&fa.w4[i]);
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, SG_W);
        umma::tmem_relinquish();
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint64_t deadline = umma::globaltimer_ns() + SG_TIMEOUT_NS;

    if (warp == 0) {
        if (lane == 0) {
            int g = 0;
            for (; g < nslices; ++g) {  // slice g: layer (g / 4) % 3, K block g % 4
                const int s = g % SGF_STAGES;
                if (g >= SGF_STAGES && !umma::mbar_wait(&w_empty[s], ((g / SGF_STAGES) - 1) & 1, deadline)) {
                    atomicExch(err, 1);
                    break;
                }
                umma::mbar_arrive_expect_tx(&w_full[s], SGF_WSTAGE);
                umma::tma_load_2d(sW + s * SGF_WSTAGE, &tw, &w_full[s], (g & 3) * SG_BK, ((g >> 2) % 3) * SG_W);
            }
            counts[0] = g;
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = umma::idesc_bf16_f32(SG_TM, SG_W);
            int g = 0;
            bool ok = true;
            for (int u = 0; ok && u < my_tiles * 3; ++u) {  // u: (tile, layer)
                if (!umma::mbar_wait(a_ready, u & 1, deadline)) {
                    atomicExch(err, 2);
                    break;
                }
                umma::fence_after_sync();
                for (int kb = 0; kb < 4; ++kb, ++g) {
                    const int s = g % SGF_STAGES;
                    if (!umma::mbar_wait(&w_full[s], (g / SGF_STAGES) & 1, deadline)) {
                        atomicExch(err, 2);
                        ok = false;
                        break;
                    }
                    umma::fence_after_sync();
                    const uint32_t a0 = base + kb * (SG_TM * SG_BK * 2);
                    const uint32_t b0 = base + SGF_A_BYTES + s * SGF_WSTAGE;
#pragma unroll
                    for (int k = 0; k < SG_BK / 16; ++k)
                        umma::mma_bf16(tmem, umma::sdesc_k128(a0 + 32 * k), umma::sdesc_k128(b0 + 32 * k), idesc,
                                       (kb | k) != 0);
                    umma::mma_commit(&w_empty[s]);
                }
                if (ok) umma::mma_commit(acc_full);
            }
            counts[1] = g;
        }
        __syncwarp();
    } else {
        // epilogue warps: lane group (warp % 4) = rows, part (warp - 2) / 4 = columns
        const int grp = warp & 3, part = (warp - 2) >> 2, row = grp * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(grp * 32) << 16);
        bool ok = true;
        for (int i = 0; ok && i < my_tiles; ++i) {
            const int m = ((int)blockIdx.x + i * (int)gridDim.x) * SG_TM + row;
            // layer 0 (k_sg_inputs, k_sg_layer0): BF16 inputs, FP32 sums over k in order
            float x[SG_MAXIN];
#pragma unroll
            for (int k = 0; k < SG_MAXIN; ++k) {
                float v = 0.f;
                if (m < fa.n && k < fa.in)
                    v = (float)((__ldg(&fa.states[(size_t)m * fa.in + k]) - fa.norm[SG_MAXIN + k]) * fa.norm[k]);
                x[k] = __bfloat162float(__float2bfloat16_rn(v));
            }
#pragma unroll 1
            for (int kb = part * (SGF_PCOLS / 64); kb < (part + 1) * (SGF_PCOLS / 64); ++kb) {
                // per column z = b0 + x0 w0 + x1 w1 + ... in k order, 16
                // columns at a time with the weights read as float4
                uint32_t pk[32];
#pragma unroll
                for (int c = 0; c < 64; c += 16) {
                    const int n0 = 64 * kb + c;
                    float z[16];
#pragma unroll
                    for (int j = 0; j < 16; j += 4) {
                        const float4 b = *reinterpret_cast<const float4*>(sb0 + n0 + j);
                        z[j] = b.x; z[j + 1] = b.y; z[j + 2] = b.z; z[j + 3] = b.w;
                    }
#pragma unroll
                    for (int k = 0; k < SG_MAXIN; ++k) {
                        if (k >= fa.in) break;
#pragma unroll
                        for (int j = 0; j < 16; j += 4) {
                            const float4 w = *reinterpret_cast<const float4*>(sW0 + k * SG_W + n0 + j);
                            z[j] = fmaf(x[k], w.x, z[j]);
                            z[j + 1] = fmaf(x[k], w.y, z[j + 1]);
                            z[j + 2] = fmaf(x[k], w.z, z[j + 2]);
                            z[j + 3] = fmaf(x[k], w.w, z[j + 3]);
                        }
                    }
#pragma unroll
                    for (int j = 0; j < 16; j += 2) pk[(c + j) / 2] = sgf_pack(sg_silu(z[j]), sg_silu(z[j + 1]));
                }
                sgf_store_row(sA, row, kb, pk);
            }
            umma::fence_proxy_async();
            umma::fence_before_sync();
            umma::mbar_arrive(a_ready);
            for (int l = 1; l <= 3; ++l) {
                const int u = 3 * i + (l - 1);
                if (!umma::mbar_wait(acc_full, u & 1, deadline)) {
                    if (lane == 0) atomicExch(err, 3);
                    ok = false;
                    break;
                }
                umma::fence_after_sync();
                const float* bias = sb + (l - 1) * SG_W;
                if (l < 3) {
#pragma unroll 1
                    for (int kb = part * (SGF_PCOLS / 64); kb < (part + 1) * (SGF_PCOLS / 64); ++kb) {
                        uint32_t pk[32];
#pragma unroll
                        for (int c = 0; c < 64; c += 16) {
                            float v[16];
                            umma::tmem_ld16(trow + 64 * kb + c, v);
#pragma unroll
                            for (int j = 0; j < 16; j += 2)
                                pk[(c + j) / 2] = sgf_pack(sg_silu(v[j] + bias[64 * kb + c + j]),
                                                           sg_silu(v[j + 1] + bias[64 * kb + c + j + 1]));
                        }
                        sgf_store_row(sA, row, kb, pk);
                    }
                    umma::fence_proxy_async();
                    umma::fence_before_sync();
                    umma::mbar_arrive(a_ready);
                } else {
                    float qs[SGF_PCOLS / 64];  // this thread's quarter sums
#pragma unroll
                    for (int h = 0; h < SGF_PCOLS / 64; ++h) {
                        const int kb = part * (SGF_PCOLS / 64) + h;
                        float out = 0.f;
#pragma unroll
                        for (int c = 0; c < 64; c += 16) {
                            float v[16];
                            umma::tmem_ld16(trow + 64 * kb + c, v);
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                const int nc = 64 * kb + c + j;
                                out = fmaf(__bfloat162float(__float2bfloat16_rn(sg_silu(v[j] + bias[nc]))),
                                           __bfloat162float(__float2bfloat16_rn(sw4[nc])), out);
                            }
                        }
                        qs[h] = out;
                    }
                    umma::fence_before_sync();
                    if (part) {
#pragma unroll
                        for (int h = 0; h < SGF_PCOLS / 64; ++h) spart[(part * (SGF_PCOLS / 64) + h) * SG_TM + row] = qs[h];
                        umma::mbar_arrive(pready);
                    } else if (umma::mbar_wait(pready, i & 1, deadline)) {
                        float out = qs[0];  // quarters added in order: 0, 1, 2, 3
#pragma unroll
                        for (int q = 1; q < 4; ++q) out += q < SGF_PCOLS / 64 ? qs[q < SGF_PCOLS / 64 ? q : 0] : spart[q * SG_TM + row];
                        if (m < fa.n) fa.out[m] = out + __ldg(fa.b4);
                    } else {
                        if (lane == 0) atomicExch(err, 3);
                        ok = false;
                    }
                }
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    // weight slices loaded but never consumed (a wait ran out) must land
    // before the shared memory they write is released
    if (tid == 0) {
        const uint64_t drain = umma::globaltimer_ns() + SG_TIMEOUT_NS;
        for (int g = counts[1]; g < counts[0]; ++g) umma::mbar_wait(&w_full[g % SGF_STAGES], (g / SGF_STAGES) & 1, drain);
    }
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, SG_W);
}

// ------------------------------------------------------------------ CUDA-core parts

// inputs: FP64 states -> normalised BF16 features, padded to 16
__global__ void k_sg_inputs(const double* __restrict__ s, int n, int in, const double* __restrict__ scale,
                            const double* __restrict__ shift, int cap, bf16* __restrict__ X) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cap) return;
    for (int k = 0; k < SG_MAXIN; ++k) {
        float v = 0.f;
        if (i < n && k < in) v = (float)((s[(size_t)i * in + k] - shift[k]) * scale[k]);
        X[(size_t)i * SG_MAXIN + k] = __float2bfloat16_rn(v);
    }
}

// layer 0: Z0 = X W0^T + b0 (bf16 operands, fp32 accumulate); thread per (m, n)
__global__ void k_sg_layer0(const bf16* __restrict__ X, int in, const float* __restrict__ W0,
                            const float* __restrict__ b0, int M, float* __restrict__ Z, bf16* __restrict__ H,
                            bf16* __restrict__ HT) {
    size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (idx >= (size_t)M * SG_W) return;
    int m = (int)(idx / SG_W), n = (int)(idx % SG_W);
    float z = b0[n];
    for (int k = 0; k < in; ++k)
        z = fmaf(__bfloat162float(X[(size_t)m * SG_MAXIN + k]), __bfloat162float(__float2bfloat16_rn(W0[n * in + k])), z);
    if (Z) Z[idx] = z;  // training keeps the pre-activation and the transpose; scoring does not
    bf16 h = __float2bfloat16_rn(sg_silu(z));
    H[idx] = h;
    if (HT) HT[(size_t)n * M + m] = h;
}

// output layer: zout[m] = H3[m] . w4 + b4 (warp per sample)
__global__ void k_sg_out(const bf16* __restrict__ H3, const float* __restrict__ w4, const float* __restrict__ b4,
                         int M, float* __restrict__ zout) {
    int m = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (m >= M) return;
    float s = 0.f;
    for (int k = lane; k < SG_W; k += 32)
        s = fmaf(__bfloat162float(H3[(size_t)m * SG_W + k]), __bfloat162float(__float2bfloat16_rn(w4[k])), s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) zout[m] = s + b4[0];
}

// BCE-with-logits: loss and dL/dz for the first n (real) rows
__global__ void k_sg_loss(const float* __restrict__ zout, const uint8_t* __restrict__ y, int n, float inv_n,
                          float* __restrict__ dz, float* __restrict__ loss) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (m < n) {
        float z = zout[m], t = y[m] ? 1.f : 0.f;
        l = fmaxf(z, 0.f) - z * t + log1pf(__expf(-fabsf(z)));
        dz[m] = (sg_sigmoid(z) - t) * inv_n;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l * inv_n);
}

// backprop through the output layer: dZ3 = (dz w4) * silu'(Z3); grads of w4, b4
__global__ void k_sg_out_back(const float* __restrict__ dz, const float* __restrict__ w4,
                              const float* __restrict__ Z3, const bf16* __restrict__ H3, int M, bf16* __restrict__ dZ,
                              bf16* __restrict__ dZT, float* __restrict__ gw4, float* __restrict__ gb4) {
    size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (idx >= (size_t)M * SG_W) return;
    int m = (int)(idx / SG_W), n = (int)(idx % SG_W);
    float d = dz[m];
    float dh = d * __bfloat162float(__float2bfloat16_rn(w4[n]));
    bf16 v = __float2bfloat16_rn(dh * sg_dsilu(Z3[idx]));
    dZ[idx] = v;
    dZT[(size_t)n * M + m] = v;
    if (d != 0.f) {
        atomicAdd(&gw4[n], d * __bfloat162float(H3[idx]));
        if (n == 0) atomicAdd(gb4, d);
    }
}

// bias gradient: column sums of dZ (block per column)
__global__ void k_sg_colsum(const bf16* __restrict__ dZT, int M, float* __restrict__ gb) {
    int n = blockIdx.x;
    float s = 0.f;
    for (int m = threadIdx.x; m < M; m += blockDim.x) s += __bfloat162float(dZT[(size_t)n * M + m]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        gb[n] = t;
    }
}

// layer-0 weight gradient: G0[n][k] = sum_m dZ0[m][n] X[m][k] (block per n)
__global__ void k_sg_grad0(const bf16* __restrict__ dZT0, const bf16* __restrict__ X, int M, int in,
                           float* __restrict__ G0) {
    int n = blockIdx.x;
    __shared__ float acc[SG_MAXIN][8];
    float s[SG_MAXIN];
    for (int k = 0; k < SG_MAXIN; ++k) s[k] = 0.f;
    for (int m = threadIdx.x; m < M; m += blockDim.x) {
        float d = __bfloat162float(dZT0[(size_t)n * M + m]);
        for (int k = 0; k < in; ++k) s[k] = fmaf(d, __bfloat162float(X[(size_t)m * SG_MAXIN + k]), s[k]);
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < in; ++k) {
        float v = s[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) acc[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < in) {
        float t = 0.f;
        for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww) t += acc[threadIdx.x][ww];
        G0[n * in + threadIdx.x] = t;
    }
}

// Adam (Kingma & Ba 2015) on the FP32 masters; refreshes the BF16 weight copies
__global__ void k_sg_adam(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ Mo,
                          float* __restrict__ Vo, size_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = G[i];
    float m = b1 * Mo[i] + (1.f - b1) * g;
    float v = b2 * Vo[i] + (1.f - b2) * g * g;
    Mo[i] = m;
    Vo[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

__global__ void k_sg_refresh(const float* __restrict__ P, size_t off1, size_t off2, size_t off3,
                             bf16* __restrict__ Wb, bf16* __restrict__ WTb) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * SG_W * SG_W) return;
    int l = idx / (SG_W * SG_W), r = idx % (SG_W * SG_W);
    int o = r / SG_W, i = r % SG_W;
    size_t off = l == 0 ? off1 : (l == 1 ? off2 : off3);
    bf16 w = __float2bfloat16_rn(P[off + r]);
    Wb[(size_t)l * SG_W * SG_W + (size_t)o * SG_W + i] = w;
    WTb[(size_t)l * SG_W * SG_W + (size_t)i * SG_W + o] = w;
}

// deterministic initialisation: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in))
__global__ void k_sg_init(float* __restrict__ P, size_t n, uint64_t seed, SgLayout L, int in) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int fan = SG_W;
    if (i < L.b0) fan = in;
    double u = phx_uniform(seed, (uint32_t)i, 0x5eedu, 0);
    P[i] = (float)((2.0 * u - 1.0) / sqrt((double)fan));
}

// ------------------------------------------------------------------ host

static mptg_status sg_reserve(mptg_surrogate* s, size_t cap) {
    if (cap <= s->cap) return MPTG_OK;
    mptg_ctx* ctx = s->ctx;
    MPTG_CUDA_TRY(ctx, cudaDeviceSynchronize());
    void* ptrs[] = {s->X, s->Z, s->H, s->HT, s->dZ, s->dZT, s->dH, s->zout, s->dzout, s->dstates, s->dlabels,
                    s->dlogits};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    cap = (cap + SG_TM - 1) / SG_TM * SG_TM;
    cudaError_t e = cudaSuccess;
#define A(p, b) if (e == cudaSuccess) e = cudaMalloc((void**)&(p), (b))
    A(s->X, cap * SG_MAXIN * sizeof(bf16));
    A(s->Z, 4 * cap * SG_W * sizeof(float));
    A(s->H, 4 * cap * SG_W * sizeof(bf16));
    A(s->HT, 4 * cap * SG_W * sizeof(bf16));
    A(s->dZ, cap * SG_W * sizeof(bf16));
    A(s->dZT, cap * SG_W * sizeof(bf16));
    A(s->dH, cap * SG_W * sizeof(float));
    A(s->zout, cap * sizeof(float));
    A(s->dzout, cap * sizeof(float));
    // [0, 16) scale, [16, 32) shift, then up to cap staged states
    A(s->dstates, (cap * SG_MAXIN + 2 * SG_MAXIN) * sizeof(double));
    A(s->dlabels, cap);
    A(s->dlogits, cap * sizeof(float));
#undef A
    if (e != cudaSuccess) {
        cudaGetLastError();
        return mptg_fail(ctx, MPTG_ERR_OOM, "surrogate buffers: %s", cudaGetErrorString(e));
    }
    s->cap = cap;
    return MPTG_OK;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda)
static EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// TMA map of a K-major BF16 matrix [rows][ld] whose first `cols` elements per
// row are the K extent: 64 x box_rows boxes with the 128-byte swizzle
static bool bf16_map(CUtensorMap* m, const bf16* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows) {
    EncodeTiledFn f = encode_tiled();
    if (!f) return false;
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {ld * sizeof(bf16)};
    cuuint32_t box[2] = {SG_BK, box_rows};
    cuuint32_t es[2] = {1, 1};
    return f(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// C = A B^T for A [rowsA][lda] (rowsA a multiple of 128) and B [256][ldb],
// both over K (a multiple of 64) elements; K split into CTAs of kblocks * 64
template <int EPI>
static mptg_status sg_gemm(mptg_surrogate* s, const bf16* A, int rowsA, int lda, const bf16* B, int ldb, int K,
                           int kblocks, const EpiArgs& ep, cudaStream_t st) {
    MPTG_CUDA_TRY(s->ctx, mptg_once_per_device((const void*)k_sg_umma<EPI>, [] {
        return cudaFuncSetAttribute(k_sg_umma<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, SG_SMEM);
    }));
    CUtensorMap ta, tb;
    if (!bf16_map(&ta, A, (uint64_t)rowsA, (uint64_t)K, (uint64_t)lda, SG_TM) ||
        !bf16_map(&tb, B, SG_W, (uint64_t)K, (uint64_t)ldb, SG_W))
        return mptg_fail(s->ctx, MPTG_ERR_CUDA, "surrogate GEMM: cuTensorMapEncodeTiled failed");
    dim3 grid(1, rowsA / SG_TM, (K / SG_BK) / kblocks);
    k_sg_umma<EPI><<<grid, 128, SG_SMEM, st>>>(ta, tb, kblocks, ep, s->err);
    MPTG_LAUNCHED(s->ctx);
    MPTG_CUDA_TRY(s->ctx, cudaGetLastError());
    return MPTG_OK;
}

// C = A B^T over K = 256 for A [rowsA][256] (rowsA a multiple of 128) and the
// weights B [256][256]: the persistent kernel, one CTA per SM at most
template <int EPI>
static mptg_status sg_gemm_p(mptg_surrogate* s, const bf16* A, int rowsA, const bf16* B, const EpiArgs& ep,
                             cudaStream_t st) {
    MPTG_CUDA_TRY(s->ctx, mptg_once_per_device((const void*)k_sg_umma_p<EPI>, [] {
        return cudaFuncSetAttribute(k_sg_umma_p<EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, SGP_SMEM);
    }));
    CUtensorMap ta, tb;
    if (!bf16_map(&ta, A, (uint64_t)rowsA, SG_W, SG_W, SG_TM) || !bf16_map(&tb, B, SG_W, SG_W, SG_W, SG_W))
        return mptg_fail(s->ctx, MPTG_ERR_CUDA, "surrogate GEMM: cuTensorMapEncodeTiled failed");
    const int tiles = rowsA / SG_TM;
    const int grid = std::min(tiles, std::max(1, s->ctx->sms));
    k_sg_umma_p<EPI><<<grid, SGP_THREADS, SGP_SMEM, st>>>(ta, tb, tiles, ep, s->err);
    MPTG_LAUNCHED(s->ctx);
    MPTG_CUDA_TRY(s->ctx, cudaGetLastError());
    return MPTG_OK;
}

// reads and clears the device error word (synchronises the stream)
static mptg_status sg_check(mptg_surrogate* s, cudaStream_t st) {
    int e = 0;
    MPTG_CUDA_TRY(s->ctx, cudaMemcpyAsync(&e, s->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    MPTG_CUDA_TRY(s->ctx, cudaStreamSynchronize(st));
    if (e) {
        MPTG_CUDA_TRY(s->ctx, cudaMemsetAsync(s->err, 0, sizeof(int), st));
        return mptg_fail(s->ctx, MPTG_ERR_TIMEOUT, "surrogate tensor-core GEMM: a pipeline wait ran out (%s)",
                         e == 1 ? "operand load" : e == 2 ? "UMMA issue" : "accumulator");
    }
    return MPTG_OK;
}

// forward over M (multiple of 128) rows already in s->X.  Training keeps every
// layer's pre-activations, activations and transposes for the backward pass;
// scoring (train = false) writes only the BF16 activations and the logits.
static mptg_status sg_forward(mptg_surrogate* s, int M, bool train, cudaStream_t st) {
    SgLayout L = sg_layout(s->in);
    const size_t MW = (size_t)M * SG_W;
    k_sg_layer0<<<mptg_blocks(MW, 256), 256, 0, st>>>(s->X, s->in, s->P + L.W0, s->P + L.b0, M,
                                                      train ? s->Z : nullptr, s->H, train ? s->HT : nullptr);
    MPTG_LAUNCHED(s->ctx);
    mptg_status r;
    for (int l = 1; l <= 3; ++l) {
        EpiArgs ep{};
        ep.bias = s->P + L.b[l];
        ep.ldt = M;
        const bf16* A = s->H + (l - 1) * MW;
        const bf16* B = s->Wb + (size_t)(l - 1) * SG_W * SG_W;
        if (train) {
            ep.Z = s->Z + l * MW;
            ep.H = s->H + l * MW;
            ep.HT = s->HT + l * MW;
            r = sg_gemm_p<EPI_FWD>(s, A, M, B, ep, st);
        } else if (l < 3) {
            ep.H = s->H + l * MW;
            r = sg_gemm_p<EPI_SCORE>(s, A, M, B, ep, st);
        } else {
            ep.w4 = s->P + L.w4;
            ep.b4 = s->P + L.b4;
            ep.zout = s->zout;
            r = sg_gemm_p<EPI_SCORE_OUT>(s, A, M, B, ep, st);
        }
        if (r) return r;
    }
    if (train) {
        k_sg_out<<<mptg_blocks((size_t)M * 32, 256), 256, 0, st>>>(s->H + 3 * MW, s->P + L.w4, s->P + L.b4, M,
                                                                   s->zout);
        MPTG_LAUNCHED(s->ctx);
    }
    return MPTG_OK;
}

extern "C" {

mptg_status mptg_surrogate_create(mptg_ctx* ctx, int in_dim, const double* scale, const double* shift, uint64_t seed,
                                  mptg_surrogate** out) {
    if (!ctx || !out) return MPTG_ERR_INVALID_ARG;
    *out = nullptr;
    if (in_dim < 1 || in_dim > SG_MAXIN) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "input dimension 1..16");
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    mptg_surrogate* s = new mptg_surrogate();
    s->ctx = ctx;
    s->in = in_dim;
    for (int k = 0; k < SG_MAXIN; ++k) {
        s->scale[k] = (scale && k < in_dim) ? scale[k] : 1.0;
        s->shift[k] = (shift && k < in_dim) ? shift[k] : 0.0;
    }
    SgLayout L = sg_layout(in_dim);
    s->nparam = L.total;
    cudaError_t e = cudaSuccess;
    size_t pb = L.total * sizeof(float);
    for (float** p : {&s->P, &s->G, &s->Mo, &s->Vo})
        if (e == cudaSuccess) e = cudaMalloc((void**)p, pb);
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->Wb, 3 * SG_W * SG_W * sizeof(bf16));
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->WTb, 3 * SG_W * SG_W * sizeof(bf16));
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(s->err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->dnorm, 2 * SG_MAXIN * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(s->dnorm, s->scale, SG_MAXIN * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(s->dnorm + SG_MAXIN, s->shift, SG_MAXIN * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return mptg_fail(ctx, MPTG_ERR_OOM, "surrogate parameters: %s", cudaGetErrorString(e));
    }
    s->wmap_ok = bf16_map(&s->wmap, s->Wb, 3 * SG_W, SG_W, SG_W, SG_W);
    cudaMemset(s->Mo, 0, pb);
    cudaMemset(s->Vo, 0, pb);
    cudaMemset(s->G, 0, pb);
    k_sg_init<<<mptg_blocks(L.total, 256), 256>>>(s->P, L.total, seed, L, in_dim);
    // biases start at zero
    cudaMemset(s->P + L.b0, 0, SG_W * sizeof(float));
    for (int l = 1; l <= 3; ++l) cudaMemset(s->P + L.b[l], 0, SG_W * sizeof(float));
    cudaMemset(s->P + L.b4, 0, sizeof(float));
    k_sg_refresh<<<mptg_blocks(3 * SG_W * SG_W, 256), 256>>>(s->P, L.W[1], L.W[2], L.W[3], s->Wb, s->WTb);
    ctx->launches += 2;
    MPTG_CUDA_TRY(ctx, cudaDeviceSynchronize());
    *out = s;
    return MPTG_OK;
}

mptg_status mptg_surrogate_destroy(mptg_surrogate* s) {
    if (!s) return MPTG_ERR_INVALID_ARG;
    cudaDeviceSynchronize();
    void* ptrs[] = {s->P, s->G, s->Mo, s->Vo, s->Wb, s->WTb, s->X, s->Z, s->H, s->HT, s->dZ, s->dZT, s->dH,
                    s->zout, s->dzout, s->dstates, s->dlabels, s->dlogits, s->loss, s->err, s->dnorm};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete s;
    return MPTG_OK;
}

mptg_status mptg_surrogate_num_params(mptg_surrogate* s, size_t* n) {
    if (!s || !n) return MPTG_ERR_INVALID_ARG;
    *n = s->nparam;
    return MPTG_OK;
}

mptg_status mptg_surrogate_get(mptg_surrogate* s, int which, float* out, size_t n) {
    if (!s || !out || n != s->nparam || which < 0 || which > 1) return MPTG_ERR_INVALID_ARG;
    MPTG_CUDA_TRY(s->ctx, cudaDeviceSynchronize());
    MPTG_CUDA_TRY(s->ctx, cudaMemcpy(out, which == 0 ? s->P : s->G, n * sizeof(float), cudaMemcpyDeviceToHost));
    return MPTG_OK;
}

mptg_status mptg_surrogate_set(mptg_surrogate* s, const float* in, size_t n) {
    if (!s || !in || n != s->nparam) return MPTG_ERR_INVALID_ARG;
    SgLayout L = sg_layout(s->in);
    MPTG_CUDA_TRY(s->ctx, cudaMemcpy(s->P, in, n * sizeof(float), cudaMemcpyHostToDevice));
    k_sg_refresh<<<mptg_blocks(3 * SG_W * SG_W, 256), 256>>>(s->P, L.W[1], L.W[2], L.W[3], s->Wb, s->WTb);
    MPTG_LAUNCHED(s->ctx);
    MPTG_CUDA_TRY(s->ctx, cudaDeviceSynchronize());
    return MPTG_OK;
}

// internal: logits for n device states (used by the planner): the fused
// scorer, one launch, no activation buffers
mptg_status mptg_surrogate_score_dev(mptg_surrogate* s, const double* dstates, int n, float* dlogits, cudaStream_t st) {
    if (n <= 0) return MPTG_OK;
    if (!s->wmap_ok) return mptg_fail(s->ctx, MPTG_ERR_CUDA, "surrogate scorer: cuTensorMapEncodeTiled failed");
    MPTG_CUDA_TRY(s->ctx, mptg_once_per_device((const void*)k_sg_score_fused, [] {
        cudaError_t e =
            cudaFuncSetAttribute(k_sg_score_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, SGF_SMEM(SG_MAXIN));
        // all of the SM's unified memory as shared memory, so two CTAs fit
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_sg_score_fused, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        return e;
    }));
    SgLayout L = sg_layout(s->in);
    FusedArgs fa;
    fa.states = dstates;
    fa.n = n;
    fa.in = s->in;
    fa.norm = s->dnorm;
    fa.W0 = s->P + L.W0;
    fa.b0 = s->P + L.b0;
    fa.b1 = s->P + L.b[1];
    fa.b2 = s->P + L.b[2];
    fa.b3 = s->P + L.b[3];
    fa.w4 = s->P + L.w4;
    fa.b4 = s->P + L.b4;
    fa.out = dlogits;
    const int tiles = (n + SG_TM - 1) / SG_TM;
    const int grid = std::min(tiles, SGF_CTAS * std::max(1, s->ctx->sms));
    k_sg_score_fused<<<grid, SGF_THREADS, SGF_SMEM(s->in), st>>>(s->wmap, tiles, fa, s->err);
    MPTG_LAUNCHED(s->ctx);
    MPTG_CUDA_TRY(s->ctx, cudaGetLastError());
    return MPTG_OK;
}

mptg_status mptg_surrogate_score(mptg_surrogate* s, const double* states, size_t n, float* logits, void* stream) {
    if (!s || (!states && n) || (!logits && n)) return MPTG_ERR_INVALID_ARG;
    if (n == 0) return MPTG_OK;
    if (n > (1u << 26)) return mptg_fail(s->ctx, MPTG_ERR_INVALID_ARG, "too many states");
    cudaStream_t st = (cudaStream_t)stream;
    DevBuf bq, bo;
    mptg_status r;
    if ((r = mptg_stage_in(s->ctx, states, n * s->in * sizeof(double), st, &bq))) return r;
    if ((r = mptg_stage_out_alloc(s->ctx, logits, n * sizeof(float), st, &bo))) return r;
    if ((r = mptg_surrogate_score_dev(s, (const double*)bq.dptr, (int)n, (float*)bo.dptr, st))) return r;
    MPTG_CUDA_TRY(s->ctx, cudaGetLastError());
    if ((r = mptg_stage_finish(s->ctx, st, &bo, 1, &bq, 1))) return r;
    // host buffers: the call has synchronised anyway, so report a GEMM wait that ran out
    if (!mptg_is_device_ptr(logits)) return sg_check(s, st);
    return MPTG_OK;
}

// One Adam step on a batch: loss and gradients of BCE-with-logits, labels 1 =
// in collision.  n must be a multiple of 128.  lr <= 0 computes the loss and
// the gradients (readable with mptg_surrogate_get(s, 1, ...)) without
// updating the parameters.
mptg_status mptg_surrogate_train_step(mptg_surrogate* s, const double* states, const uint8_t* labels, size_t n,
                                      double lr, float* loss_out, void* stream) {
    if (!s || !states || !labels || n == 0) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = s->ctx;
    if (n % SG_TM) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "batch must be a multiple of %d", SG_TM);
    if (n > (1u << 20)) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "batch too large");
    cudaStream_t st = (cudaStream_t)stream;
    mptg_status r = sg_reserve(s, n);
    if (r) return r;
    const int M = (int)n;
    const size_t MW = (size_t)M * SG_W;
    SgLayout L = sg_layout(s->in);
    // inputs
    const double* dq = states;
    if (!mptg_is_device_ptr(states)) {
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(s->dstates + 2 * SG_MAXIN, states, n * s->in * sizeof(double),
                                           cudaMemcpyHostToDevice, st));
        dq = s->dstates + 2 * SG_MAXIN;
    }
    const uint8_t* dy = labels;
    if (!mptg_is_device_ptr(labels)) {
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(s->dlabels, labels, n, cudaMemcpyHostToDevice, st));
        dy = s->dlabels;
    }
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(s->dstates, s->scale, sizeof(s->scale), cudaMemcpyHostToDevice, st));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(s->dstates + SG_MAXIN, s->shift, sizeof(s->shift), cudaMemcpyHostToDevice, st));
    k_sg_inputs<<<mptg_blocks(M, 256), 256, 0, st>>>(dq, M, s->in, s->dstates, s->dstates + SG_MAXIN, M, s->X);
    MPTG_LAUNCHED(ctx);
    if ((r = sg_forward(s, M, true, st))) return r;
    // loss and output-layer gradients
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(s->G, 0, s->nparam * sizeof(float), st));
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(s->loss, 0, sizeof(float), st));
    k_sg_loss<<<mptg_blocks(M, 256), 256, 0, st>>>(s->zout, dy, M, 1.f / (float)M, s->dzout, s->loss);
    k_sg_out_back<<<mptg_blocks(MW, 256), 256, 0, st>>>(s->dzout, s->P + L.w4, s->Z + 3 * MW, s->H + 3 * MW, M,
                                                        s->dZ, s->dZT, s->G + L.w4, s->G + L.b4);
    ctx->launches += 2;
    // hidden layers 3, 2, 1: weight and bias gradients, then back through W
    for (int l = 3; l >= 1; --l) {
        k_sg_colsum<<<SG_W, 256, 0, st>>>(s->dZT, M, s->G + L.b[l]);
        MPTG_LAUNCHED(ctx);
        EpiArgs eg{};
        eg.G = s->G + L.W[l];
        eg.ldc = SG_W;
        // dW[out][in] = sum_m dZ[m][out] H_{l-1}[m][in]: A = dZ^T [out][M], B = H^T [in][M];
        // K (= the batch) split over CTAs of 4 (or 2) stages, summed by the epilogue's atomics
        const int kb = (M / SG_BK) % 4 == 0 ? 4 : 2;
        if ((r = sg_gemm<EPI_GRAD>(s, s->dZT, SG_W, M, s->HT + (size_t)(l - 1) * MW, M, M, kb, eg, st))) return r;
        // dH_{l-1} = dZ_l W_l, then * silu'(Z_{l-1})
        EpiArgs eb{};
        eb.Zin = s->Z + (size_t)(l - 1) * MW;
        eb.dZ = s->dZ;
        eb.dZT = s->dZT;
        eb.ldt = M;
        // the GEMM reads dZ/dZT of layer l while writing layer l-1's into the same
        // buffers: stage through dH
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(s->dH, s->dZ, MW * sizeof(bf16), cudaMemcpyDeviceToDevice, st));
        if ((r = sg_gemm_p<EPI_BWD>(s, (const bf16*)s->dH, M, s->WTb + (size_t)(l - 1) * SG_W * SG_W, eb, st)))
            return r;
    }
    // layer 0
    k_sg_colsum<<<SG_W, 256, 0, st>>>(s->dZT, M, s->G + L.b0);
    k_sg_grad0<<<SG_W, 256, 0, st>>>(s->dZT, s->X, M, s->in, s->G + L.W0);
    ctx->launches += 2;
    if (lr > 0) {
        s->step += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        float c1 = 1.f - powf(b1, (float)s->step), c2 = 1.f - powf(b2, (float)s->step);
        k_sg_adam<<<mptg_blocks(s->nparam, 256), 256, 0, st>>>(s->P, s->G, s->Mo, s->Vo, s->nparam, (float)lr, b1, b2,
                                                                1e-8f, c1, c2);
        k_sg_refresh<<<mptg_blocks(3 * SG_W * SG_W, 256), 256, 0, st>>>(s->P, L.W[1], L.W[2], L.W[3], s->Wb, s->WTb);
        ctx->launches += 2;
    }
    if (loss_out) {
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(loss_out, s->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
        MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        if ((r = sg_check(s, st))) return r;
    }
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    return MPTG_OK;
}

}  // extern "C"
