// noalloc.cu - exact brute-force 1-NN over caller-owned device buffers that
// allocates no device memory.
//
// Some callers cannot allocate GPU memory while they run: a robot's real-time
// control loop must not call cudaMalloc after start-up (the call can block and
// synchronise the device for an unbounded time), and a plugin hosted by a
// framework that owns all device memory through its own allocator has no way
// to obtain more.  mptg_nearest_linear (tree.cu) needs the tree's FP32 copy of
// the points; this variant keeps that FP32 working copy in the file-scope
// array below instead, so the call itself allocates nothing.
//
// Scratch: one static device array of MPTG_NOALLOC_SCRATCH_FLOATS floats
// (4 MiB + 256 B), present on every GPU that loads the library until the
// process exits.  Host code must not pass the symbol itself to a kernel: on
// the host it names a host-side stand-in, not device memory.  The device
// address is looked up once per device with cudaGetSymbolAddress (on that
// device's first call) and cached; a cudaDeviceReset (or any other reset of
// the device's primary context) after that first call leaves the cached
// address stale, so the entry point must not be called again in that process.
#include "metrics.cuh"

#define MPTG_NOALLOC_MAX_POINTS 65536
#define MPTG_NOALLOC_COUNTERS 64  // [0] max |Lp coordinate| (float bits), [1] input-error flag
#define MPTG_NOALLOC_SCRATCH_FLOATS (MPTG_NOALLOC_MAX_POINTS * MPTG_MAX_DIM + MPTG_NOALLOC_COUNTERS)

static __device__ __align__(256) float mptg_noalloc_scratch[MPTG_NOALLOC_SCRATCH_FLOATS];

namespace {

std::mutex g_scratch_mu;
float* g_scratch_addr[64] = {nullptr};

mptg_status scratch_address(mptg_ctx* ctx, float** out) {
    int dev = ctx->device;
    if (dev < 0 || dev >= 64) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, mptg_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return mptg_fail(ctx, MPTG_ERR_CUDA, "cudaGetSymbolAddress(mptg_noalloc_scratch) failed: %s",
                             cudaGetErrorString(e));
        }
        g_scratch_addr[dev] = (float*)p;
    }
    *out = g_scratch_addr[dev];
    return MPTG_OK;
}

// true when p is memory that kernels on `device` can use directly: device
// memory allocated on that device, or managed memory
bool on_device(const void* p, int device) {
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (attr.type == cudaMemoryTypeManaged) return true;
    return attr.type == cudaMemoryTypeDevice && attr.device == device;
}

// FP32 copy of the points into the scratch array, input checks and the
// largest |coordinate| of the Lp / translation part (for the error bound)
__global__ void k_noalloc_convert(const double* __restrict__ pts, int n, int D, int metric, float* __restrict__ pts32,
                                  int* __restrict__ counters) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* s = pts + (size_t)i * D;
    bool bad = false;
    float mx = 0.f;
    for (int d = 0; d < D; ++d) {
        double v = s[d];
        if (!(v == v) || isinf(v)) bad = true;
        pts32[(size_t)i * D + d] = __double2float_rn(v);
        bool lp = metric == MPTG_METRIC_L2 || metric == MPTG_METRIC_L1 || (metric == MPTG_METRIC_SE3 && d >= 4);
        if (lp) mx = fmaxf(mx, __double2float_ru(fabs(v)));
        if (metric == MPTG_METRIC_SO2 && !(v >= -MPTG_PI && v <= MPTG_PI)) bad = true;
    }
    if (metric == MPTG_METRIC_SO3 || metric == MPTG_METRIC_SE3) {
        double nn = quat_dot64(s, s);
        if (!(fabs(nn - 1.0) <= MPTG_QUAT_NORM_TOL)) bad = true;
    }
    if (bad) atomicOr(&counters[1], 1);
    if (mx > 0.f) atomicMax(&counters[0], __float_as_int(mx));
}

// warp per query; the same FP32 sweep + FP64 re-rank as the tree's linear scan
template <int MK, int DMAX>
__global__ void __launch_bounds__(256) k_noalloc_linear(const double* __restrict__ pts64,
                                                        const float* __restrict__ pts32, int n, int D, double w0,
                                                        double w1, const int* __restrict__ counters,
                                                        const double* __restrict__ q64, int nq,
                                                        int* __restrict__ out_idx, double* __restrict__ out_d) {
    const int lane = threadIdx.x & 31;
    const int qi = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (qi >= nq) return;
    if (counters[1]) {  // invalid points: no answer for this call
        if (lane == 0) { out_idx[qi] = -1; out_d[qi] = __longlong_as_double(0x7ff8000000000000ll); }
        return;
    }
    const double* qd = q64 + (size_t)qi * D;
    const float w0f = (float)w0, w1f = (float)w1;
    float q[DMAX];
    float M = __int_as_float(counters[0]);
#pragma unroll
    for (int d = 0; d < DMAX; ++d) {
        float v = 0.f;
        if (d < D) v = __double2float_rn(qd[d]);
        q[d] = v;
        bool lp = MK == MPTG_METRIC_L2 || MK == MPTG_METRIC_L1 || (MK == MPTG_METRIC_SE3 && d >= 4 && d < 7);
        if (lp && d < D) M = fmaxf(M, __double2float_ru(fabs(qd[d])));
    }
    const float E = err32<MK>(D, M, w0f, w1f);
    double best = INFINITY;
    int bidx = INT_MAX;
    float bestf_up = INFINITY;
    for (int base = 0; base < n; base += 32) {
        int j = base + lane;
        bool have = j < n;
        float d32 = INFINITY;
        if (have) {
            float p[DMAX];
#pragma unroll
            for (int d = 0; d < DMAX; ++d) p[d] = d < D ? pts32[(size_t)j * D + d] : 0.f;
            d32 = dist32<MK, DMAX>(q, p, w0f, w1f);
            if (!(d32 == d32)) d32 = INFINITY;
        }
        // candidates: every point that could beat or tie the best in exact arithmetic
        float m = d32;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
        float thr = __fadd_ru(m, __fmul_ru(2.f, E));
        bool cand = have && __fsub_rd(d32, E) <= bestf_up && d32 <= thr;
        if (!__ballot_sync(0xffffffffu, cand)) continue;
        double dd = INFINITY;
        int pp = INT_MAX;
        if (cand) {
            dd = dist64(MK, D, w0, w1, qd, pts64 + (size_t)j * D);
            pp = j;
            if (!(dd == dd)) { dd = INFINITY; pp = INT_MAX; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double od = __shfl_xor_sync(0xffffffffu, dd, o);
            int op = __shfl_xor_sync(0xffffffffu, pp, o);
            if (od < dd || (od == dd && op < pp)) { dd = od; pp = op; }
        }
        if (pp != INT_MAX && (dd < best || (dd == best && pp < bidx))) {
            best = dd;
            bidx = pp;
            bestf_up = __double2float_ru(best);
        }
    }
    if (lane == 0) {
        out_idx[qi] = bidx == INT_MAX ? -1 : bidx;
        out_d[qi] = best;
    }
}

template <int MK, int DMAX>
void launch_noalloc(unsigned grid, cudaStream_t s, const double* pts, const float* pts32, int n, int D, double w0,
                    double w1, const int* counters, const double* q, int nq, int* idx, double* dist) {
    k_noalloc_linear<MK, DMAX><<<grid, 256, 0, s>>>(pts, pts32, n, D, w0, w1, counters, q, nq, idx, dist);
}

}  // namespace

extern "C" mptg_status mptg_nearest_linear_noalloc(mptg_ctx* ctx, mptg_metric metric, int dim,
                                                   const double* weights, const double* points, size_t n,
                                                   const double* queries, size_t nq, int32_t* idx_out,
                                                   double* dist_out, void* stream) {
    if (!ctx) return MPTG_ERR_INVALID_ARG;
    if (metric < MPTG_METRIC_L2 || metric > MPTG_METRIC_L1)
        return mptg_fail(ctx, MPTG_ERR_UNSUPPORTED_METRIC, "unknown metric %d", (int)metric);
    if (dim < 1 || dim > MPTG_MAX_DIM || (metric == MPTG_METRIC_SO3 && dim != 4) ||
        (metric == MPTG_METRIC_SE3 && dim != 7))
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "dimension %d does not fit metric %d", dim, (int)metric);
    if (n > MPTG_NOALLOC_MAX_POINTS)
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG,
                         "mptg_nearest_linear_noalloc takes at most %d points (got %zu): its working memory is a "
                         "fixed static array", MPTG_NOALLOC_MAX_POINTS, n);
    if (nq > (size_t)INT32_MAX / 32) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "too many queries");
    if (nq == 0) return MPTG_OK;
    const int dev = ctx->device;
    if ((n && !on_device(points, dev)) || !on_device(queries, dev) || !on_device(idx_out, dev) ||
        !on_device(dist_out, dev))
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG,
                         "mptg_nearest_linear_noalloc needs device buffers of the context's GPU %d (host buffers "
                         "would need staging memory; another GPU's buffers would need peer access)", dev);
    double w0 = weights ? weights[0] : 1.0, w1 = weights ? weights[1] : 1.0;
    if (metric == MPTG_METRIC_SE3 && !(w0 > 0 && w1 > 0))
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "SE3 weights must be positive");
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    float* scratch = nullptr;
    mptg_status st = scratch_address(ctx, &scratch);
    if (st != MPTG_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    float* pts32 = scratch;
    int* counters = (int*)(scratch + MPTG_NOALLOC_MAX_POINTS * MPTG_MAX_DIM);
    // the previous call's counters must not leak into this one
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(counters, 0, MPTG_NOALLOC_COUNTERS * sizeof(int), s));
    if (n) {
        k_noalloc_convert<<<mptg_blocks(n, 256), 256, 0, s>>>(points, (int)n, dim, metric, pts32, counters);
        MPTG_LAUNCHED(ctx);
    }
    unsigned grid = mptg_blocks(nq * 32, 256);
    int N = (int)n, Q = (int)nq;
    switch (metric) {
    case MPTG_METRIC_L2:
        if (dim <= 2) launch_noalloc<MPTG_METRIC_L2, 2>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        else if (dim <= 4) launch_noalloc<MPTG_METRIC_L2, 4>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        else if (dim <= 8) launch_noalloc<MPTG_METRIC_L2, 8>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        else launch_noalloc<MPTG_METRIC_L2, 16>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        break;
    case MPTG_METRIC_L1:
        if (dim <= 4) launch_noalloc<MPTG_METRIC_L1, 4>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        else launch_noalloc<MPTG_METRIC_L1, 16>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        break;
    case MPTG_METRIC_SO2:
        if (dim <= 4) launch_noalloc<MPTG_METRIC_SO2, 4>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        else launch_noalloc<MPTG_METRIC_SO2, 16>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        break;
    case MPTG_METRIC_SO3:
        launch_noalloc<MPTG_METRIC_SO3, 4>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        break;
    case MPTG_METRIC_SE3:
        launch_noalloc<MPTG_METRIC_SE3, 8>(grid, s, points, pts32, N, dim, w0, w1, counters, queries, Q, idx_out, dist_out);
        break;
    }
    MPTG_LAUNCHED(ctx);
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    return MPTG_OK;
}
