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
// Edge kernel: one warp per edge.  The DMV result is the AND of valid() over
// the fixed sample set {b} U {interpolate(a, b, i/steps) : 1 <= i < steps},
// so evaluation order does not change it; the warp takes 32 samples per round
// in a coarse-to-fine spread (lane j of round r tests sample j*R + r) and
// leaves as soon as a ballot sees an invalid sample.
//
// Exactness: every boolean equals the FP64 definition.  States are first
// decided in FP32 with an a-priori error margin; a state whose FP32 result
// lies inside the margin of a decision boundary is recomputed in FP64 with
// explicit round-to-nearest intrinsics (no FMA contraction) and the
// deterministic sin/cos of mptg_detmath.h, the same expressions the CPU
// checker evaluates.
#include "metrics.cuh"
#include "scene.cuh"

// ------------------------------------------------------------------ grid
__device__ __forceinline__ bool grid_valid64(const SceneView& s, const double* q) {
    double vx = __dadd_rn(q[0], 0.5), vy = __dadd_rn(q[1], 0.5);
    if (!(vx > -1.0 && vx < (double)s.width && vy > -1.0 && vy < (double)s.height)) return false;
    int x = __double2int_rz(vx), y = __double2int_rz(vy);
    return __ldg(&s.grid[(size_t)s.width * y + x]) == 0;
}

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

__device__ __forceinline__ bool state_valid64(const SceneView& s, const double* q) {
    switch (s.kind) {
    case MPTG_SCENE_GRID: return grid_valid64(s, q);
    case MPTG_SCENE_PLANAR_ARM: return arm_valid64(s, q);
    default: return false;
    }
}

// ------------------------------------------------------------------ kernels

__global__ void __launch_bounds__(256) k_valid_states(SceneView s, const double* __restrict__ q, int n,
                                                      uint8_t* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double st[MPTG_MAX_DIM];
    for (int d = 0; d < s.D; ++d) st[d] = q[(size_t)i * s.D + d];
    out[i] = state_valid64(s, st) ? 1 : 0;
}

// largest wrapped joint difference (planar-arm edge resolution)
__device__ __forceinline__ double linf_so2_64(const double* a, const double* b, int D) {
    double m = 0.0;
    for (int i = 0; i < D; ++i) {
        double d = so2_dist1_64(a[i], b[i]);
        if (d > m) m = d;
    }
    return m;
}

__global__ void __launch_bounds__(256) k_valid_edges(SceneView s, const double* __restrict__ a,
                                                     const double* __restrict__ b, int n, double inv, int resolution,
                                                     uint8_t* __restrict__ out, unsigned long long* __restrict__ nsamp) {
    const int lane = threadIdx.x & 31;
    const int e = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (e >= n) return;
    const int D = s.D;
    double A[MPTG_MAX_DIM], B[MPTG_MAX_DIM];
    for (int d = 0; d < D; ++d) { A[d] = a[(size_t)e * D + d]; B[d] = b[(size_t)e * D + d]; }
    double m = resolution == 1 ? linf_so2_64(A, B, D) : dist64(s.metric, D, s.w0, s.w1, A, B);
    double sd = ceil(__dmul_rn(m, inv));
    // steps as the reference's size_t; NaN distances make the edge invalid, and
    // so do edges needing more than MPTG_MAX_EDGE_SAMPLES samples (a bounded
    // kernel instead of the reference's unbounded loop)
    bool ok = true;
    long long steps = 0;
    if (!(sd >= 0.0) || sd > (double)MPTG_MAX_EDGE_SAMPLES) ok = false;
    else steps = (long long)sd;
    long long M = steps < 2 ? 1 : steps;  // sample 0 = b, samples 1..steps-1 interior
    double delta = steps >= 2 ? __ddiv_rn(1.0, (double)steps) : 0.0;
    long long R = (M + 31) / 32;
    unsigned long long cnt = 0;
    for (long long r = 0; ok && r < R; ++r) {
        long long k = (long long)lane * R + r;
        bool v = true;
        if (k < M) {
            ++cnt;
            if (k == 0) {
                v = state_valid64(s, B);
            } else {
                double qs[MPTG_MAX_DIM];
                interp64(s.metric, D, A, B, __dmul_rn((double)k, delta), qs);
                v = state_valid64(s, qs);
            }
        }
        if (__any_sync(0xffffffffu, !v)) ok = false;
    }
    if (nsamp) {
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
        out[e] = ok ? 1 : 0;
        if (nsamp) atomicAdd(nsamp, cnt);
    }
}

// ------------------------------------------------------------------ host

static void scene_free(mptg_scene* s) {
    void* ptrs[] = {s->grid, s->link_len64, s->discs64};
    for (void* p : ptrs)
        if (p) cudaFree(p);
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
    mesh_fill_view(s, &v);
    return v;
}

mptg_status scene_edges_dev(mptg_scene* sc, const double* da, const double* db, int n, double step, int resolution,
                            uint8_t* dout, cudaStream_t s, unsigned long long* nsamp) {
    if (n <= 0) return MPTG_OK;
    if (sc->kind == MPTG_SCENE_RIGID_MESH)
        return mesh_edges_dev(sc, da, db, n, step, resolution, dout, s, nsamp);
    SceneView v = scene_view(sc);
    k_valid_edges<<<mptg_blocks((size_t)n * 32, 256), 256, 0, s>>>(v, da, db, n, 1.0 / step, resolution, dout, nsamp);
    MPTG_LAUNCHED(sc->ctx);
    return MPTG_OK;
}

mptg_status scene_states_dev(mptg_scene* sc, const double* dq, int n, uint8_t* dout, cudaStream_t s) {
    if (n <= 0) return MPTG_OK;
    if (sc->kind == MPTG_SCENE_RIGID_MESH) return mesh_states_dev(sc, dq, n, dout, s);
    SceneView v = scene_view(sc);
    k_valid_states<<<mptg_blocks(n, 256), 256, 0, s>>>(v, dq, n, dout);
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
