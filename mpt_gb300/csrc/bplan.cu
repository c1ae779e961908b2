// bplan.cu - the wavefront PRRT as one persistent thread block per query.
//
// The multi-kernel wavefront of planner.cu spends most of a small query's
// time on launches and host round trips: a first path across the 1024^2 grid
// needs about 60 wavefronts, each of which is a handful of tiny kernels, two
// host synchronisations and a kd-tree insert.  This kernel runs the same
// wavefront loop -- PRRT::Worker::addSample of src/mpt/impl/prrt/prrt.hpp:
// 411-452 for W samples at once -- without leaving the GPU: one 1024-thread
// block per query, the tree's FP32 node copy in shared memory, every phase
// separated by a block barrier, and the stop conditions (solved, node budget,
// wavefront count, time) decided on the device.
//
// Per wavefront (identical, bit for bit, to plan_wavefront in planner.cu):
//   goal pick and samples   the Philox stream of sampler.cuh, sample i of
//                           wavefront w; at most one goal sample (the lowest
//                           i whose bias draw hits) until the first solution
//   nearest                 exact FP64 nearest node, lowest id on ties,
//                           over the FP32 node copy in shared memory: while
//                           W x nodes is small, an exhaustive FP32 sweep
//                           (four samples per node read) and an FP64 re-rank
//                           of the nodes within 2 err32 of the least; beyond
//                           that, groups of threads per sample over a bucket
//                           grid (cells searched in rings until the ring's
//                           distance bound passes the best), FP32 deciding
//                           wherever distances are 2 err32 apart
//   steer and link set-up   per sample, as soon as its nearest node is known
//                           (steer_setup): interpolate to `range` (skip when
//                           d == 0), then the DMV's end state and step count
//   link samples            the DMV's interior samples (scene.cu's phase B,
//                           a warp per edge, the same sample order and counts)
//   insert                  block scan of the accepted flags in sample order,
//                           node budget, parent ids, goal flags
// The kd-tree is brought up to date by the host after the block returns.
#include "bplan.cuh"
#include "grid.cuh"
#include "sampler.cuh"
#include "umma.cuh"

namespace {

struct BSmem {
    float2* pts;    // [cap] FP32 node copy
    double* q;      // [W][2] samples
    double* nw;     // [W][2] new states
    double* nd;     // [W] nearest distance
    int* ni;        // [W] nearest id (-1: none)
    int* fl;        // [W] bit 0 link valid, bit 1 skipped (d == 0)
    int* head;      // [BPLAN_CELLS] first node of each bucket-grid cell (-1: empty)
    int* ccount;    // [BPLAN_CELLS / 16] nodes in each block of 4 x 4 cells
    short* nxt;     // [cap] next node in the same cell (-1: end)
};

__device__ __forceinline__ BSmem carve(unsigned char* base, int cap, int W) {
    BSmem s;
    size_t o = 0;
    // the node copy is padded to 16 bytes: the link phase reads q as float4
    s.pts = reinterpret_cast<float2*>(base + o); o += (size_t)((cap + 1) & ~1) * sizeof(float2);
    s.q = reinterpret_cast<double*>(base + o); o += (size_t)W * 2 * sizeof(double);
    s.nw = reinterpret_cast<double*>(base + o); o += (size_t)W * 2 * sizeof(double);
    s.nd = reinterpret_cast<double*>(base + o); o += (size_t)W * sizeof(double);
    s.ni = reinterpret_cast<int*>(base + o); o += (size_t)W * sizeof(int);
    s.fl = reinterpret_cast<int*>(base + o); o += (size_t)W * sizeof(int);
    s.head = reinterpret_cast<int*>(base + o); o += (size_t)BPLAN_CELLS * sizeof(int);
    s.ccount = reinterpret_cast<int*>(base + o); o += (size_t)(BPLAN_CELLS / 16) * sizeof(int);
    s.nxt = reinterpret_cast<short*>(base + o);
    return s;
}

size_t smem_bytes(int cap, int W) {
    return (size_t)((cap + 1) & ~1) * sizeof(float2) + (size_t)W * (2 + 2 + 1) * sizeof(double) + (size_t)W * 2 * sizeof(int) +
           (size_t)(BPLAN_CELLS + BPLAN_CELLS / 16) * sizeof(int) + (size_t)cap * sizeof(short);
}

// bucket-grid cell of an FP32 point (clamped to the grid: a point outside the
// sampling box lands in a border cell, which only brings it nearer in cell
// distance, so the ring bounds below stay lower bounds)
__device__ __forceinline__ int cell_of(const BPlanJob& J, float x, float y, int* cx, int* cy) {
    int ix = (int)floorf((x - J.cell_ox) * J.cell_inv), iy = (int)floorf((y - J.cell_oy) * J.cell_inv);
    ix = min(max(ix, 0), J.gx - 1);
    iy = min(max(iy, 0), J.gy - 1);
    *cx = ix;
    *cy = iy;
    return iy * J.gx + ix;
}

// node j into its cell's list, its block's count and the cell rectangle of
// all nodes (bb: min x, max x, min y, max y)
__device__ __forceinline__ void bucket_insert(const BPlanJob& J, const BSmem& S, int* bb, int j) {
    int cx, cy;
    const float2 p = S.pts[j];
    const int c = cell_of(J, p.x, p.y, &cx, &cy);
    S.nxt[j] = (short)atomicExch(&S.head[c], j);
    atomicAdd(&S.ccount[(cy >> 2) * ((J.gx + 3) >> 2) + (cx >> 2)], 1);
    atomicMin(&bb[0], cx);
    atomicMax(&bb[1], cx);
    atomicMin(&bb[2], cy);
    atomicMax(&bb[3], cy);
}

// FP32 distance from q to the rectangle [x0, x1] x [y0, y1] (0 inside)
__device__ __forceinline__ float rect_dist(const float* q, float x0, float x1, float y0, float y1) {
    const float dx = fmaxf(fmaxf(x0 - q[0], q[0] - x1), 0.f), dy = fmaxf(fmaxf(y0 - q[1], q[1] - y1), 0.f);
    return sqrtf(dx * dx + dy * dy);
}

// Nearest-node search state of one sample.  The winner is kept by its FP32
// distance: a node whose FP32 distance lies more than 2E below the winner's
// is certainly nearer in FP64 as well (|d32 - d64| <= E), so it replaces the
// winner without any FP64 arithmetic; only a near tie (within 2E) computes
// both FP64 distances and compares (distance, id) as the FP64 search does.
// bup stays an upper bound of the winner's FP64 distance.  The FP64 distance
// of the final winner is computed once, by the steer step.
struct NNState {
    int wid = INT_MAX;      // winner (INT_MAX: none yet)
    float wd32 = INFINITY;  // its FP32 distance
    double wd64 = -1.0;     // its FP64 distance once computed (< 0: not yet)
    float bup = INFINITY;
};

// The nodes of one cell against the winner so far; gb, an upper bound of
// the FP64 distance of a node found by another thread of the group, prunes
// as well (a node beyond it cannot win).
__device__ __forceinline__ void scan_cell(const BPlanJob& J, const BSmem& S, int c, const float* q32, const double* qd,
                                          float E, NNState& st, float gb, unsigned long long* ties) {
    for (int j = S.head[c]; j >= 0; j = S.nxt[j]) {
        const float2 pj = S.pts[j];
        const float p32[2] = {pj.x, pj.y};
        const float d32 = dist32<MPTG_METRIC_L2, 2>(q32, p32, 1.f, 1.f);
        const float lo = __fsub_rd(d32, E);
        if (!(lo <= st.bup) || lo > gb) continue;  // cannot beat or tie a winner (or NaN)
        if (st.wid == INT_MAX || __fadd_ru(d32, E) < __fsub_rd(st.wd32, E)) {
            st.wid = j;
            st.wd32 = d32;
            st.wd64 = -1.0;
            st.bup = __fadd_ru(d32, E);
            continue;
        }
        atomicAdd(ties, 1ull);
        if (st.wd64 < 0.0) st.wd64 = l2_dist64(qd, J.states + 2 * st.wid, 2);
        const double d = l2_dist64(qd, J.states + 2 * j, 2);
        if (d < st.wd64 || (d == st.wd64 && j < st.wid)) {
            st.wid = j;
            st.wd32 = d32;
            st.wd64 = d;
        }
        st.bup = __double2float_ru(st.wd64);
    }
}

// The exact winner of a group (lowest FP64 distance, then lowest id) from its
// threads' winners: a thread whose winner's lower bound exceeds another's
// upper bound cannot hold it; the one thread left, or else the FP64
// distances of the ones left, decide.  The winning thread writes the id to
// S.ni[g] and its FP64 distance to S.nd[g] (-1 when not yet computed; -1 id
// and INFINITY without any node).
__device__ __forceinline__ void nn_group_winner(const BPlanJob& J, const BSmem& S, int g, int r, int G, unsigned gmask,
                                                const double* qd, float E, NNState& st) {
    const bool have = st.wid != INT_MAX;
    const float up = !have ? INFINITY : st.wd64 >= 0.0 ? __double2float_ru(st.wd64) : __fadd_ru(st.wd32, E);
    const float lo = !have ? INFINITY : st.wd64 >= 0.0 ? __double2float_rd(st.wd64) : __fsub_rd(st.wd32, E);
    float U = up;
    for (int o = 1; o < G; o <<= 1) U = fminf(U, __shfl_xor_sync(gmask, U, o));
    const bool cont = have && lo <= U;
    const unsigned cm = __ballot_sync(gmask, cont) & gmask;
    if (cm == 0) {  // no node in the tree
        if (r == 0) {
            S.ni[g] = -1;
            S.nd[g] = INFINITY;
        }
        return;
    }
    if (__popc(cm) == 1) {
        if (cont) {
            S.ni[g] = st.wid;
            S.nd[g] = st.wd64;
        }
        return;
    }
    double d = INFINITY;
    int id = INT_MAX;
    if (cont) {
        if (st.wd64 < 0.0) st.wd64 = l2_dist64(qd, J.states + 2 * st.wid, 2);
        d = st.wd64;
        id = st.wid;
    }
    for (int o = 1; o < G; o <<= 1) {
        const double od = __shfl_xor_sync(gmask, d, o);
        const int oi = __shfl_xor_sync(gmask, id, o);
        if (od < d || (od == d && oi < id)) {
            d = od;
            id = oi;
        }
    }
    if (r == 0) {
        S.ni[g] = id;
        S.nd[g] = d;
    }
}

__device__ __forceinline__ float maxabs_ru(double x, double y) {
    return fmaxf(__double2float_ru(fabs(x)), __double2float_ru(fabs(y)));
}

// Squared FP32 distance, evaluated as dist32<L2, 2> evaluates it before its
// square root.  sqrtf is correctly rounded and so monotone: the node with the
// least squared value has the least dist32, and sqrtf of the least squared
// value is the least dist32 itself.
__device__ __forceinline__ float sq32(float qx, float qy, float2 p) {
    const float tx = qx - p.x, ty = qy - p.y;
    return fmaf(ty, ty, fmaf(tx, tx, 0.f));
}

// The nearest search's per-sample slots, laid over the bucket grid's cell
// heads (16 KB, 16 bytes per sample), which only the ring search uses; a
// wavefront that runs the ring search rebuilds the grid first.
struct BruteSlots {
    int* cnt;       // [W] candidates of each sample (pass 2)
    float* maxabs;  // [W] largest |coordinate| of the sample, rounded up
    float2* q32;    // [W] the sample rounded to FP32
};
static_assert(BPLAN_THREADS * 16 <= BPLAN_CELLS * 4, "the per-sample slots fit over the cell heads");
__device__ __forceinline__ BruteSlots brute_slots(const BSmem& S, int W) {
    unsigned char* base = reinterpret_cast<unsigned char*>(S.head);
    return BruteSlots{reinterpret_cast<int*>(base), reinterpret_cast<float*>(base + 4 * (size_t)W),
                      reinterpret_cast<float2*>(base + 8 * (size_t)W)};
}

// Steer and the link set-up of sample t, whose nearest node is id (INT_MAX or
// -1: none) at FP64 distance best (< 0: not computed yet).  Steer as
// k_plan_steer (prrt.hpp:425-435): skip when d == 0, else interpolate from
// the node to `range`; then phase A of the grid DMV (k_grid_edges_a): the end
// state, the step count and the FP32 set-up of the interior samples, all the
// FP64 work of the edge.  Everything it reads or writes belongs to sample t
// (S.q / S.nd slots t, which take the set-up, S.nw, S.fl, S.ni), so threads
// may run it for different samples without a barrier between the steps.
__device__ void steer_setup(const BPlanJob& J, const BSmem& S, int t, int id, double best,
                            unsigned long long* steps64) {
    if (id == INT_MAX) id = -1;
    S.ni[t] = id;
    const double s[2] = {S.q[2 * t], S.q[2 * t + 1]};
    double A[2] = {s[0], s[1]};
    if (id >= 0) {
        A[0] = J.states[2 * id];
        A[1] = J.states[2 * id + 1];
        if (best < 0.0) best = l2_dist64(s, A, 2);
    }
    double B[2];
    const bool skip = id < 0 || best == 0.0 || !(best == best);  // prrt.hpp:425
    if (!skip && best > J.range) {
        interp64(MPTG_METRIC_L2, 2, A, s, __ddiv_rn(J.range, best), B);
    } else {
        B[0] = s[0];
        B[1] = s[1];
    }
    if (skip) {  // the edge of a skipped sample starts at the sample itself
        A[0] = s[0];
        A[1] = s[1];
    }
    S.nw[2 * t] = B[0];
    S.nw[2 * t + 1] = B[1];
    bool ok = grid_valid_f(J.scene, B);
    bool used64 = false;
    long long steps = ok ? grid_edge_steps(A, B, J.inv_step, &used64) : 0;
    if (used64) atomicAdd(steps64, 1ull);
    if (steps < 0) ok = false;
    float4 setup = make_float4(0.f, 0.f, 0.f, 0.f);
    float eps = 0.f;
    if (ok && steps >= 2) {
        setup = make_float4(__double2float_rn(A[0]), __double2float_rn(A[1]),
                            __double2float_rn(__dsub_rn(B[0], A[0])), __double2float_rn(__dsub_rn(B[1], A[1])));
        eps = 8.f * U32 * (fabsf(setup.x) + fabsf(setup.y) + fabsf(setup.z) + fabsf(setup.w) + 1.f);
    } else {
        steps = 0;
    }
    reinterpret_cast<float4*>(S.q)[t] = setup;
    reinterpret_cast<float2*>(S.nd)[t] = make_float2(eps, __int_as_float((int)steps));
    S.fl[t] = (skip ? 2 : 0) | (ok ? 1 : 0);
}

// The pass-2 bound of one sample: (min32 + 2E)^2 (1 + 2^-21), each step
// rounded up, with min32 the sqrt of the sample's least squared FP32 distance
// (S.fl) and E the FP32 error bound for its coordinates and the tree's.  Every
// node whose correctly rounded dist32 is within min32 + 2E has its squared
// value within this bound (sqrtf is off by at most half an ulp).
__device__ __forceinline__ float brute_thr2(const BSmem& S, const BruteSlots& B, int s, float maxabs) {
    const float M = fmaxf(maxabs, B.maxabs[s]);
    const float E = err32<MPTG_METRIC_L2>(2, M, 1.f, 1.f);
    const float thr = __fadd_ru(sqrtf(__int_as_float(S.fl[s])), __fmul_ru(2.f, E));
    return __fmul_ru(__fmul_ru(thr, thr), 1.0000005f);
}

// Exhaustive nearest-node search for small wavefronts on small trees, where
// the ring search spends its time walking cell lists.  Samples go in groups
// of four; the P threads of a group (a power of two, all the block's threads
// shared out) each take every P-th node of the FP32 copy, so a node read from
// shared memory serves four distances.
//   pass 1  per thread and sample, the least squared FP32 distance over its
//           nodes, that node, and the second least; the least over the
//           block's threads is min32 squared;
//   pass 2  the candidates of each sample, the nodes with dist32 <= min32 + 2E
//           (squared, against brute_thr2): a thread's least is one, and a
//           thread whose second least is one as well holds two or more, so
//           the count is exact up to two and the lowest id of a sole
//           candidate is known without a second sweep;
//   pass 3  a sample with two or more candidates gets a warp, which sweeps
//           all nodes again, gathers the candidates into lanes and ranks them
//           by (FP64 distance, id).
// The exact winner p* has dist32(p*) <= d64(p*) + E <= d64(argmin32) + E <=
// min32 + 2E, and so does every node that ties it in FP64, so the candidates
// hold all of them: the result is the FP64 argmin with the lowest id, the
// ring search's answer.  A sole candidate is the winner without any FP64
// arithmetic; its FP64 distance is computed by steer_setup, which thread s
// runs for sample s, one lane per sample.  The FP64 pipe costs the same per
// warp instruction however few lanes are active, so FP64 work is kept to
// full warps wherever it is not a single sample's own chain.  Each sample's
// steer and link set-up (steer_setup) run as soon as its winner is known, by
// the warp that ranked it or by thread s, with no barrier in between, so the
// FP64 chains of different samples overlap with each other and with pass 3.
// On entry S.fl[s] holds +inf (FP32 bits), S.ni[s] INT_MAX and the slots
// (brute_slots) a zero count and the sample in FP32 for every sample s < W;
// on return every sample has been through steer_setup.  Every thread of the
// block calls this.
__device__ void nn_brute(const BPlanJob& J, const BSmem& S, int W, int n, float maxabs,
                         unsigned long long* fp64_evals, unsigned long long* steps64) {
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int NG = (W + 3) >> 2;
    int P = 1;
    while (2 * P * NG <= T) P <<= 1;
    const int g = t / P, r = t % P, s0 = 4 * g;
    const int PW = P < 32 ? P : 32;  // lanes of a group within one warp
    const BruteSlots B = brute_slots(S, W);
    int* cnt = B.cnt;
    float qx[4], qy[4], m[4];
    bool act[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        act[k] = g < NG && s0 + k < W;
        const float2 q = B.q32[act[k] ? s0 + k : 0];
        qx[k] = q.x;
        qy[k] = q.y;
        m[k] = INFINITY;
    }
    // per sample: the least squared distance of this thread's nodes, its node
    // and the second least (a second node within the bound needs pass 3)
    float m2[4];
    int id[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        m2[k] = INFINITY;
        id[k] = INT_MAX;
    }
    const int jstart = g < NG ? r : n;
#pragma unroll 2
    for (int j = jstart; j < n; j += P) {
        const float2 p = S.pts[j];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float sq = sq32(qx[k], qy[k], p);
            const bool lt = sq < m[k];
            m2[k] = fminf(m2[k], fmaxf(sq, m[k]));
            m[k] = fminf(m[k], sq);
            id[k] = lt ? j : id[k];
        }
    }
    float mw[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        mw[k] = m[k];
        for (int o = 1; o < PW; o <<= 1) mw[k] = fminf(mw[k], __shfl_xor_sync(0xffffffffu, mw[k], o));
        if (act[k] && (lane & (PW - 1)) == 0 && mw[k] < INFINITY) atomicMin(&S.fl[s0 + k], __float_as_int(mw[k]));
    }
    __syncthreads();
    // candidates: a thread whose second least lies within the bound holds two
    // or more; otherwise it holds its least alone, or none
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!act[k]) continue;
        const float thr2 = brute_thr2(S, B, s0 + k, maxabs);
        const int c = (m[k] <= thr2 ? 1 : 0) + (m2[k] <= thr2 ? 1 : 0);
        if (!c) continue;
        atomicAdd(&cnt[s0 + k], c);
        atomicMin(&S.ni[s0 + k], id[k]);
    }
    __syncthreads();
    const int nwarps = T >> 5;
    unsigned long long evals = 0;
    for (int s = warp; s < W; s += nwarps) {
        if (cnt[s] < 2) continue;
        const double* qd = S.q + 2 * s;
        const float t2 = brute_thr2(S, B, s, maxabs);
        const float sx = B.q32[s].x, sy = B.q32[s].y;
        // best (FP64 distance bits, id): non-negative doubles order as their bits
        long long bk = LLONG_MAX;
        int bid = INT_MAX;
        int myc = -1, nc = 0;  // candidate held by this lane; candidates held
        auto flush = [&]() {
            long long key = LLONG_MAX;
            int cid = INT_MAX;
            if (myc >= 0) {
                key = __double_as_longlong(l2_dist64(qd, J.states + 2 * myc, 2));
                cid = myc;
            }
            for (int o = 16; o > 0; o >>= 1) {
                const long long ok = __shfl_xor_sync(0xffffffffu, key, o);
                const int oi = __shfl_xor_sync(0xffffffffu, cid, o);
                if (ok < key || (ok == key && oi < cid)) {
                    key = ok;
                    cid = oi;
                }
            }
            if (key < bk || (key == bk && cid < bid)) {
                bk = key;
                bid = cid;
            }
            evals += (unsigned long long)nc;
            myc = -1;
            nc = 0;
        };
        for (int base = 0; base < n; base += 32) {
            const int j = base + lane;
            unsigned mask = __ballot_sync(0xffffffffu, j < n && sq32(sx, sy, S.pts[j < n ? j : 0]) <= t2);
            while (mask) {
                const int b = __ffs(mask) - 1;
                mask &= mask - 1;
                if (lane == nc) myc = base + b;
                if (++nc == 32) flush();
            }
        }
        if (nc) flush();
        __syncwarp();
        if (lane == 0) steer_setup(J, S, s, bid, __longlong_as_double(bk), steps64);
    }
    if (lane == 0 && evals) atomicAdd(fp64_evals, evals);
    // a sole candidate (S.ni) is the winner; its FP64 distance is computed by
    // steer_setup, one lane per sample
    if (t < W && cnt[t] < 2) steer_setup(J, S, t, S.ni[t], -1.0, steps64);
}

// GoalState's test d(q, goal) <= radius in FP64, decided by the FP32 distance
// wherever it lies farther than its error bound E from the radius:
// d64 >= d32 - E > radius, or d64 <= d32 + E < radius.  Only a state within E
// of the goal sphere computes the FP64 distance.
__device__ __forceinline__ bool goal_reached(const double* q, const double* goal, double radius) {
    const float a[2] = {__double2float_rn(q[0]), __double2float_rn(q[1])};
    const float b[2] = {__double2float_rn(goal[0]), __double2float_rn(goal[1])};
    const float d32 = dist32<MPTG_METRIC_L2, 2>(a, b, 1.f, 1.f);
    const float E = err32<MPTG_METRIC_L2>(2, fmaxf(maxabs_ru(q[0], q[1]), maxabs_ru(goal[0], goal[1])), 1.f, 1.f);
    if (__fsub_rd(d32, E) > __double2float_ru(radius)) return false;
    if (__fadd_ru(d32, E) < __double2float_rd(radius)) return true;
    return dist64(MPTG_METRIC_L2, 2, 1.0, 1.0, q, goal) <= radius;
}

// cap_alloc / W_alloc: the shared-memory layout of this launch (the largest
// job's); every job of the launch fits in it
__global__ void __launch_bounds__(BPLAN_THREADS, 1) k_bplan_grid(const BPlanJob* __restrict__ jobs, int cap_alloc,
                                                                 int W_alloc) {
    static_assert(BPLAN_MAX_NODES <= 32767, "node ids are kept as short in the cell lists");
    extern __shared__ __align__(16) unsigned char bp_smem[];
    __shared__ int s_n, s_goals, s_maxabs, s_stop, s_total;
    __shared__ int s_gidx[2];  // goal sample of the wavefronts of even / odd index
    __shared__ int s_wsum[32];
    __shared__ int s_bb[4];
    __shared__ unsigned long long s_prof[3];  // FP64 fallbacks: near ties, unsure samples, step counts
    __shared__ unsigned long long s_cnt;
    const BPlanJob& J = jobs[blockIdx.x];
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5, nwarps = T >> 5;
    const int W = J.W, cap = J.cap;
    int G = 1;  // threads per sample in the nearest search
    while (G < 32 && 2 * G * W <= T) G <<= 1;
    const BSmem S = carve(bp_smem, cap_alloc, W_alloc);
    if (t == 0) {
        s_n = J.ctr->n;
        s_goals = J.ctr->goals;
        s_maxabs = 0;
        s_cnt = 0;
        s_prof[0] = s_prof[1] = s_prof[2] = 0;
        s_bb[0] = s_bb[2] = INT_MAX;
        s_bb[1] = s_bb[3] = -1;
        s_gidx[0] = s_gidx[1] = INT_MAX;
    }
    __syncthreads();
    for (int j = t; j < s_n; j += T) {
        const double x = J.states[2 * j], y = J.states[2 * j + 1];
        S.pts[j] = make_float2(__double2float_rn(x), __double2float_rn(y));
        atomicMax(&s_maxabs, __float_as_int(maxabs_ru(x, y)));
    }
    uint32_t wave = J.ctr->wave;
    int waves_run = 0, status = BPLAN_DONE;
    unsigned long long samples = 0, accepted = 0;
    unsigned long long cyc[6] = {0, 0, 0, 0, 0, 0}, tc = 0;  // phase cycles, kept by thread 0
    // thread 0, after a barrier: the cycles since the last mark go to phase i
    auto mark = [&](int i) {
        if (t == 0) {
            const unsigned long long c = clock64();
            cyc[i] += c - tc;
            tc = c;
        }
    };
    const uint64_t t0 = umma::globaltimer_ns();
    __syncthreads();
    for (;;) {
        // goal sample: the lowest index whose bias draw hits (k_plan_goalpick),
        // gathered before the stop check's barrier into this wavefront's slot
        // (the other slot is cleared for the next wavefront meanwhile)
        const bool bias_on = s_goals == 0 && J.has_goal && J.goal_bias > 0;
        if (bias_on && t < W && phx_uniform(J.seed, (uint32_t)t, wave, 16) < J.goal_bias)
            atomicMin(&s_gidx[wave & 1], t);
        // the run loop's stop checks (mptg_planner_run), decided by one thread
        if (t == 0) {
            int st = 0;
            if (J.stop_when_solved && s_goals > 0) st = 1;
            else if ((size_t)s_n >= J.max_nodes) st = 1;
            else if (J.max_waves > 0 && waves_run >= J.max_waves) st = 1;
            else if ((size_t)s_n + (size_t)W > (size_t)cap && (size_t)cap < J.max_nodes) st = 2;
            else if (J.deadline_ns && umma::globaltimer_ns() - t0 >= J.deadline_ns) st = 1;
            s_stop = st;
            s_gidx[(wave + 1) & 1] = INT_MAX;
        }
        __syncthreads();
        if (s_stop) {
            status = s_stop == 2 ? BPLAN_FULL : BPLAN_DONE;
            break;
        }
        if (t == 0) tc = clock64();
        const int n = s_n;
        if (t < W) {
            double* q = S.q + 2 * t;
            if (bias_on && t == s_gidx[wave & 1]) {
                q[0] = J.goal[0];
                q[1] = J.goal[1];
            } else {
                sample_uniform_state(MPTG_METRIC_L2, 2, J.seed, (uint32_t)t, wave, J.lo, J.hi, q);
            }
            // the exhaustive search's per-sample slots (nn_brute): its FP32
            // copy of the sample and the sample's largest |coordinate|, made
            // here by one thread per sample, so that the search converts no
            // double (conversions from FP64 use the slow FP64 pipe)
            S.fl[t] = 0x7f800000;
            S.nd[t] = INFINITY;
            S.ni[t] = INT_MAX;
            const BruteSlots b = brute_slots(S, W);
            b.cnt[t] = 0;
            b.maxabs[t] = maxabs_ru(q[0], q[1]);
            b.q32[t] = make_float2(__double2float_rn(q[0]), __double2float_rn(q[1]));
        }
        __syncthreads();
        mark(0);
        // nearest: a group of G threads per sample (G = 1024 / W rounded down
        // to a power of two, at most 32) over the bucket grid, two levels:
        // blocks of 4 x 4 cells in rings of growing Chebyshev distance around
        // the sample's block, clipped to the blocks that hold nodes (s_bb),
        // the (block, cell) pairs of a ring dealt round-robin to the group.
        // A block or cell whose rectangle lies farther than the group's best
        // (less the boundary fuzz and E) holds no node that can reach it; a
        // block R >= 1 rings out lies at least (R - 1) blocks away, which ends
        // the search.  The group's winner is then exact (nn_group_winner).
        if ((long long)W * n <= J.brute_pairs) {
            nn_brute(J, S, W, n, __int_as_float(s_maxabs), &s_prof[0], &s_prof[2]);
        } else {
            // the bucket grid of the n nodes, built for this wavefront (the
            // exhaustive search keeps its per-sample slots over the cell heads)
            for (int c = t; c < J.gx * J.gy; c += T) S.head[c] = -1;
            for (int c = t; c < BPLAN_CELLS / 16; c += T) S.ccount[c] = 0;
            if (t == 0) {
                s_bb[0] = s_bb[2] = INT_MAX;
                s_bb[1] = s_bb[3] = -1;
            }
            __syncthreads();
            for (int j = t; j < n; j += T) bucket_insert(J, S, s_bb, j);
            __syncthreads();
            const int g = t / G, r = t % G;
            if (g < W) {
                const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
                const double* qd = S.q + 2 * g;
                const float q32[2] = {__double2float_rn(qd[0]), __double2float_rn(qd[1])};
                const float M = fmaxf(__int_as_float(s_maxabs), maxabs_ru(qd[0], qd[1]));
                const float E = err32<MPTG_METRIC_L2>(2, M, 1.f, 1.f);
                const float cs = J.cell_size, fuzz = 1e-3f * cs + 1e-3f;
                const int bgx = (J.gx + 3) >> 2;
                NNState st;
                float gb = INFINITY;  // the group's best upper bound, as of the last ring
                int cx, cy;
                cell_of(J, q32[0], q32[1], &cx, &cy);
                const int bx = cx >> 2, by = cy >> 2;
                const int X0 = s_bb[0] >> 2, X1 = s_bb[1] >> 2, Y0 = s_bb[2] >> 2, Y1 = s_bb[3] >> 2;
                if (X0 <= X1) {
                    // rings nearer than the node blocks' rectangle are empty
                    const int R0 = max(max(X0 - bx, bx - X1), max(max(Y0 - by, by - Y1), 0));
                    const int Rmax = max(max(bx - X0, X1 - bx), max(by - Y0, Y1 - by));
                    for (int R = R0; R <= Rmax; ++R) {
                        if (R >= 1 && (float)(R - 1) * 4.f * cs - fuzz - E > gb) break;
                        // ring R within [X0, X1] x [Y0, Y1]: top row, bottom row, left and right columns
                        const int xa = max(bx - R, X0), xb = min(bx + R, X1);
                        const int ya = max(by - R + 1, Y0), yb = min(by + R - 1, Y1);
                        const int nrow = xb >= xa ? xb - xa + 1 : 0, ncol = yb >= ya ? yb - ya + 1 : 0;
                        const int ntop = (by - R >= Y0 && by - R <= Y1) ? nrow : 0;
                        const int nbot = (R > 0 && by + R >= Y0 && by + R <= Y1) ? nrow : 0;
                        const int nlft = (R > 0 && bx - R >= X0 && bx - R <= X1) ? ncol : 0;
                        const int nrgt = (R > 0 && bx + R >= X0 && bx + R <= X1) ? ncol : 0;
                        const int nb = ntop + nbot + nlft + nrgt;
                        for (int f = r; f < 16 * nb; f += G) {
                            int k = f >> 4, X, Y;
                            if (k < ntop) { X = xa + k; Y = by - R; }
                            else if ((k -= ntop) < nbot) { X = xa + k; Y = by + R; }
                            else if ((k -= nbot) < nlft) { X = bx - R; Y = ya + k; }
                            else { X = bx + R; Y = ya + (k - nlft); }
                            if (S.ccount[Y * bgx + X] == 0) continue;
                            const float cap = fminf(st.bup, gb);
                            const float x0 = J.cell_ox + (float)(4 * X) * cs, y0 = J.cell_oy + (float)(4 * Y) * cs;
                            if (rect_dist(q32, x0, x0 + 4.f * cs, y0, y0 + 4.f * cs) - fuzz - E > cap) continue;
                            const int x = 4 * X + (f & 3), y = 4 * Y + ((f >> 2) & 3);
                            if (x >= J.gx || y >= J.gy) continue;
                            const int c = y * J.gx + x;
                            if (S.head[c] < 0) continue;
                            const float fx = J.cell_ox + (float)x * cs, fy = J.cell_oy + (float)y * cs;
                            if (rect_dist(q32, fx, fx + cs, fy, fy + cs) - fuzz - E > cap) continue;
                            scan_cell(J, S, c, q32, qd, E, st, gb, &s_prof[0]);
                        }
                        float b = st.bup;
                        for (int o = 1; o < G; o <<= 1) b = fminf(b, __shfl_xor_sync(gmask, b, o));
                        gb = b;
                    }
                }
                nn_group_winner(J, S, g, r, G, gmask, qd, E, st);
            }
            __syncthreads();
            if (t < W) steer_setup(J, S, t, S.ni[t], S.nd[t], &s_prof[2]);
        }
        __syncthreads();
        mark(1);  // nearest search, steer and link set-up
        for (int e = warp; e < W; e += nwarps) {
            const float2 es = reinterpret_cast<const float2*>(S.nd)[e];
            const int steps = __float_as_int(es.y);
            unsigned long long cnt = 1;
            if (steps >= 2) {
                const float4 su = reinterpret_cast<const float4*>(S.q)[e];
                const float eps = es.x;
                const int Mi = steps - 1;
                const int R = (Mi + 31) / 32;
                bool ok = true;
                unsigned long long lc = 0;
                for (int r = 0; ok && r < R; ++r) {
                    const int k = 1 + lane * R + r;
                    bool v = true;
                    if (k <= Mi) {
                        ++lc;
                        const float tt = (float)k / (float)steps;
                        const int res = grid_valid32(J.scene, fmaf(su.z, tt, su.x), fmaf(su.w, tt, su.y), eps);
                        if (res == VF_UNSURE) {
                            atomicAdd(&s_prof[1], 1ull);
                            // the exact FP64 sample, as the CPU checker computes it
                            const int id = S.ni[e];
                            const double A[2] = {J.states[2 * id], J.states[2 * id + 1]};
                            const double B[2] = {S.nw[2 * e], S.nw[2 * e + 1]};
                            double qs[2];
                            interp64(MPTG_METRIC_L2, 2, A, B, __dmul_rn((double)k, __ddiv_rn(1.0, (double)steps)), qs);
                            v = grid_valid64(J.scene, qs);
                        } else {
                            v = res == VF_VALID;
                        }
                    }
                    if (__any_sync(0xffffffffu, !v)) ok = false;
                }
                for (int o = 16; o > 0; o >>= 1) lc += __shfl_xor_sync(0xffffffffu, lc, o);
                cnt += lc;
                if (lane == 0 && !ok) S.fl[e] &= ~1;
            }
            if (lane == 0 && J.nsamp) atomicAdd(&s_cnt, cnt);
        }
        __syncthreads();
        mark(4);
        // accepted samples in sample order (k_plan_scan / k_plan_scatter);
        // a wavefront of at most 32 samples lies in warp 0, whose ballot is
        // the whole scan (no barrier), others take a block scan of the warps
        const int f = (t < W && S.fl[t] == 1) ? 1 : 0;
        const unsigned m = __ballot_sync(0xffffffffu, f);
        const size_t room = J.max_nodes - (size_t)n;
        int keep = 0, base = 0;
        if (W <= 32) {
            const int nacc = __popc(m);  // warp 0's; the other warps hold no sample
            keep = (size_t)nacc > room ? (int)room : nacc;
        } else {
            if (lane == 0) s_wsum[warp] = __popc(m);
            __syncthreads();
            if (warp == 0) {
                const int v = lane < nwarps ? s_wsum[lane] : 0;
                int x = v;
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                s_wsum[lane] = x - v;
                if (lane == 31) s_total = x;
            }
            __syncthreads();
            const int nacc = s_total;
            keep = (size_t)nacc > room ? (int)room : nacc;  // node budget: the first accepted samples
            base = s_wsum[warp];
        }
        if (f) {
            const int pos = base + __popc(m & ((1u << lane) - 1u));
            if (pos < keep) {
                const int id = n + pos;
                const double* nw = S.nw + 2 * t;
                J.states[2 * id] = nw[0];
                J.states[2 * id + 1] = nw[1];
                S.pts[id] = make_float2(__double2float_rn(nw[0]), __double2float_rn(nw[1]));
                J.parent[id] = S.ni[t];
                // GoalState::operator() (src/mpt/goal_state.hpp:64-69): d <= radius
                const uint8_t g = J.has_goal && goal_reached(nw, J.goal, J.goal_radius) ? 1 : 0;
                J.goalf[id] = g;
                if (g) atomicAdd(&s_goals, 1);
                atomicMax(&s_maxabs, __float_as_int(maxabs_ru(nw[0], nw[1])));
            }
        }
        __syncthreads();
        if (t == 0) s_n = n + keep;
        samples += (unsigned long long)W;
        accepted += (unsigned long long)keep;
        ++waves_run;
        ++wave;
        __syncthreads();
        mark(5);
    }
    if (t == 0) {
        J.ctr->n = s_n;
        J.ctr->wave = wave;
        J.ctr->goals = s_goals;
        J.ctr->maxabs_bits = s_maxabs;
        J.ctr->status = status;
        J.ctr->waves_run = waves_run;
        J.ctr->samples = samples;
        J.ctr->accepted = accepted;
        for (int i = 0; i < 6; ++i) J.ctr->cyc[i] = cyc[i];
        J.ctr->ties = s_prof[0];
        J.ctr->unsure = s_prof[1];
        J.ctr->steps64 = s_prof[2];
        J.ctr->start_ns = t0;
        J.ctr->end_ns = umma::globaltimer_ns();
        if (J.nsamp) atomicAdd(J.nsamp, s_cnt);
    }
}

}  // namespace

bool bplan_supported(const mptg_scene* sc, int wavefront, int resolution) {
    return sc->kind == MPTG_SCENE_GRID && resolution == 0 && wavefront >= 1 && wavefront <= BPLAN_THREADS;
}

mptg_status bplan_configure(mptg_ctx* ctx) {
    // the caller has made ctx's device current (and may be capturing a graph,
    // so nothing here may change the device)
    MPTG_CUDA_TRY(ctx, mptg_once_per_device((const void*)k_bplan_grid, [] {
        return cudaFuncSetAttribute(k_bplan_grid, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem_bytes(BPLAN_MAX_NODES, BPLAN_THREADS));
    }));
    return MPTG_OK;
}

mptg_status bplan_launch(mptg_ctx* ctx, const BPlanJob* djobs, int njobs, int max_W, int max_cap, cudaStream_t s,
                         bool configure) {
    if (njobs <= 0) return MPTG_OK;
    if (max_W < 1 || max_W > BPLAN_THREADS || max_cap < 1 || max_cap > BPLAN_MAX_NODES)
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "block planner: wavefront %d / capacity %d out of range", max_W,
                         max_cap);
    const size_t bytes = smem_bytes(max_cap, max_W);
    if (configure) {
        mptg_status st = bplan_configure(ctx);
        if (st) return st;
    }
    k_bplan_grid<<<njobs, BPLAN_THREADS, bytes, s>>>(djobs, max_cap, max_W);
    MPTG_LAUNCHED(ctx);
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    return MPTG_OK;
}
