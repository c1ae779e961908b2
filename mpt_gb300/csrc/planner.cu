// planner.cu - the PRRT worker loop as GPU wavefronts.
//
// Replaces Worker::solve / addSample of src/mpt/impl/prrt/prrt.hpp:358-452
// (and the WorkerPool of src/mpt/impl/worker_pool_openmp.hpp:101-129).  One
// wavefront draws W samples at once and runs, batched on the device:
//   sample (uniform box / SO(2) / Shoemake SO(3); goal with probability
//     goalBias until the first solution, prrt.hpp:363-389)
//   -> nearest over the tree as it stood before the wavefront (prrt.hpp:416)
//   -> skip if d == 0 (:425); steer to `range` with interpolate (:430-434)
//   -> valid(new) and link(near, new) through the DMV (:439-442)
//   -> goal test GoalState(radius) (:443-445) -> insert with parent (:447)
// Accepted samples are compacted in sample order, so a wavefront is a pure
// function of (seed, wavefront index, tree): the CPU checker replays it
// exactly.  Unlike the reference's concurrent workers, samples of one
// wavefront do not see each other's new nodes.
#include "metrics.cuh"
#include "scene.cuh"
#include "tree.cuh"
#include "sampler.cuh"
#include "bplan.cuh"
#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <numeric>
#include <thread>

#define PLAN_SCAN_BLOCK 1024

struct PlanView {
    int D, metric;
    double w0, w1;
    const double* lo;
    const double* hi;
    const double* goal;
    int has_goal;
    double goal_bias, range, goal_radius;
    uint64_t seed;
};

struct mptg_planner {
    mptg_ctx* ctx = nullptr;
    mptg_scene* scene = nullptr;
    mptg_tree* tree = nullptr;
    mptg_plan_params prm{};
    int D = 0, metric = 0;
    double w0 = 1, w1 = 1;
    double* lo = nullptr;
    double* hi = nullptr;
    double* goal = nullptr;
    int has_goal = 0;
    std::vector<double> goal_host;
    double lo_host[MPTG_MAX_DIM] = {0}, hi_host[MPTG_MAX_DIM] = {0};  // sampling bounds
    int* parent = nullptr;
    // wavefront buffers
    double* samp = nullptr;
    int* nidx = nullptr;
    double* ndist = nullptr;
    double* nearst = nullptr;
    double* newst = nullptr;
    uint8_t* skip = nullptr;
    uint8_t* ok = nullptr;
    int* scan = nullptr;      // per-sample exclusive offsets
    int* bsum = nullptr;      // per-block sums, then offsets; [nblk] = total
    double* acc_states = nullptr;
    int* acc_parent = nullptr;
    uint8_t* acc_goal = nullptr;
    int* hbuf = nullptr;      // pinned
    uint8_t* hgoal = nullptr; // pinned
    unsigned long long* nsamp = nullptr;
    uint32_t wave = 0;
    std::vector<int> goals;   // node ids of goal nodes, in discovery order
    uint64_t stat_samples = 0, stat_goal_samples = 0, stat_accepted = 0, stat_wavefronts = 0;
    uint64_t stat_skipped = 0;
    double stat_seconds = 0;
    bool solving = false;
    // learned surrogate: cull edges whose new state is predicted in collision
    mptg_surrogate* sg = nullptr;
    float sg_thr = 0.f;
    float* logits = nullptr;
    double* near_c = nullptr;
    double* new_c = nullptr;
    int* cmap = nullptr;
    uint8_t* ok_c = nullptr;
    uint8_t* keep = nullptr;
    uint64_t stat_culled = 0;
    int sg_points = 1;          // states scored per candidate edge
    double* sg_pts = nullptr;   // [sg_points][cap_wave][D] when sg_points > 1
    int sg_pts_cap = 1;         // sg_points the logits/sg_pts buffers hold
    // surrogate-biased sampling: each wavefront slot takes the lowest-risk of
    // sg_bias candidate edges (candidate buffers hold cap_wave * sg_bias)
    int sg_bias = 1;
    int sg_bias_cap = 0;
    double* b_samp = nullptr;
    int* b_nidx = nullptr;
    double* b_ndist = nullptr;
    double* b_near = nullptr;
    double* b_new = nullptr;
    uint8_t* b_skip = nullptr;
    double* b_pts = nullptr;    // [P][W * sg_bias][D]
    float* b_logits = nullptr;  // [P][W * sg_bias]
    int b_pts_cap = 0;          // P the two buffers above hold
    // every call of this planner runs on its own non-blocking stream, with its
    // own validity scratch, so planners on one scene can run concurrently
    cudaStream_t stream = nullptr;
    EdgeScratch scratch;
    size_t cap_nodes = 0;     // tree capacity and parent array length
    int cap_wave = 0;         // wavefront buffers
    int* path_ids = nullptr;  // [cap_nodes]
    double* path_out = nullptr;  // [2]
    // phase timing on the stream's timeline (WorkerStats' nearest_ and
    // validMotion_ timers, prrt.hpp:72-101): events at the phase boundaries
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    double t_phase[4] = {0, 0, 0, 0};  // nearest, surrogate, valid motion, insert (seconds)
    // PRRT* (mptg_planner_set_rewire)
    int star = 0;
    double rewire_factor = 1.1;
    double* cost = nullptr;             // [cap_nodes]
    double* elen = nullptr;             // [cap_nodes] length of the edge to the parent
    double* pj_s = nullptr;             // [cap_nodes] pointer-jumping buffers
    int* pj_a = nullptr;
    int* pj_a2 = nullptr;
    unsigned long long* bbits = nullptr;  // [cap_nodes] best rewire proposal per node
    int* bid = nullptr;
    int* knn_i = nullptr;               // [cap_wave][64]
    double* knn_d = nullptr;
    uint8_t* pv = nullptr;
    int* s_pair = nullptr;
    double* s_rcost = nullptr;
    uint8_t* s_ok = nullptr;
    double* s_ea = nullptr;             // [cap_wave * 64][D]
    double* s_eb = nullptr;
    double* dnear = nullptr;            // [cap_wave]
    int* cpar = nullptr;
    double* ccost = nullptr;
    double* celen = nullptr;
    int* s_cnt = nullptr;               // [2]
    int* rank = nullptr;                // [cap_wave][64] choose-parent rank (-1: no candidate)
    uint8_t* decided = nullptr;         // [cap_wave]
    unsigned long long* nrw = nullptr;  // rewires applied
    uint64_t stat_rewire_tests = 0;
    cudaEvent_t sev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double t_star[4] = {0, 0, 0, 0};    // k-NN, choose parent, rewire, costs (seconds)
    bool star_timed = false;            // sev recorded in the current wavefront
    // persistent block planner (bplan.cu): grid scenes, wavefronts <= 1024
    int bp_mode = 1;                    // 0 off, 1 used wherever it applies
    int bp_cap = 0;                     // node capacity of the buffers below
    double bp_prof[9] = {};             // block planner: SM cycles per phase, FP64 fallback counts
    double* bp_states = nullptr;        // [bp_cap][2]
    uint8_t* bp_goalf = nullptr;        // [bp_cap]
    BPlanCounters* bp_ctr = nullptr;
    BPlanJob* bp_job = nullptr;
    BPlanJob* bp_hjob = nullptr;        // pinned: the job's copy is asynchronous
    long long bp_brute_pairs = BPLAN_BRUTE_PAIRS;
    // a run of the block planner as a CUDA graph (job and counters in from the
    // pinned host copies, the block, the counters out), captured on the first
    // run and replayed after; bp_graph_W: the wavefront it was captured for
    cudaGraphExec_t bp_graph = nullptr;
    int bp_graph_W = 0;
    bool bp_graph_off = false;
    uint64_t bp_graph_runs = 0;
    BPlanCounters* bp_hctr = nullptr;   // pinned
    uint8_t* bp_hgoal = nullptr;        // pinned [bp_cap]
    uint64_t stat_bp_waves = 0;         // wavefronts run inside the block planner
    // bp_states[0, bp_n) mirrors the planner's first bp_n nodes; the kd-tree
    // holds a prefix of them and takes the rest (bp_flush) only when
    // something other than the block planner needs it
    size_t bp_n = 0;
};

extern "C" mptg_status mptg_surrogate_score_dev(mptg_surrogate* s, const double* dstates, int n, float* dlogits,
                                                cudaStream_t st);
std::mutex* mptg_surrogate_mutex(mptg_surrogate* s);

// ------------------------------------------------------------------ kernels

// At most one goal sample per wavefront: the lowest-index sample whose bias
// draw hits.  Identical goal samples would all steer from the same nearest
// node to the same new state; the reference draws goal samples on one worker
// and its d == 0 test rejects repeats (prrt.hpp:363-389,425).
__global__ void k_plan_goalpick(PlanView p, int W, uint32_t wave, int* __restrict__ first) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W) return;
    if (phx_uniform(p.seed, (uint32_t)i, wave, 16) < p.goal_bias) atomicMin(first, i);
}

__global__ void k_plan_sample(PlanView p, int W, uint32_t wave, const int* __restrict__ goal_index,
                              double* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W) return;
    double* q = out + (size_t)i * p.D;
    bool goal = goal_index != nullptr && i == *goal_index;
    if (goal) {
        for (int d = 0; d < p.D; ++d) q[d] = p.goal[d];
        return;
    }
    sample_uniform_state(p.metric, p.D, p.seed, (uint32_t)i, wave, p.lo, p.hi, q);
}

__global__ void k_plan_steer(PlanView p, int W, const double* __restrict__ samp, const int* __restrict__ nidx,
                             const double* __restrict__ ndist, const double* __restrict__ states64,
                             double* __restrict__ nearst, double* __restrict__ newst, uint8_t* __restrict__ skip) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W) return;
    const int D = p.D;
    const double* s = samp + (size_t)i * D;
    double* nr = nearst + (size_t)i * D;
    double* nw = newst + (size_t)i * D;
    int id = nidx[i];
    double d = ndist[i];
    if (id < 0 || d == 0.0 || !(d == d)) {  // prrt.hpp:425: avoid adding the same state twice
        skip[i] = 1;
        for (int k = 0; k < D; ++k) { nr[k] = s[k]; nw[k] = s[k]; }
        return;
    }
    skip[i] = 0;
    const double* ns = states64 + (size_t)id * D;
    double a[MPTG_MAX_DIM], b[MPTG_MAX_DIM];
    for (int k = 0; k < D; ++k) { a[k] = ns[k]; b[k] = s[k]; nr[k] = a[k]; }
    if (d > p.range) {
        double q[MPTG_MAX_DIM];
        interp64(p.metric, D, a, b, __ddiv_rn(p.range, d), q);
        for (int k = 0; k < D; ++k) nw[k] = q[k];
    } else {
        for (int k = 0; k < D; ++k) nw[k] = b[k];
    }
}

// block-local exclusive scan of the acceptance flags
__global__ void __launch_bounds__(PLAN_SCAN_BLOCK) k_plan_scan(int W, const uint8_t* __restrict__ ok,
                                                               const uint8_t* __restrict__ skip,
                                                               int* __restrict__ scan, int* __restrict__ bsum) {
    __shared__ int wsum[32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int f = (i < W && ok[i] && !skip[i]) ? 1 : 0;
    unsigned m = __ballot_sync(0xffffffffu, f);
    int pre = __popc(m & ((1u << lane) - 1u));
    if (lane == 0) wsum[w] = __popc(m);
    __syncthreads();
    if (w == 0) {
        int v = wsum[lane];
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        wsum[lane] = x - v;
        if (lane == 31) bsum[blockIdx.x] = x;
    }
    __syncthreads();
    if (i < W) scan[i] = f ? wsum[w] + pre : -1;
}

// exclusive scan over the (<= 1024) block sums; total at bsum[nblk]
__global__ void k_plan_scan_top(int nblk, int* __restrict__ bsum) {
    __shared__ int s[1024];
    int t = threadIdx.x;
    s[t] = t < nblk ? bsum[t] : 0;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        int v = t >= o ? s[t - o] : 0;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    if (t < nblk) bsum[t] = t == 0 ? 0 : s[t - 1];
    if (t == 0) bsum[nblk] = s[1023];
}

__global__ void k_plan_scatter(PlanView p, int W, const int* __restrict__ scan, const int* __restrict__ bsum,
                               const double* __restrict__ newst, const int* __restrict__ nidx,
                               double* __restrict__ acc_states, int* __restrict__ acc_parent,
                               uint8_t* __restrict__ acc_goal) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W) return;
    int l = scan[i];
    if (l < 0) return;
    int pos = bsum[i / PLAN_SCAN_BLOCK] + l;
    const double* s = newst + (size_t)i * p.D;
    double* o = acc_states + (size_t)pos * p.D;
    for (int k = 0; k < p.D; ++k) o[k] = s[k];
    acc_parent[pos] = nidx[i];
    uint8_t g = 0;
    if (p.has_goal) {
        // GoalState::operator() (src/mpt/goal_state.hpp:64-69): d <= radius
        double d = dist64(p.metric, p.D, p.w0, p.w1, s, p.goal);
        g = d <= p.goal_radius ? 1 : 0;
    }
    acc_goal[pos] = g;
}

// surrogate culling: flag the edges that go to the exact check
// the states the surrogate scores for each candidate edge (near -> new): the
// new state first, then interpolate(near, new, j/P) for 1 <= j < P; layout
// [j][W][D] so that pts[0] is the new-state block
__global__ void k_plan_edge_points(PlanView p, int W, int P, const double* __restrict__ nearst,
                                   const double* __restrict__ newst, double* __restrict__ pts) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * (P - 1)) return;
    const int e = i % W, j = 1 + i / W;
    const int D = p.D;
    double a[MPTG_MAX_DIM], b[MPTG_MAX_DIM], q[MPTG_MAX_DIM];
    for (int k = 0; k < D; ++k) { a[k] = nearst[(size_t)e * D + k]; b[k] = newst[(size_t)e * D + k]; }
    interp64(p.metric, D, a, b, __ddiv_rn((double)j, (double)P), q);
    double* out = pts + ((size_t)j * W + e) * D;
    for (int k = 0; k < D; ++k) out[k] = q[k];
}

// an edge goes to the exact check unless skipped or some scored point's
// collision logit exceeds thr (logits [P][W])
__global__ void k_plan_keep(int W, int P, const uint8_t* __restrict__ skip, const float* __restrict__ logit, float thr,
                            uint8_t* __restrict__ keep, uint8_t* __restrict__ ok) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W) return;
    bool cull = false;
    for (int j = 0; j < P; ++j) cull = cull || logit[(size_t)j * W + i] > thr;
    keep[i] = (!skip[i] && !cull) ? 1 : 0;
    ok[i] = 0;
}

// candidate c = j*W + i (j < B) of a biased wavefront: Philox sample c of the
// wavefront (j = 0 is the plain planner's sample i; the goal sample, when
// picked, replaces candidate 0 of its slot)
__global__ void k_plan_sample_cand(PlanView p, int W, int B, uint32_t wave, const int* __restrict__ goal_index,
                                   double* __restrict__ out) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= W * B) return;
    double* q = out + (size_t)c * p.D;
    if (goal_index != nullptr && c == *goal_index) {
        for (int d = 0; d < p.D; ++d) q[d] = p.goal[d];
        return;
    }
    sample_uniform_state(p.metric, p.D, p.seed, (uint32_t)c, wave, p.lo, p.hi, q);
}

// Slot i takes, of its candidates j*W + i, the one whose highest collision
// logit over its P scored points is lowest (a skipped candidate only when all
// are; ties: the lowest j); the goal sample's slot keeps the goal.  The
// chosen candidate's sample, nearest node, edge and logits fill slot i.
__global__ void k_plan_bias_select(int W, int B, int P, int D, const int* __restrict__ goal_index,
                                   const double* __restrict__ csamp, const int* __restrict__ cnidx,
                                   const double* __restrict__ cndist, const double* __restrict__ cnear,
                                   const double* __restrict__ cnew, const uint8_t* __restrict__ cskip,
                                   const float* __restrict__ clogit, double* __restrict__ samp, int* __restrict__ nidx,
                                   double* __restrict__ ndist, double* __restrict__ nearst, double* __restrict__ newst,
                                   uint8_t* __restrict__ skip, float* __restrict__ logit) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W) return;
    const size_t WB = (size_t)W * B;
    int best = 0;
    if (!(goal_index != nullptr && i == *goal_index)) {
        float bl = INFINITY;
        bool bskip = true;
        for (int j = 0; j < B; ++j) {
            const size_t c = (size_t)j * W + i;
            float l = -INFINITY;
            for (int k = 0; k < P; ++k) l = fmaxf(l, clogit[k * WB + c]);
            const bool sk = cskip[c] != 0;
            if (j == 0 || (bskip && !sk) || (sk == bskip && l < bl)) {
                best = j;
                bl = l;
                bskip = sk;
            }
        }
    }
    const size_t c = (size_t)best * W + i;
    for (int d = 0; d < D; ++d) {
        samp[(size_t)i * D + d] = csamp[c * D + d];
        nearst[(size_t)i * D + d] = cnear[c * D + d];
        newst[(size_t)i * D + d] = cnew[c * D + d];
    }
    nidx[i] = cnidx[c];
    ndist[i] = cndist[c];
    skip[i] = cskip[c];
    for (int k = 0; k < P; ++k) logit[(size_t)k * W + i] = clogit[k * WB + c];
}

__global__ void k_plan_cgather(PlanView p, int W, const int* __restrict__ scan, const int* __restrict__ bsum,
                               const double* __restrict__ nearst, const double* __restrict__ newst,
                               double* __restrict__ near_c, double* __restrict__ new_c, int* __restrict__ cmap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W) return;
    int l = scan[i];
    if (l < 0) return;
    int pos = bsum[i / PLAN_SCAN_BLOCK] + l;
    for (int k = 0; k < p.D; ++k) {
        near_c[(size_t)pos * p.D + k] = nearst[(size_t)i * p.D + k];
        new_c[(size_t)pos * p.D + k] = newst[(size_t)i * p.D + k];
    }
    cmap[pos] = i;
}

__global__ void k_plan_cscatter(int n, const int* __restrict__ cmap, const uint8_t* __restrict__ ok_c,
                                uint8_t* __restrict__ ok) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) ok[cmap[j]] = ok_c[j];
}

// walk a goal's parent chain: path ids (start first) and the summed cost
// (PRRT::pathCost, src/mpt/impl/prrt/prrt.hpp:208-234)
__global__ void k_plan_path(int goal, const int* __restrict__ parent, const double* __restrict__ states64, int D,
                            int metric, double w0, double w1, int cap, int* __restrict__ ids, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int len = 1;
    double cost = 0.0;
    int n = goal;
    for (int guard = 0; guard < (1 << 30); ++guard) {
        int pnt = parent[n];
        if (pnt < 0) break;
        cost = __dadd_rn(cost, dist64(metric, D, w0, w1, states64 + (size_t)n * D, states64 + (size_t)pnt * D));
        n = pnt;
        ++len;
    }
    out[0] = cost;
    out[1] = (double)len;
    if (len <= cap) {
        n = goal;
        for (int k = len - 1; k >= 0; --k) {
            ids[k] = n;
            n = parent[n];
        }
    }
}

// out[k] = states64[ids[k]] for k < n (one double per thread)
__global__ void k_plan_gather(const int* __restrict__ ids, int n, const double* __restrict__ states64, int D,
                              double* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * D) return;
    int k = i / D, d = i - k * D;
    out[i] = states64[(size_t)ids[k] * D + d];
}

// ------------------------------------------------------------------ PRRT* (rewiring)
// The worker's addSample of src/mpt/impl/prrt_star/prrt_star.hpp:505-657 as
// wavefront steps (the CPU checker's orc_plan_star is the same algorithm):
// k-nearest choose-parent in (cost + d, d, id) key order, rewiring of the
// neighbours the choose loop did not reach, and costs recomputed by pointer
// jumping over the edge lengths.

__device__ __forceinline__ bool star_less(double c1, double d1, int i1, double c2, double d2, int i2) {
    if (c1 != c2) return c1 < c2;
    if (d1 != d2) return d1 < d2;
    return i1 < i2;
}

// d(near, new) of every accepted new state
__global__ void k_star_near(PlanView p, int A, const double* __restrict__ acc, const int* __restrict__ near,
                            const double* __restrict__ states64, double* __restrict__ dnear) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    dnear[a] = dist64(p.metric, p.D, p.w0, p.w1, states64 + (size_t)near[a] * p.D, acc + (size_t)a * p.D);
}

__device__ __forceinline__ void copy_state(double* __restrict__ dst, const double* __restrict__ src, int D) {
    for (int d = 0; d < D; ++d) dst[d] = src[d];
}

// choose-parent candidates: neighbour j of new state a whose key is below
// near's, ranked by key among the state's candidates (rank -1: not one)
__global__ void k_star_rank(int A, int k, const int* __restrict__ ki, const double* __restrict__ kd,
                            const int* __restrict__ near, const double* __restrict__ dnear,
                            const double* __restrict__ cost, int* __restrict__ rank) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A * k) return;
    const int a = t / k, nb = ki[t], nr = near[a];
    rank[t] = -1;
    if (nb < 0 || nb == nr) return;
    const double dj = kd[t], cj = __dadd_rn(cost[nb], dj);
    const double dn = dnear[a], cn = __dadd_rn(cost[nr], dn);
    if (!star_less(cj, dj, nb, cn, dn, nr)) return;
    int r = 0;
    for (int j = 0; j < k; ++j) {
        const int o = ki[a * k + j];
        if (o < 0 || o == nr || o == nb) continue;
        const double dd = kd[a * k + j], cc = __dadd_rn(cost[o], dd);
        if (star_less(cc, dd, o, cn, dn, nr) && star_less(cc, dd, o, cj, dj, nb)) ++r;
    }
    rank[t] = r;
}

// one round of choose-parent checks: the candidates of rank [lo, hi) of the
// states that have no valid candidate yet; their links neighbour -> new are
// gathered (in any order) for one batched DMV call.  A state stops at the
// first round with a valid candidate: every lower-ranked candidate was
// checked and failed, so the smallest valid key is the reference's choice.
__global__ void k_star_pc(PlanView p, int A, int k, int lo, int hi, const int* __restrict__ ki,
                          const int* __restrict__ rank, const uint8_t* __restrict__ decided,
                          const double* __restrict__ states64, const double* __restrict__ acc, int* __restrict__ cnt,
                          int* __restrict__ pair_of, double* __restrict__ ea, double* __restrict__ eb) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A * k) return;
    const int a = t / k, r = rank[t];
    if (r < lo || r >= hi || decided[a]) return;
    const int slot = atomicAdd(cnt, 1);  // < A * k
    pair_of[slot] = t;
    copy_state(ea + (size_t)slot * p.D, states64 + (size_t)ki[t] * p.D, p.D);
    copy_state(eb + (size_t)slot * p.D, acc + (size_t)a * p.D, p.D);
}

// states with a valid candidate among this round's are decided
__global__ void k_star_decide(int m, int k, const int* __restrict__ pair_of, const uint8_t* __restrict__ ok,
                              uint8_t* __restrict__ decided) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < m && ok[s]) decided[pair_of[s] / k] = 1;
}

__global__ void k_star_scatter(int m, const int* __restrict__ pair_of, const uint8_t* __restrict__ ok,
                               uint8_t* __restrict__ pv) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < m) pv[pair_of[s]] = ok[s];
}

// the parent: the smallest key among near and the valid candidates
__global__ void k_star_choose(int A, int k, const int* __restrict__ ki, const double* __restrict__ kd,
                              const int* __restrict__ near, const double* __restrict__ dnear,
                              const double* __restrict__ cost, const uint8_t* __restrict__ pv, int* __restrict__ cpar,
                              double* __restrict__ ccost, double* __restrict__ celen) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    int bp = near[a];
    double bd = dnear[a], bc = __dadd_rn(cost[bp], bd);
    for (int j = 0; j < k; ++j) {
        const int t = a * k + j;
        if (!pv[t]) continue;
        const int nb = ki[t];
        const double dj = kd[t], cj = __dadd_rn(cost[nb], dj);
        if (star_less(cj, dj, nb, bc, bd, bp)) { bp = nb; bc = cj; bd = dj; }
    }
    cpar[a] = bp;
    ccost[a] = bc;
    celen[a] = bd;
}

// rewire candidates: neighbours past the chosen parent in key order with
// cost(new) + d < cost(neighbour); links new -> neighbour gathered
__global__ void k_star_rw(PlanView p, int A, int k, const int* __restrict__ ki, const double* __restrict__ kd,
                          const double* __restrict__ cost, const int* __restrict__ cpar,
                          const double* __restrict__ ccost, const double* __restrict__ celen,
                          const double* __restrict__ states64, const double* __restrict__ acc, int* __restrict__ cnt,
                          int* __restrict__ pair_of, double* __restrict__ rcost, double* __restrict__ ea,
                          double* __restrict__ eb) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A * k) return;
    const int a = t / k, nb = ki[t];
    if (nb < 0) return;
    const double dj = kd[t], cj = __dadd_rn(cost[nb], dj);
    if (!star_less(ccost[a], celen[a], cpar[a], cj, dj, nb)) return;  // reached by the choose loop
    const double nc = __dadd_rn(ccost[a], dj);
    if (!(nc < cost[nb])) return;
    const int slot = atomicAdd(cnt, 1);
    pair_of[slot] = t;
    rcost[slot] = nc;
    copy_state(ea + (size_t)slot * p.D, acc + (size_t)a * p.D, p.D);
    copy_state(eb + (size_t)slot * p.D, states64 + (size_t)nb * p.D, p.D);
}

// each neighbour takes the valid proposal with the smallest (cost, new id):
// costs are >= 0, so their bit patterns order as unsigned integers
__global__ void k_star_rw_min(int m, const int* __restrict__ pair_of, const double* __restrict__ rcost,
                              const uint8_t* __restrict__ ok, const int* __restrict__ ki,
                              unsigned long long* __restrict__ bbits) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m || !ok[s]) return;
    atomicMin(&bbits[ki[pair_of[s]]], (unsigned long long)__double_as_longlong(rcost[s]));
}

__global__ void k_star_rw_id(int m, int k, const int* __restrict__ pair_of, const double* __restrict__ rcost,
                             const uint8_t* __restrict__ ok, const int* __restrict__ ki,
                             const unsigned long long* __restrict__ bbits, int* __restrict__ bid) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m || !ok[s]) return;
    const int nb = ki[pair_of[s]];
    if ((unsigned long long)__double_as_longlong(rcost[s]) == bbits[nb]) atomicMin(&bid[nb], pair_of[s] / k);
}

__global__ void k_star_rw_apply(int m, int k, int n0, const int* __restrict__ pair_of, const double* __restrict__ rcost,
                                const uint8_t* __restrict__ ok, const int* __restrict__ ki,
                                const double* __restrict__ kd, const unsigned long long* __restrict__ bbits,
                                const int* __restrict__ bid, int* __restrict__ parent, double* __restrict__ elen,
                                unsigned long long* __restrict__ nrw) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m || !ok[s]) return;
    const int t = pair_of[s], nb = ki[t], a = t / k;
    if ((unsigned long long)__double_as_longlong(rcost[s]) != bbits[nb] || bid[nb] != a) return;
    parent[nb] = n0 + a;
    elen[nb] = kd[t];
    atomicAdd(nrw, 1ull);
}

__global__ void k_star_rw_reset(int m, const int* __restrict__ pair_of, const int* __restrict__ ki,
                                unsigned long long* __restrict__ bbits, int* __restrict__ bid) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= m) return;
    const int nb = ki[pair_of[s]];
    bbits[nb] = ~0ull;
    bid[nb] = INT_MAX;
}

__global__ void k_star_insert(int A, int n0, const int* __restrict__ cpar, const double* __restrict__ celen,
                              int* __restrict__ parent, double* __restrict__ elen) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    parent[n0 + a] = cpar[a];
    elen[n0 + a] = celen[a];
}

// one pointer-jumping round: s[x] += s[a[x]], a[x] = a[a[x]]
__global__ void k_star_pj(int n, const double* __restrict__ s_in, const int* __restrict__ a_in,
                          double* __restrict__ s_out, int* __restrict__ a_out) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const int a = a_in[x];
    if (a >= 0) {
        s_out[x] = __dadd_rn(s_in[x], s_in[a]);
        a_out[x] = a_in[a];
    } else {
        s_out[x] = s_in[x];
        a_out[x] = -1;
    }
}

// ------------------------------------------------------------------ host

static PlanView plan_view(const mptg_planner* p) {
    PlanView v;
    v.D = p->D; v.metric = p->metric; v.w0 = p->w0; v.w1 = p->w1;
    v.lo = p->lo; v.hi = p->hi; v.goal = p->goal; v.has_goal = p->has_goal;
    v.goal_bias = p->prm.goal_bias;
    v.range = p->prm.range > 0 ? p->prm.range : INFINITY;
    v.goal_radius = p->prm.goal_radius;
    v.seed = p->prm.seed;
    return v;
}

static void planner_free(mptg_planner* p) {
    void* ptrs[] = {p->lo, p->hi, p->goal, p->parent, p->samp, p->nidx, p->ndist, p->nearst, p->newst, p->skip,
                    p->ok, p->scan, p->bsum, p->acc_states, p->acc_parent, p->acc_goal, p->nsamp, p->logits,
                    p->near_c, p->new_c, p->cmap, p->ok_c, p->keep, p->path_ids, p->path_out, p->sg_pts,
                    p->cost, p->elen, p->pj_s, p->pj_a, p->pj_a2, p->bbits, p->bid, p->knn_i, p->knn_d, p->pv,
                    p->s_pair, p->s_rcost, p->s_ok, p->s_ea, p->s_eb, p->dnear, p->cpar, p->ccost, p->celen,
                    p->s_cnt, p->nrw, p->rank, p->decided, p->bp_states, p->bp_goalf, p->bp_ctr, p->bp_job,
                    p->b_samp, p->b_nidx, p->b_ndist, p->b_near, p->b_new, p->b_skip, p->b_pts, p->b_logits};
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (void* x : ptrs)
        if (x) cudaFree(x);
    if (p->hbuf) cudaFreeHost(p->hbuf);
    if (p->hgoal) cudaFreeHost(p->hgoal);
    if (p->bp_graph) cudaGraphExecDestroy(p->bp_graph);
    if (p->bp_hjob) cudaFreeHost(p->bp_hjob);
    if (p->bp_hctr) cudaFreeHost(p->bp_hctr);
    if (p->bp_hgoal) cudaFreeHost(p->bp_hgoal);
    scratch_free(&p->scratch);
    for (cudaEvent_t e : p->ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : p->sev)
        if (e) cudaEventDestroy(e);
    if (p->tree) mptg_tree_destroy(p->tree);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

// nodes of the planner: the kd-tree's plus those the block planner added
// that the kd-tree has not taken yet
static size_t planner_n(const mptg_planner* p) {
    size_t n = 0;
    mptg_tree_size(p->tree, &n);
    return std::max(n, p->bp_n);
}

// the kd-tree takes the block planner's pending nodes
static mptg_status bp_flush(mptg_planner* p) {
    size_t n = 0;
    mptg_tree_size(p->tree, &n);
    if (p->bp_n <= n) return MPTG_OK;
    mptg_status st = mptg_tree_insert(p->tree, p->bp_states + n * 2, p->bp_n - n, p->stream);
    if (st) return st;
    MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
    return MPTG_OK;
}

static mptg_status check_params(mptg_ctx* ctx, const mptg_scene* scene, const mptg_plan_params* prm) {
    if (prm->wavefront < 1 || prm->wavefront > (1 << 20))
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "wavefront must be in [1, 2^20]");
    if (prm->max_nodes < 1) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "max_nodes must be positive");
    if (!(prm->edge_step > 0)) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "edge_step must be positive");
    if (!(prm->goal_bias >= 0 && prm->goal_bias <= 1))
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "goal_bias must be in [0, 1]");
    if (prm->resolution == 1 && scene->metric != MPTG_METRIC_SO2)
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "joint-step resolution needs an SO2 scene");
    return MPTG_OK;
}

// sampling bounds: given, else the metric's domain
static mptg_status set_bounds(mptg_planner* p, const double* lo, const double* hi) {
    const int D = p->D;
    double l[MPTG_MAX_DIM], h[MPTG_MAX_DIM];
    for (int d = 0; d < D; ++d) {
        l[d] = lo ? lo[d] : (p->metric == MPTG_METRIC_SO2 ? -MPTG_PI : 0.0);
        h[d] = hi ? hi[d] : (p->metric == MPTG_METRIC_SO2 ? MPTG_PI : 1.0);
    }
    for (int d = 0; d < D; ++d) {
        p->lo_host[d] = l[d];
        p->hi_host[d] = h[d];
    }
    MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(p->lo, l, D * sizeof(double), cudaMemcpyHostToDevice, p->stream));
    MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(p->hi, h, D * sizeof(double), cudaMemcpyHostToDevice, p->stream));
    MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
    return MPTG_OK;
}

// a fresh Planner(scenario, seed) on the same allocations
static mptg_status planner_reset(mptg_planner* p, const mptg_plan_params* prm, bool bounds, const double* lo,
                                 const double* hi) {
    mptg_ctx* ctx = p->ctx;
    if (p->solving) return mptg_fail(ctx, MPTG_ERR_ALREADY_SOLVING, "already solving");
    if (prm) {
        mptg_status st = check_params(ctx, p->scene, prm);
        if (st) return st;
        if (prm->wavefront > p->cap_wave || prm->max_nodes > p->cap_nodes)
            return mptg_fail(ctx, MPTG_ERR_CAPACITY, "reset needs wavefront <= %d and max_nodes <= %zu", p->cap_wave,
                             p->cap_nodes);
        p->prm = *prm;
    }
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    mptg_status st = mptg_tree_clear(p->tree, p->stream);
    if (st) return st;
    p->bp_n = 0;
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->nsamp, 0, sizeof(unsigned long long), p->stream));
    if (bounds && (st = set_bounds(p, lo, hi))) return st;
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(p->stream));
    p->has_goal = 0;
    p->goal_host.clear();
    p->goals.clear();
    p->wave = 0;
    p->stat_samples = p->stat_goal_samples = p->stat_accepted = p->stat_wavefronts = 0;
    p->stat_skipped = p->stat_culled = 0;
    p->stat_seconds = 0;
    for (double& t : p->t_phase) t = 0;
    p->stat_rewire_tests = 0;
    p->stat_bp_waves = 0;
    for (double& t : p->t_star) t = 0;
    if (p->nrw) MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->nrw, 0, sizeof(unsigned long long), p->stream));
    return MPTG_OK;
}

// PRRT* steps of one wavefront on the A accepted new states (acc_states,
// nearest node acc_parent), against the tree of n0 nodes as it stood before
// the wavefront: choose-parent (cpar / ccost / celen) and rewiring of old
// nodes (parent / elen).  The new nodes are inserted by the caller.
static mptg_status star_wave(mptg_planner* p, cudaStream_t s, int A, size_t n0) {
    mptg_ctx* ctx = p->ctx;
    const PlanView v = plan_view(p);
    const double* st64 = mptg_tree_states_dev(p->tree);
    int k = (int)ceil(p->rewire_factor * 2.718281828459045 * (1.0 + 1.0 / p->D) * log((double)n0 + 1.0));
    k = std::max(1, std::min(k, std::min(64, (int)n0)));
    const int pairs = A * k;
    mptg_status st;
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->sev[0], s));
    k_star_near<<<mptg_blocks(A, 128), 128, 0, s>>>(v, A, p->acc_states, p->acc_parent, st64, p->dnear);
    MPTG_LAUNCHED(ctx);
    if ((st = mptg_tree_nearest_k_dev(p->tree, p->acc_states, A, k, p->knn_i, p->knn_d, s))) return st;
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->sev[1], s));
    // choose parent: candidates in key order, in rounds of rank [0,1) and [1,k)
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->pv, 0, pairs, s));
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->decided, 0, A, s));
    k_star_rank<<<mptg_blocks(pairs, 128), 128, 0, s>>>(A, k, p->knn_i, p->knn_d, p->acc_parent, p->dnear, p->cost,
                                                       p->rank);
    MPTG_LAUNCHED(ctx);
    int npc = 0;
    const int bounds[3] = {0, 1, 64};
    for (int r = 0; r < 2; ++r) {
        MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->s_cnt, 0, sizeof(int), s));
        k_star_pc<<<mptg_blocks(pairs, 128), 128, 0, s>>>(v, A, k, bounds[r], bounds[r + 1], p->knn_i, p->rank,
                                                         p->decided, st64, p->acc_states, p->s_cnt, p->s_pair,
                                                         p->s_ea, p->s_eb);
        MPTG_LAUNCHED(ctx);
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hbuf + 2, p->s_cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
        MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        const int m = p->hbuf[2];
        if (m == 0) continue;
        npc += m;
        if ((st = scene_edges_dev(p->scene, p->s_ea, p->s_eb, m, p->prm.edge_step, p->prm.resolution, p->s_ok, s,
                                  p->nsamp, &p->scratch)))
            return st;
        k_star_scatter<<<mptg_blocks(m, 256), 256, 0, s>>>(m, p->s_pair, p->s_ok, p->pv);
        k_star_decide<<<mptg_blocks(m, 256), 256, 0, s>>>(m, k, p->s_pair, p->s_ok, p->decided);
        ctx->launches += 2;
    }
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->s_cnt + 1, 0, sizeof(int), s));
    k_star_choose<<<mptg_blocks(A, 128), 128, 0, s>>>(A, k, p->knn_i, p->knn_d, p->acc_parent, p->dnear, p->cost,
                                                      p->pv, p->cpar, p->ccost, p->celen);
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->sev[2], s));
    // rewire
    k_star_rw<<<mptg_blocks(pairs, 128), 128, 0, s>>>(v, A, k, p->knn_i, p->knn_d, p->cost, p->cpar, p->ccost,
                                                     p->celen, st64, p->acc_states, p->s_cnt + 1, p->s_pair,
                                                     p->s_rcost, p->s_ea, p->s_eb);
    ctx->launches += 2;
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hbuf + 3, p->s_cnt + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    const int nrc = p->hbuf[3];
    p->stat_rewire_tests += (uint64_t)(npc + nrc);
    if (nrc > 0) {
        if ((st = scene_edges_dev(p->scene, p->s_ea, p->s_eb, nrc, p->prm.edge_step, p->prm.resolution, p->s_ok, s,
                                  p->nsamp, &p->scratch)))
            return st;
        const unsigned g = mptg_blocks(nrc, 256);
        k_star_rw_min<<<g, 256, 0, s>>>(nrc, p->s_pair, p->s_rcost, p->s_ok, p->knn_i, p->bbits);
        k_star_rw_id<<<g, 256, 0, s>>>(nrc, k, p->s_pair, p->s_rcost, p->s_ok, p->knn_i, p->bbits, p->bid);
        k_star_rw_apply<<<g, 256, 0, s>>>(nrc, k, (int)n0, p->s_pair, p->s_rcost, p->s_ok, p->knn_i, p->knn_d,
                                          p->bbits, p->bid, p->parent, p->elen, p->nrw);
        k_star_rw_reset<<<g, 256, 0, s>>>(nrc, p->s_pair, p->knn_i, p->bbits, p->bid);
        ctx->launches += 4;
    }
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->sev[3], s));
    p->star_timed = true;
    return MPTG_OK;
}

// every node's cost from the edge lengths by pointer jumping,
// ceil(log2(n + 1)) rounds (the depth is below n)
static mptg_status star_costs(mptg_planner* p, cudaStream_t s, size_t n) {
    mptg_ctx* ctx = p->ctx;
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->sev[4], s));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->pj_s, p->elen, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->pj_a, p->parent, n * sizeof(int), cudaMemcpyDeviceToDevice, s));
    int rounds = 0;
    while (((size_t)1 << rounds) < n + 1) ++rounds;
    double* sa = p->pj_s;
    double* sb = p->cost;
    int* aa = p->pj_a;
    int* ab = p->pj_a2;
    for (int r = 0; r < rounds; ++r) {
        k_star_pj<<<mptg_blocks(n, 256), 256, 0, s>>>((int)n, sa, aa, sb, ab);
        std::swap(sa, sb);
        std::swap(aa, ab);
    }
    ctx->launches += rounds;
    if (sa != p->cost) MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->cost, sa, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->sev[5], s));
    return MPTG_OK;
}

// one wavefront; returns the number of nodes added
static mptg_status plan_wavefront(mptg_planner* p, cudaStream_t s, int* added) {
    mptg_ctx* ctx = p->ctx;
    const int W = p->prm.wavefront;
    *added = 0;
    mptg_status st0 = bp_flush(p);
    if (st0) return st0;
    size_t n0 = 0;
    mptg_tree_size(p->tree, &n0);
    if (n0 >= p->prm.max_nodes) return MPTG_OK;
    PlanView v = plan_view(p);
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->ev[0], s));
    bool bias_on = p->goals.empty() && p->has_goal && p->prm.goal_bias > 0;
    int* gidx = nullptr;
    if (bias_on) {
        gidx = p->bsum + 1024 + 1;  // scratch word after the scan block sums
        MPTG_CUDA_TRY(ctx, cudaMemsetAsync(gidx, 0x7f, sizeof(int), s));
        k_plan_goalpick<<<mptg_blocks(W, 128), 128, 0, s>>>(v, W, p->wave, gidx);
        MPTG_LAUNCHED(ctx);
    }
    const bool biased = p->sg && p->sg_bias > 1;
    mptg_status st;
    if (biased) {
        // W * B candidate edges, NN and steer for all of them
        const int B = p->sg_bias, WB = W * B;
        k_plan_sample_cand<<<mptg_blocks(WB, 128), 128, 0, s>>>(v, W, B, p->wave, gidx, p->b_samp);
        MPTG_LAUNCHED(ctx);
        if ((st = mptg_tree_nearest_dev(p->tree, p->b_samp, WB, p->b_nidx, p->b_ndist, s, false))) return st;
        k_plan_steer<<<mptg_blocks(WB, 128), 128, 0, s>>>(v, WB, p->b_samp, p->b_nidx, p->b_ndist,
                                                          mptg_tree_states_dev(p->tree), p->b_near, p->b_new,
                                                          p->b_skip);
        MPTG_LAUNCHED(ctx);
    } else {
        k_plan_sample<<<mptg_blocks(W, 128), 128, 0, s>>>(v, W, p->wave, gidx, p->samp);
        st = mptg_tree_nearest_dev(p->tree, p->samp, W, p->nidx, p->ndist, s, false);
        if (st) return st;
        k_plan_steer<<<mptg_blocks(W, 128), 128, 0, s>>>(v, W, p->samp, p->nidx, p->ndist,
                                                         mptg_tree_states_dev(p->tree), p->nearst, p->newst, p->skip);
        ctx->launches += 2;
    }
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->ev[1], s));
    int nblk = (W + PLAN_SCAN_BLOCK - 1) / PLAN_SCAN_BLOCK;
    if (p->sg) {
        // score the new states; only edges the surrogate does not reject go to the exact check
        int nk = 0;
        {
            // the surrogate's activation buffers are shared between planners:
            // hold it until this stream has consumed its logits
            const int P = p->sg_points;
            std::lock_guard<std::mutex> lock(*mptg_surrogate_mutex(p->sg));
            if (biased) {
                // score every candidate edge, then each slot takes its lowest-risk candidate
                const int B = p->sg_bias, WB = W * B;
                if (P > 1) {
                    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->b_pts, p->b_new, (size_t)WB * p->D * sizeof(double),
                                                       cudaMemcpyDeviceToDevice, s));
                    k_plan_edge_points<<<mptg_blocks((size_t)WB * (P - 1), 128), 128, 0, s>>>(v, WB, P, p->b_near,
                                                                                              p->b_new, p->b_pts);
                    MPTG_LAUNCHED(ctx);
                }
                if ((st = mptg_surrogate_score_dev(p->sg, P > 1 ? p->b_pts : p->b_new, WB * P, p->b_logits, s)))
                    return st;
                k_plan_bias_select<<<mptg_blocks(W, 128), 128, 0, s>>>(
                    W, B, P, p->D, gidx, p->b_samp, p->b_nidx, p->b_ndist, p->b_near, p->b_new, p->b_skip,
                    p->b_logits, p->samp, p->nidx, p->ndist, p->nearst, p->newst, p->skip, p->logits);
                MPTG_LAUNCHED(ctx);
            } else {
                if (P > 1) {
                    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->sg_pts, p->newst, (size_t)W * p->D * sizeof(double),
                                                       cudaMemcpyDeviceToDevice, s));
                    k_plan_edge_points<<<mptg_blocks((size_t)W * (P - 1), 128), 128, 0, s>>>(v, W, P, p->nearst,
                                                                                             p->newst, p->sg_pts);
                    MPTG_LAUNCHED(ctx);
                }
                if ((st = mptg_surrogate_score_dev(p->sg, P > 1 ? p->sg_pts : p->newst, W * P, p->logits, s)))
                    return st;
            }
            k_plan_keep<<<mptg_blocks(W, 256), 256, 0, s>>>(W, P, p->skip, p->logits, p->sg_thr, p->keep, p->ok);
            k_plan_scan<<<nblk, PLAN_SCAN_BLOCK, 0, s>>>(W, p->keep, p->skip, p->scan, p->bsum);
            k_plan_scan_top<<<1, 1024, 0, s>>>(nblk, p->bsum);
            k_plan_cgather<<<mptg_blocks(W, 128), 128, 0, s>>>(v, W, p->scan, p->bsum, p->nearst, p->newst,
                                                               p->near_c, p->new_c, p->cmap);
            ctx->launches += 4;
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hbuf + 1, p->bsum + nblk, sizeof(int), cudaMemcpyDeviceToHost, s));
            MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
            nk = p->hbuf[1];
        }
        p->stat_culled += (uint64_t)(W - nk);
        MPTG_CUDA_TRY(ctx, cudaEventRecord(p->ev[2], s));
        if (nk > 0) {
            st = scene_edges_dev(p->scene, p->near_c, p->new_c, nk, p->prm.edge_step, p->prm.resolution, p->ok_c, s,
                                 p->nsamp, &p->scratch);
            if (st) return st;
            k_plan_cscatter<<<mptg_blocks(nk, 256), 256, 0, s>>>(nk, p->cmap, p->ok_c, p->ok);
            MPTG_LAUNCHED(ctx);
        }
    } else {
        MPTG_CUDA_TRY(ctx, cudaEventRecord(p->ev[2], s));
        st = scene_edges_dev(p->scene, p->nearst, p->newst, W, p->prm.edge_step, p->prm.resolution, p->ok, s,
                             p->nsamp, &p->scratch);
        if (st) return st;
    }
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->ev[3], s));
    k_plan_scan<<<nblk, PLAN_SCAN_BLOCK, 0, s>>>(W, p->ok, p->skip, p->scan, p->bsum);
    k_plan_scan_top<<<1, 1024, 0, s>>>(nblk, p->bsum);
    k_plan_scatter<<<mptg_blocks(W, 128), 128, 0, s>>>(v, W, p->scan, p->bsum, p->newst, p->nidx, p->acc_states,
                                                       p->acc_parent, p->acc_goal);
    ctx->launches += 3;
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hbuf, p->bsum + nblk, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    int nacc = p->hbuf[0];
    size_t room = p->prm.max_nodes - n0;
    if ((size_t)nacc > room) nacc = (int)room;  // node budget: keep the first accepted samples
    p->stat_samples += W;
    p->stat_accepted += nacc;
    p->stat_wavefronts += 1;
    p->wave += 1;
    if (nacc > 0) {
        if (p->star) {
            // choose-parent and rewiring against the tree before the insert
            if ((st = star_wave(p, s, nacc, n0))) return st;
            k_star_insert<<<mptg_blocks(nacc, 128), 128, 0, s>>>(nacc, (int)n0, p->cpar, p->celen, p->parent, p->elen);
            MPTG_LAUNCHED(ctx);
        } else {
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->parent + n0, p->acc_parent, nacc * sizeof(int),
                                               cudaMemcpyDeviceToDevice, s));
        }
        // enqueued ahead of the insert, whose counter read-back synchronises
        // the stream, so the goal flags are on the host when it returns
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hgoal, p->acc_goal, nacc, cudaMemcpyDeviceToHost, s));
        st = mptg_tree_insert(p->tree, p->acc_states, nacc, s);
        if (st) return st;
        if (p->star && (st = star_costs(p, s, n0 + nacc))) return st;
        for (int k = 0; k < nacc; ++k)
            if (p->hgoal[k]) p->goals.push_back((int)(n0 + k));
    }
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->ev[4], s));
    MPTG_CUDA_TRY(ctx, cudaEventSynchronize(p->ev[4]));
    for (int k = 0; k < 4; ++k) {
        float ms = 0.f;
        MPTG_CUDA_TRY(ctx, cudaEventElapsedTime(&ms, p->ev[k], p->ev[k + 1]));
        p->t_phase[k] += 1e-3 * ms;
    }
    if (p->star_timed) {
        const int pairs[4][2] = {{0, 1}, {1, 2}, {2, 3}, {4, 5}};
        for (int k = 0; k < 4; ++k) {
            float ms = 0.f;
            MPTG_CUDA_TRY(ctx, cudaEventElapsedTime(&ms, p->sev[pairs[k][0]], p->sev[pairs[k][1]]));
            p->t_star[k] += 1e-3 * ms;
        }
        p->star_timed = false;
    }
    *added = nacc;
    return MPTG_OK;
}

// the block planner's buffers (node capacity min(max_nodes, BPLAN_MAX_NODES))
static mptg_status bp_alloc(mptg_planner* p) {
    const int cap = (int)std::min<size_t>(p->prm.max_nodes, BPLAN_MAX_NODES);
    cudaError_t e = cudaMalloc((void**)&p->bp_states, (size_t)cap * 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->bp_goalf, cap);
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->bp_ctr, sizeof(BPlanCounters));
    if (e == cudaSuccess) e = cudaMalloc((void**)&p->bp_job, sizeof(BPlanJob));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->bp_hjob, sizeof(BPlanJob));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->bp_hctr, sizeof(BPlanCounters));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->bp_hgoal, cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return mptg_fail(p->ctx, MPTG_ERR_OOM, "block planner buffers: %s", cudaGetErrorString(e));
    }
    p->bp_cap = cap;
    return MPTG_OK;
}

static bool bp_applies(const mptg_planner* p) {
    return p->bp_mode && !p->star && !p->sg && bplan_supported(p->scene, p->prm.wavefront, p->prm.resolution);
}

// Captures a block-planner run as a CUDA graph on the planner's stream: the
// job and counters copied in from the pinned host copies (read when the graph
// runs, so the host fills them before each launch), the block, the counters
// copied out.  A capture or instantiation that fails leaves the planner on the
// direct launches for good (bp_graph_off); either way the work is the same.
static void bp_capture(mptg_planner* p, int W) {
    mptg_ctx* ctx = p->ctx;
    cudaStream_t s = p->stream;
    if (bplan_configure(ctx) != MPTG_OK) {  // the attribute call is not allowed inside a capture
        p->bp_graph_off = true;
        return;
    }
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        bool counted = false;  // bplan_launch counted a launch that the capture only recorded
        ok = cudaMemcpyAsync(p->bp_job, p->bp_hjob, sizeof(BPlanJob), cudaMemcpyHostToDevice, s) == cudaSuccess &&
             cudaMemcpyAsync(p->bp_ctr, p->bp_hctr, sizeof(BPlanCounters), cudaMemcpyHostToDevice, s) ==
                 cudaSuccess &&
             (counted = bplan_launch(ctx, p->bp_job, 1, W, p->bp_cap, s, false) == MPTG_OK) &&
             cudaMemcpyAsync(p->bp_hctr, p->bp_ctr, sizeof(BPlanCounters), cudaMemcpyDeviceToHost, s) == cudaSuccess;
        const cudaError_t e = cudaStreamEndCapture(s, &g);
        ok = ok && e == cudaSuccess && g;
        if (counted) ctx->launches.fetch_sub(1, std::memory_order_relaxed);  // each replay counts one launch
    }
    if (ok && cudaGraphInstantiate(&p->bp_graph, g, 0) == cudaSuccess) {
        p->bp_graph_W = W;
    } else {
        p->bp_graph = nullptr;
        p->bp_graph_off = true;
    }
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
}

// the ring search's bucket grid: 64 x 64 cells over the sampling box (square
// cells on its longer side)
static void bp_cells(BPlanJob& j, const double* lo, const double* hi) {
    const double sx = hi[0] - lo[0], sy = hi[1] - lo[1];
    double cs = std::max(sx, sy) / 64.0;
    if (!(cs > 0) || !std::isfinite(cs)) cs = 1.0;
    j.cell_size = (float)cs;
    j.cell_inv = (float)(1.0 / cs);
    j.cell_ox = (float)lo[0];
    j.cell_oy = (float)lo[1];
    j.gx = std::max(1, std::min(64, (int)std::ceil(sx / cs)));
    j.gy = std::max(1, std::min(64, (int)std::ceil(sy / cs)));
}

// Longest launch of the block planner (s of device time) when its caller sets
// no limit: the launch stops at the first wavefront boundary past it.
static constexpr double kBPlanSliceS = 1.0;

// Wavefronts inside the persistent block planner until a stop condition
// (solved, node budget, wavefront count, time) or its node capacity; then the
// kd-tree takes the new nodes and the host its goals.  *waves: wavefronts run.
static mptg_status run_persistent(mptg_planner* p, int max_waves, double time_limit_s, int stop_when_solved,
                                  int* waves) {
    mptg_ctx* ctx = p->ctx;
    cudaStream_t s = p->stream;
    *waves = 0;
    mptg_status st0 = MPTG_OK;
    const size_t n0 = planner_n(p);
    const int W = p->prm.wavefront;
    const int cap = p->bp_states ? p->bp_cap : (int)std::min<size_t>(p->prm.max_nodes, BPLAN_MAX_NODES);
    if (n0 >= p->prm.max_nodes || std::min<size_t>(n0 + W, p->prm.max_nodes) > (size_t)cap) return MPTG_OK;
    if (!p->bp_states && (st0 = bp_alloc(p))) return st0;
    const PlanView v = plan_view(p);
    BPlanJob j{};
    j.scene = scene_view(p->scene);
    j.lo = p->lo;
    j.hi = p->hi;
    j.goal = p->goal;
    j.has_goal = p->has_goal;
    j.goal_bias = v.goal_bias;
    j.range = v.range;
    j.goal_radius = v.goal_radius;
    j.inv_step = 1.0 / p->prm.edge_step;
    j.seed = v.seed;
    j.states = p->bp_states;
    j.parent = p->parent;
    j.goalf = p->bp_goalf;
    j.ctr = p->bp_ctr;
    j.nsamp = p->nsamp;
    j.max_nodes = p->prm.max_nodes;
    j.cap = p->bp_cap;
    j.W = W;
    j.max_waves = max_waves;
    j.stop_when_solved = stop_when_solved;
    j.deadline_ns = time_limit_s > 0 ? (uint64_t)(time_limit_s * 1e9) : 0;
    j.brute_pairs = p->bp_brute_pairs;
    bp_cells(j, p->lo_host, p->hi_host);
    BPlanCounters* h = p->bp_hctr;
    *h = BPlanCounters{};
    h->n = (int)n0;
    h->wave = p->wave;
    h->goals = (int)p->goals.size();
    mptg_status st = MPTG_OK;
    if (p->bp_n != n0) {  // nodes added elsewhere since the last block run: mirror the tree
        if ((st = mptg_tree_states(p->tree, 0, n0, p->bp_states, s))) return st;
        p->bp_n = n0;
    }
    *p->bp_hjob = j;  // the previous run's copy ended at its synchronisation
    if (p->bp_graph && p->bp_graph_W != W) {
        cudaGraphExecDestroy(p->bp_graph);
        p->bp_graph = nullptr;
    }
    if (!p->bp_graph && !p->bp_graph_off) bp_capture(p, W);
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->ev[0], s));
    if (p->bp_graph) {
        MPTG_CUDA_TRY(ctx, cudaGraphLaunch(p->bp_graph, s));
        MPTG_LAUNCHED(ctx);
        ++p->bp_graph_runs;
    } else {
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->bp_job, p->bp_hjob, sizeof(j), cudaMemcpyHostToDevice, s));
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->bp_ctr, h, sizeof(*h), cudaMemcpyHostToDevice, s));
        if ((st = bplan_launch(ctx, p->bp_job, 1, W, p->bp_cap, s))) return st;
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(h, p->bp_ctr, sizeof(*h), cudaMemcpyDeviceToHost, s));
    }
    MPTG_CUDA_TRY(ctx, cudaEventRecord(p->ev[1], s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    {
        // the phase timers (nearest, valid motion, insert) share the block's
        // time in proportion to the SM cycles it spent in each phase
        float ms = 0.f;
        MPTG_CUDA_TRY(ctx, cudaEventElapsedTime(&ms, p->ev[0], p->ev[1]));
        double tot = 0;
        for (int i = 0; i < 6; ++i) tot += (double)h->cyc[i];
        if (tot > 0) {
            p->t_phase[0] += 1e-3 * ms * (double)(h->cyc[0] + h->cyc[1] + h->cyc[2]) / tot;
            p->t_phase[2] += 1e-3 * ms * (double)(h->cyc[3] + h->cyc[4]) / tot;
            p->t_phase[3] += 1e-3 * ms * (double)h->cyc[5] / tot;
        }
        for (int i = 0; i < 6; ++i) p->bp_prof[i] += (double)h->cyc[i];
        p->bp_prof[6] += (double)h->ties;
        p->bp_prof[7] += (double)h->unsure;
        p->bp_prof[8] += (double)h->steps64;
    }
    const size_t n1 = (size_t)h->n;
    p->wave = h->wave;
    p->stat_samples += h->samples;
    p->stat_accepted += h->accepted;
    p->stat_wavefronts += (uint64_t)h->waves_run;
    p->stat_bp_waves += (uint64_t)h->waves_run;
    *waves = h->waves_run;
    if (n1 > n0) {
        const size_t k = n1 - n0;
        p->bp_n = n1;  // the kd-tree takes them when it is next needed (bp_flush)
        if (h->goals > (int)p->goals.size()) {
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->bp_hgoal, p->bp_goalf + n0, k, cudaMemcpyDeviceToHost, s));
            MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
            for (size_t i = 0; i < k; ++i)
                if (p->bp_hgoal[i]) p->goals.push_back((int)(n0 + i));
        }
    }
    return MPTG_OK;
}

extern "C" {

mptg_status mptg_planner_set_persistent(mptg_planner* p, int mode) {
    if (!p || mode < 0 || mode > 1) return MPTG_ERR_INVALID_ARG;
    p->bp_mode = mode;
    return MPTG_OK;
}

mptg_status mptg_planner_graph_runs(mptg_planner* p, uint64_t* runs) {
    if (!p || !runs) return MPTG_ERR_INVALID_ARG;
    *runs = p->bp_graph_runs;
    return MPTG_OK;
}

mptg_status mptg_planner_set_block_search(mptg_planner* p, long long brute_pairs) {
    if (!p || brute_pairs < 0) return MPTG_ERR_INVALID_ARG;
    p->bp_brute_pairs = brute_pairs;
    return MPTG_OK;
}

mptg_status mptg_planner_create(mptg_ctx* ctx, mptg_scene* scene, const mptg_plan_params* prm, const double* lo,
                                const double* hi, mptg_planner** out) {
    if (!ctx || !scene || !prm || !out) return MPTG_ERR_INVALID_ARG;
    *out = nullptr;
    mptg_status st = check_params(ctx, scene, prm);
    if (st) return st;
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    mptg_planner* p = new mptg_planner();
    p->ctx = ctx;
    p->scene = scene;
    p->prm = *prm;
    p->D = scene->D;
    p->metric = scene->metric;
    p->w0 = scene->w0;
    p->w1 = scene->w1;
    p->cap_nodes = prm->max_nodes;
    p->cap_wave = prm->wavefront;
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete p;
        return mptg_fail(ctx, MPTG_ERR_CUDA, "planner stream: %s", cudaGetErrorString(e));
    }
    for (cudaEvent_t& ev : p->ev)
        if (e == cudaSuccess) e = cudaEventCreate(&ev);
    if (e != cudaSuccess) {
        planner_free(p);
        return mptg_fail(ctx, MPTG_ERR_CUDA, "planner events: %s", cudaGetErrorString(e));
    }
    double w[2] = {p->w0, p->w1};
    if ((st = mptg_tree_create(ctx, (mptg_metric)p->metric, p->D, w, prm->max_nodes, &p->tree))) {
        planner_free(p);
        return st;
    }
    const size_t W = prm->wavefront, D = p->D, N = prm->max_nodes;
#define ALLOC(ptr, bytes) if (e == cudaSuccess) e = cudaMalloc((void**)&(ptr), (bytes))
    ALLOC(p->lo, D * sizeof(double));
    ALLOC(p->hi, D * sizeof(double));
    ALLOC(p->goal, D * sizeof(double));
    ALLOC(p->parent, N * sizeof(int));
    ALLOC(p->samp, W * D * sizeof(double));
    ALLOC(p->nidx, W * sizeof(int));
    ALLOC(p->ndist, W * sizeof(double));
    ALLOC(p->nearst, W * D * sizeof(double));
    ALLOC(p->newst, W * D * sizeof(double));
    ALLOC(p->skip, W);
    ALLOC(p->ok, W);
    ALLOC(p->scan, W * sizeof(int));
    ALLOC(p->bsum, (1024 + 2) * sizeof(int));
    ALLOC(p->acc_states, W * D * sizeof(double));
    ALLOC(p->acc_parent, W * sizeof(int));
    ALLOC(p->acc_goal, W);
    ALLOC(p->nsamp, sizeof(unsigned long long));
    ALLOC(p->path_ids, N * sizeof(int));
    ALLOC(p->path_out, 2 * sizeof(double));
#undef ALLOC
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->hbuf, 16 * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->hgoal, W);
    if (e != cudaSuccess) {
        cudaGetLastError();
        planner_free(p);
        return mptg_fail(ctx, MPTG_ERR_OOM, "planner allocation failed: %s", cudaGetErrorString(e));
    }
    if ((st = set_bounds(p, lo, hi))) { planner_free(p); return st; }
    // grid planners run on the block planner: its buffers now, not in the first solve
    if (bplan_supported(scene, prm->wavefront, prm->resolution) && (st = bp_alloc(p))) {
        planner_free(p);
        return st;
    }
    e = cudaMemsetAsync(p->nsamp, 0, sizeof(unsigned long long), p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
        planner_free(p);
        return mptg_fail(ctx, MPTG_ERR_CUDA, "planner init failed: %s", cudaGetErrorString(e));
    }
    *out = p;
    return MPTG_OK;
}

mptg_status mptg_planner_destroy(mptg_planner* p) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    planner_free(p);
    return MPTG_OK;
}

mptg_status mptg_planner_reset(mptg_planner* p, const mptg_plan_params* params) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    return planner_reset(p, params, false, nullptr, nullptr);
}

mptg_status mptg_planner_add_start(mptg_planner* p, const double* q) {
    if (!p || !q) return MPTG_ERR_INVALID_ARG;
    mptg_status st = bp_flush(p);
    if (st) return st;
    size_t n = 0;
    mptg_tree_size(p->tree, &n);
    if (n >= p->prm.max_nodes) return mptg_fail(p->ctx, MPTG_ERR_CAPACITY, "node budget reached");
    st = mptg_tree_insert(p->tree, q, 1, p->stream);
    if (st) return st;
    const int minus1 = -1;
    MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(p->parent + n, &minus1, sizeof(int), cudaMemcpyHostToDevice, p->stream));
    if (p->star) {
        MPTG_CUDA_TRY(p->ctx, cudaMemsetAsync(p->cost + n, 0, sizeof(double), p->stream));
        MPTG_CUDA_TRY(p->ctx, cudaMemsetAsync(p->elen + n, 0, sizeof(double), p->stream));
    }
    MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
    return MPTG_OK;
}

mptg_status mptg_planner_set_goal(mptg_planner* p, const double* q, double radius) {
    if (!p || !q) return MPTG_ERR_INVALID_ARG;
    if (!(radius >= 0)) return mptg_fail(p->ctx, MPTG_ERR_INVALID_ARG, "goal radius must be >= 0");
    MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(p->goal, q, p->D * sizeof(double), cudaMemcpyDefault, p->stream));
    MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
    p->goal_host.assign(q, q + p->D);
    p->has_goal = 1;
    p->prm.goal_radius = radius;
    return MPTG_OK;
}

mptg_status mptg_planner_run(mptg_planner* p, int max_wavefronts, double time_limit_s, int stop_when_solved,
                             int* solved) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = p->ctx;
    size_t n = planner_n(p);
    if (n == 0) return mptg_fail(ctx, MPTG_ERR_NO_START, "there are no valid initial states");
    if (p->solving) return mptg_fail(ctx, MPTG_ERR_ALREADY_SOLVING, "already solving");
    p->solving = true;
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    auto t0 = std::chrono::steady_clock::now();
    mptg_status st = MPTG_OK;
    int it = 0;
    if (bp_applies(p) && !(stop_when_solved && !p->goals.empty())) {
        // a call with neither a wavefront count nor a time limit runs the block
        // planner in launches of at most kBPlanSliceS seconds of device time,
        // relaunched while the tree can still grow: a start the tree never
        // leaves (every link invalid) would otherwise keep one launch running
        // for ever.  The launches run the same wavefronts one launch would.
        const bool unbounded = max_wavefronts <= 0 && !(time_limit_s > 0);
        for (;;) {
            int w = 0;
            st = run_persistent(p, max_wavefronts, unbounded ? kBPlanSliceS : time_limit_s, stop_when_solved, &w);
            it += w;
            if (st || !unbounded || w == 0 || p->bp_hctr->status == BPLAN_FULL) break;
            if ((stop_when_solved && !p->goals.empty()) || planner_n(p) >= p->prm.max_nodes) break;
        }
    }
    // the multi-kernel wavefront: every other case, and what remains of this
    // call once the block planner's node capacity is reached
    for (; !st && (max_wavefronts <= 0 || it < max_wavefronts); ++it) {
        if (stop_when_solved && !p->goals.empty()) break;
        n = planner_n(p);
        if (n >= p->prm.max_nodes) break;
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (time_limit_s > 0 && el >= time_limit_s) break;
        int added = 0;
        st = plan_wavefront(p, p->stream, &added);
        if (st) break;
    }
    p->stat_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    p->solving = false;
    if (solved) *solved = p->goals.empty() ? 0 : 1;
    return st;
}

mptg_status mptg_planner_size(mptg_planner* p, size_t* n) {
    if (!p || !n) return MPTG_ERR_INVALID_ARG;
    *n = planner_n(p);
    return MPTG_OK;
}

mptg_status mptg_planner_goals(mptg_planner* p, size_t* n) {
    if (!p || !n) return MPTG_ERR_INVALID_ARG;
    *n = p->goals.size();
    return MPTG_OK;
}

// PRRT::bestSolution + solution() (prrt.hpp:219-274) on the planner's stream
static mptg_status planner_solution(mptg_planner* p, double* path, size_t cap, size_t* len, double* cost,
                                    bool path_must_fit) {
    mptg_ctx* ctx = p->ctx;
    cudaStream_t s = p->stream;
    *len = 0;
    if (cost) *cost = INFINITY;
    if (p->goals.empty()) return MPTG_OK;
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    double* hd = reinterpret_cast<double*>(p->hbuf + 8);  // 2 doubles of the pinned words
    size_t tn = 0;
    mptg_tree_size(p->tree, &tn);
    // the block planner's mirror holds every node when the kd-tree lags behind it
    const double* states = p->bp_n > tn ? p->bp_states : mptg_tree_states_dev(p->tree);
    // best goal by path cost; goals are visited newest first with strict <,
    // as PRRT::bestSolution walks its push_front list (prrt.hpp:219-234)
    double best = INFINITY;
    int bestg = -1, bestlen = 0;
    for (size_t k = p->goals.size(); k-- > 0;) {
        k_plan_path<<<1, 1, 0, s>>>(p->goals[k], p->parent, states, p->D, p->metric, p->w0, p->w1, 0, nullptr,
                                    p->path_out);
        MPTG_LAUNCHED(ctx);
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(hd, p->path_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        if (hd[0] < best || bestg < 0) { best = hd[0]; bestg = p->goals[k]; bestlen = (int)hd[1]; }
    }
    *len = (size_t)bestlen;
    if (cost) *cost = best;
    if (!path) return MPTG_OK;
    if ((size_t)bestlen > cap) {
        if (!path_must_fit) return MPTG_OK;
        return mptg_fail(ctx, MPTG_ERR_CAPACITY, "path of %d states does not fit %zu", bestlen, cap);
    }
    k_plan_path<<<1, 1, 0, s>>>(bestg, p->parent, states, p->D, p->metric, p->w0, p->w1, bestlen, p->path_ids,
                                p->path_out);
    MPTG_LAUNCHED(ctx);
    // gather the waypoints through the wavefront state buffer, cap_wave states at a time
    for (int c = 0; c < bestlen; c += p->cap_wave) {
        int m = std::min(p->cap_wave, bestlen - c);
        k_plan_gather<<<mptg_blocks(m * p->D, 256), 256, 0, s>>>(p->path_ids + c, m, states, p->D, p->acc_states);
        MPTG_LAUNCHED(ctx);
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(path + (size_t)c * p->D, p->acc_states, (size_t)m * p->D * sizeof(double),
                                           cudaMemcpyDefault, s));
    }
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return MPTG_OK;
}

mptg_status mptg_planner_solution(mptg_planner* p, double* path, size_t cap, size_t* len, double* cost) {
    if (!p || !len) return MPTG_ERR_INVALID_ARG;
    return planner_solution(p, path, cap, len, cost, true);
}

mptg_status mptg_planner_tree(mptg_planner* p, mptg_tree** tree) {
    if (!p || !tree) return MPTG_ERR_INVALID_ARG;
    mptg_status st = bp_flush(p);
    if (st) return st;
    *tree = p->tree;
    return MPTG_OK;
}

mptg_status mptg_planner_graph(mptg_planner* p, double* states, int32_t* parents, size_t cap, size_t* n) {
    if (!p || !n) return MPTG_ERR_INVALID_ARG;
    size_t tn = 0;
    mptg_tree_size(p->tree, &tn);
    const size_t sz = planner_n(p);
    *n = sz;
    if (!states && !parents) return MPTG_OK;
    if (sz > cap) return mptg_fail(p->ctx, MPTG_ERR_CAPACITY, "graph of %zu nodes does not fit %zu", sz, cap);
    if (states && p->bp_n > tn) {  // the block planner's mirror holds every node
        MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(states, p->bp_states, sz * 2 * sizeof(double), cudaMemcpyDefault,
                                              p->stream));
    } else if (states) {
        mptg_status st = mptg_tree_states(p->tree, 0, sz, states, p->stream);
        if (st) return st;
    }
    if (parents)
        MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(parents, p->parent, sz * sizeof(int), cudaMemcpyDefault, p->stream));
    MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
    return MPTG_OK;
}

mptg_status mptg_planner_set_surrogate(mptg_planner* p, mptg_surrogate* sg, double threshold) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    if (sg && (!p->logits || !p->near_c)) {
        const size_t W = p->cap_wave, D = p->D;
        cudaError_t e = cudaSuccess;
        if (!p->logits) e = cudaMalloc((void**)&p->logits, W * p->sg_pts_cap * sizeof(float));
        if (!p->near_c) {
            if (e == cudaSuccess) e = cudaMalloc((void**)&p->near_c, W * D * sizeof(double));
            if (e == cudaSuccess) e = cudaMalloc((void**)&p->new_c, W * D * sizeof(double));
            if (e == cudaSuccess) e = cudaMalloc((void**)&p->cmap, W * sizeof(int));
            if (e == cudaSuccess) e = cudaMalloc((void**)&p->ok_c, W);
            if (e == cudaSuccess) e = cudaMalloc((void**)&p->keep, W);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            return mptg_fail(p->ctx, MPTG_ERR_OOM, "surrogate buffers: %s", cudaGetErrorString(e));
        }
    }
    p->sg = sg;
    p->sg_thr = (float)threshold;
    return MPTG_OK;
}

mptg_status mptg_planner_set_surrogate_points(mptg_planner* p, int points) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    if (points < 1 || points > 8) return mptg_fail(p->ctx, MPTG_ERR_INVALID_ARG, "surrogate points must be in [1, 8]");
    if (points > p->sg_pts_cap) {
        const size_t W = p->cap_wave, D = p->D;
        MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
        cudaFree(p->logits);
        cudaFree(p->sg_pts);
        p->logits = nullptr;
        p->sg_pts = nullptr;
        p->sg_pts_cap = 0;
        cudaError_t e = cudaMalloc((void**)&p->logits, W * points * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc((void**)&p->sg_pts, W * points * D * sizeof(double));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return mptg_fail(p->ctx, MPTG_ERR_OOM, "surrogate point buffers: %s", cudaGetErrorString(e));
        }
        p->sg_pts_cap = points;
    }
    p->sg_points = points;
    if (p->sg_bias > 1 && points > p->b_pts_cap) return mptg_planner_set_surrogate_bias(p, p->sg_bias);
    return MPTG_OK;
}

mptg_status mptg_planner_set_surrogate_bias(mptg_planner* p, int candidates) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    if (candidates < 1 || candidates > 16)
        return mptg_fail(p->ctx, MPTG_ERR_INVALID_ARG, "candidates per wavefront slot must be in [1, 16]");
    const size_t W = p->cap_wave, D = p->D, P = (size_t)std::max(p->sg_points, p->sg_pts_cap);
    if (candidates > 1 && (candidates > p->sg_bias_cap || (int)P > p->b_pts_cap)) {
        MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
        void* old[] = {p->b_samp, p->b_nidx, p->b_ndist, p->b_near, p->b_new, p->b_skip, p->b_pts, p->b_logits};
        for (void* x : old)
            if (x) cudaFree(x);
        const int B = std::max(candidates, p->sg_bias_cap);
        const size_t WB = W * B;
        cudaError_t e = cudaSuccess;
#define ALLOC(ptr, bytes) if (e == cudaSuccess) e = cudaMalloc((void**)&(ptr), (bytes))
        ALLOC(p->b_samp, WB * D * sizeof(double));
        ALLOC(p->b_nidx, WB * sizeof(int));
        ALLOC(p->b_ndist, WB * sizeof(double));
        ALLOC(p->b_near, WB * D * sizeof(double));
        ALLOC(p->b_new, WB * D * sizeof(double));
        ALLOC(p->b_skip, WB);
        ALLOC(p->b_pts, WB * P * D * sizeof(double));
        ALLOC(p->b_logits, WB * P * sizeof(float));
#undef ALLOC
        if (e != cudaSuccess) {
            cudaGetLastError();
            p->sg_bias_cap = 0;
            p->b_pts_cap = 0;
            return mptg_fail(p->ctx, MPTG_ERR_OOM, "surrogate bias buffers: %s", cudaGetErrorString(e));
        }
        p->sg_bias_cap = B;
        p->b_pts_cap = (int)P;
    }
    p->sg_bias = candidates;
    return MPTG_OK;
}

mptg_status mptg_planner_set_rewire(mptg_planner* p, int enabled, double rewire_factor) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = p->ctx;
    if (!(rewire_factor > 0) || !std::isfinite(rewire_factor))
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "rewire factor must be positive");
    if (p->stat_wavefronts > 0)
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "rewiring must be chosen before the first wavefront");
    p->rewire_factor = rewire_factor;
    if (!enabled) { p->star = 0; return MPTG_OK; }
    if (!p->cost) {
        const size_t N = p->cap_nodes, W = p->cap_wave, D = p->D, P = W * 64;
        cudaError_t e = cudaSuccess;
#define ALLOC(ptr, bytes) if (e == cudaSuccess) e = cudaMalloc((void**)&(ptr), (bytes))
        ALLOC(p->cost, N * sizeof(double));
        ALLOC(p->elen, N * sizeof(double));
        ALLOC(p->pj_s, N * sizeof(double));
        ALLOC(p->pj_a, N * sizeof(int));
        ALLOC(p->pj_a2, N * sizeof(int));
        ALLOC(p->bbits, N * sizeof(unsigned long long));
        ALLOC(p->bid, N * sizeof(int));
        ALLOC(p->knn_i, P * sizeof(int));
        ALLOC(p->knn_d, P * sizeof(double));
        ALLOC(p->pv, P);
        ALLOC(p->s_pair, P * sizeof(int));
        ALLOC(p->s_rcost, P * sizeof(double));
        ALLOC(p->s_ok, P);
        ALLOC(p->s_ea, P * D * sizeof(double));
        ALLOC(p->s_eb, P * D * sizeof(double));
        ALLOC(p->dnear, W * sizeof(double));
        ALLOC(p->cpar, W * sizeof(int));
        ALLOC(p->ccost, W * sizeof(double));
        ALLOC(p->celen, W * sizeof(double));
        ALLOC(p->s_cnt, 2 * sizeof(int));
        ALLOC(p->nrw, sizeof(unsigned long long));
        ALLOC(p->rank, P * sizeof(int));
        ALLOC(p->decided, W);
#undef ALLOC
        if (e != cudaSuccess) {
            cudaGetLastError();
            return mptg_fail(ctx, MPTG_ERR_OOM, "rewiring buffers: %s", cudaGetErrorString(e));
        }
        MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->bbits, 0xff, N * sizeof(unsigned long long), p->stream));
        MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->bid, 0x7f, N * sizeof(int), p->stream));
        for (cudaEvent_t& ev : p->sev) MPTG_CUDA_TRY(ctx, cudaEventCreate(&ev));
    }
    // every node so far is a start: no parent, cost 0
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->cost, 0, p->cap_nodes * sizeof(double), p->stream));
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->elen, 0, p->cap_nodes * sizeof(double), p->stream));
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->nrw, 0, sizeof(unsigned long long), p->stream));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(p->stream));
    p->star = 1;
    p->stat_rewire_tests = 0;
    return MPTG_OK;
}

mptg_status mptg_planner_costs(mptg_planner* p, double* out, size_t cap, size_t* n) {
    if (!p || !n) return MPTG_ERR_INVALID_ARG;
    size_t sz = 0;
    mptg_tree_size(p->tree, &sz);
    *n = sz;
    if (!out) return MPTG_OK;
    if (!p->star) return mptg_fail(p->ctx, MPTG_ERR_INVALID_ARG, "node costs are kept with rewiring only");
    if (sz > cap) return mptg_fail(p->ctx, MPTG_ERR_CAPACITY, "%zu costs do not fit %zu", sz, cap);
    MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(out, p->cost, sz * sizeof(double), cudaMemcpyDefault, p->stream));
    MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
    return MPTG_OK;
}

mptg_status mptg_planner_rewire_stats(mptg_planner* p, double out[6]) {
    if (!p || !out) return MPTG_ERR_INVALID_ARG;
    unsigned long long n = 0;
    if (p->nrw) {
        MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(&n, p->nrw, sizeof(n), cudaMemcpyDeviceToHost, p->stream));
        MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
    }
    out[0] = (double)n;
    out[1] = (double)p->stat_rewire_tests;
    for (int k = 0; k < 4; ++k) out[2 + k] = p->t_star[k];
    return MPTG_OK;
}

mptg_status mptg_planner_timers(mptg_planner* p, double out[4]) {
    if (!p || !out) return MPTG_ERR_INVALID_ARG;
    for (int k = 0; k < 4; ++k) out[k] = p->t_phase[k];
    return MPTG_OK;
}

mptg_status mptg_planner_block_profile(mptg_planner* p, double out[9]) {
    if (!p || !out) return MPTG_ERR_INVALID_ARG;
    for (int i = 0; i < 9; ++i) out[i] = p->bp_prof[i];
    return MPTG_OK;
}

mptg_status mptg_planner_stats(mptg_planner* p, double out[8]) {
    if (!p || !out) return MPTG_ERR_INVALID_ARG;
    unsigned long long ns = 0;
    MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(&ns, p->nsamp, sizeof(ns), cudaMemcpyDeviceToHost, p->stream));
    MPTG_CUDA_TRY(p->ctx, cudaStreamSynchronize(p->stream));
    const size_t n = planner_n(p);
    out[0] = (double)p->stat_wavefronts;
    out[1] = (double)p->stat_samples;
    out[2] = (double)p->stat_accepted;
    out[3] = (double)n;
    out[4] = (double)p->goals.size();
    out[5] = (double)ns;
    out[6] = p->stat_seconds;
    out[7] = (double)p->wave;
    return MPTG_OK;
}

// ------------------------------------------------------------- batch serving

using BatchCaps = std::map<mptg_scene*, std::pair<size_t, int>>;  // scene -> (max budget, max wavefront)

static double seconds_since(std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}

// one query on this worker's planner for its scene (created on first use with
// the batch's largest budget and wavefront for that scene)
static mptg_status batch_query(mptg_ctx* ctx, const mptg_query& q, const BatchCaps& caps,
                               std::map<mptg_scene*, mptg_planner*>& mine, mptg_result& r) {
    mptg_planner*& p = mine[q.scene];
    mptg_status st;
    if (!p) {
        mptg_plan_params c = q.params;
        const auto& cap = caps.at(q.scene);
        c.max_nodes = cap.first;
        c.wavefront = cap.second;
        if ((st = mptg_planner_create(ctx, q.scene, &c, q.lo, q.hi, &p))) return st;
    }
    if ((st = planner_reset(p, &q.params, true, q.lo, q.hi))) return st;
    if ((st = mptg_planner_set_surrogate(p, q.surrogate, q.surrogate_threshold))) return st;
    if ((st = mptg_planner_set_surrogate_points(p, q.surrogate ? std::max(1, q.surrogate_points) : 1))) return st;
    if ((st = mptg_planner_set_surrogate_bias(p, q.surrogate ? std::max(1, q.surrogate_candidates) : 1))) return st;
    if ((st = mptg_planner_add_start(p, q.start))) return st;
    if ((st = mptg_planner_set_goal(p, q.goal, q.goal_radius))) return st;
    const auto t = std::chrono::steady_clock::now();
    int solved = 0;
    st = mptg_planner_run(p, 0, q.time_limit_s, 1, &solved);
    r.solve_s = seconds_since(t);
    r.solved = solved;
    r.nodes = planner_n(p);
    r.wavefronts = (size_t)p->stat_wavefronts;
    if (st) return st;
    return planner_solution(p, q.path, q.path_cap, &r.path_len, &r.cost, false);
}

// ---- the grid queries of a batch as one persistent launch
// The batch's grid queries that the block planner takes (a grid scene at
// resolution 0, W <= 1024, no surrogate) run together: one k_bplan_grid block
// per query, all in one launch on a stream of their own, while the host
// workers take the other queries.  Each block runs exactly the wavefronts a
// single planner runs (run_persistent with stop_when_solved), so it builds
// the same tree, and the solution is read as planner_solution reads it
// (k_plan_path over the goals, newest first, strict <).  A query whose block
// fills its 16,384 nodes unsolved goes back to the workers, which run it from
// its start (the same tree again, so the same answer; only the block's time
// is lost).
struct GridBatch {
    std::vector<size_t> idx;        // query indices, one block each
    std::vector<size_t> retry;      // queries the workers must run (capacity reached)
    std::vector<BPlanJob> jobs;
    std::vector<size_t> off;        // arena offset of each job's buffers
    unsigned char* arena = nullptr;
    BPlanCounters* hctr = nullptr;  // pinned
    cudaStream_t s = nullptr;
    std::chrono::steady_clock::time_point t_launch;
    int maxW = 0, maxcap = 0;
    size_t ctr_off = 0, job_off = 0, scratch_off = 0;
};

static bool grid_batch_eligible(const mptg_query& q) {
    if (q.surrogate || q.params.max_nodes < 1) return false;
    if (!bplan_supported(q.scene, q.params.wavefront, q.params.resolution)) return false;
    for (int d = 0; d < 2; ++d)
        if (!std::isfinite(q.start[d]) || !std::isfinite(q.goal[d])) return false;
    return true;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// each job's node 0 (the start, no parent, no goal flag) and its goal and
// sampling bounds, from rec[k] = start, goal, lo, hi (8 doubles)
__global__ void k_gb_init(const BPlanJob* __restrict__ jobs, int K, const double* __restrict__ rec) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const BPlanJob& j = jobs[k];
    const double* r = rec + 8 * (size_t)k;
    j.states[0] = r[0];
    j.states[1] = r[1];
    j.parent[0] = -1;
    j.goalf[0] = 0;
    double* v = const_cast<double*>(j.goal);  // goal, lo, hi: 6 doubles in the job's buffers
    for (int i = 0; i < 6; ++i) v[i] = r[2 + i];
}

static void grid_batch_free(GridBatch& g) {
    if (g.s) cudaStreamSynchronize(g.s);
    if (g.arena) cudaFree(g.arena);
    if (g.hctr) cudaFreeHost(g.hctr);
    if (g.s) cudaStreamDestroy(g.s);
    g.arena = nullptr;
    g.hctr = nullptr;
    g.s = nullptr;
}

// buffers, jobs and the launch (asynchronous)
static mptg_status grid_batch_launch(mptg_ctx* ctx, const mptg_query* qs, GridBatch& g) {
    const size_t K = g.idx.size();
    size_t o = 0;
    g.off.resize(K);
    for (size_t k = 0; k < K; ++k) {
        const mptg_query& q = qs[g.idx[k]];
        const int cap = (int)std::min<size_t>(q.params.max_nodes, BPLAN_MAX_NODES);
        g.maxcap = std::max(g.maxcap, cap);
        g.maxW = std::max(g.maxW, q.params.wavefront);
        g.off[k] = o;  // states [cap][2], parent [cap], goal flags [cap], goal / lo / hi
        o += align256((size_t)cap * 16) + align256((size_t)cap * 4) + align256((size_t)cap) + 256;
    }
    g.ctr_off = o;
    o += align256(K * sizeof(BPlanCounters));
    g.job_off = o;
    o += align256(K * sizeof(BPlanJob));
    g.scratch_off = o;  // k_plan_path: cost and length, path ids, gathered states
    o += 256 + align256((size_t)g.maxcap * 4) + align256((size_t)g.maxcap * 16);
    const size_t rec_off = o;  // the jobs' start, goal and bounds for k_gb_init
    o += align256(K * 8 * sizeof(double));
    cudaError_t e = cudaMalloc((void**)&g.arena, o);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&g.hctr, K * sizeof(BPlanCounters));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g.s, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return mptg_fail(ctx, MPTG_ERR_OOM, "batch of grid queries: %s", cudaGetErrorString(e));
    }
    std::vector<double> rec(K * 8);
    g.jobs.resize(K);
    for (size_t k = 0; k < K; ++k) {
        const mptg_query& q = qs[g.idx[k]];
        const mptg_plan_params& prm = q.params;
        const int cap = (int)std::min<size_t>(prm.max_nodes, BPLAN_MAX_NODES);
        unsigned char* base = g.arena + g.off[k];
        const size_t o_par = align256((size_t)cap * 16), o_gf = o_par + align256((size_t)cap * 4),
                     o_vec = o_gf + align256((size_t)cap);
        double* vec = rec.data() + 8 * k + 2;  // goal, lo, hi: the planner's bounds rule (set_bounds)
        rec[8 * k] = q.start[0];
        rec[8 * k + 1] = q.start[1];
        for (int d = 0; d < 2; ++d) {
            vec[d] = q.goal[d];
            vec[2 + d] = q.lo ? q.lo[d] : 0.0;
            vec[4 + d] = q.hi ? q.hi[d] : 1.0;
        }
        BPlanJob& j = g.jobs[k];
        j = BPlanJob{};
        j.scene = scene_view(q.scene);
        j.goal = reinterpret_cast<const double*>(base + o_vec);
        j.lo = j.goal + 2;
        j.hi = j.goal + 4;
        j.has_goal = 1;
        j.goal_bias = prm.goal_bias;
        j.range = prm.range > 0 ? prm.range : INFINITY;
        j.goal_radius = q.goal_radius;
        j.inv_step = 1.0 / prm.edge_step;
        j.seed = prm.seed;
        j.states = reinterpret_cast<double*>(base);
        j.parent = reinterpret_cast<int*>(base + o_par);
        j.goalf = base + o_gf;
        j.ctr = reinterpret_cast<BPlanCounters*>(g.arena + g.ctr_off) + k;
        j.nsamp = nullptr;
        j.max_nodes = prm.max_nodes;
        j.cap = cap;
        j.W = prm.wavefront;
        j.max_waves = 0;
        j.stop_when_solved = 1;
        // a query without a time limit gets one slice (grid_batch_finish sends
        // a block that ends on it unsolved back to the workers)
        j.deadline_ns = (uint64_t)((q.time_limit_s > 0 ? q.time_limit_s : kBPlanSliceS) * 1e9);
        j.brute_pairs = BPLAN_BRUTE_PAIRS;
        bp_cells(j, vec + 2, vec + 4);
        g.hctr[k] = BPlanCounters{};
        g.hctr[k].n = 1;
    }
    // pageable copies are staged before they return, so `rec` may go
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(g.arena + rec_off, rec.data(), rec.size() * sizeof(double),
                                       cudaMemcpyHostToDevice, g.s));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(g.arena + g.ctr_off, g.hctr, K * sizeof(BPlanCounters), cudaMemcpyHostToDevice,
                                       g.s));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(g.arena + g.job_off, g.jobs.data(), K * sizeof(BPlanJob),
                                       cudaMemcpyHostToDevice, g.s));
    k_gb_init<<<mptg_blocks(K, 128), 128, 0, g.s>>>(reinterpret_cast<const BPlanJob*>(g.arena + g.job_off), (int)K,
                                                   reinterpret_cast<const double*>(g.arena + rec_off));
    MPTG_LAUNCHED(ctx);
    g.t_launch = std::chrono::steady_clock::now();
    mptg_status st = bplan_launch(ctx, reinterpret_cast<const BPlanJob*>(g.arena + g.job_off), (int)K, g.maxW,
                                  g.maxcap, g.s);
    if (st) return st;
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(g.hctr, g.arena + g.ctr_off, K * sizeof(BPlanCounters), cudaMemcpyDeviceToHost,
                                       g.s));
    return MPTG_OK;
}

// waits for the launch and fills the results; queries to run again go to g.retry
static mptg_status grid_batch_finish(mptg_ctx* ctx, const mptg_query* qs, GridBatch& g, mptg_result* out,
                                     std::chrono::steady_clock::time_point t0) {
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(g.s));
    const size_t K = g.idx.size();
    unsigned long long first = ~0ull;
    for (size_t k = 0; k < K; ++k) first = std::min(first, g.hctr[k].start_ns);
    const double launch_s = std::chrono::duration<double>(g.t_launch - t0).count();
    double hd[2];
    std::vector<uint8_t> gf;
    mptg_status st = MPTG_OK;
    for (size_t k = 0; k < K && !st; ++k) {
        const BPlanCounters& h = g.hctr[k];
        const mptg_query& q = qs[g.idx[k]];
        // unsolved with its block full, or (no time limit) stopped by the slice
        // below its node budget: the workers run it from its start
        if (h.goals == 0 &&
            (h.status == BPLAN_FULL || (!(q.time_limit_s > 0) && (size_t)h.n < q.params.max_nodes))) {
            g.retry.push_back(g.idx[k]);
            continue;
        }
        mptg_result& r = out[g.idx[k]];
        r = mptg_result{};
        r.cost = INFINITY;
        r.solved = h.goals > 0;
        r.nodes = (size_t)h.n;
        r.wavefronts = (size_t)h.waves_run;
        // from the launch's first block to this block's end: a query that
        // waited for a free SM counts its wait
        r.solve_s = 1e-9 * (double)(h.end_ns - first);
        r.finish_s = launch_s + r.solve_s;
        if (!r.solved) continue;
        const BPlanJob& j = g.jobs[k];
        gf.resize((size_t)h.n);
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(gf.data(), j.goalf, (size_t)h.n, cudaMemcpyDeviceToHost, g.s));
        MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(g.s));
        double* sc = reinterpret_cast<double*>(g.arena + g.scratch_off);
        int* ids = reinterpret_cast<int*>(g.arena + g.scratch_off + 256);
        double* gath = reinterpret_cast<double*>(g.arena + g.scratch_off + 256 + align256((size_t)g.maxcap * 4));
        double best = INFINITY;
        int bestg = -1, bestlen = 0;
        for (int i = h.n; i-- > 1;) {  // goals newest first, strict < (planner_solution); 0 is the start
            if (!gf[i]) continue;
            k_plan_path<<<1, 1, 0, g.s>>>(i, j.parent, j.states, 2, MPTG_METRIC_L2, 1.0, 1.0, 0, nullptr, sc);
            MPTG_LAUNCHED(ctx);
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(hd, sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, g.s));
            MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(g.s));
            if (hd[0] < best || bestg < 0) { best = hd[0]; bestg = i; bestlen = (int)hd[1]; }
        }
        r.cost = best;
        r.path_len = (size_t)bestlen;
        if (q.path && (size_t)bestlen <= q.path_cap) {
            k_plan_path<<<1, 1, 0, g.s>>>(bestg, j.parent, j.states, 2, MPTG_METRIC_L2, 1.0, 1.0, bestlen, ids, sc);
            MPTG_LAUNCHED(ctx);
            k_plan_gather<<<mptg_blocks(bestlen * 2, 256), 256, 0, g.s>>>(ids, bestlen, j.states, 2, gath);
            MPTG_LAUNCHED(ctx);
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(q.path, gath, (size_t)bestlen * 2 * sizeof(double), cudaMemcpyDefault,
                                               g.s));
            MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(g.s));
        }
    }
    return st;
}

mptg_status mptg_plan_batch(mptg_ctx* ctx, const mptg_query* qs, size_t n, int concurrency, mptg_result* out) {
    if (!ctx) return MPTG_ERR_INVALID_ARG;
    if (n == 0) return MPTG_OK;
    if (!qs || !out) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "null queries or results");
    BatchCaps caps;
    for (size_t i = 0; i < n; ++i) {
        const mptg_query& q = qs[i];
        if (!q.scene || !q.start || !q.goal)
            return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "query %zu: null scene, start or goal", i);
        if (q.scene->ctx != ctx) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "query %zu: scene of another context", i);
        if (!(q.goal_radius >= 0)) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "query %zu: goal radius < 0", i);
        mptg_status st = check_params(ctx, q.scene, &q.params);
        if (st) return st;
        auto& c = caps[q.scene];
        c.first = std::max(c.first, q.params.max_nodes);
        c.second = std::max(c.second, q.params.wavefront);
    }
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    // the grid queries the block planner takes run as one launch; the workers
    // take the rest
    GridBatch gb;
    std::vector<size_t> rest;
    for (size_t i = 0; i < n; ++i) (grid_batch_eligible(qs[i]) ? gb.idx : rest).push_back(i);
    const auto t0 = std::chrono::steady_clock::now();
    bool grid_launched = false;
    if (!gb.idx.empty()) {
        if (grid_batch_launch(ctx, qs, gb) == MPTG_OK) {
            grid_launched = true;
        } else {  // no room for the launch: the workers take these queries as well
            grid_batch_free(gb);
            rest.insert(rest.end(), gb.idx.begin(), gb.idx.end());
            std::sort(rest.begin(), rest.end());
        }
    }
    size_t workers = concurrency > 0 ? (size_t)concurrency : 8;
    workers = std::max<size_t>(1, std::min(workers, rest.size()));
    std::atomic<size_t> next{0};
    std::mutex mu;
    mptg_status first = MPTG_OK;
    auto one = [&](size_t i, std::map<mptg_scene*, mptg_planner*>& mine, bool dev_ok) {
        mptg_result& r = out[i];
        r = mptg_result{};
        r.cost = INFINITY;
        mptg_status st = dev_ok ? batch_query(ctx, qs[i], caps, mine, r)
                                : mptg_fail(ctx, MPTG_ERR_CUDA, "cudaSetDevice failed in a batch worker");
        r.status = st;
        r.finish_s = seconds_since(t0);
        if (st) {
            std::lock_guard<std::mutex> lock(mu);
            if (first == MPTG_OK) first = st;
        }
    };
    auto work = [&](bool main_thread) {
        std::map<mptg_scene*, mptg_planner*> mine;
        const bool dev_ok = cudaSetDevice(ctx->device) == cudaSuccess;
        if (main_thread && grid_launched) {
            // the launch's results; the queries that filled their block run here
            mptg_status st = grid_batch_finish(ctx, qs, gb, out, t0);
            if (st) {
                std::lock_guard<std::mutex> lock(mu);
                if (first == MPTG_OK) first = st;
                for (size_t i : gb.idx) out[i].status = st;
            } else {
                for (size_t i : gb.retry) one(i, mine, dev_ok);
            }
        }
        for (size_t k; (k = next.fetch_add(1)) < rest.size();) one(rest[k], mine, dev_ok);
        for (auto& kv : mine)
            if (kv.second) planner_free(kv.second);
    };
    std::vector<std::thread> pool;
    for (size_t k = 1; k < workers; ++k) pool.emplace_back(work, false);
    work(true);
    for (auto& th : pool) th.join();
    grid_batch_free(gb);
    return first;
}

// ------------------------------------------------------------- wavefront autotuner

mptg_status mptg_autotune_wavefront(mptg_ctx* ctx, mptg_scene* scene, const mptg_plan_params* params,
                                    const double* lo, const double* hi, const double* start, const double* goal,
                                    double goal_radius, const int* candidates, int ncand, int trials,
                                    double time_limit_s, int* best, double* median_s) {
    if (!ctx || !scene || !params || !start || !goal || !candidates || ncand < 1 || trials < 1 || !best)
        return MPTG_ERR_INVALID_ARG;
    int wmax = 0;
    for (int c = 0; c < ncand; ++c) {
        if (candidates[c] < 1 || candidates[c] > (1 << 20))
            return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "wavefront candidate %d out of [1, 2^20]", candidates[c]);
        wmax = std::max(wmax, candidates[c]);
    }
    mptg_plan_params cp = *params;
    cp.wavefront = wmax;
    mptg_planner* p = nullptr;
    mptg_status st = mptg_planner_create(ctx, scene, &cp, lo, hi, &p);
    if (st) return st;
    // times to solution of `n` more seeds from seed offset `first` at size W
    // (unsolved: the limit)
    auto trial_times = [&](int W, int first, int n, std::vector<double>& ts) -> mptg_status {
        for (int t = first; t < first + n; ++t) {
            mptg_plan_params q = *params;
            q.wavefront = W;
            q.seed = params->seed + (uint64_t)t;
            mptg_status r;
            if ((r = planner_reset(p, &q, false, nullptr, nullptr))) return r;
            if ((r = mptg_planner_set_goal(p, goal, goal_radius))) return r;
            if ((r = mptg_planner_add_start(p, start))) return r;
            int solved = 0;
            const auto t0 = std::chrono::steady_clock::now();
            if ((r = mptg_planner_run(p, 0, time_limit_s, 1, &solved))) return r;
            const double dt = seconds_since(t0);
            ts.push_back(solved ? dt : std::max(dt, time_limit_s));
        }
        return MPTG_OK;
    };
    auto median = [](std::vector<double> v) {
        std::sort(v.begin(), v.end());
        return v[v.size() / 2];
    };
    // stage 1: `trials` seeds per candidate; stage 2: the three best get twice
    // as many seeds more, and the lowest median over all their seeds wins
    // (heavy-tailed scenes make a median of a few seeds noisy)
    std::vector<std::vector<double>> times(ncand);
    std::vector<double> med(ncand, INFINITY);
    for (int c = 0; c < ncand && !st; ++c) {
        st = trial_times(candidates[c], 0, trials, times[c]);
        if (!st) med[c] = median(times[c]);
    }
    std::vector<int> order(ncand);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return med[a] < med[b]; });
    for (int r = 0; r < std::min(3, ncand) && ncand > 1 && !st; ++r) {
        const int c = order[r];
        st = trial_times(candidates[c], trials, 2 * trials, times[c]);
        if (!st) med[c] = median(times[c]);
    }
    double best_t = INFINITY;
    *best = candidates[0];
    for (int c = 0; c < ncand && !st; ++c) {
        if (median_s) median_s[c] = med[c];
        const bool finalist = ncand == 1 || times[c].size() > (size_t)trials;
        if (finalist && med[c] < best_t) {
            best_t = med[c];
            *best = candidates[c];
        }
    }
    planner_free(p);
    return st;
}

}  // extern "C"
