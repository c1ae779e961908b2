// prm.cu - PPRM (parallel k-nearest probabilistic roadmap) as GPU wavefronts.
//
// Replaces Worker::addSample / solve of src/mpt/impl/pprm/pprm.hpp:298-371
// (and the component union of :341-363, src/mpt/impl/pprm/component.hpp).
// One wavefront draws W samples (the Philox stream of the PRRT planner, no
// goal samples) and, batched on the device:
//   valid(q) for every sample -> compaction of the valid ones in sample order
//   -> k nearest of each among the roadmap before the wavefront (the tree's
//      exact k-NN) and among the wavefront's earlier valid samples (a warp
//      per sample over its predecessors) -> skip near-duplicates (:306-308)
//   -> per kept sample of rank r: the top k_r = ceil((e + e/dim) ln(n0+r+1))
//      of the two sorted lists (the one-at-a-time neighbourhood)
//   -> link(q, nbr) for every pair through the DMV -> edges appended and
//      components united with a lock-free union-find -> tree insert
//   -> solved when a start and a goal node share a component that a union
//      formed (component.hpp isSolution).
// The roadmap (nodes, edges) is therefore the one the reference's worker
// builds from the same sample sequence one sample at a time; the CPU
// restatement replays it exactly.  The solution is Dijkstra's on the host
// over the edge list (src/mpt/impl/djikstras.hpp, pprm.hpp:230-240).
#include "metrics.cuh"
#include "scene.cuh"
#include "tree.cuh"
#include "knn.cuh"
#include "sampler.cuh"
#include <algorithm>
#include <chrono>
#include <float.h>
#include <queue>
#include <vector>

#define PRM_KMAX 64
#define PRM_MAX_STARTS 1024
#define PRM_DUP_CAP 4096

struct PrmView {
    int D, metric;
    double w0, w1;
    const double* lo;
    const double* hi;
    uint64_t seed;
};

struct mptg_prm {
    mptg_ctx* ctx = nullptr;
    mptg_scene* scene = nullptr;
    mptg_tree* tree = nullptr;
    mptg_plan_params prm{};
    int D = 0, metric = 0;
    double w0 = 1, w1 = 1;
    cudaStream_t stream = nullptr;
    EdgeScratch scratch;
    double* lo = nullptr;
    double* hi = nullptr;
    double* goal = nullptr;  // GoalState of the scenario (nullptr: none)
    std::vector<double> goal_host;
    size_t n = 0;            // roadmap nodes (= tree size)
    uint32_t wave = 0;
    // per node [max_nodes]
    int* uf = nullptr;
    uint8_t* flags = nullptr;     // 1 start, 2 goal
    uint8_t* has_edge = nullptr;
    int* goal_ids = nullptr;
    int* start_ids = nullptr;     // [PRM_MAX_STARTS]
    std::vector<int> starts;
    size_t ngoals = 0;
    // edges
    int* efrom = nullptr;
    int* eto = nullptr;
    double* edist = nullptr;
    size_t ecap = 0, ne = 0;
    // per wavefront [W]
    double* samp = nullptr;
    uint8_t* sok = nullptr;
    int* cidx = nullptr;
    double* cand = nullptr;
    uint8_t* kept = nullptr;
    int* rank = nullptr;
    int* knn_i = nullptr;   // [W][64]
    double* knn_d = nullptr;
    int* iknn_i = nullptr;  // [W][64]
    double* iknn_d = nullptr;
    double* newst = nullptr;
    int* ktab = nullptr;    // [W] k and offsets of ranks
    int* koff = nullptr;
    int* dups = nullptr;    // [PRM_DUP_CAP][2]
    // per pair [W * 64]
    int* pa = nullptr;
    int* pb = nullptr;
    double* pd = nullptr;
    double* ea = nullptr;
    double* eb = nullptr;
    uint8_t* eok = nullptr;
    size_t pcap = 0;
    int* dcnt = nullptr;    // device counters: 0 valid, 1 dups, 2 kept, 3 goals, 4 solved, 5 edges
    int* hbuf = nullptr;    // pinned mirror of dcnt
    int* hk = nullptr;      // pinned [2W]: ktab, koff
    bool solving = false;
    uint64_t stat[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

// ------------------------------------------------------------------ kernels

__global__ void k_prm_sample(PrmView v, int W, uint32_t wave, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W) return;
    sample_uniform_state(v.metric, v.D, v.seed, (uint32_t)i, wave, v.lo, v.hi, out + (size_t)i * v.D);
}

// One block: exclusive prefix count of flag[0, n) into pos (may be null), the
// indices of the set flags into compact (may be null), the total into *total.
__global__ void __launch_bounds__(1024) k_prm_scan(const uint8_t* __restrict__ flag, int n, int* __restrict__ pos,
                                                   int* __restrict__ compact, int* __restrict__ total) {
    __shared__ int wsum[32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        const int i = base + threadIdx.x;
        const int f = (i < n && flag[i]) ? 1 : 0;
        int v = f;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += t;
        }
        if (lane == 31) wsum[w] = v;
        __syncthreads();
        if (w == 0) {
            int s = wsum[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += t;
            }
            wsum[lane] = s;
        }
        __syncthreads();
        const int excl = carry + (w ? wsum[w - 1] : 0) + v - f;
        if (i < n) {
            if (pos) pos[i] = excl;
            if (f && compact) compact[excl] = i;
        }
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + f;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_prm_gather(int V, int D, const int* __restrict__ cidx, const double* __restrict__ src,
                             double* __restrict__ dst) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= V) return;
    const double* s = src + (size_t)cidx[j] * D;
    for (int d = 0; d < D; ++d) dst[(size_t)j * D + d] = s[d];
}

// tentatively kept: no old node within DBL_EPSILON (pprm.hpp:306-308)
__global__ void k_prm_tent(int V, int kold, const double* __restrict__ knn_d, uint8_t* __restrict__ kept) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= V) return;
    kept[j] = (kold > 0 && knn_d[(size_t)j * kold] < DBL_EPSILON) ? 0 : 1;
}

// Warp per valid sample j: the kk nearest (FP64, (distance, index) order) of
// the kept samples i < j of the wavefront, and the pairs closer than
// DBL_EPSILON (recorded up to PRM_DUP_CAP; *ndup counts all).
__global__ void __launch_bounds__(256) k_prm_intra(PrmView v, int V, const double* __restrict__ cand, int kk,
                                                   const uint8_t* __restrict__ kept, int* __restrict__ oi,
                                                   double* __restrict__ od, int* __restrict__ dups,
                                                   int* __restrict__ ndup) {
    const int lane = threadIdx.x & 31;
    const int j = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (j >= V) return;  // warp-uniform
    const int D = v.D;
    const double* qj = cand + (size_t)j * D;
    double ld0 = INFINITY, ld1 = INFINITY, tau = INFINITY;
    int li0 = INT_MAX, li1 = INT_MAX, cnt = 0;
    float tauf = INFINITY;
    for (int i0 = 0; i0 < j; i0 += 32) {
        const int i = i0 + lane;
        const bool have = i < j && kept[i];
        double dd = INFINITY;
        if (have) {
            dd = dist64(v.metric, D, v.w0, v.w1, qj, cand + (size_t)i * D);
            if (dd < DBL_EPSILON) {
                const int s = atomicAdd(ndup, 1);
                if (s < PRM_DUP_CAP) { dups[2 * s] = i; dups[2 * s + 1] = j; }
            }
        }
        knn_insert(lane, kk, INFINITY, have && dd <= tau, dd, i, ld0, ld1, li0, li1, cnt, tau, tauf);
    }
    int* o = oi + (size_t)j * kk;
    double* odd = od + (size_t)j * kk;
    if (lane < kk) { const bool ok = lane < cnt; o[lane] = ok ? li0 : -1; odd[lane] = ok ? ld0 : INFINITY; }
    if (lane + 32 < kk) { const bool ok = lane + 32 < cnt; o[lane + 32] = ok ? li1 : -1; odd[lane + 32] = ok ? ld1 : INFINITY; }
}

// Thread per valid sample j of rank r < K: node id n0 + r, the top ktab[r] of
// the old list (ids < n0) and the wavefront list (ids n0 + rank), both sorted
// by (distance, id), as pairs at koff[r]; the node's flags and union-find
// entry; its state into newst[r].
struct PrmMerge {
    int V, n0, K, kold, kin, D;
    const int* knn_i; const double* knn_d;
    const int* iknn_i; const double* iknn_d;
    const uint8_t* kept; const int* rank; const int* ktab; const int* koff;
    const double* cand; const double* states64;
    int* pa; int* pb; double* pd; double* ea; double* eb;
    double* newst; int* uf; uint8_t* flags; uint8_t* has_edge; int* goal_ids; int* ngoal;
    const double* goal; double goal_radius; int metric; double w0, w1; uint8_t flag;
};

__global__ void k_prm_merge(PrmMerge m) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m.V || !m.kept[j]) return;
    const int r = m.rank[j];
    if (r >= m.K) return;  // beyond the node budget
    const int D = m.D;
    const int id = m.n0 + r;
    const double* q = m.cand + (size_t)j * D;
    const int kj = m.ktab[r];
    const size_t off = (size_t)m.koff[r];
    int io = 0, in = 0;
    for (int t = 0; t < kj; ++t) {
        double dO = INFINITY, dN = INFINITY;
        int idO = INT_MAX, idN = INT_MAX;
        if (io < m.kold && m.knn_i[(size_t)j * m.kold + io] >= 0) {
            dO = m.knn_d[(size_t)j * m.kold + io];
            idO = m.knn_i[(size_t)j * m.kold + io];
        }
        if (in < m.kin && m.iknn_i[(size_t)j * m.kin + in] >= 0) {
            dN = m.iknn_d[(size_t)j * m.kin + in];
            idN = m.n0 + m.rank[m.iknn_i[(size_t)j * m.kin + in]];
        }
        const bool takeO = dO < dN || (dO == dN && idO < idN);
        const int nb = takeO ? idO : idN;
        const double d = takeO ? dO : dN;
        const double* bs = takeO ? m.states64 + (size_t)idO * D : m.cand + (size_t)m.iknn_i[(size_t)j * m.kin + in] * D;
        if (takeO) ++io; else ++in;
        m.pa[off + t] = id;
        m.pb[off + t] = nb;
        m.pd[off + t] = d;
        for (int k = 0; k < D; ++k) {
            m.ea[(off + t) * D + k] = q[k];
            m.eb[(off + t) * D + k] = bs[k];
        }
    }
    for (int k = 0; k < D; ++k) m.newst[(size_t)r * D + k] = q[k];
    uint8_t f = m.flag;
    if ((f & 2) || (m.goal && dist64(m.metric, D, m.w0, m.w1, q, m.goal) <= m.goal_radius)) {
        f |= 2;
        m.goal_ids[atomicAdd(m.ngoal, 1)] = id;
    }
    m.flags[id] = f;
    m.uf[id] = id;
    m.has_edge[id] = 0;
}

// lock-free union-find: roots hooked larger index under smaller with CAS,
// path halving on the way up (parents only ever move to ancestors)
__device__ __forceinline__ int uf_find(int* uf, int x) {
    while (true) {
        const int p = __ldcg(&uf[x]);
        if (p == x) return x;
        const int gp = __ldcg(&uf[p]);
        if (gp != p) atomicCAS(&uf[x], p, gp);
        x = gp;
    }
}

__device__ __forceinline__ void uf_unite(int* uf, int a, int b) {
    while (true) {
        a = uf_find(uf, a);
        b = uf_find(uf, b);
        if (a == b) return;
        if (a > b) { const int t = a; a = b; b = t; }
        if (atomicCAS(&uf[b], b, a) == b) return;
    }
}

// every pair whose link is valid: an edge (pprm.hpp:325-334) and a union
__global__ void k_prm_link(int M, const int* __restrict__ pa, const int* __restrict__ pb,
                           const double* __restrict__ pd, const uint8_t* __restrict__ eok, int* uf,
                           uint8_t* __restrict__ has_edge, int* __restrict__ efrom, int* __restrict__ eto,
                           double* __restrict__ edist, int* __restrict__ ne) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M || !eok[m]) return;
    const int a = pa[m], b = pb[m];
    const int e = atomicAdd(ne, 1);
    efrom[e] = a;
    eto[e] = b;
    edist[e] = pd[m];
    has_edge[a] = 1;
    has_edge[b] = 1;
    uf_unite(uf, a, b);
}

// solved: a start s and a goal g in one component, formed by a union (s != g,
// or the start-goal node has an edge)
__global__ void k_prm_solved(int* uf, const uint8_t* __restrict__ has_edge, const int* __restrict__ starts, int ns,
                             const int* __restrict__ goals, const int* __restrict__ ngoals, int* __restrict__ solved) {
    const int ng = *ngoals;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x) {
        const int g = goals[t];
        const int rg = uf_find(uf, g);
        for (int i = 0; i < ns; ++i) {
            const int s = starts[i];
            if ((s != g || has_edge[s]) && uf_find(uf, s) == rg) { *solved = 1; break; }
        }
    }
}

// ------------------------------------------------------------------ host

static int prm_k(size_t n, int dim) {
    // ceil(kRRG * log(n + 1)), kRRG = e + e/dim (pprm.hpp:145,302-303), at most 64 and n
    if (n == 0) return 0;
    const double e = 2.718281828459045, kRRG = e + e / dim;
    const double kd = std::ceil(kRRG * std::log((double)n + 1.0));
    int k = kd > (double)PRM_KMAX ? PRM_KMAX : (int)kd;
    if ((size_t)k > n) k = (int)n;
    return k < 1 ? 1 : k;
}

static void prm_free(mptg_prm* p) {
    if (!p) return;
    void* ptrs[] = {p->lo, p->hi, p->goal, p->uf, p->flags, p->has_edge, p->goal_ids, p->start_ids, p->efrom,
                    p->eto, p->edist, p->samp, p->sok, p->cidx, p->cand, p->kept, p->rank, p->knn_i, p->knn_d,
                    p->iknn_i, p->iknn_d, p->newst, p->ktab, p->koff, p->dups, p->pa, p->pb, p->pd, p->ea,
                    p->eb, p->eok, p->dcnt};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (p->hbuf) cudaFreeHost(p->hbuf);
    if (p->hk) cudaFreeHost(p->hk);
    scratch_free(&p->scratch);
    if (p->tree) mptg_tree_destroy(p->tree);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

// replaces a device array by one of `need` elements, keeping its first `keep`
template <typename T>
static mptg_status grow(mptg_ctx* ctx, cudaStream_t s, T** ptr, size_t need, size_t keep) {
    T* q = nullptr;
    MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&q, need * sizeof(T)));
    if (*ptr && keep) MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(q, *ptr, keep * sizeof(T), cudaMemcpyDeviceToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (*ptr) cudaFree(*ptr);
    *ptr = q;
    return MPTG_OK;
}

static mptg_status prm_reserve_pairs(mptg_prm* p, size_t M) {
    if (M <= p->pcap) return MPTG_OK;
    mptg_ctx* ctx = p->ctx;
    const size_t cap = std::max(M, p->pcap + p->pcap / 2);
    const size_t D = p->D;
    mptg_status st;
    if ((st = grow(ctx, p->stream, &p->pa, cap, 0))) return st;
    if ((st = grow(ctx, p->stream, &p->pb, cap, 0))) return st;
    if ((st = grow(ctx, p->stream, &p->pd, cap, 0))) return st;
    if ((st = grow(ctx, p->stream, &p->ea, cap * D, 0))) return st;
    if ((st = grow(ctx, p->stream, &p->eb, cap * D, 0))) return st;
    if ((st = grow(ctx, p->stream, &p->eok, cap, 0))) return st;
    p->pcap = cap;
    return MPTG_OK;
}

static mptg_status prm_reserve_edges(mptg_prm* p, size_t need) {
    if (need <= p->ecap) return MPTG_OK;
    mptg_ctx* ctx = p->ctx;
    const size_t cap = std::max(need, p->ecap * 2);
    mptg_status st;
    if ((st = grow(ctx, p->stream, &p->efrom, cap, p->ne))) return st;
    if ((st = grow(ctx, p->stream, &p->eto, cap, p->ne))) return st;
    if ((st = grow(ctx, p->stream, &p->edist, cap, p->ne))) return st;
    p->ecap = cap;
    return MPTG_OK;
}

// One wavefront over the W states in p->samp (random samples, or one explicit
// start / goal with flag 1 / 2).  *first_id: the id of the first new node or -1.
static mptg_status prm_wave(mptg_prm* p, int W, uint8_t flag, int* first_id) {
    mptg_ctx* ctx = p->ctx;
    cudaStream_t s = p->stream;
    const int D = p->D;
    mptg_status st;
    if (first_id) *first_id = -1;
    p->stat[1] += (uint64_t)W;
    if ((st = scene_states_dev(p->scene, p->samp, W, p->sok, s, &p->scratch))) return st;
    k_prm_scan<<<1, 1024, 0, s>>>(p->sok, W, nullptr, p->cidx, p->dcnt + 0);
    MPTG_LAUNCHED(ctx);
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hbuf, p->dcnt, sizeof(int), cudaMemcpyDeviceToHost, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    const int V = p->hbuf[0];
    p->stat[2] += (uint64_t)V;
    if (V == 0) return MPTG_OK;
    k_prm_gather<<<mptg_blocks(V, 128), 128, 0, s>>>(V, D, p->cidx, p->samp, p->cand);
    const size_t n0 = p->n;
    const int kmax = prm_k(n0 + V - 1, D);
    const int kold = std::min<int>(kmax, (int)n0);
    if (kold > 0 && (st = mptg_tree_nearest_k_dev(p->tree, p->cand, V, kold, p->knn_i, p->knn_d, s))) return st;
    k_prm_tent<<<mptg_blocks(V, 128), 128, 0, s>>>(V, kold, p->knn_d, p->kept);
    const int kin = std::min(kmax, V - 1);
    const PrmView v{D, p->metric, p->w0, p->w1, p->lo, p->hi, p->prm.seed};
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(p->dcnt + 1, 0, sizeof(int), s));
    if (kin > 0)
        k_prm_intra<<<mptg_blocks((size_t)V * 32, 256), 256, 0, s>>>(v, V, p->cand, kin, p->kept, p->iknn_i,
                                                                     p->iknn_d, p->dups, p->dcnt + 1);
    k_prm_scan<<<1, 1024, 0, s>>>(p->kept, V, p->rank, nullptr, p->dcnt + 2);
    ctx->launches += 4;
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hbuf + 1, p->dcnt + 1, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (p->hbuf[1] > 0) {
        // near-duplicates inside the wavefront (pprm.hpp:306-308 one at a
        // time): sample j is kept iff no kept earlier sample is that close
        const int nd = p->hbuf[1];
        if (nd > PRM_DUP_CAP)
            return mptg_fail(ctx, MPTG_ERR_CAPACITY, "%d near-duplicate samples in one wavefront", nd);
        std::vector<int> dp(2 * (size_t)nd);
        std::vector<uint8_t> kept(V);
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(dp.data(), p->dups, dp.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(kept.data(), p->kept, V, cudaMemcpyDeviceToHost, s));
        MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        std::vector<std::pair<int, int>> pr;
        for (int t = 0; t < nd; ++t) pr.push_back({dp[2 * t + 1], dp[2 * t]});
        std::sort(pr.begin(), pr.end());
        for (const auto& x : pr)
            if (kept[x.second]) kept[x.first] = 0;
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->kept, kept.data(), V, cudaMemcpyHostToDevice, s));
        k_prm_intra<<<mptg_blocks((size_t)V * 32, 256), 256, 0, s>>>(v, V, p->cand, kin, p->kept, p->iknn_i,
                                                                     p->iknn_d, p->dups, p->dcnt + 1);
        k_prm_scan<<<1, 1024, 0, s>>>(p->kept, V, p->rank, nullptr, p->dcnt + 2);
        ctx->launches += 2;
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hbuf + 2, p->dcnt + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
        MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    }
    const int Kall = p->hbuf[2];
    p->stat[3] += (uint64_t)(V - Kall);
    const int K = (int)std::min<size_t>((size_t)Kall, p->prm.max_nodes - n0);
    if (K <= 0) return MPTG_OK;
    // k and pair offsets per rank (the same formula as the one-at-a-time loop)
    size_t M = 0;
    for (int r = 0; r < K; ++r) {
        p->hk[r] = prm_k(n0 + r, D);
        p->hk[W + r] = (int)M;
        M += (size_t)p->hk[r];
    }
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->ktab, p->hk, K * sizeof(int), cudaMemcpyHostToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->koff, p->hk + W, K * sizeof(int), cudaMemcpyHostToDevice, s));
    if ((st = prm_reserve_pairs(p, std::max<size_t>(M, 1)))) return st;
    if ((st = prm_reserve_edges(p, p->ne + M))) return st;
    PrmMerge m;
    m.V = V; m.n0 = (int)n0; m.K = K; m.kold = kold; m.kin = kin; m.D = D;
    m.knn_i = p->knn_i; m.knn_d = p->knn_d; m.iknn_i = p->iknn_i; m.iknn_d = p->iknn_d;
    m.kept = p->kept; m.rank = p->rank; m.ktab = p->ktab; m.koff = p->koff;
    m.cand = p->cand; m.states64 = mptg_tree_states_dev(p->tree);
    m.pa = p->pa; m.pb = p->pb; m.pd = p->pd; m.ea = p->ea; m.eb = p->eb;
    m.newst = p->newst; m.uf = p->uf; m.flags = p->flags; m.has_edge = p->has_edge;
    m.goal_ids = p->goal_ids; m.ngoal = p->dcnt + 3;
    m.goal = p->goal; m.goal_radius = p->prm.goal_radius; m.metric = p->metric; m.w0 = p->w0; m.w1 = p->w1;
    m.flag = flag;
    k_prm_merge<<<mptg_blocks(V, 128), 128, 0, s>>>(m);
    MPTG_LAUNCHED(ctx);
    if (M > 0) {
        if ((st = scene_edges_dev(p->scene, p->ea, p->eb, (int)M, p->prm.edge_step, p->prm.resolution, p->eok, s,
                                  nullptr, &p->scratch)))
            return st;
        k_prm_link<<<mptg_blocks(M, 256), 256, 0, s>>>((int)M, p->pa, p->pb, p->pd, p->eok, p->uf, p->has_edge,
                                                      p->efrom, p->eto, p->edist, p->dcnt + 5);
        MPTG_LAUNCHED(ctx);
    }
    p->stat[4] += M;
    if ((st = mptg_tree_insert(p->tree, p->newst, K, s))) return st;
    p->n = n0 + K;
    if (flag & 1) {
        if (p->starts.size() >= PRM_MAX_STARTS)
            return mptg_fail(ctx, MPTG_ERR_CAPACITY, "more than %d start nodes", PRM_MAX_STARTS);
        const int id = (int)n0;
        MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->start_ids + p->starts.size(), &id, sizeof(int), cudaMemcpyHostToDevice, s));
        p->starts.push_back(id);
    }
    if (!p->starts.empty()) {
        k_prm_solved<<<16, 128, 0, s>>>(p->uf, p->has_edge, p->start_ids, (int)p->starts.size(), p->goal_ids,
                                        p->dcnt + 3, p->dcnt + 4);
        MPTG_LAUNCHED(ctx);
    }
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(p->hbuf + 3, p->dcnt + 3, 3 * sizeof(int), cudaMemcpyDeviceToHost, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    p->ngoals = (size_t)p->hbuf[3];
    p->ne = (size_t)p->hbuf[5];
    p->stat[5] = p->ne;
    p->stat[6] = p->ngoals;
    p->stat[7] = p->hbuf[4] ? 1 : 0;
    if (first_id) *first_id = (int)n0;
    return MPTG_OK;
}

static mptg_status prm_add(mptg_prm* p, const double* q, uint8_t flag, int32_t* id) {
    if (!p || !q) return MPTG_ERR_INVALID_ARG;
    if (p->solving) return mptg_fail(p->ctx, MPTG_ERR_ALREADY_SOLVING, "already solving");
    // a state outside the space (the tree's insert rules) is an error before
    // anything joins the roadmap, not a dropped sample
    std::vector<double> h(p->D);
    MPTG_CUDA_TRY(p->ctx, cudaMemcpy(h.data(), q, p->D * sizeof(double), cudaMemcpyDefault));
    bool bad = false;
    for (int d = 0; d < p->D; ++d) {
        bad = bad || !std::isfinite(h[d]);
        if (p->metric == MPTG_METRIC_SO2) bad = bad || !(h[d] >= -MPTG_PI && h[d] <= MPTG_PI);
    }
    if (p->metric == MPTG_METRIC_SO3 || p->metric == MPTG_METRIC_SE3) {
        const double nn = h[0] * h[0] + h[1] * h[1] + h[2] * h[2] + h[3] * h[3];
        bad = bad || !(std::fabs(nn - 1.0) <= MPTG_QUAT_NORM_TOL);
    }
    if (bad)
        return mptg_fail(p->ctx, MPTG_ERR_INVALID_ARG,
                         "invalid state (NaN/inf, SO2 angle outside [-pi,pi], or non-unit quaternion)");
    MPTG_CUDA_TRY(p->ctx, cudaMemcpyAsync(p->samp, h.data(), p->D * sizeof(double), cudaMemcpyHostToDevice, p->stream));
    int first = -1;
    mptg_status st = prm_wave(p, 1, flag, &first);
    if (id) *id = first;
    return st;
}

// Dijkstra over the roadmap from the start nodes to the first goal node
// settled: heap order (distance, id), adjacency in (from, to) edge order with
// each edge listed at both ends, predecessors changed on strict improvement.
static void prm_dijkstra(size_t n, const std::vector<uint8_t>& flags, const std::vector<int>& ef,
                         const std::vector<int>& et, const std::vector<double>& ed, std::vector<int>& path,
                         double* cost) {
    const size_t ne = ef.size();
    std::vector<size_t> order(ne);
    for (size_t e = 0; e < ne; ++e) order[e] = e;
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) {
        return ef[x] != ef[y] ? ef[x] < ef[y] : et[x] < et[y];
    });
    std::vector<size_t> deg(n + 1, 0);
    for (size_t e = 0; e < ne; ++e) { deg[ef[e] + 1]++; deg[et[e] + 1]++; }
    for (size_t v = 0; v < n; ++v) deg[v + 1] += deg[v];
    std::vector<size_t> fill(deg.begin(), deg.end() - 1);
    std::vector<int> adj(2 * ne);
    std::vector<double> adjw(2 * ne);
    for (size_t e : order) {
        const int a = ef[e], b = et[e];
        adj[fill[a]] = b; adjw[fill[a]++] = ed[e];
        adj[fill[b]] = a; adjw[fill[b]++] = ed[e];
    }
    std::vector<double> dist(n, INFINITY);
    std::vector<int> pred(n, -1);
    std::vector<uint8_t> done(n, 0);
    using Item = std::pair<double, int>;
    std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
    for (size_t v = 0; v < n; ++v)
        if (flags[v] & 1) { dist[v] = 0.0; heap.push({0.0, (int)v}); }
    int found = -1;
    while (!heap.empty()) {
        const Item it = heap.top();
        heap.pop();
        const int u = it.second;
        if (done[u] || it.first != dist[u]) continue;
        done[u] = 1;
        if (flags[u] & 2) { found = u; break; }
        for (size_t t = deg[u]; t < deg[u + 1]; ++t) {
            const int w = adj[t];
            const double nd = it.first + adjw[t];
            if (nd < dist[w]) { dist[w] = nd; pred[w] = u; heap.push({nd, w}); }
        }
    }
    path.clear();
    *cost = INFINITY;
    if (found < 0) return;
    *cost = dist[found];
    for (int v = found; v >= 0; v = pred[v]) path.push_back(v);
    std::reverse(path.begin(), path.end());
}

static mptg_status prm_fetch(mptg_prm* p, std::vector<double>* states, std::vector<uint8_t>* flags,
                             std::vector<int>* ef, std::vector<int>* et, std::vector<double>* ed) {
    mptg_ctx* ctx = p->ctx;
    cudaStream_t s = p->stream;
    const size_t n = p->n, ne = p->ne;
    if (states) {
        states->resize(n * p->D);
        if (n) MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(states->data(), mptg_tree_states_dev(p->tree),
                                                  n * p->D * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    if (flags) {
        flags->resize(n);
        if (n) MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(flags->data(), p->flags, n, cudaMemcpyDeviceToHost, s));
    }
    if (ef) {
        ef->resize(ne);
        et->resize(ne);
        ed->resize(ne);
        if (ne) {
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(ef->data(), p->efrom, ne * sizeof(int), cudaMemcpyDeviceToHost, s));
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(et->data(), p->eto, ne * sizeof(int), cudaMemcpyDeviceToHost, s));
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(ed->data(), p->edist, ne * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
    }
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return MPTG_OK;
}

extern "C" {

mptg_status mptg_prm_create(mptg_ctx* ctx, mptg_scene* scene, const mptg_plan_params* prm, const double* lo,
                            const double* hi, const double* goal, mptg_prm** out) {
    if (!ctx || !scene || !prm || !out) return MPTG_ERR_INVALID_ARG;
    *out = nullptr;
    if (prm->wavefront < 1 || prm->wavefront > (1 << 20))
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "wavefront must be in [1, 2^20]");
    if (prm->max_nodes < 1 || prm->max_nodes > (size_t)INT_MAX)
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "max_nodes must be in [1, 2^31)");
    if (!(prm->edge_step > 0)) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "edge_step must be positive");
    if (!(prm->goal_radius >= 0)) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "goal_radius must be >= 0");
    if (prm->resolution == 1 && scene->metric != MPTG_METRIC_SO2)
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "joint-step resolution needs an SO2 scene");
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    mptg_prm* p = new mptg_prm();
    p->ctx = ctx;
    p->scene = scene;
    p->prm = *prm;
    p->D = scene->D;
    p->metric = scene->metric;
    p->w0 = scene->w0;
    p->w1 = scene->w1;
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete p;
        return mptg_fail(ctx, MPTG_ERR_CUDA, "prm stream: %s", cudaGetErrorString(e));
    }
    double w[2] = {p->w0, p->w1};
    mptg_status st = mptg_tree_create(ctx, (mptg_metric)p->metric, p->D, w, prm->max_nodes, &p->tree);
    if (st) { prm_free(p); return st; }
    const size_t W = prm->wavefront, D = p->D, N = prm->max_nodes;
#define ALLOC(ptr, bytes) if (e == cudaSuccess) e = cudaMalloc((void**)&(ptr), (bytes))
    ALLOC(p->lo, D * sizeof(double));
    ALLOC(p->hi, D * sizeof(double));
    ALLOC(p->uf, N * sizeof(int));
    ALLOC(p->flags, N);
    ALLOC(p->has_edge, N);
    ALLOC(p->goal_ids, N * sizeof(int));
    ALLOC(p->start_ids, PRM_MAX_STARTS * sizeof(int));
    ALLOC(p->samp, W * D * sizeof(double));
    ALLOC(p->sok, W);
    ALLOC(p->cidx, W * sizeof(int));
    ALLOC(p->cand, W * D * sizeof(double));
    ALLOC(p->kept, W);
    ALLOC(p->rank, W * sizeof(int));
    ALLOC(p->knn_i, W * PRM_KMAX * sizeof(int));
    ALLOC(p->knn_d, W * PRM_KMAX * sizeof(double));
    ALLOC(p->iknn_i, W * PRM_KMAX * sizeof(int));
    ALLOC(p->iknn_d, W * PRM_KMAX * sizeof(double));
    ALLOC(p->newst, W * D * sizeof(double));
    ALLOC(p->ktab, W * sizeof(int));
    ALLOC(p->koff, W * sizeof(int));
    ALLOC(p->dups, 2 * PRM_DUP_CAP * sizeof(int));
    ALLOC(p->dcnt, 8 * sizeof(int));
    if (goal) ALLOC(p->goal, D * sizeof(double));
#undef ALLOC
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->hbuf, 8 * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->hk, 2 * W * sizeof(int));
    if (e != cudaSuccess) {
        cudaGetLastError();
        prm_free(p);
        return mptg_fail(ctx, MPTG_ERR_OOM, "prm allocation failed: %s", cudaGetErrorString(e));
    }
    double l[MPTG_MAX_DIM], h[MPTG_MAX_DIM];
    for (size_t d = 0; d < D; ++d) {
        l[d] = lo ? lo[d] : (p->metric == MPTG_METRIC_SO2 ? -MPTG_PI : 0.0);
        h[d] = hi ? hi[d] : (p->metric == MPTG_METRIC_SO2 ? MPTG_PI : 1.0);
    }
    e = cudaMemcpyAsync(p->lo, l, D * sizeof(double), cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->hi, h, D * sizeof(double), cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess && goal) {
        p->goal_host.assign(goal, goal + D);
        e = cudaMemcpyAsync(p->goal, p->goal_host.data(), D * sizeof(double), cudaMemcpyHostToDevice, p->stream);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(p->dcnt, 0, 8 * sizeof(int), p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
        prm_free(p);
        return mptg_fail(ctx, MPTG_ERR_CUDA, "prm init failed: %s", cudaGetErrorString(e));
    }
    *out = p;
    return MPTG_OK;
}

mptg_status mptg_prm_destroy(mptg_prm* p) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    prm_free(p);
    return MPTG_OK;
}

mptg_status mptg_prm_add_start(mptg_prm* p, const double* q, int32_t* id) { return prm_add(p, q, 1, id); }

mptg_status mptg_prm_add_goal(mptg_prm* p, const double* q, int32_t* id) { return prm_add(p, q, 2, id); }

mptg_status mptg_prm_run(mptg_prm* p, int max_wavefronts, double time_limit_s, int stop_when_solved, int* solved) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = p->ctx;
    if (p->starts.empty() || p->ngoals == 0)
        return mptg_fail(ctx, MPTG_ERR_NO_START, "PPRM requires both start and goal configurations");
    if (p->solving) return mptg_fail(ctx, MPTG_ERR_ALREADY_SOLVING, "already solving");
    p->solving = true;
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const auto t0 = std::chrono::steady_clock::now();
    mptg_status st = MPTG_OK;
    const int W = p->prm.wavefront;
    const PrmView v{p->D, p->metric, p->w0, p->w1, p->lo, p->hi, p->prm.seed};
    for (int it = 0; max_wavefronts <= 0 || it < max_wavefronts; ++it) {
        if (stop_when_solved && p->stat[7]) break;
        if (p->n >= p->prm.max_nodes) break;
        if (time_limit_s > 0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() >= time_limit_s)
            break;
        k_prm_sample<<<mptg_blocks(W, 128), 128, 0, p->stream>>>(v, W, p->wave, p->samp);
        MPTG_LAUNCHED(ctx);
        if ((st = prm_wave(p, W, 0, nullptr))) break;
        ++p->wave;
        ++p->stat[0];
    }
    p->solving = false;
    if (solved) *solved = p->stat[7] ? 1 : 0;
    return st;
}

mptg_status mptg_prm_size(mptg_prm* p, size_t* nodes, size_t* edges) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    if (nodes) *nodes = p->n;
    if (edges) *edges = p->ne;
    return MPTG_OK;
}

mptg_status mptg_prm_graph(mptg_prm* p, double* states, size_t cap_nodes, int32_t* from, int32_t* to, double* dist,
                           size_t cap_edges, size_t* n, size_t* ne) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    if (n) *n = p->n;
    if (ne) *ne = p->ne;
    const bool want_states = states && cap_nodes >= p->n;
    const bool want_edges = (from || to || dist) && cap_edges >= p->ne;
    if (!want_states && !want_edges) return MPTG_OK;
    std::vector<double> st;
    std::vector<int> ef, et;
    std::vector<double> ed;
    mptg_status s = prm_fetch(p, want_states ? &st : nullptr, nullptr, want_edges ? &ef : nullptr, &et, &ed);
    if (s) return s;
    if (want_states) std::copy(st.begin(), st.end(), states);
    if (want_edges) {
        std::vector<size_t> order(ef.size());
        for (size_t e = 0; e < order.size(); ++e) order[e] = e;
        std::sort(order.begin(), order.end(), [&](size_t x, size_t y) {
            return ef[x] != ef[y] ? ef[x] < ef[y] : et[x] < et[y];
        });
        for (size_t i = 0; i < order.size(); ++i) {
            if (from) from[i] = ef[order[i]];
            if (to) to[i] = et[order[i]];
            if (dist) dist[i] = ed[order[i]];
        }
    }
    return MPTG_OK;
}

mptg_status mptg_prm_solution(mptg_prm* p, double* path, size_t cap, size_t* len, double* cost) {
    if (!p) return MPTG_ERR_INVALID_ARG;
    std::vector<double> st;
    std::vector<uint8_t> fl;
    std::vector<int> ef, et, ids;
    std::vector<double> ed;
    mptg_status s = prm_fetch(p, &st, &fl, &ef, &et, &ed);
    if (s) return s;
    double c = INFINITY;
    prm_dijkstra(p->n, fl, ef, et, ed, ids, &c);
    if (len) *len = ids.size();
    if (cost) *cost = c;
    if (path && cap >= ids.size())
        for (size_t i = 0; i < ids.size(); ++i)
            std::copy(st.begin() + (size_t)ids[i] * p->D, st.begin() + (size_t)(ids[i] + 1) * p->D, path + i * p->D);
    return MPTG_OK;
}

mptg_status mptg_prm_stats(mptg_prm* p, uint64_t out[8]) {
    if (!p || !out) return MPTG_ERR_INVALID_ARG;
    for (int i = 0; i < 8; ++i) out[i] = p->stat[i];
    return MPTG_OK;
}

}  // extern "C"
