// tree.cu - device-resident bucketed kd-tree: batched incremental insert and
// warp-per-query exact nearest-neighbour search.
//
// Replaces nigh::Nigh<..., KDTreeBatch<>> behind src/mpt/impl/prrt/prrt.hpp
// (insert :186,447; nearest :406-409) and nearest(nbh,q,k,r) behind
// src/mpt/impl/rrg_rewire_neighbors.hpp:64-67,124-128.
//
// Layout in HBM (per tree, capacity N states of dimension D):
//   states64 [N][D]  double  master copy, ids = insertion order
//   pts32    [N][D]  float   FP32 copy used by the builder
//   nodes    [M]     int4    {split dim | -1 for a leaf, left child | bucket,
//                             split value bits, leaf point count}
//                             right child = left child + 1
//   cell_lo/hi [M][D] float  closed cell bounds of every node
//   bpts  [B][D][32] float   leaf buckets, SoA per bucket: lane j reads point j
//   bids  [B][32]    int     point ids of the bucket entries
// A leaf holds at most 32 points.  Inserting a batch descends every new point
// to its leaf (k_locate) and appends it (k_append); leaves that overflow are
// rebuilt into subtrees by a level-synchronous segment builder (sliding
// midpoint split on the widest axis of the points), so the tree is exact and
// complete after every insert.
#include "metrics.cuh"
#include "knn.cuh"
#include <algorithm>
#include <vector>

namespace {

enum { CNT_NODES = 0, CNT_BUCKETS = 1, CNT_NSEG_NEXT = 2, CNT_ERR = 3, CNT_OVF = 4, CNT_NREG = 5,
       CNT_PERM = 6, CNT_MAXABS = 7, CNT_MAXDEPTH = 8, CNT_N = 9 };

// a leaf deeper than this triggers a rebuild of the whole tree
#define MPTG_REBUILD_DEPTH 40
// inserts up to this many states queue the first build level without a round trip
#define MPTG_INSERT_PENDING_MAX 65536

enum { SEG_SPLIT = 0, SEG_LEAF = 1 };

struct SegState {
    int node, start, count, depth;
    int parent, side, kind, dim;
    float split;
    int lc, rc, next;
    int bucket, degenerate, pad0, pad1;
};

}  // namespace

struct mptg_tree {
    mptg_ctx* ctx = nullptr;
    int metric = 0, D = 0;
    double w0 = 1, w1 = 1;
    size_t cap = 0, n = 0;
    int node_cap = 0, bucket_cap = 0, seg_cap = 0;
    double* states64 = nullptr;
    float* pts32 = nullptr;
    int4* nodes = nullptr;
    float* cell_lo = nullptr;
    float* cell_hi = nullptr;
    int* node_depth = nullptr;
    float* bpts = nullptr;
    int* bids = nullptr;
    int* dcnt = nullptr;
    unsigned long long* dstats = nullptr;
    int* perm = nullptr; int* perm2 = nullptr; int* pseg = nullptr; int* pseg2 = nullptr;
    SegState* segA = nullptr; SegState* segB = nullptr;
    int* seg_box = nullptr;
    int* leaf_of = nullptr; int* ovf_pts = nullptr; int* ovf_leaf = nullptr; int* leaf_reg = nullptr;
    int* seg_cursor = nullptr;
    int* hcnt = nullptr;  // pinned
    uint64_t rebuilds = 0;
    int strategy = MPTG_NN_AUTO;  // mptg_nn_strategy
    // exhaustive sweep scratch: [split][BRUTE_K][queries] candidates
    float* bcd = nullptr;
    int* bci = nullptr;
    size_t bcap = 0;
    // split k-NN scratch: [split][queries][k] lists
    double* kcd = nullptr;
    int* kci = nullptr;
    size_t kcap = 0;
    // query ordering scratch (grown on demand)
    int* qkey = nullptr;
    int* qorder = nullptr;
    int* qhist = nullptr;
    size_t qcap = 0;
};

struct TreeView {
    int metric, D;
    float w0f, w1f;
    double w0, w1;
    const int4* __restrict__ nodes;
    const float* __restrict__ cell_lo;
    const float* __restrict__ cell_hi;
    const float* __restrict__ bpts;
    const int* __restrict__ bids;
    const double* __restrict__ states64;
    const float* __restrict__ pts32;
    const int* __restrict__ dcnt;
    unsigned long long* stats;
    int n;
};

static TreeView view_of(const mptg_tree* t) {
    TreeView v;
    v.metric = t->metric; v.D = t->D;
    v.w0 = t->w0; v.w1 = t->w1; v.w0f = (float)t->w0; v.w1f = (float)t->w1;
    v.nodes = t->nodes; v.cell_lo = t->cell_lo; v.cell_hi = t->cell_hi;
    v.bpts = t->bpts; v.bids = t->bids; v.states64 = t->states64; v.pts32 = t->pts32;
    v.dcnt = t->dcnt; v.stats = t->dstats; v.n = (int)t->n;
    return v;
}

// ------------------------------------------------------------------ insert

// FP64 -> FP32 copy plus input checks (NaN, SO2 range, unit quaternions) and
// the running maximum |coordinate| of the Lp / translation part.
__global__ void k_convert(const double* __restrict__ in, float* __restrict__ out, int n, int D, int metric,
                          int* __restrict__ dcnt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* s = in + (size_t)i * D;
    float* o = out + (size_t)i * D;
    bool bad = false;
    float mx = 0.f;
    for (int d = 0; d < D; ++d) {
        double v = s[d];
        if (!(v == v) || isinf(v)) bad = true;
        o[d] = __double2float_rn(v);
        bool lp = metric == MPTG_METRIC_L2 || metric == MPTG_METRIC_L1 || (metric == MPTG_METRIC_SE3 && d >= 4);
        if (lp) mx = fmaxf(mx, __double2float_ru(fabs(v)));
        if (metric == MPTG_METRIC_SO2 && !(v >= -MPTG_PI && v <= MPTG_PI)) bad = true;
    }
    if (metric == MPTG_METRIC_SO3 || metric == MPTG_METRIC_SE3) {
        double nn = quat_dot64(s, s);
        if (!(fabs(nn - 1.0) <= MPTG_QUAT_NORM_TOL)) bad = true;
    }
    if (bad) atomicOr((unsigned*)&dcnt[CNT_ERR], MPTG_DEVERR_BAD_STATE);
    if (mx > 0.f) atomicMax(&dcnt[CNT_MAXABS], __float_as_int(mx));
}

__global__ void k_locate(const int4* __restrict__ nodes, const float* __restrict__ pts32, int first, int n, int D,
                         int* __restrict__ leaf_of) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = pts32 + (size_t)(first + i) * D;
    int node = 0;
    for (int guard = 0; guard < 4 * MPTG_MAX_DEPTH; ++guard) {
        int4 nd = nodes[node];
        if (nd.x < 0) break;
        node = p[nd.x] < __int_as_float(nd.z) ? nd.y : nd.y + 1;
    }
    leaf_of[i] = node;
}

__global__ void k_append(int4* __restrict__ nodes, const float* __restrict__ pts32, float* __restrict__ bpts,
                         int* __restrict__ bids, int first, int n, int D, const int* __restrict__ leaf_of,
                         int* __restrict__ dcnt, int* __restrict__ ovf_pts, int* __restrict__ ovf_leaf,
                         int* __restrict__ leaf_reg) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // k_convert rejected a state of this batch: leave the tree untouched
    if (dcnt[CNT_ERR] & MPTG_DEVERR_BAD_STATE) return;
    int L = leaf_of[i];
    int slot = atomicAdd(&nodes[L].w, 1);
    if (slot < MPTG_BUCKET) {
        int b = nodes[L].y;
        const float* p = pts32 + (size_t)(first + i) * D;
        for (int d = 0; d < D; ++d) bpts[((size_t)b * D + d) * MPTG_BUCKET + slot] = p[d];
        bids[(size_t)b * MPTG_BUCKET + slot] = first + i;
    } else {
        int k = atomicAdd(&dcnt[CNT_OVF], 1);
        ovf_pts[k] = i;
        if (slot == MPTG_BUCKET) {
            int r = atomicAdd(&dcnt[CNT_NREG], 1);
            ovf_leaf[r] = L;
            leaf_reg[L] = r;
        }
    }
}

// one thread per overflowing leaf: open a build segment holding the leaf's
// bucket points followed by its overflow points
// Counts the host has not read yet: the first builder launches of an insert
// are queued behind k_append without a round trip, with -1 for the count,
// and read it from the device counters.  More overflowing leaves than build
// segments make every such launch a no-op (k_ovf_segs flags the capacity
// error, which the host reads with the next counters).
__device__ __forceinline__ int pending_nreg(const int* dcnt, int seg_cap) {
    const int r = dcnt[CNT_NREG];
    return r <= seg_cap ? r : 0;
}
__device__ __forceinline__ int pending_total(const int* dcnt, int seg_cap) {
    const int r = pending_nreg(dcnt, seg_cap);
    return r ? MPTG_BUCKET * r + dcnt[CNT_OVF] : 0;
}

__global__ void k_ovf_segs(const int4* __restrict__ nodes, const int* __restrict__ bids,
                           const int* __restrict__ node_depth, int nreg, const int* __restrict__ ovf_leaf,
                           int* __restrict__ dcnt, SegState* __restrict__ seg, int* __restrict__ perm,
                           int* __restrict__ pseg, int* __restrict__ seg_cursor, int seg_cap) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (nreg < 0) {
        if (dcnt[CNT_NREG] > seg_cap && r == 0) atomicOr((unsigned*)&dcnt[CNT_ERR], MPTG_DEVERR_CAPACITY);
        nreg = pending_nreg(dcnt, seg_cap);
    }
    if (r >= nreg) return;
    int L = ovf_leaf[r];
    int4 nd = nodes[L];
    int total = nd.w;
    int base = atomicAdd(&dcnt[CNT_PERM], total);
    SegState s;
    memset(&s, 0, sizeof(s));
    s.node = L; s.start = base; s.count = total; s.depth = node_depth[L]; s.parent = -1;
    seg[r] = s;
    for (int j = 0; j < MPTG_BUCKET; ++j) {
        perm[base + j] = bids[(size_t)nd.y * MPTG_BUCKET + j];
        pseg[base + j] = r;
    }
    seg_cursor[r] = MPTG_BUCKET;
}

__global__ void k_ovf_scatter(int novf, int first, const int* __restrict__ ovf_pts, const int* __restrict__ leaf_of,
                              const int* __restrict__ leaf_reg, const SegState* __restrict__ seg,
                              int* __restrict__ seg_cursor, int* __restrict__ perm, int* __restrict__ pseg,
                              const int* __restrict__ dcnt, int seg_cap) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (novf < 0) novf = pending_nreg(dcnt, seg_cap) ? dcnt[CNT_OVF] : 0;
    if (k >= novf) return;
    int i = ovf_pts[k];
    int r = leaf_reg[leaf_of[i]];
    int pos = seg[r].start + atomicAdd(&seg_cursor[r], 1);
    perm[pos] = first + i;
    pseg[pos] = r;
}

// level step A (per segment): finalise start/count from the parent split and
// decide leaf vs split
__global__ void k_seg_a(SegState* __restrict__ cur, int nseg, const SegState* __restrict__ prev,
                        int4* __restrict__ nodes, int* __restrict__ dcnt, int bucket_cap, int* __restrict__ box,
                        int D, int seg_cap) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (nseg < 0) nseg = pending_nreg(dcnt, seg_cap);
    if (s >= nseg) return;
    SegState S = cur[s];
    if (S.parent >= 0) {
        const SegState& P = prev[S.parent];
        if (S.side == 0) { S.start = P.start; S.count = P.lc; }
        else { S.start = P.start + P.lc; S.count = P.count - P.lc; }
    }
    if (S.count <= MPTG_BUCKET || S.depth >= MPTG_MAX_DEPTH) {
        if (S.count > MPTG_BUCKET) atomicOr((unsigned*)&dcnt[CNT_ERR], MPTG_DEVERR_DEPTH);
        int b = atomicAdd(&dcnt[CNT_BUCKETS], 1);
        if (b >= bucket_cap) {
            atomicOr((unsigned*)&dcnt[CNT_ERR], MPTG_DEVERR_CAPACITY);
            b = -1;
        }
        int c = S.count < MPTG_BUCKET ? S.count : MPTG_BUCKET;
        nodes[S.node] = make_int4(-1, b < 0 ? 0 : b, 0, b < 0 ? 0 : c);
        S.kind = SEG_LEAF;
        S.bucket = b;
    } else {
        S.kind = SEG_SPLIT;
        S.lc = 0; S.rc = 0;
        int* bx = box + (size_t)s * 2 * D;
        for (int d = 0; d < D; ++d) {
            bx[d] = mptg_f2ord(INFINITY);
            bx[D + d] = mptg_f2ord(-INFINITY);
        }
    }
    cur[s] = S;
}

// level step B (per position): fill leaf buckets, accumulate split boxes
__global__ void k_seg_b(const SegState* __restrict__ cur, const int* __restrict__ perm, const int* __restrict__ pseg,
                        int* __restrict__ pseg2, int total, const float* __restrict__ pts32, int D,
                        float* __restrict__ bpts, int* __restrict__ bids, int* __restrict__ box,
                        const int* __restrict__ dcnt, int seg_cap) {
    if (total < 0) total = pending_total(dcnt, seg_cap);
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = threadIdx.x & 31;
    int s = pos < total ? pseg[pos] : -1;
    bool split = false;
    int p = -1;
    if (s >= 0) {
        const SegState& S = cur[s];
        p = perm[pos];
        if (S.kind == SEG_LEAF) {
            int slot = pos - S.start;
            if (S.bucket >= 0 && slot < MPTG_BUCKET) {
                for (int d = 0; d < D; ++d)
                    bpts[((size_t)S.bucket * D + d) * MPTG_BUCKET + slot] = pts32[(size_t)p * D + d];
                bids[(size_t)S.bucket * MPTG_BUCKET + slot] = p;
            }
            pseg2[pos] = -1;
        } else {
            split = true;
        }
    } else if (pos < total) {
        pseg2[pos] = -1;
    }
    unsigned act = __ballot_sync(0xffffffffu, split);
    if (split) {
        unsigned grp = __match_any_sync(act, s);
        int leader = __ffs(grp) - 1;
        int* bx = box + (size_t)s * 2 * D;
        for (int d = 0; d < D; ++d) {
            int o = mptg_f2ord(pts32[(size_t)p * D + d]);
            int mn = __reduce_min_sync(grp, o);
            int mx = __reduce_max_sync(grp, o);
            if (lane == leader) {
                atomicMin(&bx[d], mn);
                atomicMax(&bx[D + d], mx);
            }
        }
    }
}

// level step C (per segment): choose the split, allocate children
__global__ void k_seg_c(SegState* __restrict__ cur, int nseg, SegState* __restrict__ next,
                        int4* __restrict__ nodes, float* __restrict__ cell_lo, float* __restrict__ cell_hi,
                        int* __restrict__ node_depth, int* __restrict__ dcnt, int node_cap, int seg_cap,
                        const int* __restrict__ box, int D, int metric, float w0, float w1) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (nseg < 0) nseg = pending_nreg(dcnt, seg_cap);
    if (s >= nseg) return;
    SegState S = cur[s];
    if (S.kind != SEG_SPLIT) return;
    const int* bx = box + (size_t)s * 2 * D;
    int dim = 0;
    float bext = -1.f, blo = 0.f, bhi = 0.f;
    for (int d = 0; d < D; ++d) {
        float lo = mptg_ord2f(bx[d]), hi = mptg_ord2f(bx[D + d]);
        float sc = 1.f;
        if (metric == MPTG_METRIC_SE3) sc = d < 4 ? w0 : w1;
        float ext = (hi - lo) * sc;
        if (ext > bext) { bext = ext; dim = d; blo = lo; bhi = hi; }
    }
    float split;
    int degenerate = 0;
    if (bext > 0.f) {
        split = blo + (bhi - blo) * 0.5f;
        if (!(split > blo)) split = bhi;
        if (split > bhi) split = bhi;
    } else {
        degenerate = 1;
        dim = 0;
        split = mptg_ord2f(bx[0]);
    }
    int c = atomicAdd(&dcnt[CNT_NODES], 2);
    if (c + 2 > node_cap) {
        atomicOr((unsigned*)&dcnt[CNT_ERR], MPTG_DEVERR_CAPACITY);
        // make the segment a truncated leaf so that the build terminates
        S.kind = SEG_LEAF; S.bucket = -1;
        cur[s] = S;
        nodes[S.node] = make_int4(-1, 0, 0, 0);
        return;
    }
    nodes[S.node] = make_int4(dim, c, __float_as_int(split), 0);
    atomicMax(&dcnt[CNT_MAXDEPTH], S.depth + 1);
    node_depth[c] = S.depth + 1;
    node_depth[c + 1] = S.depth + 1;
    for (int d = 0; d < D; ++d) {
        float lo = cell_lo[(size_t)S.node * D + d], hi = cell_hi[(size_t)S.node * D + d];
        cell_lo[(size_t)c * D + d] = lo;
        cell_hi[(size_t)c * D + d] = d == dim ? split : hi;
        cell_lo[(size_t)(c + 1) * D + d] = d == dim ? split : lo;
        cell_hi[(size_t)(c + 1) * D + d] = hi;
    }
    int nx = atomicAdd(&dcnt[CNT_NSEG_NEXT], 2);
    if (nx + 2 > seg_cap) {
        // no room for the children's segments: stop here (the insert reports
        // a capacity error); k_seg_d skips non-split segments
        atomicOr((unsigned*)&dcnt[CNT_ERR], MPTG_DEVERR_CAPACITY);
        S.kind = SEG_LEAF; S.bucket = -1;
        cur[s] = S;
        return;
    }
    SegState a;
    memset(&a, 0, sizeof(a));
    a.node = c; a.parent = s; a.side = 0; a.depth = S.depth + 1;
    next[nx] = a;
    a.node = c + 1; a.side = 1;
    next[nx + 1] = a;
    S.dim = dim; S.split = split; S.degenerate = degenerate; S.next = nx;
    cur[s] = S;
}

// level step D (per position): partition the points of split segments
__global__ void k_seg_d(SegState* __restrict__ cur, const int* __restrict__ perm, const int* __restrict__ pseg,
                        int* __restrict__ perm2, int* __restrict__ pseg2, int total, const float* __restrict__ pts32,
                        int D, const int* __restrict__ dcnt, int seg_cap) {
    if (total < 0) total = pending_total(dcnt, seg_cap);
    int pos = blockIdx.x * blockDim.x + threadIdx.x;
    int lane = threadIdx.x & 31;
    int s = pos < total ? pseg[pos] : -1;
    bool act = false;
    bool left = false;
    int p = -1;
    SegState S;
    if (s >= 0) {
        S = cur[s];
        if (S.kind == SEG_SPLIT) {
            act = true;
            p = perm[pos];
            left = S.degenerate ? (pos - S.start < S.count / 2) : (pts32[(size_t)p * D + S.dim] < S.split);
        }
    }
    if (s >= 0 && !act) pseg2[pos] = -1;
    unsigned am = __ballot_sync(0xffffffffu, act);
    if (act) {
        unsigned grp = __match_any_sync(am, s);
        unsigned lm = __ballot_sync(grp, left);
        unsigned rm = grp & ~lm;
        int leader = __ffs(grp) - 1;
        int lbase = 0, rbase = 0;
        if (lane == leader) {
            if (lm) lbase = atomicAdd(&cur[s].lc, __popc(lm));
            if (rm) rbase = atomicAdd(&cur[s].rc, __popc(rm));
        }
        lbase = __shfl_sync(grp, lbase, leader);
        rbase = __shfl_sync(grp, rbase, leader);
        unsigned below = (1u << lane) - 1u;
        int slot;
        if (left) slot = S.start + lbase + __popc(lm & below);
        else slot = S.start + S.count - 1 - (rbase + __popc(rm & below));
        perm2[slot] = p;
        pseg2[slot] = S.next + (left ? 0 : 1);
    }
}

// ------------------------------------------------------------------ search

__device__ __forceinline__ float warp_sum16(float v) {
    v += __shfl_xor_sync(0xffffffffu, v, 8);
    v += __shfl_xor_sync(0xffffffffu, v, 4);
    v += __shfl_xor_sync(0xffffffffu, v, 2);
    v += __shfl_xor_sync(0xffffffffu, v, 1);
    return __shfl_sync(0xffffffffu, v, 0);
}

__device__ __forceinline__ float so2_w32(float x) {
    x = fabsf(x);
    return fminf(x, TWO_PI_F - x);
}

// lower bound of the distance from the query to a cell whose interval on
// dimension d is [lo, hi] in lane d (lanes >= D ignored)
template <int MK>
__device__ __forceinline__ float cell_lb_vals(const TreeView& t, float myq, float lo, float hi, int lane) {
    const int D = t.D;
    if constexpr (MK == MPTG_METRIC_L2 || MK == MPTG_METRIC_L1) {
        float o = lane < D ? fmaxf(fmaxf(lo - myq, myq - hi), 0.f) : 0.f;
        if constexpr (MK == MPTG_METRIC_L2) return sqrtf(warp_sum16(o * o));
        else return warp_sum16(o);
    } else if constexpr (MK == MPTG_METRIC_SO2) {
        float o = 0.f;
        if (lane < D && (myq < lo || myq > hi)) o = fminf(so2_w32(myq - lo), so2_w32(myq - hi));
        return warp_sum16(o);
    } else {
        float cp = 0.f, cm = 0.f, tt = 0.f;
        if (lane < 4) {
            float o = fmaxf(fmaxf(lo - myq, myq - hi), 0.f);
            float om = fmaxf(fmaxf(lo + myq, -myq - hi), 0.f);
            cp = o * o; cm = om * om;
        } else if (lane < 7 && MK == MPTG_METRIC_SE3) {
            float o = fmaxf(fmaxf(lo - myq, myq - hi), 0.f);
            tt = o * o;
        }
        cp = warp_sum16(cp);
        cm = warp_sum16(cm);
        float rot = 2.f * asinf(fminf(1.f, 0.5f * sqrtf(fminf(cp, cm))));
        if constexpr (MK == MPTG_METRIC_SO3) {
            return rot;
        } else {
            tt = warp_sum16(tt);
            return t.w0f * rot + t.w1f * sqrtf(tt);
        }
    }
}

// cell_lb_vals for L1, L2 and SO(2)^n with every dimension held twice, by
// lanes d and d + 16 (dl = lane & 15): the xor reduction over 16 lanes then
// leaves the sum in all 32 lanes, with no broadcast (the same additions in
// the same order as warp_sum16, so the same bound bit for bit).
template <int MK>
__device__ __forceinline__ float cell_lb_half(int D, float myq, float lo, float hi, int dl) {
    float o = 0.f;
    if constexpr (MK == MPTG_METRIC_SO2) {
        if (dl < D && (myq < lo || myq > hi)) o = fminf(so2_w32(myq - lo), so2_w32(myq - hi));
    } else {
        o = dl < D ? fmaxf(fmaxf(lo - myq, myq - hi), 0.f) : 0.f;
        if constexpr (MK == MPTG_METRIC_L2) o = o * o;
    }
    o += __shfl_xor_sync(0xffffffffu, o, 8);
    o += __shfl_xor_sync(0xffffffffu, o, 4);
    o += __shfl_xor_sync(0xffffffffu, o, 2);
    o += __shfl_xor_sync(0xffffffffu, o, 1);
    if constexpr (MK == MPTG_METRIC_L2) return sqrtf(o);
    else return o;
}

// lower bound of the distance from the query to node `c`'s stored cell
template <int MK>
__device__ __forceinline__ float cell_lb(const TreeView& t, int c, float myq, int lane) {
    const int D = t.D;
    float lo = 0.f, hi = 0.f;
    if (lane < D) {
        lo = __ldg(&t.cell_lo[(size_t)c * D + lane]);
        hi = __ldg(&t.cell_hi[(size_t)c * D + lane]);
    }
    return cell_lb_vals<MK>(t, myq, lo, hi, lane);
}

// Candidate step shared by the tree and the linear scan: each lane holds one
// point (id pid, FP32 distance d32).  Every point that could beat or tie the
// current best in exact arithmetic is re-ranked in FP64.
// ids: when not null, the lane's point id is ids[lane], read only for a
// candidate (most buckets have none), and pid is ignored.
__device__ __forceinline__ void rerank_step(const TreeView& t, const double* __restrict__ qd, int lane, bool have,
                                            int pid, float d32, float E, double& best, int& bidx, float& bestf_up,
                                            unsigned long long& nrerank, const int* __restrict__ ids = nullptr) {
    // most buckets hold no point that can reach the current best: leave
    // before the bucket-minimum reduction (the candidate set is unchanged)
    if (!__any_sync(0xffffffffu, have && __fsub_rd(d32, E) <= bestf_up)) return;
    float m = d32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    float thr = __fadd_ru(m, __fmul_ru(2.f, E));
    bool cand = have && __fsub_rd(d32, E) <= bestf_up && d32 <= thr;
    unsigned cm = __ballot_sync(0xffffffffu, cand);
    if (!cm) return;
    nrerank += __popc(cm);
    double dd = INFINITY;
    int pp = INT_MAX;
    if (cand) {
        if (ids) pid = __ldg(&ids[lane]);
        dd = dist64(t.metric, t.D, t.w0, t.w1, qd, t.states64 + (size_t)pid * t.D);
        pp = pid;
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

template <int MK, int DMAX>
__device__ __forceinline__ void load_query(const double* __restrict__ qd, int D, int lane, float (&q)[DMAX],
                                           float& myq, float& M, const TreeView& t) {
    M = __int_as_float(t.dcnt[CNT_MAXABS]);
#pragma unroll
    for (int d = 0; d < DMAX; ++d) {
        float v = 0.f;
        if (d < D) v = __double2float_rn(qd[d]);
        q[d] = v;
        bool lp = MK == MPTG_METRIC_L2 || MK == MPTG_METRIC_L1 || (MK == MPTG_METRIC_SE3 && d >= 4 && d < 7);
        if (lp && d < D) M = fmaxf(M, __double2float_ru(fabs(qd[d])));
    }
    myq = 0.f;
#pragma unroll
    for (int d = 0; d < DMAX; ++d)
        if (lane == d) myq = q[d];
}

// One query (index qi) answered by the calling warp.
template <int MK, int DMAX>
__device__ __forceinline__ void nearest_one(const TreeView& t, const double* __restrict__ q64, int qi, int lane,
                                            int* __restrict__ out_idx, double* __restrict__ out_d) {
    const int D = t.D;
    const double* qd = q64 + (size_t)qi * D;
    float q[DMAX];
    float myq, M;
    load_query<MK, DMAX>(qd, D, lane, q, myq, M, t);
    const float E = err32<MK>(D, M, t.w0f, t.w1f);
    // L1 / L2 / SO(2)^n: each half-warp holds every dimension (cell_lb_half)
    constexpr bool HALF = (MK == MPTG_METRIC_L1 || MK == MPTG_METRIC_L2 || MK == MPTG_METRIC_SO2) && DMAX <= 16;
    const int dl = HALF ? (lane & 15) : lane;
    if constexpr (HALF) {
#pragma unroll
        for (int d = 0; d < DMAX; ++d)
            if (dl == d) myq = q[d];
    }

    double best = INFINITY;
    int bidx = INT_MAX;
    float bestf_up = INFINITY;
    unsigned long long n_int = 0, n_leaf = 0, n_pts = 0, n_rr = 0;

    int sp = 0;
    int s0n = 0, s1n = 0;
    float s0l = 0.f, s1l = 0.f;
    int node = 0;
    // The current node's record and cell live in registers: lane d < D (and
    // d + 16 under HALF) holds the cell's interval on dimension d.  A child's
    // cell is its parent's with one bound replaced by the split (as k_seg_c
    // builds them), so descending needs no cell load; only a pop reloads a
    // cell.  The near child's record is loaded (one address for the whole
    // warp) as soon as the side is known, and arrives while the far child's
    // bound is computed, so each level costs one round trip.
    int4 nd = __ldg(&t.nodes[0]);
    float clo = 0.f, chi = 0.f;
    if (dl < D) { clo = __ldg(&t.cell_lo[dl]); chi = __ldg(&t.cell_hi[dl]); }
    while (true) {
        if (nd.x >= 0) {
            ++n_int;
            const int c = nd.y, s = nd.x;
            const float split = __int_as_float(nd.z);
            const float qv = __shfl_sync(0xffffffffu, myq, s);
            const bool goLeft = qv < split;
            const int nearc = goLeft ? c : c + 1;
            const int4 nn = __ldg(&t.nodes[nearc]);
            float flo = clo, fhi = chi;
            if (dl == s) {
                if (goLeft) flo = split;
                else fhi = split;
            }
            float lb;
            if constexpr (HALF) lb = cell_lb_half<MK>(D, myq, flo, fhi, dl);
            else lb = cell_lb_vals<MK>(t, myq, flo, fhi, lane);
            const int farc = goLeft ? c + 1 : c;
            // the builder keeps depth <= MPTG_MAX_DEPTH < 64, so the stack never fills
            if (__fsub_rd(lb, E) <= bestf_up && sp < 64) {
                if (sp < 32) {
                    if (lane == sp) { s0n = farc; s0l = lb; }
                } else {
                    if (lane == sp - 32) { s1n = farc; s1l = lb; }
                }
                ++sp;
            }
            if (dl == s) {
                if (goLeft) chi = split;
                else clo = split;
            }
            nd = nn;
            node = nearc;
            continue;
        }
        // leaf
        ++n_leaf;
        int cnt = nd.w < MPTG_BUCKET ? nd.w : MPTG_BUCKET;
        n_pts += cnt;
        bool have = lane < cnt;
        float d32 = INFINITY;
        const size_t b = (size_t)nd.y;
        if (have) {
            const float* bp = t.bpts + b * (size_t)D * MPTG_BUCKET + lane;  // dimension d at bp[32 d]
            float p[DMAX];
            if (D == DMAX) {  // the exact-dimension instantiation: no per-dimension guard
#pragma unroll
                for (int d = 0; d < DMAX; ++d) p[d] = __ldg(bp + d * MPTG_BUCKET);
            } else {
#pragma unroll
                for (int d = 0; d < DMAX; ++d) p[d] = d < D ? __ldg(bp + d * MPTG_BUCKET) : 0.f;
            }
            d32 = dist32<MK, DMAX>(q, p, t.w0f, t.w1f);
            if (!(d32 == d32)) d32 = INFINITY;
        }
        rerank_step(t, qd, lane, have, -1, d32, E, best, bidx, bestf_up, n_rr, t.bids + b * MPTG_BUCKET);
        // pop the next far child whose bound can still beat the best
        bool found = false;
        while (sp > 0) {
            --sp;
            int src = sp & 31;
            int nn;
            float lb;
            if (sp < 32) { nn = __shfl_sync(0xffffffffu, s0n, src); lb = __shfl_sync(0xffffffffu, s0l, src); }
            else { nn = __shfl_sync(0xffffffffu, s1n, src); lb = __shfl_sync(0xffffffffu, s1l, src); }
            if (__fsub_rd(lb, E) <= bestf_up) { node = nn; found = true; break; }
        }
        if (!found) break;
        nd = __ldg(&t.nodes[node]);
        if (dl < D) {
            clo = __ldg(&t.cell_lo[(size_t)node * D + dl]);
            chi = __ldg(&t.cell_hi[(size_t)node * D + dl]);
        }
    }
    if (lane == 0) {
        out_idx[qi] = bidx == INT_MAX ? -1 : bidx;
        out_d[qi] = best;
        if (t.stats) {
            atomicAdd(&t.stats[0], 1ull);
            atomicAdd(&t.stats[1], n_int);
            atomicAdd(&t.stats[2], n_leaf);
            atomicAdd(&t.stats[3], n_pts);
            atomicAdd(&t.stats[4], n_rr);
        }
    }
}

// Warp per query.  order (may be null): the w-th query answered is
// order[w], so that neighbouring warps, sorted by tree region, reuse each
// other's nodes in L1.  qnext (may be null, else zeroed before the launch):
// a grid of resident warps only; each warp answers query w = its warp id,
// then takes w = (warps in the grid) + atomicAdd(qnext, 1) until w >= nq, so
// no warp slot idles while the slowest query of its block finishes (query
// costs vary several-fold).
template <int MK, int DMAX>
__global__ void __launch_bounds__(256, 4) k_nearest(TreeView t, const double* __restrict__ q64, int nq,
                                                 const int* __restrict__ order, int* __restrict__ out_idx,
                                                 double* __restrict__ out_d, int* __restrict__ qnext) {
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)(((size_t)gridDim.x * blockDim.x) >> 5);
    int wi = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    while (wi < nq) {
        nearest_one<MK, DMAX>(t, q64, order ? __ldg(&order[wi]) : wi, lane, out_idx, out_d);
        if (!qnext) break;
        int nx = 0;
        if (lane == 0) nx = atomicAdd(qnext, 1);
        wi = nwarps + __shfl_sync(0xffffffffu, nx, 0);
    }
}

// ------------------------------------------------------------------ packets
// Packet traversal for large, spatially ordered batches: one warp answers 32
// neighbouring queries (one per lane) and walks the union of their search
// trees once.  Every node and bucket it touches is loaded by all lanes from
// the same address (one L1 transaction, shared by 32 queries), instead of
// each query following its own dependent chain through L2.  Pruning is per
// lane; a node is entered when any lane's bound admits it (ballot).

// lower bound of the distance from this lane's query to node c's cell
template <int MK, int DMAX>
__device__ __forceinline__ float lane_cell_lb(const TreeView& t, int c, const float (&q)[DMAX], float w0,
                                              float w1) {
    const float* lo = t.cell_lo + (size_t)c * t.D;
    const float* hi = t.cell_hi + (size_t)c * t.D;
    if constexpr (MK == MPTG_METRIC_L2 || MK == MPTG_METRIC_L1) {
        float s = 0.f;
#pragma unroll
        for (int d = 0; d < DMAX; ++d) {
            if (d < t.D) {
                float o = fmaxf(fmaxf(__ldg(&lo[d]) - q[d], q[d] - __ldg(&hi[d])), 0.f);
                if constexpr (MK == MPTG_METRIC_L2) s = fmaf(o, o, s);
                else s += o;
            }
        }
        if constexpr (MK == MPTG_METRIC_L2) return sqrtf(s);
        else return s;
    } else if constexpr (MK == MPTG_METRIC_SO2) {
        float s = 0.f;
#pragma unroll
        for (int d = 0; d < DMAX; ++d) {
            if (d < t.D) {
                float l = __ldg(&lo[d]), h = __ldg(&hi[d]);
                if (q[d] < l || q[d] > h) s += fminf(so2_w32(q[d] - l), so2_w32(q[d] - h));
            }
        }
        return s;
    } else {
        float cp = 0.f, cm = 0.f;
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            float l = __ldg(&lo[d]), h = __ldg(&hi[d]);
            float o = fmaxf(fmaxf(l - q[d], q[d] - h), 0.f);
            float om = fmaxf(fmaxf(l + q[d], -q[d] - h), 0.f);
            cp = fmaf(o, o, cp);
            cm = fmaf(om, om, cm);
        }
        float rot = 2.f * asinf(fminf(1.f, 0.5f * sqrtf(fminf(cp, cm))));
        if constexpr (MK == MPTG_METRIC_SO3) {
            return rot;
        } else {
            float s = 0.f;
#pragma unroll
            for (int d = 4; d < 7; ++d) {
                float o = fmaxf(fmaxf(__ldg(&lo[d]) - q[d], q[d] - __ldg(&hi[d])), 0.f);
                s = fmaf(o, o, s);
            }
            return w0 * rot + w1 * sqrtf(s);
        }
    }
}

template <int MK, int DMAX>
__global__ void __launch_bounds__(256, 4) k_nearest_packet(TreeView t, const double* __restrict__ q64, int nq,
                                                           const int* __restrict__ order, int* __restrict__ out_idx,
                                                           double* __restrict__ out_d) {
    const int lane = threadIdx.x & 31;
    const int base = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5) * 32;
    if (base >= nq) return;
    const int D = t.D;
    const int slot = base + lane;
    const bool act = slot < nq;
    const int qi = act ? __ldg(&order[slot]) : 0;
    const double* qd = q64 + (size_t)qi * D;
    float q[DMAX];
    float M = __int_as_float(t.dcnt[CNT_MAXABS]);
#pragma unroll
    for (int d = 0; d < DMAX; ++d) {
        float v = 0.f;
        if (act && d < D) v = __double2float_rn(qd[d]);
        q[d] = v;
        bool lp = MK == MPTG_METRIC_L2 || MK == MPTG_METRIC_L1 || (MK == MPTG_METRIC_SE3 && d >= 4 && d < 7);
        if (lp && act && d < D) M = fmaxf(M, __double2float_ru(fabs(qd[d])));
    }
    const float E = err32<MK>(D, M, t.w0f, t.w1f);
    const float E2 = __fmul_ru(2.f, E);
    double best = INFINITY;
    int bidx = INT_MAX;
    float bestf_up = act ? INFINITY : -INFINITY;  // inactive lanes never admit a node
    float run32 = INFINITY;
    unsigned long long n_int = 0, n_leaf = 0, n_pts = 0, n_rr = 0;

    int sp = 0;
    int s0n = 0, s1n = 0;
    int node = 0;
    while (true) {
        int4 nd = __ldg(&t.nodes[node]);
        if (nd.x >= 0) {
            ++n_int;
            int c = nd.y;
            float lbL = lane_cell_lb<MK, DMAX>(t, c, q, t.w0f, t.w1f);
            float lbR = lane_cell_lb<MK, DMAX>(t, c + 1, q, t.w0f, t.w1f);
            bool nL = __fsub_rd(lbL, E) <= bestf_up;
            bool nR = __fsub_rd(lbR, E) <= bestf_up;
            unsigned bL = __ballot_sync(0xffffffffu, nL), bR = __ballot_sync(0xffffffffu, nR);
            if (bL && bR) {
                // enter the child most lanes are closer to; keep the other
                unsigned pl = __ballot_sync(0xffffffffu, nL && (!nR || lbL <= lbR));
                unsigned pr = __ballot_sync(0xffffffffu, nR && (!nL || lbR < lbL));
                int first = __popc(pl) >= __popc(pr) ? c : c + 1;
                int second = 2 * c + 1 - first;
                if (sp < 64) {
                    if (sp < 32) { if (lane == sp) s0n = second; }
                    else if (lane == sp - 32) s1n = second;
                    ++sp;
                }
                node = first;
                continue;
            } else if (bL || bR) {
                node = bL ? c : c + 1;
                continue;
            }
        } else {
            ++n_leaf;
            int cnt = nd.w < MPTG_BUCKET ? nd.w : MPTG_BUCKET;
            n_pts += cnt;
            const size_t b = (size_t)nd.y;
            const float* bp = t.bpts + b * D * MPTG_BUCKET;
            for (int j = 0; j < cnt; ++j) {
                float p[DMAX];
#pragma unroll
                for (int d = 0; d < DMAX; ++d) p[d] = d < D ? __ldg(&bp[d * MPTG_BUCKET + j]) : 0.f;
                float d32 = dist32<MK, DMAX>(q, p, t.w0f, t.w1f);
                if (!(d32 == d32)) continue;
                run32 = fminf(run32, d32);
                // a point that could beat or tie this lane's best in exact arithmetic
                if (act && __fsub_rd(d32, E) <= bestf_up && d32 <= __fadd_ru(run32, E2)) {
                    int pid = __ldg(&t.bids[b * MPTG_BUCKET + j]);
                    double dd = dist64(t.metric, D, t.w0, t.w1, qd, t.states64 + (size_t)pid * D);
                    ++n_rr;
                    if (dd < best || (dd == best && pid < bidx)) {
                        best = dd;
                        bidx = pid;
                        bestf_up = __double2float_ru(best);
                    }
                }
            }
        }
        // pop until a node some lane still needs
        bool found = false;
        while (sp > 0) {
            --sp;
            int src = sp & 31;
            int nn = sp < 32 ? __shfl_sync(0xffffffffu, s0n, src) : __shfl_sync(0xffffffffu, s1n, src);
            float lb = lane_cell_lb<MK, DMAX>(t, nn, q, t.w0f, t.w1f);
            if (__any_sync(0xffffffffu, __fsub_rd(lb, E) <= bestf_up)) { node = nn; found = true; break; }
        }
        if (!found) break;
    }
    if (act) {
        out_idx[qi] = bidx == INT_MAX ? -1 : bidx;
        out_d[qi] = best;
    }
    if (t.stats) {
        // per-query accounting: every lane paid for the whole packet walk
        unsigned na = __popc(__ballot_sync(0xffffffffu, act));
        unsigned long long rr = n_rr;
        for (int o = 16; o > 0; o >>= 1) rr += __shfl_xor_sync(0xffffffffu, rr, o);
        if (lane == 0) {
            atomicAdd(&t.stats[0], (unsigned long long)na);
            atomicAdd(&t.stats[1], n_int * na);
            atomicAdd(&t.stats[2], n_leaf * na);
            atomicAdd(&t.stats[3], n_pts * na);
            atomicAdd(&t.stats[4], rr);
        }
    }
}

// exhaustive scan (nigh::Linear): warp per query, 32 points per step
template <int MK, int DMAX>
__global__ void __launch_bounds__(256) k_nearest_linear(TreeView t, const double* __restrict__ q64, int nq,
                                                        int* __restrict__ out_idx, double* __restrict__ out_d) {
    const int lane = threadIdx.x & 31;
    const int qi = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (qi >= nq) return;
    const int D = t.D;
    const double* qd = q64 + (size_t)qi * D;
    float q[DMAX];
    float myq, M;
    load_query<MK, DMAX>(qd, D, lane, q, myq, M, t);
    const float E = err32<MK>(D, M, t.w0f, t.w1f);
    double best = INFINITY;
    int bidx = INT_MAX;
    float bestf_up = INFINITY;
    unsigned long long nrr = 0;
    for (int base = 0; base < t.n; base += 32) {
        int j = base + lane;
        bool have = j < t.n;
        float d32 = INFINITY;
        if (have) {
            float p[DMAX];
#pragma unroll
            for (int d = 0; d < DMAX; ++d) p[d] = d < D ? t.pts32[(size_t)j * D + d] : 0.f;
            d32 = dist32<MK, DMAX>(q, p, t.w0f, t.w1f);
            if (!(d32 == d32)) d32 = INFINITY;
        }
        rerank_step(t, qd, lane, have, j, d32, E, best, bidx, bestf_up, nrr);
    }
    if (lane == 0) {
        out_idx[qi] = bidx == INT_MAX ? -1 : bidx;
        out_d[qi] = best;
    }
}

// ------------------------------------------------------------------ tiled exhaustive 1-NN
// For trees in high dimension the kd-tree visits a large share of the points
// at a high cost per point (dependent node loads, divergent lanes).  This
// sweep is thread per query and runs in two passes.
//  Pass 1 (k_nearest_tiled): block (query tile, point split) stages its split
//   of the FP32 points through shared memory, BRUTE_TILE at a time, so each
//   point is read once per 256 queries, and every thread keeps the BRUTE_K
//   smallest FP32 distances (distance, id) of the split in registers.
//   Splitting the points keeps the GPU full when there are few queries.
//  Pass 2 (k_nearest_tiled_merge): the exact argmin p* satisfies
//   d32(p*) <= d64(p*) + E <= d64(argmin32) + E <= min32 + 2E
//   (|d32 - d64| <= E for every point), and so does every point tied with it.
//   When every split's K-th kept distance exceeds min32 + 2E, each such point
//   is in some list and the FP64 re-rank runs on the lists alone; otherwise
//   (more than K points within 2E in a split, e.g. duplicates) the thread
//   sweeps all points again and re-ranks every one within min32 + 2E.
// Ties go to the lowest id, as in k_nearest.
#define BRUTE_K 8
#define BRUTE_TILE 256

template <int MK, int DMAX>
__device__ __forceinline__ float load_query32(const TreeView& t, const double* __restrict__ qd, bool active,
                                              float (&q)[DMAX]) {
    float M = __int_as_float(t.dcnt[CNT_MAXABS]);
#pragma unroll
    for (int d = 0; d < DMAX; ++d) {
        float v = 0.f;
        if (d < t.D && active) v = __double2float_rn(qd[d]);
        q[d] = v;
        bool lp = MK == MPTG_METRIC_L2 || MK == MPTG_METRIC_L1 || (MK == MPTG_METRIC_SE3 && d >= 4 && d < 7);
        if (lp && d < t.D && active) M = fmaxf(M, __double2float_ru(fabs(qd[d])));
    }
    return err32<MK>(t.D, M, t.w0f, t.w1f);
}

// cd / ci: [split][BRUTE_K][nq]
template <int MK, int DMAX>
__global__ void __launch_bounds__(BRUTE_TILE) k_nearest_tiled(TreeView t, const double* __restrict__ q64, int nq,
                                                              int chunk, float* __restrict__ cd,
                                                              int* __restrict__ ci) {
    __shared__ float tile[DMAX][BRUTE_TILE];
    const int qi = blockIdx.x * BRUTE_TILE + threadIdx.x;
    const int split = blockIdx.y;
    const bool active = qi < nq;
    const int D = t.D;
    float q[DMAX];
    load_query32<MK, DMAX>(t, q64 + (size_t)(active ? qi : 0) * D, active, q);
    float kd[BRUTE_K];
    int ki[BRUTE_K];
#pragma unroll
    for (int s = 0; s < BRUTE_K; ++s) { kd[s] = INFINITY; ki[s] = -1; }
    const int lo = split * chunk, hi = min(t.n, lo + chunk);
    for (int base = lo; base < hi; base += BRUTE_TILE) {
        __syncthreads();
        const int j = base + threadIdx.x;
#pragma unroll
        for (int d = 0; d < DMAX; ++d) tile[d][threadIdx.x] = (j < hi && d < D) ? t.pts32[(size_t)j * D + d] : 0.f;
        __syncthreads();
        if (!active) continue;
        const int cnt = min(BRUTE_TILE, hi - base);
        for (int k = 0; k < cnt; ++k) {
            float p[DMAX];
#pragma unroll
            for (int d = 0; d < DMAX; ++d) p[d] = tile[d][k];
            float d32 = dist32<MK, DMAX>(q, p, t.w0f, t.w1f);
            if (d32 < kd[BRUTE_K - 1]) {  // false for NaN
                float xd = d32;
                int xi = base + k;
#pragma unroll
                for (int s = 0; s < BRUTE_K; ++s) {
                    if (xd < kd[s]) {
                        float td = kd[s]; kd[s] = xd; xd = td;
                        int ti = ki[s]; ki[s] = xi; xi = ti;
                    }
                }
            }
        }
    }
    if (!active) return;
#pragma unroll
    for (int s = 0; s < BRUTE_K; ++s) {
        cd[((size_t)split * BRUTE_K + s) * nq + qi] = kd[s];
        ci[((size_t)split * BRUTE_K + s) * nq + qi] = ki[s];
    }
}

// Warp per query: the lanes take the splits round-robin.  Each split's list is
// sorted, so a split whose first entry exceeds min32 + 2E holds no candidate
// and is complete, and the common case reads one value per split.
template <int MK, int DMAX>
__global__ void __launch_bounds__(256) k_nearest_tiled_merge(TreeView t, const double* __restrict__ q64, int nq,
                                                             int nsplit, const float* __restrict__ cd,
                                                             const int* __restrict__ ci, int* __restrict__ out_idx,
                                                             double* __restrict__ out_d) {
    const int lane = threadIdx.x & 31;
    const int qi = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (qi >= nq) return;  // warp-uniform
    const int D = t.D;
    const double* qd = q64 + (size_t)qi * D;
    float q[DMAX];
    const float E = load_query32<MK, DMAX>(t, qd, true, q);
    float m = INFINITY;
    for (int sp = lane; sp < nsplit; sp += 32) m = fminf(m, cd[((size_t)sp * BRUTE_K) * nq + qi]);
    for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
    double best = INFINITY;
    int bidx = INT_MAX;
    unsigned long long nrr = 0;
    if (m < INFINITY) {
        const float thr = __fadd_ru(m, __fmul_ru(2.f, E));
        auto consider = [&](int id) {
            ++nrr;
            double dd = dist64(t.metric, D, t.w0, t.w1, qd, t.states64 + (size_t)id * D);
            if (dd == dd && (dd < best || (dd == best && id < bidx))) { best = dd; bidx = id; }
        };
        bool complete = true;
        for (int sp = lane; sp < nsplit; sp += 32) {
            const size_t o0 = ((size_t)sp * BRUTE_K) * nq + qi;
            if (!(cd[o0] <= thr)) continue;
            complete = complete && cd[o0 + (size_t)(BRUTE_K - 1) * nq] > thr;
            for (int s = 0; s < BRUTE_K; ++s) {
                const size_t o = o0 + (size_t)s * nq;
                if (!(cd[o] <= thr)) break;
                if (ci[o] >= 0) consider(ci[o]);
            }
        }
        if (!__all_sync(0xffffffffu, complete)) {
            // more than BRUTE_K points within 2E in some split: every point
            // again, lanes round-robin
            best = INFINITY;
            bidx = INT_MAX;
            for (int j = lane; j < t.n; j += 32) {
                float p[DMAX];
#pragma unroll
                for (int d = 0; d < DMAX; ++d) p[d] = d < D ? t.pts32[(size_t)j * D + d] : 0.f;
                if (dist32<MK, DMAX>(q, p, t.w0f, t.w1f) <= thr) consider(j);
            }
        }
    }
    // (distance, id) minimum over the lanes
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (ob < best || (ob == best && oi < bidx)) { best = ob; bidx = oi; }
    }
    for (int o = 16; o > 0; o >>= 1) nrr += __shfl_xor_sync(0xffffffffu, nrr, o);
    if (lane == 0) {
        out_idx[qi] = bidx == INT_MAX ? -1 : bidx;
        out_d[qi] = best;
        if (t.stats) {
            atomicAdd(&t.stats[0], 1ull);
            atomicAdd(&t.stats[3], (unsigned long long)t.n);
            atomicAdd(&t.stats[4], nrr);
        }
    }
}

// ------------------------------------------------------------------ k-NN

// One batch of up to 32 candidate points (lane: have, pid, d32) against the
// warp's sorted k-NN list: every point whose FP32 distance is within E of the
// bound tau gets its FP64 distance, and those within tau join the list in
// (distance, id) order, one at a time (the list lives two entries per lane).
__device__ __forceinline__ void knn_consider(const TreeView& t, const double* __restrict__ qd, int lane, int k,
                                             double radius, bool have, int pid, float d32, float E, double& ld0,
                                             double& ld1, int& li0, int& li1, int& cnt, double& tau, float& tauf) {
    bool cand = have && __fsub_rd(d32, E) <= tauf;
    double dd = INFINITY;
    if (cand) {
        dd = dist64(t.metric, t.D, t.w0, t.w1, qd, t.states64 + (size_t)pid * t.D);
        cand = dd <= tau;
    }
    knn_insert(lane, k, radius, cand, dd, pid, ld0, ld1, li0, li1, cnt, tau, tauf);
}

// FP32 twin of knn_insert for k_nearest_k_tiled's running list: the 64 best
// (d32, id) pairs, entry j in lane j (fd0/fi0) or lane j - 32 (fd1/fi1)
__device__ __forceinline__ void fknn_insert(int lane, bool cand, float d32, int pid, float& fd0, float& fd1, int& fi0,
                                            int& fi1, int& fcnt, float& ftau) {
    unsigned cmask = __ballot_sync(0xffffffffu, cand);
    while (cmask) {
        const int src = __ffs(cmask) - 1;
        cmask &= cmask - 1;
        const float cd = __shfl_sync(0xffffffffu, d32, src);
        const int ci = __shfl_sync(0xffffffffu, pid, src);
        if (fcnt == 64) {
            const float kd = __shfl_sync(0xffffffffu, fd1, 31);
            const int ki = __shfl_sync(0xffffffffu, fi1, 31);
            if (!(cd < kd || (cd == kd && ci < ki))) continue;
        }
        const bool ahead0 = lane < fcnt && (fd0 < cd || (fd0 == cd && fi0 < ci));
        const bool ahead1 = lane + 32 < fcnt && (fd1 < cd || (fd1 == cd && fi1 < ci));
        const int pos = __popc(__ballot_sync(0xffffffffu, ahead0)) + __popc(__ballot_sync(0xffffffffu, ahead1));
        const float p0d = __shfl_up_sync(0xffffffffu, fd0, 1), p1d = __shfl_up_sync(0xffffffffu, fd1, 1);
        const int p0i = __shfl_up_sync(0xffffffffu, fi0, 1), p1i = __shfl_up_sync(0xffffffffu, fi1, 1);
        const float l0d = __shfl_sync(0xffffffffu, fd0, 31);
        const int l0i = __shfl_sync(0xffffffffu, fi0, 31);
        if (lane > pos) { fd0 = p0d; fi0 = p0i; }
        else if (lane == pos) { fd0 = cd; fi0 = ci; }
        const int j1 = lane + 32;
        if (j1 > pos) { fd1 = lane == 0 ? l0d : p1d; fi1 = lane == 0 ? l0i : p1i; }
        else if (j1 == pos) { fd1 = cd; fi1 = ci; }
        if (fcnt < 64) ++fcnt;
        if (fcnt == 64) ftau = __shfl_sync(0xffffffffu, fd1, 31);
    }
}

// Exhaustive k nearest for high-dimensional trees (the strategy rule of the
// 1-NN sweep), warp per (query, point split): a block of 8 queries stages the
// split's FP32 points through shared memory, 256 at a time, and each warp
// keeps the 64 best FP32 (distance, id) pairs, FP32 work only.  With
// dk = the k-th kept FP32 distance, every member p of the exact top k has
//   d32(p) <= d64(p) + E <= dk + 2E
// (the k FP32-best points lie within dk + E in FP64, or one of them lies
// beyond the radius, which then is below dk + E), so when the list holds the
// whole split or its 64th entry exceeds dk + 2E, the exact top k is the
// knn_insert ranking of the kept entries within dk + 2E by their FP64
// distances.  Otherwise (more than 64 - k points within 2E of dk, e.g.
// duplicates) the warp sweeps the split again through knn_consider, the list
// logic of the tree walk.  Either way the list is the exact (distance,
// id)-ordered top k of the split.  With one split it is the answer (equal to
// k_nearest_k's); with several, each split's list goes to out + split * nq * k
// and k_nearest_k_merge keeps the top k of their union, which holds the
// global top k.  The list's slack is 64 - k entries, so with k near 64 the
// second sweep runs more often.
template <int MK, int DMAX>
__global__ void __launch_bounds__(256) k_nearest_k_tiled(TreeView t, const double* __restrict__ q64, int nq, int k,
                                                         double radius, int chunk, int* __restrict__ out_idx,
                                                         double* __restrict__ out_d) {
    __shared__ float tile[DMAX][256];
    const int lane = threadIdx.x & 31;
    const int qi = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int split = blockIdx.y;
    const bool active = qi < nq;  // warp-uniform
    const int D = t.D;
    const double* qd = q64 + (size_t)(active ? qi : 0) * D;
    float q[DMAX];
    float myq, M;
    load_query<MK, DMAX>(qd, D, lane, q, myq, M, t);
    const float E = err32<MK>(D, M, t.w0f, t.w1f);
    float fd0 = INFINITY, fd1 = INFINITY, ftau = INFINITY;
    int fi0 = INT_MAX, fi1 = INT_MAX, fcnt = 0;
    const int lo = split * chunk, n = min(t.n, lo + chunk);
    for (int base = lo; base < n; base += 256) {
        __syncthreads();
        const int j = base + threadIdx.x;
#pragma unroll
        for (int d = 0; d < DMAX; ++d) tile[d][threadIdx.x] = (j < n && d < D) ? t.pts32[(size_t)j * D + d] : 0.f;
        __syncthreads();
        if (!active) continue;
        const int cntp = min(256, n - base);
        for (int sub = 0; sub < cntp; sub += 32) {
            const int off = sub + lane;
            const bool have = off < cntp;
            float d32 = INFINITY;
            if (have) {
                float p[DMAX];
#pragma unroll
                for (int d = 0; d < DMAX; ++d) p[d] = tile[d][off];
                d32 = dist32<MK, DMAX>(q, p, t.w0f, t.w1f);
                if (!(d32 == d32)) d32 = INFINITY;
            }
            fknn_insert(lane, have && d32 <= ftau, d32, base + off, fd0, fd1, fi0, fi1, fcnt, ftau);
        }
    }
    if (!active) return;
    double ld0 = INFINITY, ld1 = INFINITY;
    int li0 = INT_MAX, li1 = INT_MAX;
    int cnt = 0;
    double tau = radius;
    float tauf = __double2float_ru(tau);
    const float dk = __shfl_sync(0xffffffffu, k - 1 < 32 ? fd0 : fd1, (k - 1) & 31);
    const float thr = __fadd_ru(dk, __fmul_ru(2.f, E));
    const bool whole = fcnt < 64;
    if (whole || (thr < INFINITY && __shfl_sync(0xffffffffu, fd1, 31) > thr)) {
        // exact re-rank of the kept entries within thr (all of them for a whole split)
        for (int slot = 0; slot < 2; ++slot) {
            const int e = lane + 32 * slot;
            const float fd = slot ? fd1 : fd0;
            const int fi = slot ? fi1 : fi0;
            bool cand = e < fcnt && (whole || fd <= thr);
            double dd = INFINITY;
            if (cand) {
                dd = dist64(t.metric, D, t.w0, t.w1, qd, t.states64 + (size_t)fi * D);
                cand = dd <= tau;
            }
            knn_insert(lane, k, radius, cand, dd, fi, ld0, ld1, li0, li1, cnt, tau, tauf);
        }
    } else {
        for (int base = lo; base < n; base += 32) {
            const int j = base + lane;
            const bool have = j < n;
            float d32 = INFINITY;
            if (have) {
                float p[DMAX];
#pragma unroll
                for (int d = 0; d < DMAX; ++d) p[d] = d < D ? t.pts32[(size_t)j * D + d] : 0.f;
                d32 = dist32<MK, DMAX>(q, p, t.w0f, t.w1f);
                if (!(d32 == d32)) d32 = INFINITY;
            }
            knn_consider(t, qd, lane, k, radius, have, j, d32, E, ld0, ld1, li0, li1, cnt, tau, tauf);
        }
    }
    int* oi = out_idx + ((size_t)split * nq + qi) * k;
    double* od = out_d + ((size_t)split * nq + qi) * k;
    if (lane < k) { bool v = lane < cnt; oi[lane] = v ? li0 : -1; od[lane] = v ? ld0 : INFINITY; }
    if (lane + 32 < k) { bool v = lane + 32 < cnt; oi[lane + 32] = v ? li1 : -1; od[lane + 32] = v ? ld1 : INFINITY; }
}

// Top k of the per-split lists of k_nearest_k_tiled (cd / ci: [split][nq][k],
// FP64 distances), warp per query, through the same insertion logic.
__global__ void __launch_bounds__(256) k_nearest_k_merge(int nq, int k, double radius, int nsplit,
                                                         const double* __restrict__ cd, const int* __restrict__ ci,
                                                         int* __restrict__ out_idx, double* __restrict__ out_d) {
    const int lane = threadIdx.x & 31;
    const int qi = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (qi >= nq) return;  // warp-uniform
    double ld0 = INFINITY, ld1 = INFINITY;
    int li0 = INT_MAX, li1 = INT_MAX;
    int cnt = 0;
    double tau = radius;
    float tauf = __double2float_ru(tau);
    const int total = nsplit * k;
    for (int c0 = 0; c0 < total; c0 += 32) {
        const int c = c0 + lane;
        const int sp = c / k, j = c - sp * k;
        const size_t o = ((size_t)sp * nq + qi) * k + j;
        const int pid = c < total ? ci[o] : -1;
        const double dd = pid >= 0 ? cd[o] : INFINITY;
        knn_insert(lane, k, radius, pid >= 0 && dd <= tau, dd, pid, ld0, ld1, li0, li1, cnt, tau, tauf);
    }
    int* oi = out_idx + (size_t)qi * k;
    double* od = out_d + (size_t)qi * k;
    if (lane < k) { bool v = lane < cnt; oi[lane] = v ? li0 : -1; od[lane] = v ? ld0 : INFINITY; }
    if (lane + 32 < k) { bool v = lane + 32 < cnt; oi[lane + 32] = v ? li1 : -1; od[lane + 32] = v ? ld1 : INFINITY; }
}

// Exact k nearest (k <= 64) sorted by (distance, id), warp per query.  The
// running list lives in registers: entry j in lane j (j < 32) / lane j-32 of
// the second slot.  tau = the k-th best exact distance (or the radius).
template <int MK, int DMAX>
__global__ void __launch_bounds__(256) k_nearest_k(TreeView t, const double* __restrict__ q64, int nq, int k,
                                                   double radius, int* __restrict__ out_idx,
                                                   double* __restrict__ out_d) {
    const int lane = threadIdx.x & 31;
    const int qi = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (qi >= nq) return;
    const int D = t.D;
    const double* qd = q64 + (size_t)qi * D;
    float q[DMAX];
    float myq, M;
    load_query<MK, DMAX>(qd, D, lane, q, myq, M, t);
    const float E = err32<MK>(D, M, t.w0f, t.w1f);
    // sorted list: (d, id) in two register slots
    double ld0 = INFINITY, ld1 = INFINITY;
    int li0 = INT_MAX, li1 = INT_MAX;
    int cnt = 0;
    double tau = radius;  // prune bound: k-th distance once full, else radius
    float tauf = __double2float_ru(tau);

    int sp = 0;
    int s0n = 0, s1n = 0;
    float s0l = 0.f, s1l = 0.f;
    int node = 0;
    while (true) {
        int4 nd = __ldg(&t.nodes[node]);
        if (nd.x >= 0) {
            float qv = __shfl_sync(0xffffffffu, myq, nd.x);
            float split = __int_as_float(nd.z);
            int nearc = qv < split ? nd.y : nd.y + 1;
            int farc = 2 * nd.y + 1 - nearc;
            float lb = cell_lb<MK>(t, farc, myq, lane);
            if (__fsub_rd(lb, E) <= tauf && sp < 64) {
                if (sp < 32) { if (lane == sp) { s0n = farc; s0l = lb; } }
                else if (lane == sp - 32) { s1n = farc; s1l = lb; }
                ++sp;
            }
            node = nearc;
            continue;
        }
        int c = nd.w < MPTG_BUCKET ? nd.w : MPTG_BUCKET;
        bool have = lane < c;
        float d32 = INFINITY;
        int pid = -1;
        if (have) {
            size_t b = (size_t)nd.y;
            pid = __ldg(&t.bids[b * MPTG_BUCKET + lane]);
            const float* bp = t.bpts + b * (size_t)D * MPTG_BUCKET + lane;  // dimension d at bp[32 d]
            float p[DMAX];
            if (D == DMAX) {  // the exact-dimension instantiation: no per-dimension guard
#pragma unroll
                for (int d = 0; d < DMAX; ++d) p[d] = __ldg(bp + d * MPTG_BUCKET);
            } else {
#pragma unroll
                for (int d = 0; d < DMAX; ++d) p[d] = d < D ? __ldg(bp + d * MPTG_BUCKET) : 0.f;
            }
            d32 = dist32<MK, DMAX>(q, p, t.w0f, t.w1f);
            if (!(d32 == d32)) d32 = INFINITY;
        }
        knn_consider(t, qd, lane, k, radius, have, pid, d32, E, ld0, ld1, li0, li1, cnt, tau, tauf);
        bool found = false;
        while (sp > 0) {
            --sp;
            int src = sp & 31;
            int nn;
            float lb;
            if (sp < 32) { nn = __shfl_sync(0xffffffffu, s0n, src); lb = __shfl_sync(0xffffffffu, s0l, src); }
            else { nn = __shfl_sync(0xffffffffu, s1n, src); lb = __shfl_sync(0xffffffffu, s1l, src); }
            if (__fsub_rd(lb, E) <= tauf) { node = nn; found = true; break; }
        }
        if (!found) break;
    }
    int* oi = out_idx + (size_t)qi * k;
    double* od = out_d + (size_t)qi * k;
    if (lane < k) { bool v = lane < cnt; oi[lane] = v ? li0 : -1; od[lane] = v ? ld0 : INFINITY; }
    if (lane + 32 < k) { bool v = lane + 32 < cnt; oi[lane + 32] = v ? li1 : -1; od[lane + 32] = v ? ld1 : INFINITY; }
}

// ------------------------------------------------------------------ query order
// Queries are answered in the order of the tree region they fall in: the key
// is the first `bits` left/right decisions of the query's descent (10 to 16,
// about twice as many bins as queries), and a counting sort groups queries of
// the same subtree, so the warps of a block share the nodes and buckets they
// visit.
#define MPTG_QSORT_BITS 16
#define MPTG_QSORT_BINS (1 << MPTG_QSORT_BITS)
#define MPTG_QSORT_MIN 2048  // smaller batches are answered in input order

static int qsort_bits(int nq) {
    int b = 1;
    while ((1 << b) < nq && b < MPTG_QSORT_BITS) ++b;
    return std::min(MPTG_QSORT_BITS, std::max(10, b + 1));
}

__global__ void k_qkey(TreeView t, const double* __restrict__ q64, int nq, int bits, int* __restrict__ key,
                       int* __restrict__ hist) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const double* qd = q64 + (size_t)i * t.D;
    int node = 0;
    unsigned k = 0;
    int lev = 0;
    for (; lev < bits; ++lev) {
        int4 nd = __ldg(&t.nodes[node]);
        if (nd.x < 0) break;
        int right = !(__double2float_rn(qd[nd.x]) < __int_as_float(nd.z));
        k = (k << 1) | (unsigned)right;
        node = nd.y + right;
    }
    k <<= (bits - lev);
    key[i] = (int)k;
    atomicAdd(&hist[k], 1);
}

// in-place exclusive scan of the 2^bits-bin histogram: one block, bins/1024 per thread
__global__ void __launch_bounds__(1024) k_qscan(int* __restrict__ hist, int bins) {
    __shared__ int s[1024];
    const int t = threadIdx.x;
    const int per = bins / 1024;
    const int base = t * per;
    int sum = 0;
    for (int j = 0; j < per; ++j) sum += hist[base + j];
    s[t] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        int v = t >= o ? s[t - o] : 0;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    int run = t ? s[t - 1] : 0;
    for (int j = 0; j < per; ++j) {
        int c = hist[base + j];
        hist[base + j] = run;
        run += c;
    }
}

__global__ void k_qscatter(int nq, const int* __restrict__ key, int* __restrict__ hist, int* __restrict__ order) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    order[atomicAdd(&hist[key[i]], 1)] = i;
}

// ------------------------------------------------------------------ host side

// exact-size register arrays for the common dimensions keep register use
// (and so occupancy) proportional to D
#define DISPATCH_DIMS(MK, D, KERNEL, grid, block, stream, ...)                                          \
    if (D <= 2) KERNEL<MK, 2><<<grid, block, 0, stream>>>(__VA_ARGS__);                                 \
    else if (D <= 3) KERNEL<MK, 3><<<grid, block, 0, stream>>>(__VA_ARGS__);                            \
    else if (D <= 4) KERNEL<MK, 4><<<grid, block, 0, stream>>>(__VA_ARGS__);                            \
    else if (D <= 6) KERNEL<MK, 6><<<grid, block, 0, stream>>>(__VA_ARGS__);                            \
    else if (D <= 8) KERNEL<MK, 8><<<grid, block, 0, stream>>>(__VA_ARGS__);                            \
    else if (D <= 10) KERNEL<MK, 10><<<grid, block, 0, stream>>>(__VA_ARGS__);                          \
    else if (D <= 12) KERNEL<MK, 12><<<grid, block, 0, stream>>>(__VA_ARGS__);                          \
    else KERNEL<MK, 16><<<grid, block, 0, stream>>>(__VA_ARGS__);

#define DISPATCH_METRIC(metric, D, KERNEL, grid, block, stream, ...)                                      \
    do {                                                                                                \
        switch (metric) {                                                                               \
        case MPTG_METRIC_L2:                                                                            \
            DISPATCH_DIMS(MPTG_METRIC_L2, D, KERNEL, grid, block, stream, __VA_ARGS__)                  \
            break;                                                                                      \
        case MPTG_METRIC_L1:                                                                            \
            DISPATCH_DIMS(MPTG_METRIC_L1, D, KERNEL, grid, block, stream, __VA_ARGS__)                  \
            break;                                                                                      \
        case MPTG_METRIC_SO2:                                                                           \
            DISPATCH_DIMS(MPTG_METRIC_SO2, D, KERNEL, grid, block, stream, __VA_ARGS__)                 \
            break;                                                                                      \
        case MPTG_METRIC_SO3: KERNEL<MPTG_METRIC_SO3, 4><<<grid, block, 0, stream>>>(__VA_ARGS__); break; \
        case MPTG_METRIC_SE3: KERNEL<MPTG_METRIC_SE3, 8><<<grid, block, 0, stream>>>(__VA_ARGS__); break; \
        }                                                                                               \
    } while (0)

static void tree_free(mptg_tree* t) {
    void* ptrs[] = {t->states64, t->pts32, t->nodes, t->cell_lo, t->cell_hi, t->node_depth, t->bpts, t->bids,
                    t->dcnt, t->dstats, t->perm, t->perm2, t->pseg, t->pseg2, t->segA, t->segB, t->seg_box,
                    t->leaf_of, t->ovf_pts, t->ovf_leaf, t->leaf_reg, t->seg_cursor, t->qkey, t->qorder,
                    t->qhist, t->bcd, t->bci, t->kcd, t->kci};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (t->hcnt) cudaFreeHost(t->hcnt);
    delete t;
}

extern "C" {

mptg_status mptg_tree_create(mptg_ctx* ctx, mptg_metric metric, int dim, const double* weights, size_t capacity,
                             mptg_tree** out) {
    if (!ctx || !out) return MPTG_ERR_INVALID_ARG;
    *out = nullptr;
    if (metric < MPTG_METRIC_L2 || metric > MPTG_METRIC_L1)
        return mptg_fail(ctx, MPTG_ERR_UNSUPPORTED_METRIC, "unknown metric %d", (int)metric);
    if (metric == MPTG_METRIC_SO3 && dim != 4) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "SO3 needs dim 4");
    if (metric == MPTG_METRIC_SE3 && dim != 7) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "SE3 needs dim 7");
    if (dim < 1 || dim > MPTG_MAX_DIM) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "dim %d out of [1,16]", dim);
    if (capacity < 1 || capacity > (size_t)1 << 30)
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "capacity %zu out of range", capacity);
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    mptg_tree* t = new mptg_tree();
    t->ctx = ctx;
    t->metric = metric;
    t->D = dim;
    if (weights) { t->w0 = weights[0]; t->w1 = weights[1]; }
    if (metric == MPTG_METRIC_SE3 && !(t->w0 > 0 && t->w1 > 0)) {
        delete t;
        return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "SE3 weights must be positive");
    }
    t->cap = capacity;
    t->bucket_cap = (int)(capacity / 2 + 1024);
    t->node_cap = 2 * t->bucket_cap + 16;
    t->seg_cap = (int)(capacity / 16 + 1024);
    size_t N = capacity, D = dim;
    cudaError_t e = cudaSuccess;
#define ALLOC(ptr, bytes) if (e == cudaSuccess) e = cudaMalloc((void**)&(ptr), (bytes))
    ALLOC(t->states64, N * D * sizeof(double));
    ALLOC(t->pts32, N * D * sizeof(float));
    ALLOC(t->nodes, (size_t)t->node_cap * sizeof(int4));
    ALLOC(t->cell_lo, (size_t)t->node_cap * D * sizeof(float));
    ALLOC(t->cell_hi, (size_t)t->node_cap * D * sizeof(float));
    ALLOC(t->node_depth, (size_t)t->node_cap * sizeof(int));
    ALLOC(t->bpts, (size_t)t->bucket_cap * D * MPTG_BUCKET * sizeof(float));
    ALLOC(t->bids, (size_t)t->bucket_cap * MPTG_BUCKET * sizeof(int));
    ALLOC(t->dcnt, CNT_N * sizeof(int));
    ALLOC(t->dstats, 8 * sizeof(unsigned long long));
    ALLOC(t->perm, N * sizeof(int));
    ALLOC(t->perm2, N * sizeof(int));
    ALLOC(t->pseg, N * sizeof(int));
    ALLOC(t->pseg2, N * sizeof(int));
    ALLOC(t->segA, (size_t)t->seg_cap * sizeof(SegState));
    ALLOC(t->segB, (size_t)t->seg_cap * sizeof(SegState));
    ALLOC(t->seg_box, (size_t)t->seg_cap * 2 * D * sizeof(int));
    ALLOC(t->leaf_of, N * sizeof(int));
    ALLOC(t->ovf_pts, N * sizeof(int));
    ALLOC(t->ovf_leaf, N * sizeof(int));
    ALLOC(t->leaf_reg, (size_t)t->node_cap * sizeof(int));
    ALLOC(t->seg_cursor, (size_t)t->seg_cap * sizeof(int));
#undef ALLOC
    if (e == cudaSuccess) e = cudaMallocHost((void**)&t->hcnt, CNT_N * sizeof(int));
    if (e != cudaSuccess) {
        cudaGetLastError();
        tree_free(t);
        return mptg_fail(ctx, MPTG_ERR_OOM, "tree allocation failed: %s", cudaGetErrorString(e));
    }
    // root = empty leaf on bucket 0; root cell = the metric's domain
    int hc[CNT_N] = {1, 1, 0, 0, 0, 0, 0, 0, 0};
    int4 root = make_int4(-1, 0, 0, 0);
    std::vector<float> lo(D), hi(D);
    for (size_t d = 0; d < D; ++d) {
        lo[d] = -INFINITY; hi[d] = INFINITY;
        if (metric == MPTG_METRIC_SO2) { lo[d] = -PI_F; hi[d] = PI_F; }
        if ((metric == MPTG_METRIC_SO3 || metric == MPTG_METRIC_SE3) && d < 4) { lo[d] = -1.f; hi[d] = 1.f; }
    }
    // -pi/pi as floats may round inward of the double range: widen by one ulp
    for (size_t d = 0; d < D; ++d) {
        if (metric == MPTG_METRIC_SO2) { lo[d] = nextafterf(lo[d], -INFINITY); hi[d] = nextafterf(hi[d], INFINITY); }
    }
    int zero = 0;
    e = cudaMemcpy(t->dcnt, hc, sizeof(hc), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->nodes, &root, sizeof(root), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->cell_lo, lo.data(), D * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->cell_hi, hi.data(), D * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->node_depth, &zero, sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(t->dstats, 0, 8 * sizeof(unsigned long long));
    if (e != cudaSuccess) {
        tree_free(t);
        return mptg_fail(ctx, MPTG_ERR_CUDA, "tree init failed: %s", cudaGetErrorString(e));
    }
    *out = t;
    return MPTG_OK;
}

mptg_status mptg_tree_destroy(mptg_tree* t) {
    if (!t) return MPTG_ERR_INVALID_ARG;
    cudaDeviceSynchronize();
    tree_free(t);
    return MPTG_OK;
}

mptg_status mptg_tree_size(mptg_tree* t, size_t* n) {
    if (!t || !n) return MPTG_ERR_INVALID_ARG;
    *n = t->n;
    return MPTG_OK;
}

mptg_status mptg_tree_set_strategy(mptg_tree* t, int strategy) {
    if (!t) return MPTG_ERR_INVALID_ARG;
    if (strategy < MPTG_NN_AUTO || strategy > MPTG_NN_EXHAUSTIVE)
        return mptg_fail(t->ctx, MPTG_ERR_INVALID_ARG, "unknown nearest-neighbour strategy %d", strategy);
    t->strategy = strategy;
    return MPTG_OK;
}

// Back to the empty tree of mptg_tree_create, keeping every allocation: the
// root becomes an empty leaf on bucket 0 again.  The root cell (the metric's
// domain) is never written by inserts or rebuilds, so it stays as created.
mptg_status mptg_tree_clear(mptg_tree* t, void* stream) {
    if (!t) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = t->ctx;
    cudaStream_t s = (cudaStream_t)stream;
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int hc[CNT_N] = {1, 1, 0, 0, 0, 0, 0, 0, 0};
    const int4 root = make_int4(-1, 0, 0, 0);
    const int zero = 0;
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(t->dcnt, hc, sizeof(hc), cudaMemcpyHostToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(t->nodes, &root, sizeof(root), cudaMemcpyHostToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(t->node_depth, &zero, sizeof(int), cudaMemcpyHostToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    t->n = 0;
    return MPTG_OK;
}

static mptg_status read_counters(mptg_tree* t, cudaStream_t s) {
    mptg_ctx* ctx = t->ctx;
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(t->hcnt, t->dcnt, CNT_N * sizeof(int), cudaMemcpyDeviceToHost, s));
    MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return MPTG_OK;
}

// level-synchronous build of the `nseg` segments in segA over positions
// [0, total) of perm/pseg.  nseg = total = -1: the first level runs on the
// counts k_append left on the device (the overflowing leaves, see
// pending_nreg), in grids of bound_seg / bound_total threads, and the host
// learns the counts with that level's counters.
static mptg_status build_levels(mptg_tree* t, cudaStream_t s, int nseg, int total, int bound_seg = 0,
                                int bound_total = 0) {
    mptg_ctx* ctx = t->ctx;
    const int D = t->D;
    SegState* cur = t->segA;
    SegState* prev = t->segB;
    int* perm = t->perm; int* perm2 = t->perm2; int* pseg = t->pseg; int* pseg2 = t->pseg2;
    const unsigned tb = 256;
    mptg_status st;
    for (int level = 0; nseg != 0 && level < 4 * MPTG_MAX_DEPTH; ++level) {
        const bool pending = nseg < 0;
        const int gs = pending ? bound_seg : nseg, gt = pending ? bound_total : total;
        MPTG_CUDA_TRY(ctx, cudaMemsetAsync(t->dcnt + CNT_NSEG_NEXT, 0, sizeof(int), s));
        if (gs > 0) {
            k_seg_a<<<mptg_blocks(gs, 128), 128, 0, s>>>(cur, nseg, prev, t->nodes, t->dcnt, t->bucket_cap,
                                                         t->seg_box, D, t->seg_cap);
            k_seg_b<<<mptg_blocks(gt, tb), tb, 0, s>>>(cur, perm, pseg, pseg2, total, t->pts32, D, t->bpts,
                                                       t->bids, t->seg_box, t->dcnt, t->seg_cap);
            k_seg_c<<<mptg_blocks(gs, 128), 128, 0, s>>>(cur, nseg, prev, t->nodes, t->cell_lo, t->cell_hi,
                                                         t->node_depth, t->dcnt, t->node_cap, t->seg_cap,
                                                         t->seg_box, D, t->metric, (float)t->w0, (float)t->w1);
            k_seg_d<<<mptg_blocks(gt, tb), tb, 0, s>>>(cur, perm, pseg, perm2, pseg2, total, t->pts32, D, t->dcnt,
                                                       t->seg_cap);
            ctx->launches += 4;
        }
        st = read_counters(t, s);
        if (st) return st;
        if (pending) {
            const int r = t->hcnt[CNT_NREG];
            total = r <= t->seg_cap && r > 0 ? MPTG_BUCKET * r + t->hcnt[CNT_OVF] : 0;
        }
        nseg = t->hcnt[CNT_NSEG_NEXT];
        if (nseg > t->seg_cap || (t->hcnt[CNT_ERR] & MPTG_DEVERR_CAPACITY))
            return mptg_fail(ctx, MPTG_ERR_CAPACITY, "kd-tree build ran out of node/segment capacity");
        // next level: the children just written to `prev` become current
        SegState* tmp = cur; cur = prev; prev = tmp;
        int* tp = perm; perm = perm2; perm2 = tp;
        tp = pseg; pseg = pseg2; pseg2 = tp;
    }
    if (nseg > 0) return mptg_fail(ctx, MPTG_ERR_CAPACITY, "kd-tree build did not converge");
    return MPTG_OK;
}

__global__ void k_rebuild_init(int n, int* __restrict__ perm, int* __restrict__ pseg) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    perm[i] = i;
    pseg[i] = 0;
}

// drop every node and bucket and build the tree again from all t->n points
static mptg_status rebuild_all(mptg_tree* t, cudaStream_t s) {
    mptg_ctx* ctx = t->ctx;
    int n = (int)t->n;
    // node 0 stays the root (its cell is the metric's domain); buckets restart at 0
    int hc[3] = {1, 0, 0};
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(t->dcnt + CNT_NODES, hc, 2 * sizeof(int), cudaMemcpyHostToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(t->dcnt + CNT_MAXDEPTH, hc + 2, sizeof(int), cudaMemcpyHostToDevice, s));
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(t->dcnt + CNT_ERR, 0, sizeof(int), s));
    k_rebuild_init<<<mptg_blocks(n, 256), 256, 0, s>>>(n, t->perm, t->pseg);
    MPTG_LAUNCHED(ctx);
    SegState root;
    memset(&root, 0, sizeof(root));
    root.node = 0; root.start = 0; root.count = n; root.depth = 0; root.parent = -1;
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(t->segA, &root, sizeof(root), cudaMemcpyHostToDevice, s));
    mptg_status st = build_levels(t, s, 1, n);
    if (st) return st;
    t->rebuilds += 1;
    return read_counters(t, s);
}

mptg_status mptg_tree_insert(mptg_tree* t, const double* states, size_t n, void* stream) {
    if (!t) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = t->ctx;
    if (n == 0) return MPTG_OK;
    if (!states) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "null states");
    if (t->n + n > t->cap) return mptg_fail(ctx, MPTG_ERR_CAPACITY, "tree capacity %zu exceeded", t->cap);
    cudaStream_t s = (cudaStream_t)stream;
    const int D = t->D;
    const int first = (int)t->n;
    const int nn = (int)n;
    MPTG_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(t->states64 + (size_t)first * D, states, n * D * sizeof(double),
                                       cudaMemcpyDefault, s));
    // clear per-insert counters and the error word
    MPTG_CUDA_TRY(ctx, cudaMemsetAsync(t->dcnt + CNT_ERR, 0, 4 * sizeof(int), s));
    k_convert<<<mptg_blocks(n, 256), 256, 0, s>>>(t->states64 + (size_t)first * D, t->pts32 + (size_t)first * D, nn,
                                                  D, t->metric, t->dcnt);
    MPTG_LAUNCHED(ctx);
    // one host round trip: k_append does nothing when k_convert flagged a bad
    // state, and the flag is read together with the overflow counts
    k_locate<<<mptg_blocks(n, 256), 256, 0, s>>>(t->nodes, t->pts32, first, nn, D, t->leaf_of);
    k_append<<<mptg_blocks(n, 256), 256, 0, s>>>(t->nodes, t->pts32, t->bpts, t->bids, first, nn, D, t->leaf_of,
                                                 t->dcnt, t->ovf_pts, t->ovf_leaf, t->leaf_reg);
    ctx->launches += 2;
    mptg_status st;
    if (nn <= MPTG_INSERT_PENDING_MAX) {
        // small batches (a planner's wavefront): the overflow segments and the
        // first builder level are queued on the counts k_append leaves on the
        // device, so the first counter read comes after that level
        const int rb = std::min(nn, t->seg_cap);
        k_ovf_segs<<<mptg_blocks(rb, 128), 128, 0, s>>>(t->nodes, t->bids, t->node_depth, -1, t->ovf_leaf, t->dcnt,
                                                        t->segA, t->perm, t->pseg, t->seg_cursor, t->seg_cap);
        k_ovf_scatter<<<mptg_blocks(nn, 256), 256, 0, s>>>(-1, first, t->ovf_pts, t->leaf_of, t->leaf_reg, t->segA,
                                                           t->seg_cursor, t->perm, t->pseg, t->dcnt, t->seg_cap);
        ctx->launches += 2;
        st = build_levels(t, s, -1, -1, rb, MPTG_BUCKET * rb + nn);
        if (st) return st;
        if (t->hcnt[CNT_ERR] & MPTG_DEVERR_BAD_STATE)
            return mptg_fail(ctx, MPTG_ERR_INVALID_ARG,
                             "invalid state (NaN/inf, SO2 angle outside [-pi,pi], or non-unit quaternion)");
    } else {
        st = read_counters(t, s);
        if (st) return st;
        if (t->hcnt[CNT_ERR] & MPTG_DEVERR_BAD_STATE)
            return mptg_fail(ctx, MPTG_ERR_INVALID_ARG,
                             "invalid state (NaN/inf, SO2 angle outside [-pi,pi], or non-unit quaternion)");
        int nreg = t->hcnt[CNT_NREG];
        int novf = t->hcnt[CNT_OVF];
        if (nreg > 0) {
            if (nreg > t->seg_cap) return mptg_fail(ctx, MPTG_ERR_CAPACITY, "too many overflowing leaves");
            k_ovf_segs<<<mptg_blocks(nreg, 128), 128, 0, s>>>(t->nodes, t->bids, t->node_depth, nreg, t->ovf_leaf,
                                                              t->dcnt, t->segA, t->perm, t->pseg, t->seg_cursor,
                                                              t->seg_cap);
            k_ovf_scatter<<<mptg_blocks(novf, 256), 256, 0, s>>>(novf, first, t->ovf_pts, t->leaf_of, t->leaf_reg,
                                                                 t->segA, t->seg_cursor, t->perm, t->pseg, t->dcnt,
                                                                 t->seg_cap);
            ctx->launches += 2;
            st = build_levels(t, s, nreg, MPTG_BUCKET * nreg + novf);
            if (st) return st;
        }
    }
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    // hcnt is current: read after k_append, or after the builder's last level
    t->n += n;
    // Leaf splits only see the points of one leaf, so a tree that keeps
    // growing at one frontier (a planner extending a corridor) degenerates
    // into a chain.  When any leaf gets deeper than MPTG_REBUILD_DEPTH (or hit
    // the depth limit) the whole tree is rebuilt from all its points.
    if (t->hcnt[CNT_MAXDEPTH] > MPTG_REBUILD_DEPTH || (t->hcnt[CNT_ERR] & MPTG_DEVERR_DEPTH)) {
        st = rebuild_all(t, s);
        if (st) return st;
    }
    int err = t->hcnt[CNT_ERR];
    if (err & MPTG_DEVERR_CAPACITY) return mptg_fail(ctx, MPTG_ERR_CAPACITY, "kd-tree node/bucket capacity exceeded");
    if (err & MPTG_DEVERR_DEPTH) return mptg_fail(ctx, MPTG_ERR_CAPACITY, "kd-tree depth limit reached");
    return MPTG_OK;
}

mptg_status mptg_tree_states(mptg_tree* t, size_t first, size_t n, double* out, void* stream) {
    if (!t || (!out && n)) return MPTG_ERR_INVALID_ARG;
    if (first + n > t->n) return mptg_fail(t->ctx, MPTG_ERR_INVALID_ARG, "range beyond tree size");
    cudaStream_t s = (cudaStream_t)stream;
    MPTG_CUDA_TRY(t->ctx, cudaMemcpyAsync(out, t->states64 + first * t->D, n * t->D * sizeof(double),
                                          cudaMemcpyDefault, s));
    if (!mptg_is_device_ptr(out)) MPTG_CUDA_TRY(t->ctx, cudaStreamSynchronize(s));
    return MPTG_OK;
}

mptg_status mptg_tree_counters(mptg_tree* t, uint64_t out[5], int reset) {
    if (!t || !out) return MPTG_ERR_INVALID_ARG;
    unsigned long long h[8];
    MPTG_CUDA_TRY(t->ctx, cudaDeviceSynchronize());
    MPTG_CUDA_TRY(t->ctx, cudaMemcpy(h, t->dstats, sizeof(h), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 5; ++i) out[i] = h[i];
    if (reset) MPTG_CUDA_TRY(t->ctx, cudaMemset(t->dstats, 0, sizeof(h)));
    return MPTG_OK;
}

const double* mptg_tree_states_dev(const mptg_tree* t) { return t->states64; }

// The tiled exhaustive sweep beats the kd-tree where the tree must visit a
// large share of its points: Lp / SO(2)^n spaces of six or more dimensions.
// Measured on SO(2)^10 (GB300): the sweep evaluates ~4.3e11 (query, point)
// pairs/s, the tree ~0.1-2 us per query; the sweep is chosen while
// points x queries x dimensions stays below MPTG_TILED_MAX_WORK.  Rotation
// metrics keep the tree (it prunes well there).
#define MPTG_TILED_MAX_WORK 2.5e11
static bool tree_use_tiled(const mptg_tree* t, int nq) {
    if (t->strategy == MPTG_NN_KDTREE || t->n == 0) return false;
    if (t->strategy == MPTG_NN_EXHAUSTIVE) return true;
    const bool lp = t->metric == MPTG_METRIC_L2 || t->metric == MPTG_METRIC_L1 || t->metric == MPTG_METRIC_SO2;
    return lp && t->D >= 6 && (double)t->n * nq * t->D <= MPTG_TILED_MAX_WORK;
}

// internal: launch the 1-NN search on device buffers (used by the planner too)
mptg_status mptg_tree_nearest_dev(mptg_tree* t, const double* dq, int nq, int* didx, double* dd, cudaStream_t s,
                                  bool count) {
    if (nq <= 0) return MPTG_OK;
    mptg_ctx* ctx = t->ctx;
    TreeView v = view_of(t);
    if (!count) v.stats = nullptr;
    if (tree_use_tiled(t, nq)) {
        // enough (query tile, point split) blocks to fill the GPU four times over
        const int qblocks = (int)mptg_blocks((size_t)nq, BRUTE_TILE);
        const int maxsplit = std::max(1, (int)((t->n + BRUTE_TILE - 1) / BRUTE_TILE));
        const int nsplit = std::min(maxsplit, std::max(1, (4 * 152 + qblocks - 1) / qblocks));
        const int chunk = (int)((t->n + nsplit - 1) / nsplit);
        const size_t need = (size_t)nsplit * BRUTE_K * nq;
        if (need > t->bcap) {
            MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
            cudaFree(t->bcd);
            cudaFree(t->bci);
            t->bcd = nullptr;
            t->bci = nullptr;
            t->bcap = 0;
            const size_t cap = need + need / 2;
            MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&t->bcd, cap * sizeof(float)));
            MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&t->bci, cap * sizeof(int)));
            t->bcap = cap;
        }
        dim3 grid(qblocks, nsplit);
        DISPATCH_METRIC(t->metric, t->D, k_nearest_tiled, grid, BRUTE_TILE, s, v, dq, nq, chunk, t->bcd, t->bci);
        DISPATCH_METRIC(t->metric, t->D, k_nearest_tiled_merge, mptg_blocks((size_t)nq * 32, 256), 256, s, v, dq, nq,
                        nsplit, t->bcd, t->bci, didx, dd);
        ctx->launches += 2;
        return MPTG_OK;
    }
    const int* order = nullptr;
    if (nq >= MPTG_QSORT_MIN && t->n > 4 * MPTG_BUCKET) {
        if ((size_t)nq > t->qcap) {
            cudaStreamSynchronize(s);
            cudaFree(t->qkey);
            cudaFree(t->qorder);
            t->qkey = t->qorder = nullptr;
            t->qcap = 0;
            if (!t->qhist) MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&t->qhist, (MPTG_QSORT_BINS + 1) * sizeof(int)));
            MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&t->qkey, (size_t)nq * sizeof(int)));
            MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&t->qorder, (size_t)nq * sizeof(int)));
            t->qcap = (size_t)nq;
        }
        const int bits = qsort_bits(nq);
        MPTG_CUDA_TRY(ctx, cudaMemsetAsync(t->qhist, 0, ((size_t)1 << bits) * sizeof(int), s));
        k_qkey<<<mptg_blocks(nq, 256), 256, 0, s>>>(v, dq, nq, bits, t->qkey, t->qhist);
        k_qscan<<<1, 1024, 0, s>>>(t->qhist, 1 << bits);
        k_qscatter<<<mptg_blocks(nq, 256), 256, 0, s>>>(nq, t->qkey, t->qhist, t->qorder);
        ctx->launches += 3;
        order = t->qorder;
    }
    // Packets pay off where neighbouring queries' search balls overlap (low
    // dimension); in SO(2)^10 the union of 32 balls is ~6x one ball, so
    // higher dimensions keep one query per warp (still in sorted order).
    // Below 32k queries a packet launch has too few warps to fill the GPU.
    if (order && t->D <= 3 && nq >= 32768) {
        // 32 sorted queries per warp
        unsigned grid = mptg_blocks((size_t)nq, 256);
        DISPATCH_METRIC(t->metric, t->D, k_nearest_packet, grid, 256, s, v, dq, nq, order, didx, dd);
    } else {
        // more queries than resident warps (4 blocks of 8 per SM): a resident
        // grid taking queries from a counter (qhist's last slot)
        unsigned grid = mptg_blocks((size_t)nq * 32, 256);
        int* qnext = nullptr;
        const unsigned resident = 4u * (unsigned)ctx->sms;
        if (grid > 2 * resident) {
            if (!t->qhist) MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&t->qhist, (MPTG_QSORT_BINS + 1) * sizeof(int)));
            qnext = t->qhist + MPTG_QSORT_BINS;
            MPTG_CUDA_TRY(ctx, cudaMemsetAsync(qnext, 0, sizeof(int), s));
            grid = resident;
        }
        DISPATCH_METRIC(t->metric, t->D, k_nearest, grid, 256, s, v, dq, nq, order, didx, dd, qnext);
    }
    MPTG_LAUNCHED(ctx);
    return MPTG_OK;
}

mptg_status mptg_nearest(mptg_tree* t, const double* q, size_t nq, int32_t* idx, double* dist, void* stream) {
    if (!t) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = t->ctx;
    if (nq == 0) return MPTG_OK;
    if (!q || !idx || !dist) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "null buffer");
    if (nq > (size_t)INT32_MAX / 32) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "too many queries");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf bq, bi, bd;
    mptg_status st;
    if ((st = mptg_stage_in(ctx, q, nq * t->D * sizeof(double), s, &bq))) return st;
    if ((st = mptg_stage_out_alloc(ctx, idx, nq * sizeof(int32_t), s, &bi))) return st;
    if ((st = mptg_stage_out_alloc(ctx, dist, nq * sizeof(double), s, &bd))) return st;
    mptg_tree_nearest_dev(t, (const double*)bq.dptr, (int)nq, (int*)bi.dptr, (double*)bd.dptr, s, true);
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    DevBuf outs[2] = {bi, bd};
    return mptg_stage_finish(ctx, s, outs, 2, &bq, 1);
}

mptg_status mptg_nearest_linear(mptg_tree* t, const double* q, size_t nq, int32_t* idx, double* dist,
                                void* stream) {
    if (!t) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = t->ctx;
    if (nq == 0) return MPTG_OK;
    if (!q || !idx || !dist) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf bq, bi, bd;
    mptg_status st;
    if ((st = mptg_stage_in(ctx, q, nq * t->D * sizeof(double), s, &bq))) return st;
    if ((st = mptg_stage_out_alloc(ctx, idx, nq * sizeof(int32_t), s, &bi))) return st;
    if ((st = mptg_stage_out_alloc(ctx, dist, nq * sizeof(double), s, &bd))) return st;
    TreeView v = view_of(t);
    unsigned grid = mptg_blocks(nq * 32, 256);
    DISPATCH_METRIC(t->metric, t->D, k_nearest_linear, grid, 256, s, v, (const double*)bq.dptr, (int)nq,
                    (int*)bi.dptr, (double*)bd.dptr);
    MPTG_LAUNCHED(ctx);
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    DevBuf outs[2] = {bi, bd};
    return mptg_stage_finish(ctx, s, outs, 2, &bq, 1);
}

// k nearest on device buffers: the tree walk, or the exhaustive sweep with
// the points split over blocks while the queries alone give fewer than two
// blocks per SM (at least 2048 points per split), then the merge of the lists
static mptg_status knn_launch(mptg_tree* t, const TreeView& v, const double* dq, int nq, int k, double radius,
                              int* didx, double* dd, cudaStream_t s) {
    mptg_ctx* ctx = t->ctx;
    if (!tree_use_tiled(t, nq)) {
        unsigned grid = mptg_blocks((size_t)nq * 32, 256);
        DISPATCH_METRIC(t->metric, t->D, k_nearest_k, grid, 256, s, v, dq, nq, k, radius, didx, dd);
        MPTG_LAUNCHED(ctx);
        return MPTG_OK;
    }
    const int qblocks = (int)mptg_blocks((size_t)nq, 8);
    const int maxsplit = std::max(1, (int)(t->n / 2048));
    const int nsplit = std::min(maxsplit, std::max(1, (2 * ctx->sms + qblocks - 1) / qblocks));
    const int chunk = (int)((t->n + nsplit - 1) / nsplit);
    if (nsplit == 1) {
        DISPATCH_METRIC(t->metric, t->D, k_nearest_k_tiled, dim3(qblocks, 1), 256, s, v, dq, nq, k, radius, chunk,
                        didx, dd);
        MPTG_LAUNCHED(ctx);
        return MPTG_OK;
    }
    const size_t need = (size_t)nsplit * nq * k;
    if (need > t->kcap) {
        MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        cudaFree(t->kcd);
        cudaFree(t->kci);
        t->kcd = nullptr;
        t->kci = nullptr;
        t->kcap = 0;
        const size_t cap = need + need / 2;
        MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&t->kcd, cap * sizeof(double)));
        MPTG_CUDA_TRY(ctx, cudaMalloc((void**)&t->kci, cap * sizeof(int)));
        t->kcap = cap;
    }
    DISPATCH_METRIC(t->metric, t->D, k_nearest_k_tiled, dim3(qblocks, nsplit), 256, s, v, dq, nq, k, radius, chunk,
                    t->kci, t->kcd);
    k_nearest_k_merge<<<mptg_blocks((size_t)nq * 32, 256), 256, 0, s>>>(nq, k, radius, nsplit, t->kcd, t->kci, didx,
                                                                         dd);
    ctx->launches += 2;
    return MPTG_OK;
}

mptg_status mptg_tree_nearest_k_dev(mptg_tree* t, const double* dq, int nq, int k, int* didx, double* dd,
                                    cudaStream_t s) {
    if (nq <= 0) return MPTG_OK;
    if (k < 1 || k > 64) return mptg_fail(t->ctx, MPTG_ERR_INVALID_ARG, "k=%d outside [1,64]", k);
    TreeView v = view_of(t);
    v.stats = nullptr;
    return knn_launch(t, v, dq, nq, k, (double)INFINITY, didx, dd, s);
}

mptg_status mptg_nearest_k(mptg_tree* t, const double* q, size_t nq, int k, double r, int32_t* idx, double* dist,
                           void* stream) {
    if (!t) return MPTG_ERR_INVALID_ARG;
    mptg_ctx* ctx = t->ctx;
    if (k < 1 || k > 64) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "k=%d outside [1,64]", k);
    if (nq == 0) return MPTG_OK;
    if (!q || !idx || !dist) return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "null buffer");
    if (!(r > 0)) r = INFINITY;
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf bq, bi, bd;
    mptg_status st;
    if ((st = mptg_stage_in(ctx, q, nq * t->D * sizeof(double), s, &bq))) return st;
    if ((st = mptg_stage_out_alloc(ctx, idx, nq * k * sizeof(int32_t), s, &bi))) return st;
    if ((st = mptg_stage_out_alloc(ctx, dist, nq * k * sizeof(double), s, &bd))) return st;
    TreeView v = view_of(t);
    if ((st = knn_launch(t, v, (const double*)bq.dptr, (int)nq, k, r, (int*)bi.dptr, (double*)bd.dptr, s)))
        return st;
    MPTG_CUDA_TRY(ctx, cudaGetLastError());
    DevBuf outs[2] = {bi, bd};
    return mptg_stage_finish(ctx, s, outs, 2, &bq, 1);
}

}  // extern "C"
