/*
 * mptg.h - C ABI of the GB300-native MPT planner hot path.
 *
 * Plain C: pointers, sizes and opaque handles only.  Every call returns an
 * mptg_status; no C++ exception crosses this boundary.  Buffers are owned by
 * the caller and may live in host memory (pageable or pinned) or in device
 * memory of the context's GPU: the library inspects each pointer.  A call
 * whose buffers are all in device memory is asynchronous on `stream`
 * (a cudaStream_t passed as void*, NULL = the legacy default stream); a call
 * that touches host memory copies through a staging buffer and returns after
 * the results are in the caller's buffer.
 *
 * Each entry point names the reference interface it replaces (paths inside
 * the MPT project, file:line).
 */
#ifndef MPTG_H
#define MPTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MPTG_OK = 0,
    MPTG_ERR_INVALID_ARG = 1,
    MPTG_ERR_OOM = 2,
    MPTG_ERR_CUDA = 3,
    MPTG_ERR_TIMEOUT = 4,
    MPTG_ERR_QUEUE_OVERFLOW = 5,
    MPTG_ERR_UNSUPPORTED_METRIC = 6,
    MPTG_ERR_CAPACITY = 7,
    MPTG_ERR_NO_START = 8,
    MPTG_ERR_ALREADY_SOLVING = 9
} mptg_status;

/* Metric spaces (nigh::metric::Space<T, M> as used through
 * src/mpt/lp_space.hpp, so2_space.hpp, so3_space.hpp, se3_space.hpp):
 *  L2   sqrt(sum (a_i-b_i)^2)                      LPSpace<double, D, 2>
 *  SO2  sum_i min(|a_i-b_i|, 2pi-|a_i-b_i|)        SO2LPSpace<double, D, 1>
 *  SO3  acos(|a.b|), a,b unit quaternions (x,y,z,w)  SO3Space<double>
 *  SE3  w0*acos(|qa.qb|) + w1*|pa-pb|, state (qx,qy,qz,qw,px,py,pz)
 *                                                  SE3Space<double, w0, w1>
 *  L1   sum |a_i-b_i|                              L1Space<double, D> */
typedef enum {
    MPTG_METRIC_L2 = 0,
    MPTG_METRIC_SO2 = 1,
    MPTG_METRIC_SO3 = 2,
    MPTG_METRIC_SE3 = 3,
    MPTG_METRIC_L1 = 4
} mptg_metric;

typedef struct mptg_ctx mptg_ctx;
typedef struct mptg_tree mptg_tree;
typedef struct mptg_scene mptg_scene;

/* ---- context ------------------------------------------------------- */
/* A context on one CUDA device: its streams, scratch and error message (no
 * reference counterpart: the reference runs on the host's threads). */
mptg_status mptg_create(mptg_ctx** ctx, int device);
mptg_status mptg_destroy(mptg_ctx* ctx);
/* Message of the last failed call on this context (static storage): the text
 * the reference puts in its exceptions, e.g. "there are no valid initial
 * states" (src/mpt/impl/prrt/prrt.hpp:197-198); no exception crosses the ABI. */
const char* mptg_last_error(mptg_ctx* ctx);
/* Number of kernels this library has launched on the context (for audits;
 * no reference counterpart). */
uint64_t mptg_kernel_launches(mptg_ctx* ctx);

/* ---- nearest-neighbour tree ----------------------------------------
 * Replaces nigh::Nigh<Node*, Space, NodeKey, Concurrency, KDTreeBatch<>>
 * as constructed in src/mpt/impl/prrt/prrt.hpp:121-122 and
 * src/mpt/impl/prrt_star/prrt_star.hpp:182-183. */
mptg_status mptg_tree_create(mptg_ctx* ctx, mptg_metric metric, int dim, const double* weights,
                             size_t capacity, mptg_tree** tree);
/* the Nigh object's lifetime (a member of PRRT, src/mpt/impl/prrt/prrt.hpp:121-122) */
mptg_status mptg_tree_destroy(mptg_tree* tree);
/* nigh insert (src/mpt/impl/prrt/prrt.hpp:186,447): appends n states
 * (row-major n x dim doubles); their ids are size()..size()+n-1. */
mptg_status mptg_tree_insert(mptg_tree* tree, const double* states, size_t n, void* stream);
/* nigh size() (PRRT::size, src/mpt/impl/prrt/prrt.hpp:177-179) */
mptg_status mptg_tree_size(mptg_tree* tree, size_t* n);
/* Search strategy, as the reference picks a nigh strategy per planner
 * (src/mpt/impl/nearest_strategy.hpp:44-72; auto = nigh::auto_strategy_t).
 * KDTREE: the bucketed kd-tree walk.  EXHAUSTIVE: every stored point, staged
 * through shared memory (nigh::Linear's answer).  AUTO uses EXHAUSTIVE for
 * L2, L1 and SO2 spaces of six or more dimensions while points x queries x
 * dim <= 2.5e11, where the tree must visit a large share of the points.
 * Every strategy returns the same exact ids and distances. */
typedef enum { MPTG_NN_AUTO = 0, MPTG_NN_KDTREE = 1, MPTG_NN_EXHAUSTIVE = 2 } mptg_nn_strategy;
mptg_status mptg_tree_set_strategy(mptg_tree* tree, int strategy);
/* Remove every state, keeping the tree's allocations (no reference
 * counterpart: a reference planner is rebuilt for each query). */
mptg_status mptg_tree_clear(mptg_tree* tree, void* stream);
/* Copy states [first, first+n) out of the tree (row-major doubles); the node
 * states PRRT::visitGraph reads (src/mpt/impl/prrt/prrt.hpp:300-316). */
mptg_status mptg_tree_states(mptg_tree* tree, size_t first, size_t n, double* out, void* stream);
/* nigh nearest(q) (src/mpt/impl/prrt/prrt.hpp:406-409): for each of nq
 * queries the id of the nearest state and its exact FP64 distance; ties go to
 * the lowest id.  idx = -1 and dist = +inf when the tree is empty. */
mptg_status mptg_nearest(mptg_tree* tree, const double* queries, size_t nq, int32_t* idx_out,
                         double* dist_out, void* stream);
/* nigh nearest(nbh, q, k, r) (src/mpt/impl/rrg_rewire_neighbors.hpp:64-67,
 * 124-128): the k nearest states within distance r (r <= 0 or inf = no
 * limit), sorted by (distance, id); unused slots hold id -1 and +inf.
 * k <= 64. */
mptg_status mptg_nearest_k(mptg_tree* tree, const double* queries, size_t nq, int k, double r,
                           int32_t* idx_out, double* dist_out, void* stream);
/* Brute-force exact 1-NN over every stored state (same contract as
 * mptg_nearest); the reference nigh::Linear strategy (src/mpt/impl/
 * nearest_strategy.hpp:44-72). */
mptg_status mptg_nearest_linear(mptg_tree* tree, const double* queries, size_t nq, int32_t* idx_out,
                                double* dist_out, void* stream);

/* Exact 1-NN among n caller-owned points that allocates no device memory.
 * It has no counterpart in the reference.  It is for callers that cannot
 * allocate GPU memory while they run: a real-time control loop that must not
 * call cudaMalloc after start-up (the call can block and synchronise the
 * device), or a plugin inside a framework that owns all device memory through
 * its own allocator.  Same results as mptg_nearest_linear on a tree holding
 * the same points (ids are row indices; lowest id on ties; -1 and +inf when
 * n == 0).  points, queries, idx_out and dist_out must be device memory of
 * the context's GPU (or managed memory); host buffers and buffers of another
 * GPU return MPTG_ERR_INVALID_ARG.  weights may be NULL (1, 1) or host memory.
 * Working memory is one static device array built into the library
 * (4 MiB + 256 bytes on every GPU that loads the library, kept until the
 * process exits), so n is at most 65,536 points of at most 16 dimensions;
 * a larger n returns MPTG_ERR_INVALID_ARG.  A device's first call looks up
 * the array's device address with cudaGetSymbolAddress and caches it: make
 * that first call before any stream capture.  A cudaDeviceReset after it
 * leaves that cached address stale: do not call the entry point again in the
 * same process after a device reset.  All calls share the array and
 * it keeps the last call's contents (each call clears what must start at
 * zero), so calls whose work overlaps on the GPU race: order them on one
 * stream.  Invalid points (NaN, SO2 angles outside [-pi, pi], non-unit
 * quaternions) give id -1 and NaN for every query of that call. */
mptg_status mptg_nearest_linear_noalloc(mptg_ctx* ctx, mptg_metric metric, int dim, const double* weights,
                                        const double* points, size_t n, const double* queries, size_t nq,
                                        int32_t* idx_out, double* dist_out, void* stream);

/* Per-tree search counters accumulated since the last reset (no reference
 * counterpart: the roofline's algorithmic-byte inputs):
 * [0] queries, [1] internal nodes visited, [2] leaves visited,
 * [3] points evaluated in FP32, [4] candidates re-ranked in FP64. */
mptg_status mptg_tree_counters(mptg_tree* tree, uint64_t out[5], int reset);

/* ---- scenes and validity ------------------------------------------- */
typedef enum { MPTG_SCENE_GRID = 0, MPTG_SCENE_PLANAR_ARM = 1, MPTG_SCENE_RIGID_MESH = 2 } mptg_scene_kind;

/* Scene descriptor (all arrays are host memory, copied at creation).
 *  GRID:        width x height uint8 cells, non-zero = obstacle, row-major by y;
 *               state (x, y), L2 metric; valid(q) per
 *               demo/png_2d_scenario.hpp:104-110 with out-of-grid = invalid.
 *  PLANAR_ARM:  nlinks links of link_len[i], base at the origin, discs
 *               (cx, cy, r) x ndiscs; state = nlinks joint angles, SO2 metric;
 *               valid(q) per demo/link_manipulator_scenario.hpp:99-116 plus,
 *               when self_collision != 0, no two non-adjacent links touching.
 *  RIGID_MESH:  robot and environment triangle soups (9 doubles per
 *               triangle); state (qx,qy,qz,qw,px,py,pz), SE3 metric with
 *               weights w0 (rotation) and w1 (translation); valid(q) iff the
 *               robot placed at T(q) intersects no environment triangle
 *               (demo/se3_rigid_body_scenario.hpp:282-312). */
typedef struct {
    int kind;
    /* grid */
    const uint8_t* grid; int width; int height;
    /* planar arm */
    int nlinks; const double* link_len; int ndiscs; const double* discs;
    double robot_radius; int self_collision;
    /* rigid mesh */
    int64_t nrobot; const double* robot_tris; int64_t nenv; const double* env_tris;
    double w_rot; double w_pos;
} mptg_scene_desc;

/* The Scenario's collision world (the three demo scenarios above) copied to
 * the device; a planner's copy of its Scenario (src/mpt/impl/prrt/prrt.hpp:326). */
mptg_status mptg_scene_create(mptg_ctx* ctx, const mptg_scene_desc* desc, mptg_scene** scene);
mptg_status mptg_scene_destroy(mptg_scene* scene);
/* State dimension and metric of a scene's configuration space (Scenario::space(),
 * its Space's dimensions() and distance). */
mptg_status mptg_scene_space(mptg_scene* scene, int* dim, int* metric, double weights[2]);

/* Scenario::valid(q) batched (src/mpt/impl/prrt/prrt.hpp:439). */
mptg_status mptg_valid_states(mptg_scene* scene, const double* states, size_t n, uint8_t* out,
                              void* stream);

/* Scenario::link(a, b) through DiscreteMotionValidator
 * (src/mpt/discrete_motion_validator.hpp:71-130) batched: out[i] = 1 iff
 * valid(b_i) and every interpolate(a_i, b_i, j/steps), 1 <= j < steps, is
 * valid, where steps = ceil(m(a_i, b_i) / step).  resolution 0: m is the
 * space metric (the reference DMV); resolution 1: m is the largest wrapped
 * joint difference (planar-arm edges at a maximum joint step).  a_i is
 * assumed valid, as the reference asserts (:73).  Edges that would need
 * more than 2^22 samples are reported invalid. */
mptg_status mptg_valid_edges(mptg_scene* scene, const double* a, const double* b, size_t n,
                             double step, int resolution, uint8_t* out, void* stream);

/* ---- wavefront planner ---------------------------------------------
 * PRRT's worker loop (src/mpt/impl/prrt/prrt.hpp:358-452) as wavefronts of
 * `wavefront` samples: sample (goal with probability goal_bias until the
 * first solution) -> nearest -> skip if d == 0 -> steer to `range` ->
 * valid + link (DMV at edge_step) -> goal test -> insert.  Samples come from
 * a Philox4x32-10 stream keyed by `seed`; a wavefront sees the tree as it
 * stood before it, and accepted samples join in sample order, so a run is
 * reproducible from the seed. */
typedef struct mptg_planner mptg_planner;
typedef struct {
    double range;        /* PRRT::setRange (prrt.hpp:168-171); <= 0 means unlimited */
    double goal_bias;    /* PRRT::setGoalBias (prrt.hpp:159-162), reference default 0.01 */
    double goal_radius;  /* GoalState radius (goal_state.hpp:64-69); set by set_goal */
    double edge_step;    /* DiscreteMotionValidator step size */
    int resolution;      /* 0: space metric, 1: max wrapped joint difference */
    int wavefront;       /* samples per wavefront, 1 .. 2^20 */
    uint64_t seed;
    size_t max_nodes;    /* node budget (tree capacity) */
} mptg_plan_params;

/* Planner<Scenario, PRRT<...>>(scenario, seed) (prrt.hpp:149-157); lo/hi are
 * the sampling bounds (Scenario::bounds, src/mpt/impl/scenario_bounds.hpp);
 * NULL uses [-pi, pi] per joint for SO2 and [0, 1] otherwise (quaternion
 * dimensions of SE3 are always sampled uniformly on SO(3)). */
mptg_status mptg_planner_create(mptg_ctx* ctx, mptg_scene* scene, const mptg_plan_params* params,
                                const double* lo, const double* hi, mptg_planner** planner);
/* the Planner's destructor */
mptg_status mptg_planner_destroy(mptg_planner* planner);
/* PRRT::addStart (prrt.hpp:181-187); the start is not checked for validity, as in the reference */
mptg_status mptg_planner_add_start(mptg_planner* planner, const double* q);
/* GoalState(radius, q) as the Scenario's goal (src/mpt/goal_state.hpp:43-90) */
mptg_status mptg_planner_set_goal(mptg_planner* planner, const double* q, double radius);
/* PRRT::solve (prrt.hpp:194-201) driven by the host between wavefronts: runs
 * up to max_wavefronts (<= 0: no limit) or time_limit_s (<= 0: none), and
 * stops after the first solution when stop_when_solved.  No start ->
 * MPTG_ERR_NO_START (the reference throws "there are no valid initial
 * states"); a second concurrent call -> MPTG_ERR_ALREADY_SOLVING. */
mptg_status mptg_planner_run(mptg_planner* planner, int max_wavefronts, double time_limit_s,
                             int stop_when_solved, int* solved);
/* PRRT::size (prrt.hpp:177-179) */
mptg_status mptg_planner_size(mptg_planner* planner, size_t* n);
/* number of goal nodes found (PRRT::solved() is goals > 0, prrt.hpp:203-205) */
mptg_status mptg_planner_goals(mptg_planner* planner, size_t* n);
/* PRRT::solution() (prrt.hpp:263-274): the best goal's path, start first,
 * len states of dim doubles, and its cost (prrt.hpp:208-234).  path may be
 * NULL to query len and cost. */
mptg_status mptg_planner_solution(mptg_planner* planner, double* path, size_t cap, size_t* len,
                                  double* cost);
/* PRRT::visitGraph (prrt.hpp:300-316): all states and parent ids (-1 for starts). */
mptg_status mptg_planner_graph(mptg_planner* planner, double* states, int32_t* parents, size_t cap,
                               size_t* n);
/* Where the wavefronts run (no reference counterpart: an execution choice).
 * mode 1 (the default): on grid scenes with wavefronts of up to 1,024 samples
 * (PRRT, no surrogate), mptg_planner_run runs its wavefronts inside one
 * persistent thread block -- nearest neighbours, steering, the motion check,
 * the ordered insert and the stop conditions all on the device -- for up to
 * 16,384 nodes, then updates the kd-tree; beyond that, and everywhere else,
 * the multi-kernel wavefront runs.  mode 0: always the multi-kernel
 * wavefront.  Both build the same tree, state for state.  A run with neither a
 * wavefront count nor a time limit launches the block in slices of at most
 * 1 s of device time, relaunched while the tree can grow, so that no launch
 * runs for ever when every sample's link is invalid. */
mptg_status mptg_planner_set_persistent(mptg_planner* planner, int mode);
/* The block planner's nearest-node search (no reference counterpart: a tuning
 * knob of this planner).  A wavefront of W samples over n nodes with
 * W * n <= brute_pairs sweeps every node in FP32 and re-ranks the nodes within
 * the FP32 error bound of the least in FP64; a larger one searches rings of a
 * bucket grid.  Both return the exact FP64 nearest node (lowest id on ties),
 * so the setting changes the speed only.  Default 2^24, which covers every
 * wavefront of up to 1,024 samples over the block planner's 16,384 nodes. */
mptg_status mptg_planner_set_block_search(mptg_planner* planner, long long brute_pairs);
/* Runs of the block planner replayed through its captured CUDA graph (no
 * reference counterpart: a profile of this planner).  A planner captures one
 * run (job and counters in, the block, counters out) on its stream the first
 * time it uses the block planner, and replays it for every later run with the
 * same wavefront size; if the capture fails it launches directly. */
mptg_status mptg_planner_graph_runs(mptg_planner* planner, uint64_t* runs);
/* The planner's nearest-neighbour container -- PRRT's nn_ member, the nigh
 * tree its workers query (src/mpt/impl/prrt/prrt.hpp:121-122,406-409) -- as a
 * borrowed tree handle: mptg_nearest / mptg_nearest_k / mptg_nearest_linear /
 * mptg_tree_counters work on it; it stays owned by the planner (do not
 * destroy or insert into it) and is valid until the planner is destroyed. */
mptg_status mptg_planner_tree(mptg_planner* planner, mptg_tree** tree);
/* ---- learned collision surrogate ------------------------------------
 * No counterpart in the reference.  An MLP in -> 256 -> 256 -> 256 -> 256 -> 1
 * (SiLU, BF16 weights/activations, FP32 accumulation) predicting the logit
 * that a state is in collision, trained on states labelled by the exact
 * checker.  It only orders and culls candidate edges; edges enter the tree
 * only after the exact check.  Inputs are (state - shift) * scale. */
typedef struct mptg_surrogate mptg_surrogate;
mptg_status mptg_surrogate_create(mptg_ctx* ctx, int in_dim, const double* scale, const double* shift,
                                  uint64_t seed, mptg_surrogate** surrogate);
mptg_status mptg_surrogate_destroy(mptg_surrogate* surrogate);
mptg_status mptg_surrogate_num_params(mptg_surrogate* surrogate, size_t* n);
/* which 0: parameters, 1: gradients of the last train step (FP32, host buffer of n) */
mptg_status mptg_surrogate_get(mptg_surrogate* surrogate, int which, float* out, size_t n);
mptg_status mptg_surrogate_set(mptg_surrogate* surrogate, const float* params, size_t n);
/* One Adam step (lr <= 0: gradients only) of BCE-with-logits on n states
 * (n a multiple of 128), labels 1 = in collision; the batch loss goes to loss. */
mptg_status mptg_surrogate_train_step(mptg_surrogate* surrogate, const double* states, const uint8_t* labels,
                                      size_t n, double lr, float* loss, void* stream);
/* collision logits of n states */
mptg_status mptg_surrogate_score(mptg_surrogate* surrogate, const double* states, size_t n, float* logits,
                                 void* stream);
/* Cull edges whose new state's collision logit exceeds `threshold` before the
 * exact check (they count as rejected); NULL removes the surrogate. */
mptg_status mptg_planner_set_surrogate(mptg_planner* planner, mptg_surrogate* surrogate, double threshold);
/* Score `points` states per candidate edge (1 .. 8, default 1): the new state
 * and interpolate(near, new, j/points) for 1 <= j < points; the edge is culled
 * when any of them exceeds the threshold. */
mptg_status mptg_planner_set_surrogate_points(mptg_planner* planner, int points);
/* Surrogate-biased sampling (1 .. 16, default 1 = off): each wavefront slot
 * draws `candidates` samples, finds their nearest nodes and steers all of
 * them, the surrogate scores every candidate edge, and the slot keeps the one
 * whose highest collision logit is lowest (candidate 0 is the plain planner's
 * sample; the goal sample always keeps its slot).  The kept edge is culled or
 * exact-checked as above: an edge still enters the tree only after the exact
 * check.  No reference counterpart (the learned part of the planner). */
mptg_status mptg_planner_set_surrogate_bias(mptg_planner* planner, int candidates);

/* WorkerStats (prrt.hpp:63-101): [0] wavefronts, [1] samples, [2] nodes
 * added, [3] tree size, [4] goals, [5] states checked by link, [6] seconds in
 * run, [7] wavefront counter. */
mptg_status mptg_planner_stats(mptg_planner* planner, double out[8]);
/* Persistent block planner (grid scenes, mptg_planner_set_persistent), summed
 * over its runs: SM cycles in [0] the sample phase, [1] the nearest-search
 * phase, which also runs each sample's steer and link set-up as soon as its
 * nearest node is known, [2] and [3] unused (zero), [4] the
 * link-sample phase and [5] the insert phase; [6] FP64 distances of the
 * nearest search beyond the winners', [7] interior samples decided in FP64,
 * [8] edge step counts decided in FP64.  No reference counterpart (a profile
 * of this planner). */
mptg_status mptg_planner_block_profile(mptg_planner* planner, double out[9]);
/* Planner<Scenario, PRRTStar<...>> (src/mpt/prrt_star.hpp:56-95): wavefronts
 * with k-nearest rewiring (rewire_k_nearest, the reference default):
 * k = ceil(rewire_factor * e * (1 + 1/dim) * ln(n + 1)), at most 64
 * (src/mpt/impl/rrg_rewire_neighbors.hpp:47-66), rewire_factor default 1.1
 * (PRRTStar::setRewireFactor, src/mpt/impl/prrt_star/prrt_star.hpp:234-240).
 * Per wavefront, against the tree before it: choose-parent among the
 * accepted state's k nearest in (cost + d, d, id) order with batched link
 * checks; rewiring of the neighbours the choose step did not reach when
 * cost(new) + d < cost(neighbour) and link(new, neighbour) holds (each
 * neighbour takes the proposal with the smallest (cost, new id)); every cost
 * is then recomputed from the edge lengths by pointer jumping.  Call before
 * the first wavefront; enabled = 0 returns to plain PRRT. */
mptg_status mptg_planner_set_rewire(mptg_planner* planner, int enabled, double rewire_factor);
/* Each node's cost (Edge::cost, prrt_star.hpp) with rewiring on; out NULL
 * queries n only. */
mptg_status mptg_planner_costs(mptg_planner* planner, double* out, size_t cap, size_t* n);
/* PRRT*'s Stats (prrt_star.hpp:121-152): [0] rewires applied, [1] links checked
 * for choose-parent and rewiring; seconds on the GPU timeline in [2] k-NN,
 * [3] choose parent, [4] rewire, [5] cost recomputation */
mptg_status mptg_planner_rewire_stats(mptg_planner* planner, double out[6]);
/* WorkerStats' timers (prrt.hpp:72-101) on the GPU timeline, seconds summed
 * over wavefronts: [0] sample + nearest + steer, [1] surrogate scoring,
 * [2] valid motion (state + DMV link checks), [3] compaction + insert. */
mptg_status mptg_planner_timers(mptg_planner* planner, double out[4]);

/* Start over as a new Planner(scenario, seed) on the same scene, keeping the
 * allocations: tree, goal, solutions and statistics are cleared.  params NULL
 * keeps the current ones; otherwise wavefront and max_nodes may not exceed
 * those the planner was created with (MPTG_ERR_CAPACITY). */
mptg_status mptg_planner_reset(mptg_planner* planner, const mptg_plan_params* params);

/* ---- batched multi-query serving -------------------------------------
 * Many independent planning queries (one start, one GoalState each) over
 * shared scenes.  `concurrency` host workers (<= 0: 8) each own one CUDA
 * stream and reuse one planner per scene between queries, so the wavefronts
 * of different queries overlap on the GPU.  The grid queries that the
 * persistent block planner takes (resolution 0, wavefront <= 1,024, no
 * surrogate) do not use the workers: they run together as one launch, one
 * thread block per query, while the workers take the rest; a query whose block
 * fills its 16,384 nodes unsolved, or (no time limit) is still unsolved after
 * 1 s of device time, is then run from its start by a worker.  A
 * query behaves exactly as mptg_planner_create + add_start + set_goal +
 * run(stop_when_solved) with the same parameters: the same seed gives the
 * same tree and path. */
typedef struct {
    mptg_scene* scene;
    const double* start;        /* [dim], host */
    const double* goal;         /* [dim], host */
    double goal_radius;
    mptg_plan_params params;    /* params.max_nodes is the query's node budget */
    const double* lo;           /* sampling bounds or NULL, as mptg_planner_create */
    const double* hi;
    double time_limit_s;        /* <= 0: none */
    mptg_surrogate* surrogate;  /* NULL: plain planner */
    double surrogate_threshold;
    int surrogate_points;       /* as mptg_planner_set_surrogate_points (<= 1: the new state only) */
    double* path;               /* optional host buffer of path_cap states */
    size_t path_cap;
    int surrogate_candidates;   /* as mptg_planner_set_surrogate_bias (<= 1: off) */
} mptg_query;

typedef struct {
    mptg_status status;
    int solved;
    size_t nodes;               /* tree size at the end */
    size_t wavefronts;
    double solve_s;             /* from the query's first wavefront to its end */
    double finish_s;            /* from the batch's start to the query's end */
    double cost;                /* best path cost, +inf when unsolved */
    size_t path_len;            /* states of the best path (0 if unsolved); written to
                                   query.path only when it fits path_cap */
} mptg_result;

/* Project-written autotuner for the wavefront size of one scene and query:
 * plans `trials` seeds (params->seed, +1, ...) from start to the goal for each
 * candidate size (stop at the first solution, time_limit_s each; unsolved
 * counts as the limit), then 2 * trials more seeds for the three sizes with
 * the lowest medians, and returns in *best the one of those three with the
 * lowest median time to solution over all its seeds; median_s (ncand
 * entries, may be NULL) receives each size's median over the seeds it ran.
 * The time to solution is governed by tree depth (wavefronts needed) times
 * per-wavefront latency, so the best size is scene-dependent; the second
 * stage keeps a heavy-tailed scene's pick from resting on a few seeds. */
mptg_status mptg_autotune_wavefront(mptg_ctx* ctx, mptg_scene* scene, const mptg_plan_params* params,
                                    const double* lo, const double* hi, const double* start, const double* goal,
                                    double goal_radius, const int* candidates, int ncand, int trials,
                                    double time_limit_s, int* best, double* median_s);

/* Runs queries [0, n) and fills out[0, n).  Returns MPTG_OK when every query
 * ran (per-query failures are in out[i].status), else the first error. */
mptg_status mptg_plan_batch(mptg_ctx* ctx, const mptg_query* queries, size_t n, int concurrency,
                            mptg_result* out);

/* ---- PPRM: parallel k-nearest probabilistic roadmap ------------------
 * PPRM's Worker::addSample (src/mpt/impl/pprm/pprm.hpp:293-340) over
 * wavefronts of `wavefront` uniform samples (the Philox stream of the PRRT
 * planner, without goal samples).  Each valid sample q joins the roadmap in
 * sample order: k = ceil((e + e/dim) ln(n + 1)) (at most 64) nearest of the n
 * nodes before it, sorted by (distance, id); skipped when the nearest is
 * closer than DBL_EPSILON; a goal node when within goal_radius of the goal;
 * an edge (q, nbr, distance) for every neighbour with a valid link(q, nbr).
 * Within a wavefront a sample's neighbours include the wavefront's earlier
 * samples, so the roadmap equals the one-at-a-time roadmap of the same sample
 * sequence.  Components are a union-find; solved when a start and a goal
 * node share one.  Uses mptg_plan_params' goal_radius, edge_step,
 * resolution, wavefront, seed and max_nodes. */
typedef struct mptg_prm mptg_prm;
/* Planner<Scenario, PPRM<...>>(scenario, seed) (pprm.hpp:141-149); lo/hi as mptg_planner_create */
mptg_status mptg_prm_create(mptg_ctx* ctx, mptg_scene* scene, const mptg_plan_params* params, const double* lo,
                            const double* hi, const double* goal, mptg_prm** prm);
/* the Planner's destructor */
mptg_status mptg_prm_destroy(mptg_prm* prm);
/* PPRM::addStart / addGoal (pprm.hpp:155-170): addSample with the start or
 * goal flag; *id = the node id, or -1 when the state is invalid or a
 * duplicate (the reference returns nullptr) */
mptg_status mptg_prm_add_start(mptg_prm* prm, const double* q, int32_t* id);
mptg_status mptg_prm_add_goal(mptg_prm* prm, const double* q, int32_t* id);
/* PPRM::solve (pprm.hpp:173-183): wavefronts until max_wavefronts (<= 0: no
 * limit), time_limit_s (<= 0: none), the node budget, or the first solution
 * when stop_when_solved.  No start or no goal -> MPTG_ERR_NO_START (the
 * reference throws "PPRM requires both start and goal configurations"). */
mptg_status mptg_prm_run(mptg_prm* prm, int max_wavefronts, double time_limit_s, int stop_when_solved,
                         int* solved);
/* PPRM::size (pprm.hpp:152-154), and the roadmap's edge count */
mptg_status mptg_prm_size(mptg_prm* prm, size_t* nodes, size_t* edges);
/* The roadmap PPRM::visitGraph walks (pprm.hpp:248-251,381-388): states
 * [n][dim] (may be NULL), and the undirected edges (from, to, distance),
 * from > to, sorted by (from, to) (any may be NULL) */
mptg_status mptg_prm_graph(mptg_prm* prm, double* states, size_t cap_nodes, int32_t* from, int32_t* to,
                           double* dist, size_t cap_edges, size_t* n, size_t* ne);
/* PPRM::solution() (pprm.hpp:232-243): Dijkstra from the start nodes to the
 * nearest goal node over the edge distances; len states, start first (path
 * may be NULL to query len and cost; cost = +inf and len = 0 when unsolved) */
mptg_status mptg_prm_solution(mptg_prm* prm, double* path, size_t cap, size_t* len, double* cost);
/* counters (PPRM::printStats, pprm.hpp:242-245, and PPRM::solved,
 * pprm.hpp:185-187): [0] wavefronts, [1] samples, [2] valid samples,
 * [3] duplicates skipped, [4] links checked, [5] edges, [6] goal nodes,
 * [7] solved */
mptg_status mptg_prm_stats(mptg_prm* prm, uint64_t out[8]);

/* ---- scene ingestion helpers (host only) -------------------------------
 * PNG scanline reconstruction for the image reader of mpt_gb300.ingest (the
 * row filters libpng undoes for demo/png_2d_scenario.hpp:198-240): raw holds
 * height rows of (filter byte + stride bytes), out receives height * stride
 * bytes; bpp = bytes per complete pixel (at least 1).  An unknown filter type
 * returns MPTG_ERR_INVALID_ARG. */
mptg_status mptg_png_unfilter(const uint8_t* raw, int height, int stride, int bpp, uint8_t* out);

#ifdef __cplusplus
}
#endif
#endif /* MPTG_H */
