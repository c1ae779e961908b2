// bplan.cuh - interface of the persistent block planner (bplan.cu).
#pragma once
#include "scene.cuh"

// Counters a persistent run reads at its start and leaves at its end.
struct BPlanCounters {
    int n;                          // nodes in the tree
    uint32_t wave;                  // wavefront index of the next wavefront (the sample stream's w)
    int goals;                      // goal nodes found so far (this run and earlier ones)
    int maxabs_bits;                // largest |coordinate| of a stored state, FP32 bits (error bound)
    int status;                     // BPLAN_* below
    int waves_run;                  // wavefronts this run completed
    unsigned long long samples;     // samples drawn by this run
    unsigned long long accepted;    // nodes added by this run
    // SM cycles of this run per phase: [0] samples, [1] nearest search with
    // each sample's steer and link set-up (one phase: a sample's steer starts
    // as soon as its nearest node is known), [2] and [3] unused (zero),
    // [4] link samples (warp per edge), [5] insert
    unsigned long long cyc[6];
    // FP64 fallbacks of this run: FP64 distances of the nearest search (the
    // ring search's near ties; every candidate of the exhaustive search,
    // winners included), unsure interior samples (warps), step counts left
    // to FP64
    unsigned long long ties, unsure, steps64;
    // the device's global timer (ns) when the block started and when it ended
    unsigned long long start_ns, end_ns;
};

enum { BPLAN_DONE = 0, BPLAN_FULL = 1 };  // FULL: the next wavefront could overflow the block's node capacity

// One query of the persistent planner: the wavefront PRRT of planner.cu, with
// every step inside one thread block (the grid scene).
struct BPlanJob {
    SceneView scene;
    const double* lo;
    const double* hi;
    const double* goal;
    int has_goal;
    double goal_bias, range, goal_radius, inv_step;
    uint64_t seed;
    double* states;                 // [cap][2] node states (the first n given)
    int* parent;                    // [cap] parent ids (the planner's array)
    uint8_t* goalf;                 // [cap] goal flag per node
    BPlanCounters* ctr;
    unsigned long long* nsamp;      // link states checked (may be null)
    size_t max_nodes;               // the planner's node budget
    int cap;                        // node capacity of this block (<= BPLAN_MAX_NODES)
    int W;                          // wavefront size (<= BPLAN_THREADS)
    int max_waves;                  // wavefronts to run (<= 0: no limit)
    int stop_when_solved;
    uint64_t deadline_ns;           // time limit of the run (0: none)
    // bucket grid of the nearest-neighbour search: gx x gy cells of size
    // cell_size from (cell_ox, cell_oy), gx * gy <= BPLAN_CELLS
    float cell_ox, cell_oy, cell_size, cell_inv;
    int gx, gy;
    long long brute_pairs;          // W x nodes up to this: exhaustive nearest search (nn_brute)
};

#define BPLAN_THREADS 1024
#define BPLAN_MAX_NODES 16384       // FP32 node copy in shared memory: 128 KB
#define BPLAN_CELLS 4096            // bucket-grid cells (64 x 64 over the sampling box)
// default of BPlanJob::brute_pairs: wavefronts with W x nodes up to this many
// pairs search their nearest nodes exhaustively (nn_brute); larger ones by
// rings of the bucket grid
#define BPLAN_BRUTE_PAIRS (1LL << 24)

// Sets the kernel's shared-memory limit on the context's device (once); done
// by bplan_launch, and before a stream capture of it.
mptg_status bplan_configure(mptg_ctx* ctx);
// Runs njobs jobs (device array), one thread block each, on stream s;
// configure false: bplan_configure has run already (inside a stream capture
// the launch makes no other runtime call).
mptg_status bplan_launch(mptg_ctx* ctx, const BPlanJob* djobs, int njobs, int max_W, int max_cap, cudaStream_t s,
                         bool configure = true);
// true when the scene and parameters are ones the block planner runs
bool bplan_supported(const mptg_scene* sc, int wavefront, int resolution);
