/*
 * oracle.h - CPU restatement of MPT's planner hot path, used ONLY as the
 * checker by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
 * Nothing in the mpt_gb300 product links, loads or calls this library.
 *
 * Metric ids match include/mptg.h (MPTG_METRIC_*).
 */
#ifndef MPTG_ORACLE_H
#define MPTG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_L2 = 0, ORC_SO2 = 1, ORC_SO3 = 2, ORC_SE3 = 3, ORC_L1 = 4 };

/* Metric space description: SE3 uses w[0] (rotation weight) and w[1]
 * (translation weight); the others ignore w. */
typedef struct { int metric; int dim; double w[2]; } orc_space;

double orc_distance(const orc_space* s, const double* a, const double* b);
void orc_interpolate(const orc_space* s, const double* a, const double* b, double t, double* out);
double orc_so2_ccw(double a, double b);
double orc_so2_bound(double v);

/* Exact FP64 1-NN (lowest index on ties), brute force. */
void orc_nn_brute(const orc_space* s, const double* pts, int64_t n, const double* q,
                  int64_t nq, int32_t* idx, double* dist, int nthreads);
/* Exact FP64 k-NN sorted by (distance, index); k results per query, -1/inf padded. */
void orc_knn_brute(const orc_space* s, const double* pts, int64_t n, const double* q,
                   int64_t nq, int k, int32_t* idx, double* dist, int nthreads);

/* CPU bucketed kd-tree (the baseline NN structure: nigh is not vendored). */
void* orc_kd_build(const orc_space* s, const double* pts, int64_t n, int leaf_size);
void orc_kd_nearest(void* tree, const double* q, int64_t nq, int32_t* idx, double* dist,
                    int nthreads, int64_t* dist_evals);
void orc_kd_free(void* tree);

/* Scenes. */
typedef struct {
    int kind;                 /* 0 grid, 1 planar arm, 2 rigid mesh (SE3) */
    /* grid */
    const uint8_t* grid; int width, height;
    /* planar arm */
    int nlinks; const double* link_len; int ndiscs; const double* discs; /* (cx,cy,r)*ndiscs */
    double robot_radius; int self_collision;
    /* rigid mesh: triangles as 9 doubles each */
    int64_t nrobot; const double* robot_tris; int64_t nenv; const double* env_tris;
} orc_scene;

/* Edge resolution: 0 = the space metric (DiscreteMotionValidator),
 * 1 = max over joints of the wrapped joint difference (planar-arm edges). */
int orc_state_valid(const orc_scene* sc, const double* q);
void orc_valid_states(const orc_scene* sc, const orc_space* sp, const double* q, int64_t n,
                      uint8_t* out, int nthreads);
void orc_valid_edges(const orc_scene* sc, const orc_space* sp, const double* a, const double* b,
                     int64_t n, double step, int resolution, uint8_t* out, int64_t* samples,
                     int nthreads);

/* Wavefront planner replay (see oracle.c). */
typedef struct {
    double range, goal_bias, goal_radius, edge_step;
    int resolution, wavefront;
    uint64_t seed;
    int64_t max_nodes;
} orc_plan_params;
double orc_uniform(uint64_t seed, uint32_t i, uint32_t w, uint32_t j);
/* sample i of wavefront w of the planners' sample stream (no goal bias) */
void orc_sample_state(const orc_space* sp, const orc_plan_params* pp, const double* lo, const double* hi,
                      uint32_t i, uint32_t w, double* q);
/* nearest-neighbour search of the replays: 0 brute force (default), 1 the
 * exact kd-tree, 2 the kd-tree up to 7 dimensions (same answers; for CPU
 * timing runs) */
void orc_set_plan_nn(int mode);
int64_t orc_plan(const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp, const double* lo,
                 const double* hi, const double* start, const double* goal, int max_waves, int stop_when_solved,
                 double* states, int32_t* parents, int32_t* goals, int64_t* ngoals, int nthreads);

/* Replay of the wavefront PRRT* (rewiring) planner: as orc_plan, then per
 * wavefront k-nearest choose-parent, rewiring and pointer-jumping costs
 * (see orc_plan_star in oracle.c).  costs receives each node's cost. */
int64_t orc_plan_star(const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp, const double* lo,
                      const double* hi, const double* start, const double* goal, int max_waves,
                      double rewire_factor, double* states, int32_t* parents, double* costs, int32_t* goals,
                      int64_t* ngoals, int64_t* rewires, int nthreads);

/* Replay of the wavefront PPRM roadmap (see orc_prm in oracle.c): starts,
 * then goals, then max_waves wavefronts of the sample stream, one sample at a
 * time.  Returns the node count; edges (from = new node > to) in insertion
 * order up to ecap (*ne = all); stats as mptg_prm_stats. */
int orc_prm_k(int64_t n, int dim);
int64_t orc_prm(const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp, const double* lo,
                const double* hi, const double* goal, const double* starts, int nstarts, const double* goals,
                int ngoals, int max_waves, int stop_when_solved, double* states, uint8_t* flags, int64_t* ne,
                int32_t* efrom, int32_t* eto, double* edist, int64_t ecap, int64_t* stats);
/* Dijkstra over a roadmap (start flag 1, goal flag 2); path = node ids */
int64_t orc_prm_dijkstra(int64_t n, const uint8_t* flags, int64_t ne, const int32_t* efrom, const int32_t* eto,
                         const double* edist, int32_t* path, double* cost);

/* Triangle-triangle intersection (FP64 orientation predicates). */
int orc_tri_tri(const double* t1, const double* t2);

#ifdef __cplusplus
}
#endif
#endif
