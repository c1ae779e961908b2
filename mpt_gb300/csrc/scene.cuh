// scene.cuh - scene storage shared by the validity, mesh and planner units.
#pragma once
#include "common.cuh"

struct MeshData;  // rigid-mesh BVHs (mesh.cu)

// Working memory of one batched validity call.  A scene owns one for the
// C-ABI calls; every planner owns its own, so planners sharing a scene can run
// concurrently on their own streams.
struct EdgeScratch {
    // grid / planar-arm two-phase edges
    int* work = nullptr;
    int* wsteps = nullptr;
    int* wcount = nullptr;
    size_t work_cap = 0;
    // rigid mesh
    int* mwork = nullptr;
    int* nwork = nullptr;
    size_t mwork_cap = 0;
    double* samples = nullptr;
    int* sample_edge = nullptr;
    uint8_t* sample_ok = nullptr;
    size_t sample_cap = 0;
    int* counts = nullptr;
    int* offs = nullptr;
    uint8_t* okb = nullptr;
    size_t edge_cap = 0;
    int* hbuf = nullptr;  // pinned, 4 ints
};
void scratch_free(EdgeScratch* s);

struct mptg_scene {
    mptg_ctx* ctx = nullptr;
    int kind = 0, metric = 0, D = 0;
    double w0 = 1.0, w1 = 1.0;
    // grid
    uint8_t* grid = nullptr;
    int width = 0, height = 0;
    // planar arm
    int nlinks = 0, ndiscs = 0, self_collision = 0;
    double robot_radius = 0.0;
    double* link_len64 = nullptr;
    double* discs64 = nullptr;
    // rigid mesh
    MeshData* mesh = nullptr;
    // FP32 filter data: discs (cx, cy, (r + robot_radius)^2, unused), link lengths
    float4* discs32 = nullptr;
    float* link32 = nullptr;
    float arm_reach = 0.f;
    float arm_span = 0.f;  // bound on |x| + |y| of joint positions and disc centres
    // scratch of the C-ABI validity calls on this scene
    EdgeScratch scratch;
};

// POD view passed to kernels by value
struct SceneView {
    int kind, metric, D;
    double w0, w1;
    const uint8_t* grid;
    int width, height;
    int nlinks, ndiscs, self_collision;
    double robot_radius;
    const double* link_len64;
    const double* discs64;
    const float4* discs32;
    const float* link32;
    float arm_reach;
    float arm_span;
    // rigid mesh (see mesh.cu)
    const double* robot_tris;   // [nrobot][9]
    int nrobot;
    const double* env_tris;     // [nenv][9], BVH leaf order
    const float4* env_nodes;    // [2*nenv] {lo.xyz, left|leaf}, {hi.xyz, right|count}
    int nenv;
};

SceneView scene_view(const mptg_scene* s);
// scr == nullptr uses the scene's own scratch
mptg_status scene_edges_dev(mptg_scene* sc, const double* da, const double* db, int n, double step, int resolution,
                            uint8_t* dout, cudaStream_t s, unsigned long long* nsamp, EdgeScratch* scr = nullptr);
mptg_status scene_states_dev(mptg_scene* sc, const double* dq, int n, uint8_t* dout, cudaStream_t s,
                             EdgeScratch* scr = nullptr);

// rigid-mesh hooks (mesh.cu)
mptg_status mesh_scene_create(mptg_ctx* ctx, const mptg_scene_desc* d, mptg_scene* s);
void mesh_scene_free(mptg_scene* s);
void mesh_fill_view(const mptg_scene* s, SceneView* v);
mptg_status mesh_edges_dev(mptg_scene* sc, const double* da, const double* db, int n, double step, int resolution,
                           uint8_t* dout, cudaStream_t s, unsigned long long* nsamp, EdgeScratch* scr);
// sample_edge / edge_out: the interior samples of a batch of edges (see k_mesh_detail)
mptg_status mesh_states_dev(mptg_scene* sc, const double* dq, int n, uint8_t* dout, cudaStream_t s,
                            EdgeScratch* scr, const int* sample_edge = nullptr, uint8_t* edge_out = nullptr);
