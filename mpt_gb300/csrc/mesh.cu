// mesh.cu - rigid-body (SE(3)) mesh-vs-mesh validity.
#include "metrics.cuh"
#include "scene.cuh"

struct MeshData {
    int placeholder;
};

mptg_status mesh_scene_create(mptg_ctx* ctx, const mptg_scene_desc*, mptg_scene*) {
    return mptg_fail(ctx, MPTG_ERR_INVALID_ARG, "rigid mesh scenes are not available in this build");
}

void mesh_scene_free(mptg_scene* s) {
    delete s->mesh;
    s->mesh = nullptr;
}

void mesh_fill_view(const mptg_scene*, SceneView*) {}

mptg_status mesh_edges_dev(mptg_scene* sc, const double*, const double*, int, double, int, uint8_t*, cudaStream_t,
                           unsigned long long*) {
    return mptg_fail(sc->ctx, MPTG_ERR_INVALID_ARG, "rigid mesh scenes are not available in this build");
}

mptg_status mesh_states_dev(mptg_scene* sc, const double*, int, uint8_t*, cudaStream_t) {
    return mptg_fail(sc->ctx, MPTG_ERR_INVALID_ARG, "rigid mesh scenes are not available in this build");
}
