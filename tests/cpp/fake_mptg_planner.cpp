// A scripted CPU stand-in for the planner calls of the C ABI (mptg.h) that
// include/mptg_planner.hpp makes.  TEST CODE ONLY: it is not a planner (no
// sampling, no collision checks).  Each mptg_planner_run adds one node a
// `range` step from the newest node toward the goal, and each mptg_prm_run one
// node on the segment from the start to the goal, so that
// tests/cpp/planner_header_check.cpp can check, on a machine without a GPU,
// what the header forwards (parameters, bounds, goal, rewiring, starts), how
// its solve loops poll and stop, how it turns status codes into exceptions,
// and how it reads paths and graphs back.  Every call is recorded in
// fake_planner_log.
#include <cmath>
#include <cstring>
#include <vector>

#include "mptg.h"

// what the stand-in saw; read and steered by the check program
struct FakePlannerLog {
    int device;
    int scene_kind;
    mptg_plan_params params;      // the last mptg_planner_create / mptg_prm_create
    int has_bounds;
    double lo[8], hi[8];
    double goal[8], goal_radius;
    int rewire;
    double rewire_factor;
    int runs;                     // mptg_planner_run calls
    double min_limit, max_limit;  // their time limits
    int unlimited_runs;           // calls with neither a wavefront count nor a time limit
    int stop_after_solved;        // calls with stop_when_solved set once a goal was found
    int prm_runs;
    int live_ctx, live_scene, live_planner, live_prm;
    int fail_create;              // the next mptg_create fails
    int fail_run;                 // the next mptg_planner_run fails
};
extern "C" {
FakePlannerLog fake_planner_log;
}

struct mptg_ctx {
    const char* err = "";
};
struct mptg_scene {
    mptg_ctx* ctx;
    int dim, metric;
};
struct mptg_planner {
    mptg_ctx* ctx;
    int dim;
    mptg_plan_params p;
    std::vector<double> goal;
    std::vector<double> st;
    std::vector<int32_t> par;
    std::vector<int> goals;
    double waves = 0;
};
struct mptg_prm {
    mptg_ctx* ctx;
    int dim;
    mptg_plan_params p;
    std::vector<double> st;
    std::vector<int32_t> ef, et;  // from > to
    std::vector<double> ed;
    int start = -1, goal = -1, last = -1;
    uint64_t waves = 0;
    bool solved = false;
};

namespace {
FakePlannerLog& L = fake_planner_log;

mptg_status fail(mptg_ctx* c, const char* msg, mptg_status s) {
    c->err = msg;
    return s;
}

double l2(const double* a, const double* b, int d) {
    double s = 0;
    for (int i = 0; i < d; ++i) s += (a[i] - b[i]) * (a[i] - b[i]);
    return std::sqrt(s);
}

// copies n states and parents out with the ABI's capacity rule (NULL buffers query n)
mptg_status read_path(mptg_ctx* ctx, const std::vector<double>& st, int dim, const std::vector<int>& ids,
                      double* path, size_t cap, size_t* len) {
    *len = ids.size();
    if (!path) return MPTG_OK;
    if (cap < ids.size()) return fail(ctx, "path does not fit", MPTG_ERR_CAPACITY);
    for (size_t i = 0; i < ids.size(); ++i)
        std::memcpy(path + i * dim, &st[(size_t)ids[i] * dim], dim * sizeof(double));
    return MPTG_OK;
}
}  // namespace

extern "C" {

mptg_status mptg_create(mptg_ctx** ctx, int device) {
    if (!ctx) return MPTG_ERR_INVALID_ARG;
    if (L.fail_create) {
        L.fail_create = 0;
        return MPTG_ERR_CUDA;
    }
    L.device = device;
    *ctx = new mptg_ctx;
    ++L.live_ctx;
    return MPTG_OK;
}
mptg_status mptg_destroy(mptg_ctx* ctx) {
    if (ctx) --L.live_ctx;
    delete ctx;
    return MPTG_OK;
}
const char* mptg_last_error(mptg_ctx* ctx) { return ctx ? ctx->err : "no context"; }

mptg_status mptg_scene_create(mptg_ctx* ctx, const mptg_scene_desc* d, mptg_scene** scene) {
    if (!ctx || !d || !scene) return MPTG_ERR_INVALID_ARG;
    L.scene_kind = d->kind;
    int dim = 2, metric = MPTG_METRIC_L2;
    if (d->kind == MPTG_SCENE_PLANAR_ARM) dim = d->nlinks, metric = MPTG_METRIC_SO2;
    else if (d->kind == MPTG_SCENE_RIGID_MESH) dim = 7, metric = MPTG_METRIC_SE3;
    else if (d->kind != MPTG_SCENE_GRID || !d->grid) return fail(ctx, "bad scene", MPTG_ERR_INVALID_ARG);
    *scene = new mptg_scene{ctx, dim, metric};
    ++L.live_scene;
    return MPTG_OK;
}
mptg_status mptg_scene_destroy(mptg_scene* s) {
    if (s) --L.live_scene;
    delete s;
    return MPTG_OK;
}
mptg_status mptg_scene_space(mptg_scene* s, int* dim, int* metric, double w[2]) {
    if (!s) return MPTG_ERR_INVALID_ARG;
    if (dim) *dim = s->dim;
    if (metric) *metric = s->metric;
    if (w) w[0] = w[1] = 1.0;
    return MPTG_OK;
}

// ---- PRRT --------------------------------------------------------------
mptg_status mptg_planner_create(mptg_ctx* ctx, mptg_scene* s, const mptg_plan_params* p, const double* lo,
                                const double* hi, mptg_planner** out) {
    if (!ctx || !s || !p || !out) return MPTG_ERR_INVALID_ARG;
    if (p->wavefront < 1 || p->max_nodes < 1) return fail(ctx, "bad parameters", MPTG_ERR_INVALID_ARG);
    L.params = *p;
    L.has_bounds = lo && hi;
    for (int i = 0; L.has_bounds && i < s->dim && i < 8; ++i) L.lo[i] = lo[i], L.hi[i] = hi[i];
    mptg_planner* r = new mptg_planner;
    r->ctx = ctx;
    r->dim = s->dim;
    r->p = *p;
    *out = r;
    ++L.live_planner;
    return MPTG_OK;
}
mptg_status mptg_planner_destroy(mptg_planner* p) {
    if (p) --L.live_planner;
    delete p;
    return MPTG_OK;
}
mptg_status mptg_planner_set_goal(mptg_planner* p, const double* q, double radius) {
    p->goal.assign(q, q + p->dim);
    p->p.goal_radius = radius;
    for (int i = 0; i < p->dim && i < 8; ++i) L.goal[i] = q[i];
    L.goal_radius = radius;
    return MPTG_OK;
}
mptg_status mptg_planner_set_rewire(mptg_planner*, int enabled, double factor) {
    L.rewire = enabled;
    L.rewire_factor = factor;
    return MPTG_OK;
}
mptg_status mptg_planner_add_start(mptg_planner* p, const double* q) {
    if (p->par.size() >= p->p.max_nodes) return fail(p->ctx, "node budget", MPTG_ERR_CAPACITY);
    p->st.insert(p->st.end(), q, q + p->dim);
    p->par.push_back(-1);
    return MPTG_OK;
}
mptg_status mptg_planner_run(mptg_planner* p, int max_waves, double limit, int stop_when_solved, int* solved) {
    mptg_ctx* ctx = p->ctx;
    if (p->par.empty()) return fail(ctx, "there are no valid initial states", MPTG_ERR_NO_START);
    if (L.fail_run) {
        L.fail_run = 0;
        return fail(ctx, "injected failure", MPTG_ERR_CUDA);
    }
    if (L.runs == 0 || limit < L.min_limit) L.min_limit = limit;
    if (L.runs == 0 || limit > L.max_limit) L.max_limit = limit;
    ++L.runs;
    if (max_waves <= 0 && !(limit > 0)) ++L.unlimited_runs;
    if (stop_when_solved && !p->goals.empty()) ++L.stop_after_solved;
    const bool stop = stop_when_solved && !p->goals.empty();
    if (!stop && p->par.size() < p->p.max_nodes && !p->goal.empty()) {
        const int d = p->dim;
        const size_t last = p->par.size() - 1;
        const double* a = &p->st[last * d];
        const double dist = l2(a, p->goal.data(), d);
        const double step = p->p.range > 0 ? p->p.range : dist;
        std::vector<double> q(d);
        for (int i = 0; i < d; ++i) q[i] = dist <= step ? p->goal[i] : a[i] + (p->goal[i] - a[i]) * (step / dist);
        p->st.insert(p->st.end(), q.begin(), q.end());
        p->par.push_back((int32_t)last);
        if (l2(q.data(), p->goal.data(), d) <= p->p.goal_radius) p->goals.push_back((int)p->par.size() - 1);
        p->waves += 1;
    }
    if (solved) *solved = !p->goals.empty();
    return MPTG_OK;
}
mptg_status mptg_planner_size(mptg_planner* p, size_t* n) {
    *n = p->par.size();
    return MPTG_OK;
}
mptg_status mptg_planner_goals(mptg_planner* p, size_t* n) {
    *n = p->goals.size();
    return MPTG_OK;
}
mptg_status mptg_planner_solution(mptg_planner* p, double* path, size_t cap, size_t* len, double* cost) {
    std::vector<int> ids;
    double c = INFINITY;
    if (!p->goals.empty()) {
        c = 0;
        for (int i = p->goals.back(); i >= 0; i = p->par[i]) {
            ids.insert(ids.begin(), i);
            if (p->par[i] >= 0) c += l2(&p->st[(size_t)i * p->dim], &p->st[(size_t)p->par[i] * p->dim], p->dim);
        }
    }
    if (cost) *cost = c;
    return read_path(p->ctx, p->st, p->dim, ids, path, cap, len);
}
mptg_status mptg_planner_graph(mptg_planner* p, double* states, int32_t* parents, size_t cap, size_t* n) {
    *n = p->par.size();
    if (!states && !parents) return MPTG_OK;
    if (cap < p->par.size()) return fail(p->ctx, "graph does not fit", MPTG_ERR_CAPACITY);
    if (states) std::memcpy(states, p->st.data(), p->st.size() * sizeof(double));
    if (parents) std::memcpy(parents, p->par.data(), p->par.size() * sizeof(int32_t));
    return MPTG_OK;
}
mptg_status mptg_planner_stats(mptg_planner* p, double out[8]) {
    out[0] = out[7] = p->waves;
    out[1] = p->waves * p->p.wavefront;
    out[2] = p->waves;
    out[3] = (double)p->par.size();
    out[4] = (double)p->goals.size();
    out[5] = out[6] = 0;
    return MPTG_OK;
}
mptg_status mptg_planner_rewire_stats(mptg_planner* p, double out[6]) {
    for (int i = 0; i < 6; ++i) out[i] = 0;
    out[1] = (double)p->par.size();
    return MPTG_OK;
}

// ---- PPRM --------------------------------------------------------------
mptg_status mptg_prm_create(mptg_ctx* ctx, mptg_scene* s, const mptg_plan_params* p, const double* lo,
                            const double* hi, const double* goal, mptg_prm** out) {
    if (!ctx || !s || !p || !out) return MPTG_ERR_INVALID_ARG;
    L.params = *p;
    L.has_bounds = lo && hi;
    for (int i = 0; goal && i < s->dim && i < 8; ++i) L.goal[i] = goal[i];
    L.goal_radius = p->goal_radius;
    mptg_prm* r = new mptg_prm;
    r->ctx = ctx;
    r->dim = s->dim;
    r->p = *p;
    *out = r;
    ++L.live_prm;
    return MPTG_OK;
}
mptg_status mptg_prm_destroy(mptg_prm* r) {
    if (r) --L.live_prm;
    delete r;
    return MPTG_OK;
}
static int prm_add(mptg_prm* r, const double* q) {
    r->st.insert(r->st.end(), q, q + r->dim);
    return (int)(r->st.size() / r->dim) - 1;
}
mptg_status mptg_prm_add_start(mptg_prm* r, const double* q, int32_t* id) {
    *id = r->start = r->last = prm_add(r, q);
    return MPTG_OK;
}
mptg_status mptg_prm_add_goal(mptg_prm* r, const double* q, int32_t* id) {
    *id = r->goal = prm_add(r, q);
    return MPTG_OK;
}
mptg_status mptg_prm_run(mptg_prm* r, int, double, int, int* solved) {
    if (r->start < 0 || r->goal < 0)
        return fail(r->ctx, "PPRM requires both start and goal configurations", MPTG_ERR_NO_START);
    ++L.prm_runs;
    const size_t n = r->st.size() / r->dim;
    if (!r->solved && n < r->p.max_nodes) {
        // the next node of eight on the segment start -> goal, linked to the
        // previous one; the eighth links to the goal as well
        const int d = r->dim, k = (int)n - 1;  // 1 .. 7
        std::vector<double> q(d);
        for (int i = 0; i < d; ++i) {
            const double a = r->st[(size_t)r->start * d + i], b = r->st[(size_t)r->goal * d + i];
            q[i] = a + (b - a) * k / 8.0;
        }
        const int id = prm_add(r, q.data());
        auto link = [&](int x, int y) {
            r->ef.push_back(x > y ? x : y);
            r->et.push_back(x > y ? y : x);
            r->ed.push_back(l2(&r->st[(size_t)x * d], &r->st[(size_t)y * d], d));
        };
        link(id, r->last);
        r->last = id;
        if (k == 7) {
            link(id, r->goal);
            r->solved = true;
        }
        ++r->waves;
    }
    if (solved) *solved = r->solved;
    return MPTG_OK;
}
mptg_status mptg_prm_size(mptg_prm* r, size_t* nodes, size_t* edges) {
    if (nodes) *nodes = r->st.size() / r->dim;
    if (edges) *edges = r->ef.size();
    return MPTG_OK;
}
mptg_status mptg_prm_graph(mptg_prm* r, double* states, size_t cap_nodes, int32_t* from, int32_t* to,
                           double* dist, size_t cap_edges, size_t* n, size_t* ne) {
    const size_t nn = r->st.size() / r->dim;
    *n = nn;
    *ne = r->ef.size();
    if ((states && cap_nodes < nn) || ((from || to || dist) && cap_edges < r->ef.size()))
        return fail(r->ctx, "graph does not fit", MPTG_ERR_CAPACITY);
    if (states) std::memcpy(states, r->st.data(), r->st.size() * sizeof(double));
    for (size_t e = 0; e < r->ef.size(); ++e) {
        if (from) from[e] = r->ef[e];
        if (to) to[e] = r->et[e];
        if (dist) dist[e] = r->ed[e];
    }
    return MPTG_OK;
}
mptg_status mptg_prm_solution(mptg_prm* r, double* path, size_t cap, size_t* len, double* cost) {
    std::vector<int> ids;
    if (r->solved) {
        ids.push_back(r->start);
        for (size_t i = 2; i < r->st.size() / r->dim; ++i) ids.push_back((int)i);
        ids.push_back(r->goal);
    }
    if (cost) {
        double c = r->solved ? 0 : INFINITY;
        for (size_t i = 1; i < ids.size(); ++i)
            c += l2(&r->st[(size_t)ids[i] * r->dim], &r->st[(size_t)ids[i - 1] * r->dim], r->dim);
        *cost = c;
    }
    return read_path(r->ctx, r->st, r->dim, ids, path, cap, len);
}
mptg_status mptg_prm_stats(mptg_prm* r, uint64_t out[8]) {
    out[0] = r->waves;
    out[1] = out[2] = r->waves;
    out[3] = 0;
    out[4] = out[5] = r->ef.size();
    out[6] = r->goal >= 0;
    out[7] = r->solved;
    return MPTG_OK;
}

}  // extern "C"
