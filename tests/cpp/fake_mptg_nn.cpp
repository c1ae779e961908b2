// A CPU stand-in for the nearest-neighbour calls of the C ABI (mptg.h):
// exact brute force, ties to the lowest id, the same argument checks and
// status codes.  TEST CODE ONLY: it lets tests/cpp/nigh_adapter.cpp check the
// nigh adapter's bookkeeping (mptg_nigh.hpp) on a machine without a GPU.
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "mptg.h"

struct mptg_ctx {
    const char* err = "";
};
struct mptg_tree {
    mptg_ctx* ctx;
    int metric, dim;
    size_t cap;
    std::vector<double> pts;
};

namespace {
const double kPi = 3.14159265358979323846;

double dist(const mptg_tree* t, const double* a, const double* b) {
    double s = 0;
    for (int i = 0; i < t->dim; ++i) {
        double d = std::fabs(a[i] - b[i]);
        if (t->metric == MPTG_METRIC_SO2) s += d > kPi ? 2 * kPi - d : d;
        else if (t->metric == MPTG_METRIC_L1) s += d;
        else s += d * d;
    }
    return t->metric == MPTG_METRIC_L2 ? std::sqrt(s) : s;
}

mptg_status fail(mptg_ctx* c, const char* msg, mptg_status s) {
    c->err = msg;
    return s;
}
}  // namespace

extern "C" {

mptg_status mptg_create(mptg_ctx** ctx, int) {
    *ctx = new mptg_ctx;
    return MPTG_OK;
}

mptg_status mptg_destroy(mptg_ctx* ctx) {
    delete ctx;
    return MPTG_OK;
}

const char* mptg_last_error(mptg_ctx* ctx) { return ctx->err; }

mptg_status mptg_tree_create(mptg_ctx* ctx, mptg_metric metric, int dim, const double*, size_t capacity,
                             mptg_tree** tree) {
    if (metric != MPTG_METRIC_L2 && metric != MPTG_METRIC_L1 && metric != MPTG_METRIC_SO2)
        return fail(ctx, "unsupported metric", MPTG_ERR_UNSUPPORTED_METRIC);
    if (dim < 1 || capacity == 0) return fail(ctx, "bad dim or capacity", MPTG_ERR_INVALID_ARG);
    *tree = new mptg_tree{ctx, int(metric), dim, capacity, {}};
    return MPTG_OK;
}

mptg_status mptg_tree_destroy(mptg_tree* tree) {
    delete tree;
    return MPTG_OK;
}

mptg_status mptg_tree_insert(mptg_tree* t, const double* states, size_t n, void*) {
    if (t->pts.size() / t->dim + n > t->cap) return fail(t->ctx, "tree capacity exceeded", MPTG_ERR_CAPACITY);
    t->pts.insert(t->pts.end(), states, states + n * t->dim);
    return MPTG_OK;
}

mptg_status mptg_nearest(mptg_tree* t, const double* q, size_t nq, int32_t* idx, double* d, void*) {
    size_t n = t->pts.size() / t->dim;
    for (size_t j = 0; j < nq; ++j) {
        idx[j] = -1;
        d[j] = std::numeric_limits<double>::infinity();
        for (size_t i = 0; i < n; ++i) {
            double e = dist(t, &t->pts[i * t->dim], q + j * t->dim);
            if (e < d[j]) { d[j] = e; idx[j] = int32_t(i); }
        }
    }
    return MPTG_OK;
}

mptg_status mptg_nearest_k(mptg_tree* t, const double* q, size_t nq, int k, double r, int32_t* idx, double* d,
                           void*) {
    if (k < 1 || k > 64) return fail(t->ctx, "k must be in [1, 64]", MPTG_ERR_INVALID_ARG);
    if (!(r > 0)) r = std::numeric_limits<double>::infinity();
    size_t n = t->pts.size() / t->dim;
    for (size_t j = 0; j < nq; ++j) {
        std::vector<std::pair<double, int32_t>> all;
        for (size_t i = 0; i < n; ++i) {
            double e = dist(t, &t->pts[i * t->dim], q + j * t->dim);
            if (e <= r) all.emplace_back(e, int32_t(i));
        }
        std::sort(all.begin(), all.end());
        for (int s = 0; s < k; ++s) {
            idx[j * k + s] = s < int(all.size()) ? all[s].second : -1;
            d[j * k + s] = s < int(all.size()) ? all[s].first : std::numeric_limits<double>::infinity();
        }
    }
    return MPTG_OK;
}

}  // extern "C"
