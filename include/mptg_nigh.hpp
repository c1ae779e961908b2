// mptg_nigh.hpp - the GB300 nearest-neighbour tree as a nigh strategy, so
// that MPT's own planners run unchanged on it:
//
//   #include <mpt/prrt.hpp>
//   #include "mptg_nigh.hpp"
//   using namespace unc::robotics;
//   mpt::Planner<Scenario, mpt::PRRT<mpt_gb300::GpuKDTree>> planner(scenario);
//
// It replaces the container nigh::Nigh<Node*, Space, NodeKey, Concurrency,
// Strategy> that the planners construct (src/mpt/impl/prrt/prrt.hpp:121-122,
// src/mpt/impl/prrt_star/prrt_star.hpp:182-183, src/mpt/impl/pprm/pprm.hpp)
// and the strategy option parsed by src/mpt/impl/pack_nearest.hpp.  Every
// call goes through the C ABI (mptg.h): insert -> mptg_tree_insert,
// nearest(q) -> mptg_nearest, nearest(nbh, q, k, r) -> mptg_nearest_k.
//
// One query per call, so this is latency-bound: it exists for drop-in
// parity.  The throughput path is the wavefront planner (mptg_planner.hpp),
// which batches thousands of queries per launch.
//
// Requirements on the Space (nigh::metric::Space<T, M>): Type, Distance,
// dimensions() and the static coeff(q, i) accessor, and an mptg_metric for
// its metric through mpt_gb300::nigh_metric<Space> (L2, L1, SO(2) and SO(3)
// are provided; specialise it for others, e.g. a weighted SE(3)).  A Space
// without one is a compile-time error, not a CPU fallback.
#pragma once

#include <cstddef>
#include <limits>
#include <mutex>
#include <optional>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "mptg.h"

#if __has_include(<nigh/nigh_forward.hpp>)
#include <nigh/nigh_forward.hpp>
#endif
#if __has_include(<mpt/impl/pack_nearest.hpp>)
#include <mpt/impl/pack_nearest.hpp>
#define MPTG_NIGH_HAVE_MPT 1
#endif

namespace unc::robotics::mpt_gb300 {

// the strategy tag: PRRT<GpuKDTree>, PRRTStar<GpuKDTree>, PPRM<GpuKDTree>
struct GpuKDTree {};

// mptg_metric (and weights) of a nigh Space
template <class Space, class = void>
struct nigh_metric;  // undefined: the Space has no GPU metric

template <class T, int p>
struct nigh_metric<nigh::metric::Space<T, nigh::metric::LP<p>>> {
    static_assert(p == 1 || p == 2, "the GPU tree supports L1 and L2 spaces");
    static constexpr mptg_metric value = p == 1 ? MPTG_METRIC_L1 : MPTG_METRIC_L2;
    static const double* weights() { return nullptr; }
};

template <class T, int p>
struct nigh_metric<nigh::metric::Space<T, nigh::metric::SO2<p>>> {
    static_assert(p == 1, "the GPU tree supports SO(2)^n with the summed (p = 1) distance");
    static constexpr mptg_metric value = MPTG_METRIC_SO2;
    static const double* weights() { return nullptr; }
};

template <class T>
struct nigh_metric<nigh::metric::Space<T, nigh::metric::SO3>> {
    static constexpr mptg_metric value = MPTG_METRIC_SO3;
    static const double* weights() { return nullptr; }
};

// default tree capacity (states); the tree reports MPTG_ERR_CAPACITY past it
inline constexpr std::size_t kNighDefaultCapacity = std::size_t(1) << 22;

}  // namespace unc::robotics::mpt_gb300

#ifdef MPTG_NIGH_HAVE_MPT
namespace unc::robotics::mpt::impl {
// PRRT<GpuKDTree, ...> selects the GPU tree, like nigh::KDTreeBatch<> in
// src/mpt/impl/pack_nearest.hpp
template <typename... Rest>
struct pack_nearest<mpt_gb300::GpuKDTree, Rest...> {
    using type = mpt_gb300::GpuKDTree;
    static_assert(std::is_void_v<pack_nearest_t<Rest...>>, "multiple nearest neighbor strategies");
};
}  // namespace unc::robotics::mpt::impl
#endif

namespace unc::robotics::nigh {

template <class T, class Space, class KeyFn, class Concurrency>
class Nigh<T, Space, KeyFn, Concurrency, mpt_gb300::GpuKDTree> {
public:
    using Key = typename Space::Type;
    using Distance = typename Space::Distance;

private:
    using Metric = mpt_gb300::nigh_metric<Space>;
    static constexpr int kMaxK = 64;  // mptg_nearest_k's limit

    Space space_;
    KeyFn keyFn_;
    int dim_;
    mptg_ctx* ctx_ = nullptr;
    mptg_tree* tree_ = nullptr;
    std::vector<T> nodes_;           // id -> element
    mutable std::vector<double> q_;  // one state, row-major doubles
    // the C ABI is not re-entrant on one context: every call is serialised,
    // which also makes the container safe under nigh::Concurrent
    mutable std::mutex mutex_;

    void check(mptg_status s, const char* what) const {
        if (s != MPTG_OK)
            throw std::runtime_error(std::string(what) + ": " + (ctx_ ? mptg_last_error(ctx_) : "no context"));
    }

    template <class Q>
    const double* flatten(const Q& q) const {
        for (int i = 0; i < dim_; ++i) q_[i] = double(Space::coeff(q, i));
        return q_.data();
    }

public:
    explicit Nigh(const Space& space = Space(), const KeyFn& keyFn = KeyFn(),
                  std::size_t capacity = mpt_gb300::kNighDefaultCapacity, int device = 0)
        : space_(space), keyFn_(keyFn), dim_(int(space.dimensions())), q_(std::size_t(dim_)) {
        check(mptg_create(&ctx_, device), "mptg_create");
        mptg_status s = mptg_tree_create(ctx_, Metric::value, dim_, Metric::weights(), capacity, &tree_);
        if (s != MPTG_OK) {
            std::string msg = std::string("mptg_tree_create: ") + mptg_last_error(ctx_);
            mptg_destroy(ctx_);
            throw std::runtime_error(msg);
        }
    }

    ~Nigh() {
        if (tree_) mptg_tree_destroy(tree_);
        if (ctx_) mptg_destroy(ctx_);
    }

    Nigh(const Nigh&) = delete;
    Nigh& operator=(const Nigh&) = delete;

    // nigh insert (src/mpt/impl/prrt/prrt.hpp:186,447): the element's id is
    // its insertion index
    void insert(const T& t) {
        std::lock_guard<std::mutex> lock(mutex_);
        check(mptg_tree_insert(tree_, flatten(keyFn_(t)), 1, nullptr), "mptg_tree_insert");
        nodes_.push_back(t);
    }

    std::size_t size() const {
        std::lock_guard<std::mutex> lock(mutex_);
        return nodes_.size();
    }

    // nigh nearest(q) (src/mpt/impl/prrt/prrt.hpp:406-409): the exact nearest
    // element (earliest inserted on ties); empty when the container is empty
    template <class Q>
    std::optional<std::pair<T, Distance>> nearest(const Q& q) const {
        std::lock_guard<std::mutex> lock(mutex_);
        int32_t id = -1;
        double d = 0;
        check(mptg_nearest(tree_, flatten(q), 1, &id, &d, nullptr), "mptg_nearest");
        if (id < 0) return std::nullopt;
        return std::make_pair(nodes_[std::size_t(id)], Distance(d));
    }

    // nigh nearest(nbh, q, k, r) (src/mpt/impl/rrg_rewire_neighbors.hpp:64-67,
    // 124-128; src/mpt/impl/pprm/pprm.hpp:302-304): the k nearest within r in
    // ascending distance.  The element and its distance are placed in each
    // tuple by type, for (T, Distance) and (Distance, T) lists alike.  At most
    // 64 neighbours: a request for more than 64 that finds 64 in a container
    // holding more throws std::length_error rather than truncate silently.
    template <class Tuple, class Alloc, class Q>
    void nearest(std::vector<Tuple, Alloc>& nbh, const Q& q, std::size_t k,
                 Distance r = std::numeric_limits<Distance>::infinity()) const {
        std::lock_guard<std::mutex> lock(mutex_);
        nbh.clear();
        if (k == 0) return;
        int kk = k > std::size_t(kMaxK) ? kMaxK : int(k);
        int32_t ids[kMaxK];
        double ds[kMaxK];
        check(mptg_nearest_k(tree_, flatten(q), 1, kk, double(r), ids, ds, nullptr), "mptg_nearest_k");
        if (k > std::size_t(kMaxK) && ids[kMaxK - 1] >= 0 && nodes_.size() > std::size_t(kMaxK))
            throw std::length_error("mptg_nigh: more than 64 neighbours requested and present");
        for (int i = 0; i < kk && ids[i] >= 0; ++i) {
            Tuple e;
            std::get<T>(e) = nodes_[std::size_t(ids[i])];
            std::get<Distance>(e) = Distance(ds[i]);
            nbh.push_back(e);
        }
    }
};

}  // namespace unc::robotics::nigh
