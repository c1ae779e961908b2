// Project-written stand-in for nigh's strategy tags and its Nigh container
// (UNC-Robotics/nigh is not vendored with MPT and has no pinned version), as
// far as MPT's planners use them: insert(T), nearest(q) -> optional<pair<T,
// Distance>>, nearest(nbh, q, k, r) sorted by distance, size().  Every
// strategy tag maps to one exact container -- a forest of vantage-point trees
// over the older elements plus a linear scan of the newest, standing in for
// nigh's KDTreeBatch -- that answers with the exact minimum distance under the
// Space's own distance(), the earliest inserted element on ties, which is how
// the oracle defines NN results.  Concurrent containers guard it with a shared
// mutex.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <memory>
#include <mutex>
#include <optional>
#include <shared_mutex>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "shim_metric.hpp"

namespace unc::robotics::nigh {

struct Concurrent {};
struct NoThreadSafety {};
struct Linear {};
template <std::size_t batchSize = 8> struct KDTreeBatch {};
template <unsigned degree = 8, unsigned minDegree = 4, unsigned maxDegree = 12, unsigned maxNumPtsPerLeaf = 50,
          unsigned removedCacheSize = 500, bool rebalancing = false>
struct GNAT {};

template <class Space, class Concurrency, class = void>
struct auto_strategy { using type = Linear; };
template <class Space, class Concurrency>
using auto_strategy_t = typename auto_strategy<Space, Concurrency>::type;

namespace impl {
struct NoLock {
    void lock() {}
    void unlock() {}
    void lock_shared() {}
    void unlock_shared() {}
};
}  // namespace impl

template <class T, class Space, class KeyFn, class Concurrency = NoThreadSafety, class Strategy = Linear>
class Nigh {
public:
    using Key = typename Space::Type;
    using Distance = typename Space::Distance;

private:
    using Mutex = std::conditional_t<std::is_same_v<Concurrency, Concurrent>, std::shared_mutex, impl::NoLock>;
    // The newest elements (fewer than kBuffer) are scanned linearly; the rest
    // are indexed by a logarithmic forest of static vantage-point trees
    // (Bentley and Saxe's binary-counter method: blocks of kBuffer * 2^j
    // consecutive insertions, two equal blocks merged and rebuilt).  A VP-tree
    // node splits its points at the median distance mu from its vantage point;
    // the triangle inequality bounds the distance from a query to every point
    // of either side, so the search needs only Space::distance().
    static constexpr std::size_t kBuffer = 64;
    static constexpr std::size_t kLeaf = 12;
    struct VPNode {
        std::size_t vp;       // vantage point (insertion id); leaf: unused
        Distance mu;
        std::int64_t inner;   // child indices; -1 marks a leaf
        std::int64_t outer;
        std::size_t lo, hi;   // leaf: range of ids_
    };
    struct Block {
        std::size_t first = 0, count = 0;
        std::vector<VPNode> nodes;
        std::vector<std::size_t> ids;
    };
    Space space_;
    KeyFn keyFn_;
    std::vector<T> nodes_;
    std::vector<Block> blocks_;  // disjoint, in insertion order, sizes decreasing
    std::size_t indexed_ = 0;    // nodes_[0, indexed_) are in blocks_
    mutable Mutex mutex_;

    // Pruning is exact up to rounding: a bound is discarded only when it
    // exceeds the current best by more than the distances' worst rounding
    // error (the SO(3) angle acos(|a.b|) can be off by ~3e-8 near 0), so the
    // earliest-inserted of equally near elements is never skipped.
    static Distance slack(Distance best) { return Distance(1e-6) + Distance(1e-12) * best; }

    Distance dist(std::size_t id, const Key& q) const { return space_.distance(keyFn_(nodes_[id]), q); }

    std::int64_t build(Block& b, std::size_t lo, std::size_t hi, std::vector<std::pair<Distance, std::size_t>>& tmp) {
        std::int64_t me = (std::int64_t)b.nodes.size();
        b.nodes.push_back(VPNode{0, 0, -1, -1, lo, hi});
        if (hi - lo <= kLeaf) return me;
        std::size_t vp = b.ids[lo + (hi - lo) / 2];
        std::swap(b.ids[lo + (hi - lo) / 2], b.ids[lo]);
        tmp.clear();
        for (std::size_t i = lo + 1; i < hi; ++i)
            tmp.emplace_back(space_.distance(keyFn_(nodes_[vp]), keyFn_(nodes_[b.ids[i]])), b.ids[i]);
        std::size_t m = tmp.size() / 2;
        std::nth_element(tmp.begin(), tmp.begin() + m, tmp.end());
        for (std::size_t i = 0; i < tmp.size(); ++i) b.ids[lo + 1 + i] = tmp[i].second;
        Distance mu = tmp[m].first;
        std::size_t mid = lo + 1 + m + 1;  // inner [lo+1, mid): d <= mu; outer [mid, hi): d >= mu
        std::int64_t in = build(b, lo + 1, mid, tmp);
        std::int64_t out = build(b, mid, hi, tmp);
        b.nodes[me] = VPNode{vp, mu, in, out, 0, 0};
        return me;
    }

    void index_buffer() {
        Block nb;
        nb.first = indexed_;
        nb.count = kBuffer;
        while (!blocks_.empty() && blocks_.back().count == nb.count) {
            nb.first = blocks_.back().first;
            nb.count *= 2;
            blocks_.pop_back();
        }
        nb.ids.resize(nb.count);
        for (std::size_t i = 0; i < nb.count; ++i) nb.ids[i] = nb.first + i;
        std::vector<std::pair<Distance, std::size_t>> tmp;
        tmp.reserve(nb.count);
        build(nb, 0, nb.count, tmp);
        blocks_.push_back(std::move(nb));
        indexed_ += kBuffer;
    }

    // (distance, insertion id) order: nearer first, earlier inserted on ties
    static bool before(Distance d, std::size_t id, Distance bd, std::size_t bid) {
        return d < bd || (d == bd && id < bid);
    }

    // Visitor interface: bound() is the distance beyond which nothing is
    // wanted; offer(d, id) takes a candidate.
    template <class V>
    void search(const Block& b, std::int64_t n, const Key& q, V& v) const {
        const VPNode& nd = b.nodes[(std::size_t)n];
        if (nd.inner < 0) {
            for (std::size_t i = nd.lo; i < nd.hi; ++i) v.offer(dist(b.ids[i], q), b.ids[i]);
            return;
        }
        Distance d = dist(nd.vp, q);
        v.offer(d, nd.vp);
        auto inner_ok = [&] { return !(d - nd.mu > v.bound() + slack(v.bound())); };
        auto outer_ok = [&] { return !(nd.mu - d > v.bound() + slack(v.bound())); };
        if (d <= nd.mu) {
            if (inner_ok()) search(b, nd.inner, q, v);
            if (outer_ok()) search(b, nd.outer, q, v);
        } else {
            if (outer_ok()) search(b, nd.outer, q, v);
            if (inner_ok()) search(b, nd.inner, q, v);
        }
    }

    template <class V>
    void visit_all(const Key& q, V& v) const {
        for (const Block& b : blocks_) search(b, 0, q, v);
        for (std::size_t id = indexed_; id < nodes_.size(); ++id) v.offer(dist(id, q), id);
    }

    struct Nearest1 {
        Distance best = std::numeric_limits<Distance>::infinity();
        std::size_t bid = std::numeric_limits<std::size_t>::max();
        Distance bound() const { return best; }
        void offer(Distance d, std::size_t id) {
            if (d == d && before(d, id, best, bid)) { best = d; bid = id; }
        }
    };

    struct NearestK {
        std::size_t k;
        Distance r;
        std::vector<std::pair<Distance, std::size_t>> list;  // sorted by (d, id), at most k
        Distance bound() const { return list.size() < k ? r : std::min(r, list.back().first); }
        void offer(Distance d, std::size_t id) {
            if (!(d <= r)) return;
            if (list.size() == k && !before(d, id, list.back().first, list.back().second)) return;
            auto pos = std::upper_bound(list.begin(), list.end(), std::make_pair(d, id),
                                        [](const auto& a, const auto& b) { return before(a.first, a.second, b.first, b.second); });
            list.insert(pos, std::make_pair(d, id));
            if (list.size() > k) list.pop_back();
        }
    };

public:
    explicit Nigh(const Space& space = Space(), const KeyFn& keyFn = KeyFn()) : space_(space), keyFn_(keyFn) {}

    void insert(const T& t) {
        std::unique_lock<Mutex> lock(mutex_);
        nodes_.push_back(t);
        if (nodes_.size() - indexed_ >= kBuffer) index_buffer();
    }

    std::size_t size() const {
        std::shared_lock<Mutex> lock(mutex_);
        return nodes_.size();
    }

    template <class Q>
    std::optional<std::pair<T, Distance>> nearest(const Q& q) const {
        std::shared_lock<Mutex> lock(mutex_);
        Nearest1 v;
        visit_all(q, v);
        if (v.bid == std::numeric_limits<std::size_t>::max()) return std::nullopt;
        return std::make_pair(nodes_[v.bid], v.best);
    }

    // the k nearest within r, ascending distance, earlier insertion first on
    // ties; the element and its distance are placed in each tuple by type, so
    // both (T, Distance) and (Distance, T) neighbour lists work
    template <class Tuple, class Alloc, class Q>
    void nearest(std::vector<Tuple, Alloc>& nbh, const Q& q, std::size_t k,
                 Distance r = std::numeric_limits<Distance>::infinity()) const {
        std::shared_lock<Mutex> lock(mutex_);
        nbh.clear();
        if (k == 0) return;
        NearestK v{k, r, {}};
        visit_all(q, v);
        for (const auto& e : v.list) {
            Tuple t;
            std::get<T>(t) = nodes_[e.second];
            std::get<Distance>(t) = e.first;
            nbh.push_back(t);
        }
    }
};

}  // namespace unc::robotics::nigh
