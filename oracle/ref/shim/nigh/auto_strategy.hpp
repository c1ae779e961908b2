// Project-written stand-in for nigh's strategy tags and its Nigh container
// (UNC-Robotics/nigh is not vendored with MPT and has no pinned version), as
// far as MPT's planners use them: insert(T), nearest(q) -> optional<pair<T,
// Distance>>, nearest(nbh, q, k, r) sorted by distance, size().  Every
// strategy tag maps to one exact brute-force container: it answers with the
// exact minimum distance under the Space's own distance(), the earliest
// inserted element on ties, which is how the oracle defines NN results.
// Concurrent containers guard the element list with a shared mutex.
#pragma once
#include <cstddef>
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
    Space space_;
    KeyFn keyFn_;
    std::vector<T> nodes_;
    mutable Mutex mutex_;

public:
    explicit Nigh(const Space& space = Space(), const KeyFn& keyFn = KeyFn()) : space_(space), keyFn_(keyFn) {}

    void insert(const T& t) {
        std::unique_lock<Mutex> lock(mutex_);
        nodes_.push_back(t);
    }

    std::size_t size() const {
        std::shared_lock<Mutex> lock(mutex_);
        return nodes_.size();
    }

    template <class Q>
    std::optional<std::pair<T, Distance>> nearest(const Q& q) const {
        std::shared_lock<Mutex> lock(mutex_);
        std::optional<std::pair<T, Distance>> best;
        for (const T& t : nodes_) {
            Distance d = space_.distance(keyFn_(t), q);
            if (!best || d < best->second) best.emplace(t, d);
        }
        return best;
    }

    // the k nearest within r, ascending distance, earlier insertion first on
    // ties; the element and its distance are placed in each tuple by type, so
    // both (T, Distance) and (Distance, T) neighbour lists work
    template <class Tuple, class Alloc, class Q>
    void nearest(std::vector<Tuple, Alloc>& nbh, const Q& q, std::size_t k,
                 Distance r = std::numeric_limits<Distance>::infinity()) const {
        std::shared_lock<Mutex> lock(mutex_);
        nbh.clear();
        for (const T& t : nodes_) {
            Distance d = space_.distance(keyFn_(t), q);
            if (!(d <= r)) continue;
            std::size_t pos = nbh.size();
            while (pos > 0 && d < std::get<Distance>(nbh[pos - 1])) --pos;
            if (pos >= k) continue;
            Tuple e;
            std::get<T>(e) = t;
            std::get<Distance>(e) = d;
            nbh.insert(nbh.begin() + pos, e);
            if (nbh.size() > k) nbh.pop_back();
        }
    }
};

}  // namespace unc::robotics::nigh
