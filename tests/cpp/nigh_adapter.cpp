// The nigh adapter (include/mptg_nigh.hpp) under the reference's own planners.
// (1) The container against brute force: nearest, k-nearest with both tuple
//     orders, the radius, the 64-neighbour limit, the empty container.
// (2) MPT's PRRT, PRRT* and PPRM (src/mpt/*.hpp, compiled in place) with
//     PRRT<mpt_gb300::GpuKDTree>, ... on a 2-D world with a wall, checked by
//     the acceptance rules of test/planner_integration_test.hpp:219-291.
// Built by tests/test_nigh_adapter.py against the C ABI (the real libmptg,
// or the CPU stand-in tests/cpp/fake_mptg_nn.cpp where there is no GPU).
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <random>
#include <stdexcept>
#include <tuple>
#include <vector>

#include <mpt/lp_space.hpp>  // interpolate() before the DMV that calls it
#include <mpt/discrete_motion_validator.hpp>
#include <mpt/goal_state.hpp>
#include <mpt/pprm.hpp>
#include <mpt/prrt.hpp>
#include <mpt/prrt_star.hpp>

#include "mptg_nigh.hpp"

namespace mpt = unc::robotics::mpt;
namespace nigh = unc::robotics::nigh;
namespace nm = unc::robotics::nigh::metric;
using unc::robotics::mpt_gb300::GpuKDTree;

using State = std::array<double, 2>;
using Space = nm::Space<State, nm::LP<2>>;

#define CHECK(c)                                                        \
    do {                                                                \
        if (!(c)) {                                                     \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c); \
            return 1;                                                   \
        }                                                               \
    } while (0)

namespace {

struct Elem {
    int id;
    State q;
};
struct ElemKey {
    const State& operator()(const Elem* e) const { return e->q; }
};

int container_checks() {
    Space space;
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> u(0, 100);
    nigh::Nigh<Elem*, Space, ElemKey, nigh::Concurrent, GpuKDTree> nn(space, ElemKey{}, 4096);
    CHECK(nn.size() == 0);
    CHECK(!nn.nearest(State{1, 2}));
    std::vector<Elem> elems(1000);
    for (int i = 0; i < 1000; ++i) {
        elems[i].id = i;
        // every tenth element duplicates an earlier one: ties go to the earlier
        elems[i].q = (i % 10 == 9) ? elems[i - 5].q : State{u(rng), u(rng)};
        nn.insert(&elems[i]);
    }
    CHECK(nn.size() == 1000);
    for (int t = 0; t < 200; ++t) {
        State q = t < 20 ? elems[t * 37 + 9].q : State{u(rng), u(rng)};
        int best = -1;
        double bd = 0;
        std::vector<std::pair<double, int>> all;
        for (int i = 0; i < 1000; ++i) {
            double d = space.distance(elems[i].q, q);
            all.emplace_back(d, i);
            if (best < 0 || d < bd) { best = i; bd = d; }
        }
        auto r = nn.nearest(q);
        CHECK(r && r->first->id == best && r->second == bd);
        std::sort(all.begin(), all.end());
        std::vector<std::tuple<Elem*, double>> a;  // PRRT*'s order
        std::vector<std::tuple<double, Elem*>> b;  // PPRM's order
        nn.nearest(a, q, 10);
        nn.nearest(b, q, 10);
        CHECK(a.size() == 10 && b.size() == 10);
        for (int s = 0; s < 10; ++s) {
            CHECK(std::get<0>(a[s])->id == all[s].second && std::get<1>(a[s]) == all[s].first);
            CHECK(std::get<1>(b[s])->id == all[s].second && std::get<0>(b[s]) == all[s].first);
        }
        double rad = 6.0;
        nn.nearest(a, q, 64, rad);
        std::size_t within = 0;
        while (within < all.size() && all[within].first <= rad) ++within;
        CHECK(a.size() == std::min<std::size_t>(within, 64));
    }
    std::vector<std::tuple<Elem*, double>> many;
    bool threw = false;
    try {
        nn.nearest(many, State{50, 50}, 100);
    } catch (const std::length_error&) {
        threw = true;
    }
    CHECK(threw);
    return 0;
}

struct WallValidator {
    bool operator()(const State& q) const {
        return q[0] >= 0 && q[0] <= 100 && q[1] >= 0 && q[1] <= 100 && !(q[0] > 45 && q[0] < 55 && q[1] < 80);
    }
};

// a 2-D world [0, 100]^2 with a wall x in (45, 55), y < 80
struct WallScenario {
    using Space = ::Space;
    using State = ::State;
    Space space_;
    mpt::GoalState<Space> goal_{1.0, State{90, 10}};
    mpt::DiscreteMotionValidator<Space, WallValidator> dmv_{space_, 0.25};

    struct Sampler {
        template <class RNG>
        State operator()(RNG& rng) const {
            std::uniform_real_distribution<double> u(0, 100);
            return State{u(rng), u(rng)};
        }
    };
    Sampler sampler() const { return Sampler{}; }
    const Space& space() const { return space_; }
    const mpt::GoalState<Space>& goal() const { return goal_; }
    bool valid(const State& q) const { return WallValidator{}(q); }
    bool link(const State& a, const State& b) const { return dmv_(a, b); }
};

template <class Planner, class Setup>
int planner_checks(const char* name, Setup setup) {
    WallScenario sc;
    Planner planner(sc);
    planner.addStart(State{10, 10});
    setup(planner);
    planner.solveFor([&] { return planner.solved(); }, std::chrono::seconds(30));
    CHECK(planner.solved());
    std::vector<State> path = planner.solution();
    CHECK(path.size() >= 2 && path.front() == (State{10, 10}));
    CHECK(sc.space().distance(path.back(), State{90, 10}) <= 1.0);
    for (std::size_t i = 0; i < path.size(); ++i) {
        CHECK(sc.valid(path[i]));
        if (i) CHECK(sc.link(path[i - 1], path[i]));
    }
    std::printf("%s: %zu nodes, %zu waypoints\n", name, planner.size(), path.size());
    return 0;
}

}  // namespace

// the strategy option is found in any position of the pack, as nigh's are
// (test/pack_nearest_test.cpp)
static_assert(std::is_same_v<mpt::impl::pack_nearest_t<GpuKDTree, mpt::single_threaded>, GpuKDTree>);
static_assert(std::is_same_v<mpt::impl::pack_nearest_t<mpt::report_stats<true>, GpuKDTree>, GpuKDTree>);
static_assert(std::is_same_v<mpt::PRRT<GpuKDTree, mpt::single_threaded>, mpt::PRRT<mpt::single_threaded, GpuKDTree>>);

int main() {
    auto range = [](auto& p) { p.setRange(5); };
    auto goal = [](auto& p) { p.addGoal(State{90, 10}); };
    if (container_checks()) return 1;
    if (planner_checks<mpt::Planner<WallScenario, mpt::PRRT<GpuKDTree, mpt::single_threaded>>>("PRRT", range))
        return 1;
    if (planner_checks<mpt::Planner<WallScenario, mpt::PRRT<GpuKDTree>>>("PRRT, OpenMP workers", range)) return 1;
    if (planner_checks<mpt::Planner<WallScenario, mpt::PRRTStar<GpuKDTree, mpt::single_threaded>>>("PRRT*", range))
        return 1;
    if (planner_checks<mpt::Planner<WallScenario, mpt::PPRM<GpuKDTree, mpt::single_threaded>>>("PPRM", goal))
        return 1;
    std::printf("nigh adapter OK\n");
    return 0;
}
