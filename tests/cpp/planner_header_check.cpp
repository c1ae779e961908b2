// Host-side check of include/mptg_planner.hpp against the scripted stand-in of
// the C ABI (tests/cpp/fake_mptg_planner.cpp): the parameters, bounds, goal,
// rewiring and starts the header forwards; its solve loops (poll limits,
// deadlines, the node budget, stop_when_solved); status codes turned into the
// reference's exceptions (src/mpt/impl/prrt/prrt.hpp:197-198,
// src/mpt/impl/pprm/pprm.hpp:173-183); the vector and callback forms of
// solution() (prrt.hpp:263-285); visitGraph (prrt.hpp:300-316,
// pprm.hpp:381-388); and handle release.  Exit status 0 on success.
#include <mptg_planner.hpp>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

struct FakePlannerLog {
    int device;
    int scene_kind;
    mptg_plan_params params;
    int has_bounds;
    double lo[8], hi[8];
    double goal[8], goal_radius;
    int rewire;
    double rewire_factor;
    int runs;
    double min_limit, max_limit;
    int unlimited_runs;
    int stop_after_solved;
    int prm_runs;
    int live_ctx, live_scene, live_planner, live_prm;
    int fail_create;
    int fail_run;
};
extern "C" FakePlannerLog fake_planner_log;

using namespace unc::robotics::mpt_gb300;
using Clock = std::chrono::steady_clock;

struct GridScenario {
    using State = std::array<double, 2>;
    std::vector<uint8_t> cells = std::vector<uint8_t>(64 * 64, 0);
    State goal_state{60.0, 40.0};
    GridScene gpu_scene() const { return GridScene{cells.data(), 64, 64}; }
    std::pair<State, State> bounds() const { return {State{0, 0}, State{64, 64}}; }
    GoalState<State> goal() const { return GoalState<State>(1e-9, goal_state); }
    double link_step() const { return 0.25; }
};

#define CHECK(c)                                                             \
    do {                                                                     \
        if (!(c)) {                                                          \
            std::fprintf(stderr, "FAILED %s at line %d\n", #c, __LINE__);   \
            return 1;                                                        \
        }                                                                    \
    } while (0)

template <class Fn>
static bool throws_with(Fn fn, const char* text) {
    try {
        fn();
    } catch (const std::exception& e) {
        return std::strstr(e.what(), text) != nullptr;
    }
    return false;
}

static double l2(const std::array<double, 2>& a, const std::array<double, 2>& b) {
    return std::hypot(a[0] - b[0], a[1] - b[1]);
}

int main() {
    FakePlannerLog& L = fake_planner_log;
    const GridScenario sc;
    const GridScenario::State start{4.0, 8.0};
    {
        using Algo = PRRT<report_stats<true>, gpu_wavefront<256>, gpu_device<3>>;
        Planner<GridScenario, Algo> pl(sc, 42, 1000);
        CHECK(L.device == 3 && L.scene_kind == MPTG_SCENE_GRID && L.live_ctx == 1 && L.live_scene == 1);
        // no start: the reference's runtime_error, before any planner exists
        CHECK(throws_with([&] { pl.solve([] { return true; }); }, "there are no valid initial states"));
        CHECK(L.live_planner == 0);
        CHECK(throws_with([&] { pl.setRange(0.0); }, "range must be positive"));
        CHECK(throws_with([&] { pl.setGoalBias(1.5); }, "goal bias"));
        pl.setRange(4.0);
        pl.setGoalBias(0.05);
        CHECK(pl.getRange() == 4.0 && pl.getGoalBias() == 0.05);
        pl.addStart(start);  // queued until the first solve creates the planner
        CHECK(pl.size() == 1 && !pl.solved() && pl.solution().empty());
        L.runs = 0;
        pl.solveFor([&] { return pl.solved(); }, std::chrono::seconds(10));
        // what the header forwarded
        CHECK(L.live_planner == 1);
        CHECK(L.params.range == 4.0 && L.params.goal_bias == 0.05 && L.params.goal_radius == 1e-9);
        CHECK(L.params.edge_step == 0.25 && L.params.resolution == 0 && L.params.wavefront == 256);
        CHECK(L.params.seed == 42 && L.params.max_nodes == 1000);
        CHECK(L.has_bounds && L.lo[0] == 0 && L.lo[1] == 0 && L.hi[0] == 64 && L.hi[1] == 64);
        CHECK(L.goal[0] == 60.0 && L.goal[1] == 40.0 && L.goal_radius == 1e-9);
        CHECK(L.rewire == 0);
        // every call bounded by the poll period, none unlimited, and no call
        // asked to stop at a solution that was already there
        constexpr double poll = Planner<GridScenario, Algo>::kPollSeconds;
        CHECK(L.runs > 1 && L.min_limit > 0 && L.max_limit <= poll);
        CHECK(L.unlimited_runs == 0 && L.stop_after_solved == 0);
        CHECK(pl.solved());
        // the path: start first, goal last, steps of at most the range
        auto path = pl.solution();
        CHECK(path.size() > 2 && path.front() == start && path.back() == sc.goal_state);
        for (size_t i = 1; i < path.size(); ++i) CHECK(l2(path[i - 1], path[i]) <= 4.0 + 1e-12);
        size_t k = 0;
        bool same = true;
        pl.solution([&](const GridScenario::State& q) { same = same && k < path.size() && path[k++] == q; });
        CHECK(same && k == path.size());
        struct Counter {
            size_t v = 0, e = 0;
            void vertex(const GridScenario::State&) { ++v; }
            void edge(const GridScenario::State&) { ++e; }
        } cnt;
        pl.visitGraph(cnt);
        CHECK(cnt.v == pl.size() && cnt.e == pl.size() - 1);
        // parameters are fixed once the planner exists
        CHECK(throws_with([&] { pl.setRange(8.0); }, "must precede the first solve"));
        // a failed call surfaces as runtime_error carrying the library's message
        L.fail_run = 1;
        CHECK(throws_with([&] { pl.solveFor(std::chrono::milliseconds(50)); }, "mptg: injected failure"));
        // solved: a further solve keeps growing the tree without stopping at the
        // solution (stop_when_solved 0) and ends at the node budget
        L.stop_after_solved = 0;
        pl.solveFor(std::chrono::seconds(10));
        CHECK(L.stop_after_solved == 0 && pl.size() == 1000);
        pl.printStats();
    }
    CHECK(L.live_ctx == 0 && L.live_scene == 0 && L.live_planner == 0);
    {
        // the node budget ends a solve that has no other end
        Planner<GridScenario, PRRT<gpu_wavefront<64>>> pl(sc, 7, 5);
        pl.setRange(1e-3);
        pl.addStart(start);
        const auto t0 = Clock::now();
        pl.solve([] { return false; });
        CHECK(std::chrono::duration<double>(Clock::now() - t0).count() < 5.0);
        CHECK(pl.size() == 5 && !pl.solved() && pl.solution().empty());
    }
    {
        // a deadline ends a solve that neither solves nor fills its budget;
        // no call's time limit reaches past the deadline
        Planner<GridScenario, PRRT<>> pl(sc, 8, size_t(1) << 26);
        pl.setRange(1e-6);
        pl.addStart(start);
        L.runs = 0;
        const auto t0 = Clock::now();
        pl.solveFor(std::chrono::milliseconds(30));
        const double el = std::chrono::duration<double>(Clock::now() - t0).count();
        CHECK(el >= 0.03 && el < 2.0 && !pl.solved() && pl.size() > 1);
        CHECK(L.min_limit > 0 && L.max_limit <= 0.03);
    }
    {
        // no usable device: the constructor throws and leaks nothing
        L.fail_create = 1;
        CHECK(throws_with([&] { Planner<GridScenario, PRRT<>> pl(sc, 1); }, "no usable GPU"));
        CHECK(L.live_ctx == 0 && L.live_scene == 0);
    }
    {
        Planner<GridScenario, PRRTStar<gpu_wavefront<128>>> star(sc, 9, 1000);
        CHECK(throws_with([&] { star.setRewireFactor(-1.0); }, "rewire factor must be positive"));
        star.setRewireFactor(1.2);
        star.setRange(8.0);
        star.addStart(start);
        star.solveFor([&] { return star.solved(); }, std::chrono::seconds(10));
        CHECK(L.rewire == 1 && L.rewire_factor == 1.2 && L.params.wavefront == 128 && L.params.seed == 9);
        CHECK(star.solved() && star.solution().back() == sc.goal_state);
        CHECK(throws_with([&] { star.setRewireFactor(1.5); }, "must precede the first solve"));
        star.printStats();
    }
    {
        Planner<GridScenario, PPRM<gpu_wavefront<2048>, report_stats<true>>> prm(sc, 5, 100);
        CHECK(L.live_prm == 1 && L.params.wavefront == 2048 && L.params.seed == 5 && L.params.max_nodes == 100);
        CHECK(L.goal[0] == 60.0 && L.goal[1] == 40.0 && L.has_bounds);
        // "PPRM requires both start and goal configurations"
        CHECK(throws_with([&] { prm.solveFor(std::chrono::seconds(1)); }, "requires both start and goal"));
        prm.addStart(start);
        prm.addGoal(sc.goal_state);
        CHECK(prm.size() == 2 && !prm.solved());
        L.prm_runs = 0;
        prm.solveFor([&] { return prm.solved(); }, std::chrono::seconds(10));
        CHECK(prm.solved() && L.prm_runs == 7 && prm.size() == 9);
        auto path = prm.solution();
        CHECK(path.size() == 9 && path.front() == start && path.back() == sc.goal_state);
        struct Counter {
            size_t v = 0, e = 0;
            void vertex(const GridScenario::State&) { ++v; }
            void edge(const GridScenario::State&) { ++e; }
        } cnt;
        prm.visitGraph(cnt);
        CHECK(cnt.v == 9 && cnt.e == 2 * 8);  // every edge seen from both ends
        // a solve past the node budget ends when a wavefront adds nothing
        Planner<GridScenario, PPRM<>> small(sc, 6, 4);
        small.addStart(start);
        small.addGoal(sc.goal_state);
        small.solve([] { return false; });
        CHECK(small.size() == 4 && !small.solved());
        prm.printStats();
    }
    CHECK(L.live_ctx == 0 && L.live_scene == 0 && L.live_planner == 0 && L.live_prm == 0);
    std::printf("planner header OK\n");
    return 0;
}
