// C++ drop-in check of include/mptg_planner.hpp, modelled on the reference's
// planner acceptance test (test/planner_integration_test.hpp:219-291):
// solve until solved (10 s cap), solved() is true, the path has more than two
// waypoints, starts at the start and ends at the goal, and the callback and
// vector forms of solution() agree.  Exit status 0 on success.
#include <mptg_planner.hpp>

#include <cmath>
#include <cstdio>
#include <type_traits>

using namespace unc::robotics::mpt_gb300;

// a 1024 x 1024 grid with a wall across the middle and one gap
struct WallScenario {
    using State = std::array<double, 2>;
    std::vector<uint8_t> cells;
    WallScenario() : cells(1024 * 1024, 0) {
        for (int y = 500; y < 540; ++y)
            for (int x = 0; x < 1024; ++x)
                if (x < 700 || x > 760) cells[(size_t)y * 1024 + x] = 1;
    }
    GridScene gpu_scene() const { return GridScene{cells.data(), 1024, 1024}; }
    std::pair<State, State> bounds() const { return {State{0, 0}, State{1024, 1024}}; }
    GoalState<State> goal() const { return GoalState<State>(1e-6, State{900.0, 900.0}); }
    double link_step() const { return 1.0; }
    static State startState() { return State{100.0, 100.0}; }
};

#define CHECK(c)                                                             \
    do {                                                                     \
        if (!(c)) {                                                          \
            std::fprintf(stderr, "FAILED %s at line %d\n", #c, __LINE__);   \
            return 1;                                                        \
        }                                                                    \
    } while (0)

int main() {
    // option packs resolve independent of order (prrt_integration_test.cpp:35-42)
    static_assert(PRRT<gpu_wavefront<512>, single_threaded, report_stats<true>>::wavefront ==
                  PRRT<report_stats<true>, gpu_wavefront<512>, single_threaded>::wavefront);
    static_assert(PRRT<report_stats<true>, gpu_wavefront<512>>::stats);
    static_assert(PRRT<gpu_wavefront<64>, gpu_device<1>>::device == 1 && PRRT<gpu_wavefront<64>>::device == 0);

    WallScenario sc;
    Planner<WallScenario, PRRT<gpu_wavefront<1024>, report_stats<true>>> planner(sc, 42);
    bool threw = false;
    try {
        planner.solve([] { return true; });
    } catch (const std::runtime_error&) {
        threw = true;  // "there are no valid initial states"
    }
    CHECK(threw);
    planner.setRange(32.0);
    planner.setGoalBias(0.05);
    CHECK(planner.getRange() == 32.0);
    planner.addStart(WallScenario::startState());
    planner.solveFor([&] { return planner.solved(); }, std::chrono::seconds(10));
    planner.printStats();
    CHECK(planner.solved());
    auto path = planner.solution();
    CHECK(path.size() > 2);
    CHECK(path.front() == WallScenario::startState());
    CHECK(path.back() == sc.goal().state);
    auto it = path.begin();
    bool same = true;
    planner.solution([&](const WallScenario::State& q) { same = same && it != path.end() && *it++ == q; });
    CHECK(same && it == path.end());
    // the path crosses the wall through the gap
    bool through_gap = false;
    for (size_t i = 1; i < path.size(); ++i)
        if ((path[i - 1][1] < 520) != (path[i][1] < 520))
            through_gap = through_gap || (path[i][0] > 690 && path[i][0] < 770);
    CHECK(through_gap);
    struct Counter {
        size_t v = 0, e = 0;
        void vertex(const WallScenario::State&) { ++v; }
        void edge(const WallScenario::State&) { ++e; }
    } cnt;
    planner.visitGraph(cnt);
    CHECK(cnt.v == planner.size());
    CHECK(cnt.e == planner.size() - 1);

    // Planner<Scenario, PRRTStar<...>>: the same contract, rewiring on
    Planner<WallScenario, PRRTStar<gpu_wavefront<1024>, report_stats<true>>> star(sc, 42);
    star.setRange(32.0);
    star.setGoalBias(0.05);
    star.setRewireFactor(1.2);
    CHECK(star.getRewireFactor() == 1.2);
    star.addStart(WallScenario::startState());
    star.solveFor([&] { return star.solved(); }, std::chrono::seconds(10));
    CHECK(star.solved());
    auto spath = star.solution();
    CHECK(spath.size() > 2 && spath.front() == WallScenario::startState() && spath.back() == sc.goal().state);
    bool threw2 = false;
    try {
        star.setRewireFactor(1.5);
    } catch (const std::logic_error&) {
        threw2 = true;
    }
    CHECK(threw2);
    star.printStats();

    // Planner<Scenario, PPRM<...>>: roadmap with explicit start and goal
    Planner<WallScenario, PPRM<gpu_wavefront<2048>, report_stats<true>>> prm(sc, 7);
    bool threw3 = false;
    try {
        prm.solveFor(std::chrono::seconds(1));  // "PPRM requires both start and goal configurations"
    } catch (const std::runtime_error&) {
        threw3 = true;
    }
    CHECK(threw3);
    prm.addStart(WallScenario::startState());
    prm.addGoal(sc.goal().state);
    CHECK(prm.size() == 2);
    prm.solveFor([&] { return prm.solved(); }, std::chrono::seconds(10));
    CHECK(prm.solved());
    auto ppath = prm.solution();
    CHECK(ppath.size() >= 2 && ppath.front() == WallScenario::startState() && ppath.back() == sc.goal().state);
    Counter pc;
    prm.visitGraph(pc);
    CHECK(pc.v == prm.size() && pc.e > pc.v && pc.e % 2 == 0);
    prm.printStats();
    std::printf("C++ Planner OK: %zu waypoints, %zu nodes; PRRTStar %zu waypoints; PPRM %zu waypoints\n",
                path.size(), planner.size(), spath.size(), ppath.size());
    return 0;
}
