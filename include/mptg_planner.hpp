// mptg_planner.hpp - C++17 Planner<Scenario, PRRT<Options...>> over the mptg C ABI.
//
// Mirrors MPT's planner surface so that code written against
//   unc::robotics::mpt::Planner<Scenario, PRRT<options...>>
// (src/mpt/planner.hpp:46-47, src/mpt/prrt.hpp:56-82, src/mpt/impl/prrt/prrt.hpp:149-316,
// src/mpt/impl/planner_base.hpp:58-80) can switch namespaces:
//
//   Planner(scenario [, seed])            addStart(q)          solve(doneFn)
//   solveFor(duration) / solveFor(doneFn, duration)  solveUntil(...)
//   solved()  size()  setRange/getRange  setGoalBias/getGoalBias
//   solution() -> std::vector<State>      solution(fn) (waypoint callback)
//   printStats()                          visitGraph(visitor{vertex, edge})
//
// The Scenario contract is the reference's (State, goal(), bounds()) plus the
// GPU extension: gpu_scene() returns a description of the collision world
// (GridScene, PlanarArmScene or RigidMeshScene).  A Scenario without
// gpu_scene() does not compile: arbitrary C++ valid()/link() code cannot run
// on the device, and there is no CPU fallback.
//
// Option tags (src/mpt/planner_tags.hpp): gpu_wavefront<W>, report_stats<b>,
// gpu_device<id>;
// max_threads<N>, single_threaded and hardware_concurrency are accepted and
// have no effect (wavefronts replace the worker pool).
#pragma once

#include <algorithm>
#include <array>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <random>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "mptg.h"

namespace unc::robotics::mpt_gb300 {

// ---- option tags ---------------------------------------------------------
template <int W> struct gpu_wavefront {};
template <int N> struct max_threads {};
using single_threaded = max_threads<1>;
using hardware_concurrency = max_threads<0>;
template <bool enabled> struct report_stats {};
// the CUDA device a planner creates its context on (the constructor's default)
template <int index> struct gpu_device {};

namespace impl {
template <class... O> struct options;
template <> struct options<> {
    static constexpr int wavefront = 4096;
    static constexpr bool stats = false;
    static constexpr int device = 0;
};
template <int D, class... O> struct options<gpu_device<D>, O...> : options<O...> {
    static constexpr int device = D;
};
template <int W, class... O> struct options<gpu_wavefront<W>, O...> : options<O...> {
    static constexpr int wavefront = W;
};
template <bool b, class... O> struct options<report_stats<b>, O...> : options<O...> {
    static constexpr bool stats = b;
};
template <int N, class... O> struct options<max_threads<N>, O...> : options<O...> {};
}  // namespace impl

// PRRT<Options...> resolves to the same planner whatever the option order
// (src/mpt/prrt.hpp:56-71); compare PRRT<...>::wavefront / ::stats.
template <class... Options> struct PRRT {
    static constexpr int wavefront = impl::options<Options...>::wavefront;
    static constexpr bool stats = impl::options<Options...>::stats;
    static constexpr int device = impl::options<Options...>::device;
};

// ---- goal and scene descriptions --------------------------------------------
template <class State> struct GoalState {  // src/mpt/goal_state.hpp:43-90
    double radius;
    State state;
    GoalState(double r, const State& s) : radius(r), state(s) {}
};

struct GridScene {       // demo/png_2d_scenario.hpp
    const uint8_t* cells;  // width*height, non-zero = obstacle, row-major by y
    int width, height;
};
struct PlanarArmScene {  // demo/link_manipulator_scenario.hpp
    std::vector<double> link_len;
    std::vector<std::array<double, 3>> discs;  // (cx, cy, r)
    double robot_radius = 0.0;
    bool self_collision = true;
};
struct RigidMeshScene {  // demo/se3_rigid_body_scenario.hpp
    const double* robot_tris; int64_t nrobot;
    const double* env_tris; int64_t nenv;
    double w_rot = 1.0, w_pos = 1.0;
};

namespace impl {
inline void check(mptg_ctx* ctx, mptg_status st) {
    if (st != MPTG_OK) throw std::runtime_error(std::string("mptg: ") + mptg_last_error(ctx));
}
inline mptg_scene_desc desc_of(const GridScene& g) {
    mptg_scene_desc d{};
    d.kind = MPTG_SCENE_GRID; d.grid = g.cells; d.width = g.width; d.height = g.height;
    return d;
}
inline mptg_scene_desc desc_of(const PlanarArmScene& a) {
    mptg_scene_desc d{};
    d.kind = MPTG_SCENE_PLANAR_ARM;
    d.nlinks = (int)a.link_len.size(); d.link_len = a.link_len.data();
    d.ndiscs = (int)a.discs.size(); d.discs = a.discs.empty() ? nullptr : a.discs[0].data();
    d.robot_radius = a.robot_radius; d.self_collision = a.self_collision ? 1 : 0;
    return d;
}
inline mptg_scene_desc desc_of(const RigidMeshScene& m) {
    mptg_scene_desc d{};
    d.kind = MPTG_SCENE_RIGID_MESH;
    d.nrobot = m.nrobot; d.robot_tris = m.robot_tris; d.nenv = m.nenv; d.env_tris = m.env_tris;
    d.w_rot = m.w_rot; d.w_pos = m.w_pos;
    return d;
}
template <class S, class = void> struct has_gpu_scene : std::false_type {};
template <class S>
struct has_gpu_scene<S, std::void_t<decltype(std::declval<const S&>().gpu_scene())>> : std::true_type {};
template <class S, class = void> struct has_bounds : std::false_type {};
template <class S>
struct has_bounds<S, std::void_t<decltype(std::declval<const S&>().bounds())>> : std::true_type {};
template <class S, class = void> struct has_link_step : std::false_type {};
template <class S>
struct has_link_step<S, std::void_t<decltype(std::declval<const S&>().link_step())>> : std::true_type {};
template <class S, class = void> struct has_link_resolution : std::false_type {};
template <class S>
struct has_link_resolution<S, std::void_t<decltype(std::declval<const S&>().link_resolution())>> : std::true_type {};

template <class State> const double* data(const State& q) { return &q[0]; }
template <class State> double* data(State& q) { return &q[0]; }
}  // namespace impl

template <class Scenario, class Algorithm> class Planner;

template <class Scenario, class... Options>
class Planner<Scenario, PRRT<Options...>> {
    static_assert(impl::has_gpu_scene<Scenario>::value,
                  "the Scenario must describe its collision world with gpu_scene() "
                  "(GridScene, PlanarArmScene or RigidMeshScene): no CPU fallback exists");
    using Algo = PRRT<Options...>;

public:
    using State = typename Scenario::State;

protected:
    Scenario scenario_;
    uint64_t seed_;
    double range_ = -1.0;
    double goalBias_ = 0.01;
    bool rewire_ = false;       // PRRTStar
    double rewireFactor_ = 1.1;
    size_t maxNodes_;
    mptg_ctx* ctx_ = nullptr;
    mptg_scene* scene_ = nullptr;
    mptg_planner* planner_ = nullptr;
    std::vector<State> starts_;
    int dim_ = 0;

    void create() {
        if (planner_) return;
        mptg_plan_params p{};
        p.range = range_;
        p.goal_bias = goalBias_;
        auto goal = scenario_.goal();
        p.goal_radius = goal.radius;
        p.edge_step = 1.0;
        if constexpr (impl::has_link_step<Scenario>::value) p.edge_step = scenario_.link_step();
        p.resolution = 0;
        if constexpr (impl::has_link_resolution<Scenario>::value) p.resolution = scenario_.link_resolution();
        p.wavefront = Algo::wavefront;
        p.seed = seed_;
        p.max_nodes = maxNodes_;
        const double* lo = nullptr;
        const double* hi = nullptr;
        std::pair<State, State> b;
        if constexpr (impl::has_bounds<Scenario>::value) {
            b = scenario_.bounds();
            lo = impl::data(b.first);
            hi = impl::data(b.second);
        }
        impl::check(ctx_, mptg_planner_create(ctx_, scene_, &p, lo, hi, &planner_));
        impl::check(ctx_, mptg_planner_set_goal(planner_, impl::data(goal.state), goal.radius));
        if (rewire_) impl::check(ctx_, mptg_planner_set_rewire(planner_, 1, rewireFactor_));
        for (const State& q : starts_) impl::check(ctx_, mptg_planner_add_start(planner_, impl::data(q)));
        starts_.clear();
    }

public:
    // prrt.hpp:149-157; the default seed draws fresh entropy (random_device_seed.hpp)
    explicit Planner(const Scenario& scenario = Scenario(), uint64_t seed = std::random_device{}(),
                     size_t maxNodes = size_t(1) << 21,
                     int device = impl::options<Options...>::device)
        : scenario_(scenario), seed_(seed), maxNodes_(maxNodes) {
        if (mptg_create(&ctx_, device) != MPTG_OK) throw std::runtime_error("mptg: no usable GPU");
        auto d = impl::desc_of(scenario_.gpu_scene());
        impl::check(ctx_, mptg_scene_create(ctx_, &d, &scene_));
        double w[2];
        impl::check(ctx_, mptg_scene_space(scene_, &dim_, nullptr, w));
    }
    Planner(const Planner&) = delete;
    Planner& operator=(const Planner&) = delete;
    ~Planner() {
        if (planner_) mptg_planner_destroy(planner_);
        if (scene_) mptg_scene_destroy(scene_);
        if (ctx_) mptg_destroy(ctx_);
    }

    void setRange(double r) {  // prrt.hpp:168-171
        if (!(r > 0)) throw std::invalid_argument("range must be positive");
        if (planner_) throw std::logic_error("setRange must precede the first solve");
        range_ = r;
    }
    double getRange() const { return range_ > 0 ? range_ : std::numeric_limits<double>::infinity(); }
    void setGoalBias(double b) {  // prrt.hpp:159-162
        if (!(b >= 0 && b <= 1)) throw std::invalid_argument("goal bias must be in [0, 1]");
        if (planner_) throw std::logic_error("setGoalBias must precede the first solve");
        goalBias_ = b;
    }
    double getGoalBias() const { return goalBias_; }

    void addStart(const State& q) {  // prrt.hpp:181-187
        if (planner_) impl::check(ctx_, mptg_planner_add_start(planner_, impl::data(q)));
        else starts_.push_back(q);
    }

    std::size_t size() const {
        if (!planner_) return starts_.size();
        size_t n = 0;
        impl::check(ctx_, mptg_planner_size(planner_, &n));
        return n;
    }

    bool solved() const {
        if (!planner_) return false;
        size_t g = 0;
        impl::check(ctx_, mptg_planner_goals(planner_, &g));
        return g > 0;
    }

    // prrt.hpp:194-201: doneFn is polled between calls of up to kPollSeconds
    // of wavefronts (at least one), each of which also ends at the first
    // solution and at the node budget
    static constexpr double kPollSeconds = 0.005;
    template <class DoneFn>
    void solve(DoneFn done) {
        solve_until_(done, false, std::chrono::steady_clock::time_point{});
    }
    template <class Rep, class Period>
    void solveFor(const std::chrono::duration<Rep, Period>& d) {
        auto end = std::chrono::steady_clock::now() + d;
        solve_until_([&] { return std::chrono::steady_clock::now() >= end; }, true, end);
    }
    template <class DoneFn, class Rep, class Period>
    void solveFor(DoneFn done, const std::chrono::duration<Rep, Period>& d) {
        auto end = std::chrono::steady_clock::now() + d;
        solve_until_([&] { return std::chrono::steady_clock::now() >= end || done(); }, true, end);
    }
    template <class Clock, class Duration>
    void solveUntil(const std::chrono::time_point<Clock, Duration>& t) {
        solve([&] { return Clock::now() >= t; });
    }
    template <class DoneFn, class Clock, class Duration>
    void solveUntil(DoneFn done, const std::chrono::time_point<Clock, Duration>& t) {
        solve([&] { return Clock::now() >= t || done(); });
    }

    // with a deadline, each call's time limit is what is left until `end`
    template <class DoneFn>
    void solve_until_(DoneFn done, bool has_deadline, std::chrono::steady_clock::time_point end) {
        if (size() == 0) throw std::runtime_error("there are no valid initial states");
        create();
        while (!done()) {
            double limit = kPollSeconds;
            if (has_deadline) {
                double left = std::chrono::duration<double>(end - std::chrono::steady_clock::now()).count();
                if (left <= 0) break;
                limit = std::min(limit, left);
            }
            int s = 0;
            impl::check(ctx_, mptg_planner_run(planner_, 0, limit, solved() ? 0 : 1, &s));
            if (size() >= maxNodes_) break;  // node budget reached
        }
    }

    // prrt.hpp:263-274
    std::vector<State> solution() const {
        std::vector<State> path;
        if (!planner_) return path;
        size_t len = 0;
        double cost = 0;
        impl::check(ctx_, mptg_planner_solution(planner_, nullptr, 0, &len, &cost));
        if (!len) return path;
        std::vector<double> buf(len * dim_);
        impl::check(ctx_, mptg_planner_solution(planner_, buf.data(), len, &len, &cost));
        path.resize(len);
        for (size_t i = 0; i < len; ++i)
            for (int d = 0; d < dim_; ++d) path[i][d] = buf[i * dim_ + d];
        return path;
    }
    // waypoint callback form (prrt.hpp:276-285)
    template <class Fn>
    void solution(Fn fn) const {
        for (const State& q : solution()) fn(q);
    }

    // prrt.hpp:300-316
    template <class Visitor>
    void visitGraph(Visitor&& visitor) const {
        if (!planner_) return;
        size_t n = 0;
        impl::check(ctx_, mptg_planner_graph(planner_, nullptr, nullptr, 0, &n));
        std::vector<double> st(n * dim_);
        std::vector<int32_t> par(n);
        impl::check(ctx_, mptg_planner_graph(planner_, st.data(), par.data(), n, &n));
        State q, p;
        for (size_t i = 0; i < n; ++i) {
            for (int d = 0; d < dim_; ++d) q[d] = st[i * dim_ + d];
            visitor.vertex(q);
            if (par[i] >= 0) {
                for (int d = 0; d < dim_; ++d) p[d] = st[(size_t)par[i] * dim_ + d];
                visitor.edge(p);
            }
        }
    }

    void printStats() const {  // prrt.hpp:287-298
        std::printf("nodes in graph: %zu\n", size());
        if (!planner_) return;
        size_t len = 0;
        double cost = 0;
        impl::check(ctx_, mptg_planner_solution(planner_, nullptr, 0, &len, &cost));
        size_t g = 0;
        impl::check(ctx_, mptg_planner_goals(planner_, &g));
        std::printf("solutions: %zu, best cost=%g over %zu waypoints\n", g, cost, len);
        if constexpr (Algo::stats) {
            double st[8];
            impl::check(ctx_, mptg_planner_stats(planner_, st));
            std::printf("wavefronts: %.0f\nsamples: %.0f\nnodes added: %.0f\nlink states checked: %.0f\n", st[0],
                        st[1], st[2], st[5]);
            if (rewire_) {
                double rw[6];
                impl::check(ctx_, mptg_planner_rewire_stats(planner_, rw));
                std::printf("rewire count: %.0f of %.0f\n", rw[0], rw[1]);
            }
        }
    }
};

// Planner<Scenario, PRRTStar<Options...>> (src/mpt/prrt_star.hpp:56-95): the
// same wavefront planner with k-nearest rewiring (rewire_k_nearest)
template <class... Options> struct PRRTStar : PRRT<Options...> {};

template <class Scenario, class... Options>
class Planner<Scenario, PRRTStar<Options...>> : public Planner<Scenario, PRRT<Options...>> {
    using Base = Planner<Scenario, PRRT<Options...>>;

public:
    explicit Planner(const Scenario& scenario = Scenario(), uint64_t seed = std::random_device{}(),
                     size_t maxNodes = size_t(1) << 21,
                     int device = impl::options<Options...>::device)
        : Base(scenario, seed, maxNodes, device) {
        this->rewire_ = true;
    }
    // PRRTStar::setRewireFactor (src/mpt/impl/prrt_star/prrt_star.hpp:234-240)
    void setRewireFactor(double f) {
        if (!(f > 0)) throw std::invalid_argument("rewire factor must be positive");
        if (this->planner_) throw std::logic_error("setRewireFactor must precede the first solve");
        this->rewireFactor_ = f;
    }
    double getRewireFactor() const { return this->rewireFactor_; }
};

// Planner<Scenario, PPRM<Options...>> (src/mpt/pprm.hpp:56-84,
// src/mpt/impl/pprm/pprm.hpp:141-250): the k-nearest roadmap over wavefronts.
// addStart / addGoal run addSample at once (invalid or duplicate states are
// dropped, as the reference's nullptr); solve needs both.
template <class... Options> struct PPRM : PRRT<Options...> {};

template <class Scenario, class... Options>
class Planner<Scenario, PPRM<Options...>> {
    static_assert(impl::has_gpu_scene<Scenario>::value,
                  "the Scenario must describe its collision world with gpu_scene() "
                  "(GridScene, PlanarArmScene or RigidMeshScene): no CPU fallback exists");
    using Algo = PPRM<Options...>;

public:
    using State = typename Scenario::State;

private:
    Scenario scenario_;
    mptg_ctx* ctx_ = nullptr;
    mptg_scene* scene_ = nullptr;
    mptg_prm* prm_ = nullptr;
    int dim_ = 0;

    uint64_t stat(int i) const {
        uint64_t st[8];
        impl::check(ctx_, mptg_prm_stats(prm_, st));
        return st[i];
    }

public:
    explicit Planner(const Scenario& scenario = Scenario(), uint64_t seed = std::random_device{}(),
                     size_t maxNodes = size_t(1) << 21,
                     int device = impl::options<Options...>::device)
        : scenario_(scenario) {
        if (mptg_create(&ctx_, device) != MPTG_OK) throw std::runtime_error("mptg: no usable GPU");
        auto d = impl::desc_of(scenario_.gpu_scene());
        impl::check(ctx_, mptg_scene_create(ctx_, &d, &scene_));
        double w[2];
        impl::check(ctx_, mptg_scene_space(scene_, &dim_, nullptr, w));
        mptg_plan_params p{};
        auto goal = scenario_.goal();
        p.goal_radius = goal.radius;
        p.edge_step = 1.0;
        if constexpr (impl::has_link_step<Scenario>::value) p.edge_step = scenario_.link_step();
        p.resolution = 0;
        if constexpr (impl::has_link_resolution<Scenario>::value) p.resolution = scenario_.link_resolution();
        p.wavefront = Algo::wavefront;
        p.seed = seed;
        p.max_nodes = maxNodes;
        const double* lo = nullptr;
        const double* hi = nullptr;
        std::pair<State, State> b;
        if constexpr (impl::has_bounds<Scenario>::value) {
            b = scenario_.bounds();
            lo = impl::data(b.first);
            hi = impl::data(b.second);
        }
        impl::check(ctx_, mptg_prm_create(ctx_, scene_, &p, lo, hi, impl::data(goal.state), &prm_));
    }
    Planner(const Planner&) = delete;
    Planner& operator=(const Planner&) = delete;
    ~Planner() {
        if (prm_) mptg_prm_destroy(prm_);
        if (scene_) mptg_scene_destroy(scene_);
        if (ctx_) mptg_destroy(ctx_);
    }

    void addStart(const State& q) {  // pprm.hpp:157-165
        int32_t id;
        impl::check(ctx_, mptg_prm_add_start(prm_, impl::data(q), &id));
    }
    void addGoal(const State& q) {  // pprm.hpp:167-170
        int32_t id;
        impl::check(ctx_, mptg_prm_add_goal(prm_, impl::data(q), &id));
    }

    std::size_t size() const {
        size_t n = 0;
        impl::check(ctx_, mptg_prm_size(prm_, &n, nullptr));
        return n;
    }
    bool solved() const { return stat(7) != 0; }

    // pprm.hpp:173-183: doneFn is polled between wavefronts
    template <class DoneFn>
    void solve(DoneFn done) {
        while (!done()) {
            const uint64_t before = stat(0);
            int s = 0;
            impl::check(ctx_, mptg_prm_run(prm_, 1, 0.0, 0, &s));
            if (stat(0) == before) break;  // node budget reached
        }
    }
    template <class Rep, class Period>
    void solveFor(const std::chrono::duration<Rep, Period>& d) {
        auto end = std::chrono::steady_clock::now() + d;
        solve([&] { return std::chrono::steady_clock::now() >= end; });
    }
    template <class DoneFn, class Rep, class Period>
    void solveFor(DoneFn done, const std::chrono::duration<Rep, Period>& d) {
        auto end = std::chrono::steady_clock::now() + d;
        solve([&] { return std::chrono::steady_clock::now() >= end || done(); });
    }
    template <class Clock, class Duration>
    void solveUntil(const std::chrono::time_point<Clock, Duration>& t) {
        solve([&] { return Clock::now() >= t; });
    }
    template <class DoneFn, class Clock, class Duration>
    void solveUntil(DoneFn done, const std::chrono::time_point<Clock, Duration>& t) {
        solve([&] { return Clock::now() >= t || done(); });
    }

    // pprm.hpp:230-240: the shortest roadmap path from a start to a goal node
    std::vector<State> solution() const {
        std::vector<State> path;
        size_t len = 0;
        double cost = 0;
        impl::check(ctx_, mptg_prm_solution(prm_, nullptr, 0, &len, &cost));
        if (!len) return path;
        std::vector<double> buf(len * dim_);
        impl::check(ctx_, mptg_prm_solution(prm_, buf.data(), len, &len, &cost));
        path.resize(len);
        for (size_t i = 0; i < len; ++i)
            for (int d = 0; d < dim_; ++d) path[i][d] = buf[i * dim_ + d];
        return path;
    }
    template <class Fn>
    void solution(Fn fn) const {
        for (const State& q : solution()) fn(q);
    }

    // pprm.hpp:381-388: every node, then the far end of each of its edges
    template <class Visitor>
    void visitGraph(Visitor&& visitor) const {
        size_t n = 0, ne = 0;
        impl::check(ctx_, mptg_prm_size(prm_, &n, &ne));
        std::vector<double> st(n * dim_);
        std::vector<int32_t> ef(ne), et(ne);
        impl::check(ctx_, mptg_prm_graph(prm_, st.data(), n, ef.data(), et.data(), nullptr, ne, &n, &ne));
        std::vector<std::vector<int32_t>> adj(n);
        for (size_t e = 0; e < ne; ++e) {
            adj[ef[e]].push_back(et[e]);
            adj[et[e]].push_back(ef[e]);
        }
        State q, p;
        for (size_t i = 0; i < n; ++i) {
            for (int d = 0; d < dim_; ++d) q[d] = st[i * dim_ + d];
            visitor.vertex(q);
            for (int32_t j : adj[i]) {
                for (int d = 0; d < dim_; ++d) p[d] = st[(size_t)j * dim_ + d];
                visitor.edge(p);
            }
        }
    }

    void printStats() const {  // pprm.hpp:242-245
        std::printf("nodes in graph: %zu\n", size());
        if constexpr (Algo::stats) {
            uint64_t st[8];
            impl::check(ctx_, mptg_prm_stats(prm_, st));
            std::printf("wavefronts: %llu\nsamples: %llu\nedges: %llu\nlinks checked: %llu\n",
                        (unsigned long long)st[0], (unsigned long long)st[1], (unsigned long long)st[5],
                        (unsigned long long)st[4]);
        }
    }
};

}  // namespace unc::robotics::mpt_gb300
