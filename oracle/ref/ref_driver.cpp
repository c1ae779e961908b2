// ref_driver.cpp - C entry points around the reference's OWN headers, used to
// check the oracle's restatement.  TEST INFRASTRUCTURE ONLY.
//
// Compiled from the MPT sources where they lie (the include path points at
// the reference's src/ directory; nothing is copied), against the
// project-written nigh/Eigen stand-ins in shim/:
//   src/mpt/lp_space.hpp, so2_space.hpp, so3_space.hpp    interpolate()
//   src/mpt/discrete_motion_validator.hpp                 DMV bisection
//   src/mpt/goal_state.hpp                                GoalState
//   src/mpt/prrt.hpp, prrt_star.hpp, pprm.hpp (impl/)      the PRRT, PRRT* and PPRM planners
// State validity comes from the oracle (orc_state_valid), so a mismatch
// between ref_dmv_edges and orc_valid_edges isolates the DMV restatement.
#include <omp.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <limits>
#include <cstdint>
#include <random>
#include <tuple>
#include <type_traits>
#include <vector>

#include <mpt/lp_space.hpp>
#include <mpt/so2_space.hpp>
#include <mpt/so3_space.hpp>
#include <mpt/goal_state.hpp>
#include <mpt/discrete_motion_validator.hpp>
#include <mpt/prrt.hpp>
#include <mpt/prrt_star.hpp>
#include <mpt/pprm.hpp>

#include "../oracle.h"

namespace mpt = unc::robotics::mpt;
namespace nm = unc::robotics::nigh::metric;

namespace {

template <class Space>
struct Validator {
    const orc_scene* sc;
    long long* counter;
    Validator(const orc_scene* s, long long* c) : sc(s), counter(c) {}
    bool operator()(const typename Space::Type& q) const {
        ++*counter;
        return orc_state_valid(sc, q.data()) != 0;
    }
};

template <class Space, std::size_t D>
void dmv(const orc_scene* sc, const double* a, const double* b, long long n, double step, uint8_t* out,
         long long* samples) {
    Space space;
    for (long long i = 0; i < n; ++i) {
        long long cnt = 0;
        mpt::DiscreteMotionValidator<Space, Validator<Space>> v(space, step, sc, &cnt);
        std::array<double, D> A, B;
        for (std::size_t d = 0; d < D; ++d) { A[d] = a[i * D + d]; B[d] = b[i * D + d]; }
        out[i] = v(A, B) ? 1 : 0;
        samples[i] = cnt;
    }
}

template <class Space, std::size_t D>
void interp(const double* a, const double* b, double t, double* out) {
    Space space;
    std::array<double, D> A, B;
    for (std::size_t d = 0; d < D; ++d) { A[d] = a[d]; B[d] = b[d]; }
    std::array<double, D> q = mpt::interpolate(space, A, B, t);
    for (std::size_t d = 0; d < D; ++d) out[d] = q[d];
}

// SE(3) states (x, y, z, w, px, py, pz) under the oracle's weighted metric
// w0 * acos|q1.q2| + w1 * |p1 - p2| (cartesian_space.hpp:43-68 with SO3 and
// L2 elements).  nigh's Cartesian space and MPT's SE3 state need Eigen, so
// this project-written space stands in; its distance and interpolate are the
// oracle's, reached by the reference's templates through argument-dependent
// lookup.
struct SE3Tag {};
using SE3Space = nm::Space<std::array<double, 7>, SE3Tag>;

}  // namespace

namespace unc::robotics::nigh::metric {
template <>
struct Space<std::array<double, 7>, SE3Tag> {
    using Type = std::array<double, 7>;
    using Distance = double;
    static constexpr int kDimensions = 7;
    orc_space sp{3, 7, {2.0, 1.0}};
    constexpr unsigned dimensions() const { return 7; }
    Distance distance(const Type& a, const Type& b) const { return orc_distance(&sp, a.data(), b.data()); }
};
}  // namespace unc::robotics::nigh::metric

namespace {

std::array<double, 7> interpolate(const SE3Space& space, const std::array<double, 7>& a,
                                  const std::array<double, 7>& b, double t) {
    std::array<double, 7> q;
    orc_interpolate(&space.sp, a.data(), b.data(), t, q.data());
    return q;
}

// The same SE(3) metric evaluated with glibc's acos, and interpolated by the
// reference's own SO(3) slerp (so3_space.hpp:44-83, glibc acos/sin) on the
// quaternion and its L2 interpolate (lp_space.hpp:44-54) on the position, as
// nigh's Cartesian space combines its parts (cartesian_space.hpp:43-68).  The
// DMV over this space is the reference's SE(3) motion check with the
// reference's own transcendental functions; only valid() is the oracle's.
struct SE3GlibcTag {};
using SE3GlibcSpace = nm::Space<std::array<double, 7>, SE3GlibcTag>;

}  // namespace

namespace unc::robotics::nigh::metric {
template <>
struct Space<std::array<double, 7>, SE3GlibcTag> {
    using Type = std::array<double, 7>;
    using Distance = double;
    static constexpr int kDimensions = 7;
    double w0 = 2.0, w1 = 1.0;
    constexpr unsigned dimensions() const { return 7; }
    Distance distance(const Type& a, const Type& b) const {
        double d = std::abs(a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
        if (d > 1.0) d = 1.0;
        double s = 0;
        for (int i = 4; i < 7; ++i) {
            double x = a[i] - b[i];
            s += x * x;
        }
        return w0 * std::acos(d) + w1 * std::sqrt(s);
    }
};
}  // namespace unc::robotics::nigh::metric

namespace {

std::array<double, 7> interpolate(const SE3GlibcSpace&, const std::array<double, 7>& a,
                                  const std::array<double, 7>& b, double t) {
    nm::Space<std::array<double, 4>, nm::SO3> so3;
    nm::Space<std::array<double, 3>, nm::LP<2>> r3;
    std::array<double, 4> qa{a[0], a[1], a[2], a[3]}, qb{b[0], b[1], b[2], b[3]};
    std::array<double, 3> pa{a[4], a[5], a[6]}, pb{b[4], b[5], b[6]};
    std::array<double, 4> q = mpt::interpolate(so3, qa, qb, t);
    std::array<double, 3> p = mpt::interpolate(r3, pa, pb, t);
    return {q[0], q[1], q[2], q[3], p[0], p[1], p[2]};
}

// A SeedSequence that gives each generator seeded from it its own stream:
// the planner seeds every worker's RNG from one seed object
// (impl/prrt/prrt.hpp:341-344), in worker order.
struct WorkerSeed {
    using result_type = std::uint32_t;
    std::uint64_t seed;
    mutable std::uint32_t calls = 0;
    template <class It>
    void generate(It first, It last) const {
        std::seed_seq seq{std::uint32_t(seed), std::uint32_t(seed >> 32), calls++};
        seq.generate(first, last);
    }
};

// A Scenario (the contract of impl/scenario_*.hpp) over an oracle scene: the
// oracle's valid(), link() by the reference's DMV (resolution 0) or the
// oracle's joint-step edge check (resolution 1), uniform samples in the box,
// GoalState(radius, goal).
template <class S, std::size_t D>
struct OracleScenario {
    using Space = S;
    using State = std::array<double, D>;
    const orc_scene* sc;
    const orc_space* sp;
    std::array<double, D> lo, hi;
    double step;
    int resolution;
    Space space_;
    mpt::GoalState<Space> goal_;

    OracleScenario(const orc_scene* s, const orc_space* p, const double* l, const double* h, const double* g,
                   double radius, double st, int res)
        : sc(s), sp(p), step(st), resolution(res), space_(make_space(p)), goal_(radius, arr(g)) {
        lo = arr(l);
        hi = arr(h);
    }
    static Space make_space(const orc_space* p) {
        Space s{};
        if constexpr (std::is_same_v<Space, SE3Space>) s.sp = *p;
        return s;
    }
    static State arr(const double* v) {
        State q;
        for (std::size_t d = 0; d < D; ++d) q[d] = v[d];
        return q;
    }
    const Space& space() const { return space_; }
    const mpt::GoalState<Space>& goal() const { return goal_; }
    // uniform in the box, Shoemake's uniform rotation for SE(3)
    // (impl/uniform_sampler_so3.hpp:55-68); handed to the planners through
    // sampler() (impl/scenario_sampler.hpp, case 2)
    struct BoxSampler {
        std::array<double, D> lo, hi;
        template <class RNG>
        State operator()(RNG& rng) const {
            State q;
            std::size_t d0 = 0;
            if constexpr (std::is_same_v<Space, SE3Space>) {
                std::uniform_real_distribution<double> u01(0.0, 1.0);
                double a = u01(rng), b = 2 * M_PI * u01(rng), c = 2 * M_PI * u01(rng);
                double s1 = std::sqrt(1.0 - a), s2 = std::sqrt(a);
                q[0] = s1 * std::sin(b);
                q[1] = s1 * std::cos(b);
                q[2] = s2 * std::sin(c);
                q[3] = s2 * std::cos(c);
                d0 = 4;
            }
            for (std::size_t d = d0; d < D; ++d) q[d] = std::uniform_real_distribution<double>(lo[d], hi[d])(rng);
            return q;
        }
    };
    BoxSampler sampler() const { return BoxSampler{lo, hi}; }
    bool valid(const State& q) const { return orc_state_valid(sc, q.data()) != 0; }
    bool link(const State& a, const State& b) const {
        if (resolution == 0) {
            long long cnt = 0;
            mpt::DiscreteMotionValidator<Space, Validator<Space>> v(space_, step, sc, &cnt);
            return v(a, b);
        }
        uint8_t ok = 0;
        int64_t samples = 0;
        orc_valid_edges(sc, sp, a.data(), b.data(), 1, step, resolution, &ok, &samples, 1);
        return ok != 0;
    }
};

// The planners' sample stream (orc_sample_state) as an MPT sampler: the c-th
// call returns sample c % W of wavefront c / W and ignores the RNG, so the
// reference's one-sample-at-a-time planners see the states the oracle's
// replays draw, in the same order.  Single-threaded use only.
template <std::size_t D>
struct StreamSampler {
    const orc_space* sp;
    const orc_plan_params* pp;
    const double* lo;
    const double* hi;
    std::uint64_t* count;
    template <class RNG>
    std::array<double, D> operator()(RNG&) const {
        std::uint64_t c = (*count)++;
        std::uint64_t W = std::uint64_t(pp->wavefront);
        std::array<double, D> q;
        orc_sample_state(sp, pp, lo, hi, std::uint32_t(c % W), std::uint32_t(c / W), q.data());
        return q;
    }
};

template <class S, std::size_t D>
struct StreamScenario : OracleScenario<S, D> {
    StreamSampler<D> stream;
    StreamScenario(const OracleScenario<S, D>& base, const StreamSampler<D>& st)
        : OracleScenario<S, D>(base), stream(st) {}
    StreamSampler<D> sampler() const { return stream; }
};

// visitGraph visitor: vertex states, and one (from, to) state pair per edge
template <std::size_t D>
struct GraphCollector {
    double* v;
    long long vcap;
    long long* nv;
    double* e;
    long long ecap;
    long long* ne;
    std::array<double, D> from{};
    void vertex(const std::array<double, D>& q) {
        if (*nv < vcap)
            for (std::size_t d = 0; d < D; ++d) v[*nv * D + d] = q[d];
        ++*nv;
        from = q;
    }
    void edge(const std::array<double, D>& to) {
        if (*ne < ecap)
            for (std::size_t d = 0; d < D; ++d) {
                e[*ne * 2 * D + d] = from[d];
                e[*ne * 2 * D + D + d] = to[d];
            }
        ++*ne;
    }
};

template <class S, std::size_t D>
int stream_graph(int algo, const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp, const double* lo,
                 const double* hi, const double* start, const double* goal, long long nsamples, double* v,
                 long long vcap, long long* nv, double* e, long long ecap, long long* ne, double* path,
                 long long pcap, long long* plen) {
    OracleScenario<S, D> base(sc, sp, lo, hi, goal, pp->goal_radius, pp->edge_step, pp->resolution);
    std::uint64_t count = 0;
    StreamScenario<S, D> scen(base, StreamSampler<D>{sp, pp, lo, hi, &count});
    orc_state_valid(sc, start);
    auto done = [&] { return count >= std::uint64_t(nsamples); };
    GraphCollector<D> out{v, vcap, nv, e, ecap, ne};
    *nv = 0;
    *ne = 0;
    *plen = 0;
    auto take_path = [&](const std::vector<std::array<double, D>>& sol) {
        *plen = (long long)sol.size();
        for (long long i = 0; i < *plen && i < pcap; ++i)
            for (std::size_t d = 0; d < D; ++d) path[i * D + d] = sol[std::size_t(i)][d];
    };
    if (algo == 0) {
        mpt::Planner<StreamScenario<S, D>, mpt::PRRT<mpt::single_threaded>> planner(scen, WorkerSeed{pp->seed});
        planner.setRange(pp->range > 0 ? pp->range : std::numeric_limits<double>::infinity());
        planner.setGoalBias(0);
        planner.addStart(OracleScenario<S, D>::arr(start));
        planner.solve(done);
        planner.visitGraph(out);
    } else if (algo == 1) {
        mpt::Planner<StreamScenario<S, D>, mpt::PRRTStar<mpt::single_threaded>> planner(scen, WorkerSeed{pp->seed});
        planner.setRange(pp->range > 0 ? pp->range : std::numeric_limits<double>::infinity());
        planner.setGoalBias(0);
        planner.addStart(OracleScenario<S, D>::arr(start));
        planner.solve(done);
        planner.visitGraph(out);
    } else if (algo == 2) {
        mpt::Planner<StreamScenario<S, D>, mpt::PPRM<mpt::single_threaded>> planner(scen, WorkerSeed{pp->seed});
        planner.addStart(OracleScenario<S, D>::arr(start));
        planner.addGoal(OracleScenario<S, D>::arr(goal));
        planner.solve(done);
        planner.visitGraph(out);
        if (planner.solved()) take_path(planner.solution());
    } else {
        return -1;
    }
    return (*nv <= vcap && *ne <= ecap && *plen <= pcap) ? 0 : -2;
}

template <class P, class State, class = void>
struct has_add_goal : std::false_type {};
template <class P, class State>
struct has_add_goal<P, State, std::void_t<decltype(std::declval<P&>().addGoal(std::declval<State>()))>>
    : std::true_type {};

// addStart (and addGoal for PPRM), solve until the first solution or the time
// limit, then the solution path and its cost in the space's metric
template <class Planner, class Scen>
int run_planner(Planner& planner, const Scen& scen, const double* start, const double* goal, double range,
                double goal_bias, double time_limit_s, double* path, int path_cap, int* path_len, long long* nodes,
                double* solve_s, double* cost) {
    using State = typename Scen::State;
    constexpr std::size_t D = std::tuple_size_v<State>;
    if constexpr (!has_add_goal<Planner, State>::value) {
        planner.setRange(range);
        planner.setGoalBias(goal_bias);
    }
    planner.addStart(Scen::arr(start));
    if constexpr (has_add_goal<Planner, State>::value) planner.addGoal(Scen::arr(goal));
    auto t0 = std::chrono::steady_clock::now();
    planner.solveFor([&] { return planner.solved(); },
                     std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                         std::chrono::duration<double>(time_limit_s)));
    *solve_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *nodes = (long long)planner.size();
    std::vector<State> sol = planner.solution();
    *path_len = (int)sol.size();
    *cost = 0;
    for (std::size_t i = 0; i < sol.size(); ++i) {
        if ((int)i < path_cap)
            for (std::size_t d = 0; d < D; ++d) path[i * D + d] = sol[i][d];
        if (i) *cost += scen.space().distance(sol[i - 1], sol[i]);
    }
    return planner.solved() ? 1 : 0;
}

// Alg1 / AlgN: the planner's single-threaded and OpenMP-pool variants
template <class Space, std::size_t D, class Alg1, class AlgN>
int plan_solve(const orc_scene* sc, const orc_space* sp, const double* lo, const double* hi, const double* start,
               const double* goal, double goal_radius, double range, double goal_bias, double step, int resolution,
               std::uint64_t seed, int threads, double time_limit_s, double* path, int path_cap, int* path_len,
               long long* nodes, double* solve_s, double* cost) {
    using Scen = OracleScenario<Space, D>;
    Scen scen(sc, sp, lo, hi, goal, goal_radius, step, resolution);
    WorkerSeed ws{seed};
    orc_state_valid(sc, start);  // builds the oracle's mesh BVH before any worker thread reads it
    if (threads == 1) {
        mpt::Planner<Scen, Alg1> planner(scen, ws);
        return run_planner(planner, scen, start, goal, range, goal_bias, time_limit_s, path, path_cap, path_len,
                           nodes, solve_s, cost);
    }
    int saved = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
    mpt::Planner<Scen, AlgN> planner(scen, ws);
    omp_set_num_threads(saved);
    return run_planner(planner, scen, start, goal, range, goal_bias, time_limit_s, path, path_cap, path_len, nodes,
                       solve_s, cost);
}

template <class Space, std::size_t D, class... A>
int plan_algo(int algo, A... args) {
    switch (algo) {
    case 0: return plan_solve<Space, D, mpt::PRRT<mpt::single_threaded>, mpt::PRRT<>>(args...);
    case 1: return plan_solve<Space, D, mpt::PRRTStar<mpt::single_threaded>, mpt::PRRTStar<>>(args...);
    case 2: return plan_solve<Space, D, mpt::PPRM<mpt::single_threaded>, mpt::PPRM<>>(args...);
    }
    return -1;
}

}  // namespace

extern "C" {

// metric: 0 L2 (dim 2), 1 SO2 (dim 10), 3 SE3 with weights (2, 1) and glibc's
// acos/sin (dim 7); returns 0 on success
int ref_dmv_edges(const orc_scene* sc, int metric, int dim, const double* a, const double* b, long long n,
                  double step, uint8_t* out, long long* samples) {
    if (metric == 0 && dim == 2) dmv<nm::Space<std::array<double, 2>, nm::LP<2>>, 2>(sc, a, b, n, step, out, samples);
    else if (metric == 1 && dim == 10) dmv<nm::Space<std::array<double, 10>, nm::SO2<1>>, 10>(sc, a, b, n, step, out, samples);
    else if (metric == 3 && dim == 7) dmv<SE3GlibcSpace, 7>(sc, a, b, n, step, out, samples);
    else return 1;
    return 0;
}

// ref_dmv_edges over nthreads OpenMP threads (0 = all), edges split evenly:
// the reference's motion check timed on the host's cores
int ref_dmv_edges_mt(const orc_scene* sc, int metric, int dim, const double* a, const double* b, long long n,
                     double step, uint8_t* out, long long* samples, int nthreads) {
    if (!((metric == 0 && dim == 2) || (metric == 1 && dim == 10) || (metric == 3 && dim == 7))) return 1;
    orc_state_valid(sc, a);  // builds the oracle's mesh BVH before any thread reads it
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
    long long chunk = (n + nt - 1) / nt;
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
        long long lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo < hi) ref_dmv_edges(sc, metric, dim, a + lo * dim, b + lo * dim, hi - lo, step, out + lo, samples + lo);
    }
    return 0;
}

int ref_interpolate(int metric, int dim, const double* a, const double* b, double t, double* out) {
    if (metric == 0 && dim == 2) interp<nm::Space<std::array<double, 2>, nm::LP<2>>, 2>(a, b, t, out);
    else if (metric == 0 && dim == 3) interp<nm::Space<std::array<double, 3>, nm::LP<2>>, 3>(a, b, t, out);
    else if (metric == 1 && dim == 10) interp<nm::Space<std::array<double, 10>, nm::SO2<1>>, 10>(a, b, t, out);
    else if (metric == 1 && dim == 1) {
        nm::Space<double, nm::SO2<1>> space;
        out[0] = mpt::interpolate(space, a[0], b[0], t);
    } else if (metric == 2 && dim == 4) interp<nm::Space<std::array<double, 4>, nm::SO3>, 4>(a, b, t, out);
    else return 1;
    return 0;
}

// GoalState(radius, goal)(space, q) for the 2-D L2 space (goal_state.hpp:64-69)
int ref_goal_l2(const double* goal, double radius, const double* q, double* dist_out) {
    using S = nm::Space<std::array<double, 2>, nm::LP<2>>;
    mpt::GoalState<S> g(radius, std::array<double, 2>{goal[0], goal[1]});
    auto r = g(S{}, std::array<double, 2>{q[0], q[1]});
    *dist_out = r.second;
    return r.first ? 1 : 0;
}

// One of the reference's own planners on an oracle scene, until the first
// solution or time_limit_s.  algo 0: PRRT (src/mpt/prrt.hpp;
// impl/prrt/prrt.hpp:149-316,358-452), 1: PRRT* with k-nearest rewiring
// (src/mpt/prrt_star.hpp; impl/prrt_star/prrt_star.hpp), 2: PPRM
// (src/mpt/pprm.hpp; impl/pprm/pprm.hpp, start and goal added, no range).
// metric/dim: 0/2 (grid), 1/10 (planar arm) or 3/7 (SE(3) rigid body).
// threads 1 = single_threaded, 0 = all OpenMP threads.  Returns 1 solved,
// 0 not solved, -1 unsupported.  path receives up to path_cap waypoints;
// *path_len is the full count.
int ref_plan_solve(int algo, const orc_scene* sc, const orc_space* sp, const double* lo, const double* hi,
                   const double* start, const double* goal, double goal_radius, double range, double goal_bias,
                   double step, int resolution, unsigned long long seed, int threads, double time_limit_s,
                   double* path, int path_cap, int* path_len, long long* nodes, double* solve_s, double* cost) {
    std::uint64_t sd = seed;
    if (sp->metric == 0 && sp->dim == 2)
        return plan_algo<nm::Space<std::array<double, 2>, nm::LP<2>>, 2>(
            algo, sc, sp, lo, hi, start, goal, goal_radius, range, goal_bias, step, resolution, sd, threads,
            time_limit_s, path, path_cap, path_len, nodes, solve_s, cost);
    if (sp->metric == 1 && sp->dim == 10)
        return plan_algo<nm::Space<std::array<double, 10>, nm::SO2<1>>, 10>(
            algo, sc, sp, lo, hi, start, goal, goal_radius, range, goal_bias, step, resolution, sd, threads,
            time_limit_s, path, path_cap, path_len, nodes, solve_s, cost);
    if (sp->metric == 3 && sp->dim == 7)
        return plan_algo<SE3Space, 7>(algo, sc, sp, lo, hi, start, goal, goal_radius, range, goal_bias, step,
                                      resolution, sd, threads, time_limit_s, path, path_cap, path_len, nodes,
                                      solve_s, cost);
    return -1;
}

// The reference's PRRT (algo 0) or PRRT* (algo 1; both with setRange(pp->range)
// and goal bias 0) or PPRM (algo 2; start then goal added), single-threaded, fed nsamples states of
// the planners' sample stream (StreamSampler, wavefront size pp->wavefront).
// The graph comes back through visitGraph: *nv vertex states in v (D doubles
// each) and *ne edges in e as (from state, to state) pairs (2D doubles each;
// PRRT, PRRT*: node -> parent; PPRM: every roadmap edge from both of its ends).
// PPRM also returns its solution() (the Dijkstra path of src/mpt/impl/
// djikstras.hpp) in path when solved: *plen states, 0 when not solved.
// Returns 0, -1 unsupported, -2 when vcap, ecap or pcap was too small.
int ref_stream_graph(int algo, const orc_scene* sc, const orc_space* sp, const orc_plan_params* pp,
                     const double* lo, const double* hi, const double* start, const double* goal,
                     long long nsamples, double* v, long long vcap, long long* nv, double* e, long long ecap,
                     long long* ne, double* path, long long pcap, long long* plen) {
    if (sp->metric == 0 && sp->dim == 2)
        return stream_graph<nm::Space<std::array<double, 2>, nm::LP<2>>, 2>(algo, sc, sp, pp, lo, hi, start, goal,
                                                                           nsamples, v, vcap, nv, e, ecap, ne, path, pcap, plen);
    if (sp->metric == 1 && sp->dim == 10)
        return stream_graph<nm::Space<std::array<double, 10>, nm::SO2<1>>, 10>(
            algo, sc, sp, pp, lo, hi, start, goal, nsamples, v, vcap, nv, e, ecap, ne, path, pcap, plen);
    if (sp->metric == 3 && sp->dim == 7)
        return stream_graph<SE3Space, 7>(algo, sc, sp, pp, lo, hi, start, goal, nsamples, v, vcap, nv, e, ecap, ne, path, pcap, plen);
    return -1;
}

}  // extern "C"
