// ref_driver.cpp - C entry points around the reference's OWN headers, used to
// check the oracle's restatement.  TEST INFRASTRUCTURE ONLY.
//
// Compiled from the MPT sources where they lie (the include path points at
// the reference's src/ directory; nothing is copied), against the
// project-written nigh/Eigen stand-ins in shim/:
//   src/mpt/lp_space.hpp, so2_space.hpp, so3_space.hpp    interpolate()
//   src/mpt/discrete_motion_validator.hpp                 DMV bisection
//   src/mpt/goal_state.hpp                                GoalState
// State validity comes from the oracle (orc_state_valid), so a mismatch
// between ref_dmv_edges and orc_valid_edges isolates the DMV restatement.
#include <array>
#include <cstdint>

#include <mpt/lp_space.hpp>
#include <mpt/so2_space.hpp>
#include <mpt/so3_space.hpp>
#include <mpt/goal_state.hpp>
#include <mpt/discrete_motion_validator.hpp>

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

}  // namespace

extern "C" {

// metric: 0 L2 (dim 2 or 3), 1 SO2 (dim 1 or 10), 2 SO3 (dim 4); returns 0 on success
int ref_dmv_edges(const orc_scene* sc, int metric, int dim, const double* a, const double* b, long long n,
                  double step, uint8_t* out, long long* samples) {
    if (metric == 0 && dim == 2) dmv<nm::Space<std::array<double, 2>, nm::LP<2>>, 2>(sc, a, b, n, step, out, samples);
    else if (metric == 1 && dim == 10) dmv<nm::Space<std::array<double, 10>, nm::SO2<1>>, 10>(sc, a, b, n, step, out, samples);
    else return 1;
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

}  // extern "C"
