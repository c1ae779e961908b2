// Project-written stand-in for the parts of the nigh library (UNC-Robotics/
// nigh, not vendored with MPT and with no pinned version) that MPT's
// interpolate()/DiscreteMotionValidator headers use: the metric tags, the
// Space<T, M> accessors (Type, Distance, coeff, dimensions, distance) and
// so2::ccwDist / so2::bound.  States are std::array<double, D> (and plain
// double for a single SO(2) angle).  The formulas are the ones the oracle
// restates (oracle/oracle.c), pinned by MPT's own metric unit tests.
#pragma once
#include <array>
#include <cmath>
#include <cstddef>

namespace unc::robotics::nigh {
namespace impl {
template <class T>
constexpr T PI = T(3.14159265358979323846264338327950288419716939937510582097494459230781640628620L);
namespace so2 {
// counter-clockwise angle from a to b in [0, 2pi)
template <class T>
T ccwDist(T a, T b) {
    T d = std::fmod(b - a, 2 * PI<T>);
    if (d < 0) d += 2 * PI<T>;
    return d;
}
// reduce into [-pi, pi)
template <class T>
T bound(T v) {
    v = std::fmod(v, 2 * PI<T>);
    if (v < -PI<T>) v += 2 * PI<T>;
    else if (v >= PI<T>) v -= 2 * PI<T>;
    return v;
}
template <class T>
T dist1(T a, T b) {
    T d = std::fabs(a - b);
    if (d > 2 * PI<T>) d = std::fmod(d, 2 * PI<T>);
    return d > PI<T> ? 2 * PI<T> - d : d;
}
}  // namespace so2
}  // namespace impl

namespace metric {
template <int p> struct LP {};
template <int p> struct SO2 {};
struct SO3 {};
template <class T, class M, class = void> struct Space;

template <std::size_t D, int p>
struct Space<std::array<double, D>, LP<p>> {
    using Type = std::array<double, D>;
    using Distance = double;
    static constexpr int kDimensions = (int)D;
    static double& coeff(Type& q, int i) { return q[i]; }
    static const double& coeff(const Type& q, int i) { return q[i]; }
    constexpr unsigned dimensions() const { return D; }
    Distance distance(const Type& a, const Type& b) const {
        double s = 0;
        for (std::size_t i = 0; i < D; ++i) {
            double d = a[i] - b[i];
            if (p == 1) s += std::fabs(d);
            else s += d * d;
        }
        return p == 1 ? s : std::sqrt(s);
    }
};

template <int p>
struct Space<double, SO2<p>> {
    using Type = double;
    using Distance = double;
    static constexpr int kDimensions = 1;
    static double& coeff(Type& q, int) { return q; }
    static const double& coeff(const Type& q, int) { return q; }
    constexpr unsigned dimensions() const { return 1; }
    Distance distance(double a, double b) const { return impl::so2::dist1(a, b); }
};

template <std::size_t D, int p>
struct Space<std::array<double, D>, SO2<p>> {
    using Type = std::array<double, D>;
    using Distance = double;
    static constexpr int kDimensions = (int)D;
    static double& coeff(Type& q, int i) { return q[i]; }
    static const double& coeff(const Type& q, int i) { return q[i]; }
    constexpr unsigned dimensions() const { return D; }
    Distance distance(const Type& a, const Type& b) const {
        double s = 0;
        for (std::size_t i = 0; i < D; ++i) s += impl::so2::dist1(a[i], b[i]);
        return s;
    }
};

// unit quaternions, coefficients (x, y, z, w)
template <>
struct Space<std::array<double, 4>, SO3> {
    using Type = std::array<double, 4>;
    using Distance = double;
    static constexpr int kDimensions = 4;
    static double& coeff(Type& q, int i) { return q[i]; }
    static const double& coeff(const Type& q, int i) { return q[i]; }
    constexpr unsigned dimensions() const { return 4; }
    Distance distance(const Type& a, const Type& b) const {
        double d = std::fabs(a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
        return std::acos(d > 1 ? 1.0 : d);
    }
};
}  // namespace metric
}  // namespace unc::robotics::nigh
