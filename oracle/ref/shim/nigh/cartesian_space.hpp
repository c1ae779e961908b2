// Project-written nigh stand-in: the Cartesian metric tag and the state
// element accessors, declared so that MPT's cartesian_space.hpp and its
// Cartesian sampler compile (their templates are not instantiated here).
#pragma once
#include <cstddef>
#include "shim_metric.hpp"
namespace unc::robotics::nigh {
namespace metric {
template <class... M> struct Cartesian {};
template <std::size_t I, class T> struct cartesian_state_element;
}  // namespace metric
template <std::size_t I, class T>
using cartesian_state_element_t = typename metric::cartesian_state_element<I, T>::type;
}  // namespace unc::robotics::nigh
