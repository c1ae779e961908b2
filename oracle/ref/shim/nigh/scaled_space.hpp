// Project-written nigh stand-in: the Scaled metric tag, declared so that MPT's
// scaled_space.hpp compiles (its templates are not instantiated here).
#pragma once
#include "shim_metric.hpp"
namespace unc::robotics::nigh::metric {
template <class M, class W> struct Scaled {};
}  // namespace unc::robotics::nigh::metric
