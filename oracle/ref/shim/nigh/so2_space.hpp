// Project-written nigh stand-in (see shim_metric.hpp).
#pragma once
#include "shim_metric.hpp"
