// Project-written nigh stand-in (see auto_strategy.hpp).
#pragma once
#include "auto_strategy.hpp"
