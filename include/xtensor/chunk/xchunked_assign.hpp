// Forwarding header: the GB300 evaluator provides this part of the xtensor
// API (xtensor 0.27.1, same include path) from xtensor_gb300/xt.hpp.
#pragma once
#include "../../xtensor_gb300/xt.hpp"
