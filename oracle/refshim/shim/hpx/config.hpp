// Stand-in for <hpx/config.hpp> (TEST INFRASTRUCTURE ONLY, oracle/refshim).
#pragma once
#include "include/parallel_algorithm.hpp"
