// euler_operators drop-in for GB300: the HLLC Riemann solver tag.  In the
// reference (euler_operators/hllc.hpp:50-105) hllc::operator() is evaluated
// inside godunov's kernel; here the flux is computed by the CUDA library's
// godunov and fused-step kernels, so the tag only selects the solver.
#pragma once

#include <euler_arrays.hpp>
#include <perfect_gas.hpp>

struct hllc
{
};
