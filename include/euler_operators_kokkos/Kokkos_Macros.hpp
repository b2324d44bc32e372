// Kokkos names for builds of the euler_operators drop-in without Kokkos.
#pragma once
#include "Kokkos_Core.hpp"
