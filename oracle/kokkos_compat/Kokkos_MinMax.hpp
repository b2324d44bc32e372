// Test-only Kokkos compatibility layer: everything lives in Kokkos_Core.hpp.
#pragma once
#include "Kokkos_Core.hpp"
