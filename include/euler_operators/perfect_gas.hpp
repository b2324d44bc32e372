// euler_operators drop-in for GB300: perfect-gas equation of state, the
// reference's euler_operators/perfect_gas.hpp (sound speed :15-18, internal
// energy :20-23, pressure :25-28).  gamma() is an addition: the CUDA
// operators take the ratio of specific heats as a plain scalar.
#pragma once

#include <cmath>

#include <Kokkos_Core.hpp>

template <class T>
class PerfectGas
{
private:
    T m_gamma;

public:
    KOKKOS_FUNCTION explicit PerfectGas(T const gamma) : m_gamma(gamma) {}

    KOKKOS_FUNCTION T gamma() const noexcept { return m_gamma; }

    KOKKOS_FUNCTION T speed_of_sound(T const density, T const pressure) const noexcept
    {
        return std::sqrt(m_gamma * pressure / density);
    }

    KOKKOS_FUNCTION T internal_energy(T const /*density*/, T const pressure) const noexcept
    {
        return pressure / (m_gamma - 1);
    }

    KOKKOS_FUNCTION T pressure(T const /*density*/, T const int_e) const noexcept { return (m_gamma - 1) * int_e; }
};
