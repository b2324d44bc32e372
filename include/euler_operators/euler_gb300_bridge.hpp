// Internal to the euler_operators drop-in: maps the reference's template
// operators onto the C ABI of libeuler_gb300 (include/euler_gb300.h) for
// real_t = double (*_f64) and real_t = float (*_f32).  Failures of the C ABI
// become std::runtime_error, since the reference operators have no status.
#pragma once

#include <euler_gb300.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>

#include <Kokkos_Core.hpp>

namespace euler_gb300_bridge {

inline void check(int status, const char* what)
{
    if (status != EULR_SUCCESS) {
        throw std::runtime_error(std::string(what) + ": " + eulr_status_string(status) + ": " + eulr_last_error());
    }
}

inline eulr_stream_t stream_of(Kokkos::DefaultExecutionSpace const& exec)
{
    return reinterpret_cast<eulr_stream_t>(exec.cuda_stream());
}

template <class Span>
int extent_int(Span const& s, int r)
{
    return static_cast<int>(s.extent(r));
}

template <class T>
struct types;

template <>
struct types<double>
{
    using prim = eulr_prim_f64;
    using cons = eulr_cons_f64;
    using cprim = eulr_prim_cf64;
    using ccons = eulr_cons_cf64;
};

template <>
struct types<float>
{
    using prim = eulr_prim_f32;
    using cons = eulr_cons_f32;
    using cprim = eulr_prim_cf32;
    using ccons = eulr_cons_cf32;
};

template <class Out, class A>
Out prim_ptrs(A const& a)
{
    return Out{a.d.data_handle(), a.p.data_handle(), a.ux0.data_handle(), a.ux1.data_handle(), a.ux2.data_handle()};
}

template <class Out, class A>
Out cons_ptrs(A const& a)
{
    return Out{a.d.data_handle(), a.e.data_handle(), a.mx0.data_handle(), a.mx1.data_handle(), a.mx2.data_handle()};
}

} // namespace euler_gb300_bridge
