// euler_operators drop-in for GB300: prim_to_cons, the reference's
// euler_operators/prim_to_cons.hpp:7-33, on the GPU through
// eulr_prim_to_cons_{f64,f32} (bit-identical to the reference).  Enqueued on
// the execution space's stream; returns without waiting.
#pragma once

#include <euler_arrays.hpp>
#include <euler_gb300_bridge.hpp>
#include <perfect_gas.hpp>

template <class T, class IndexType, std::size_t E0, std::size_t E1, std::size_t E2>
void prim_to_cons(
        Kokkos::DefaultExecutionSpace const& exec_space,
        EulerPrimArrays<Kokkos::mdspan<T const, Kokkos::extents<IndexType, E0, E1, E2>, Kokkos::layout_left>> const&
                prim_arrays,
        EulerConsArrays<Kokkos::mdspan<T, Kokkos::extents<IndexType, E0, E1, E2>, Kokkos::layout_left>> const& cons_arrays,
        PerfectGas<T> const& eos)
{
    namespace b = euler_gb300_bridge;
    using ty = b::types<T>;
    auto const& s = prim_arrays.d;
    int st;
    if constexpr (std::is_same_v<T, double>) {
        st = eulr_prim_to_cons_f64(b::prim_ptrs<typename ty::cprim>(prim_arrays), b::cons_ptrs<typename ty::cons>(cons_arrays),
                                   b::extent_int(s, 0), b::extent_int(s, 1), b::extent_int(s, 2), eos.gamma(),
                                   b::stream_of(exec_space));
    } else {
        st = eulr_prim_to_cons_f32(b::prim_ptrs<typename ty::cprim>(prim_arrays), b::cons_ptrs<typename ty::cons>(cons_arrays),
                                   b::extent_int(s, 0), b::extent_int(s, 1), b::extent_int(s, 2), eos.gamma(),
                                   b::stream_of(exec_space));
    }
    b::check(st, "prim_to_cons");
}
