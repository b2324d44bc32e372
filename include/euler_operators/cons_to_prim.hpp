// euler_operators drop-in for GB300: cons_to_prim, the reference's
// euler_operators/cons_to_prim.hpp:7-33 (all cells, ghosts included), on the
// GPU through eulr_cons_to_prim_{f64,f32} (bit-identical to the reference).
// Enqueued on the execution space's stream; returns without waiting.
#pragma once

#include <euler_arrays.hpp>
#include <euler_gb300_bridge.hpp>
#include <perfect_gas.hpp>

template <class T, class IndexType, std::size_t E0, std::size_t E1, std::size_t E2>
void cons_to_prim(
        Kokkos::DefaultExecutionSpace const& exec_space,
        EulerConsArrays<Kokkos::mdspan<T const, Kokkos::extents<IndexType, E0, E1, E2>, Kokkos::layout_left>> const&
                cons_arrays,
        EulerPrimArrays<Kokkos::mdspan<T, Kokkos::extents<IndexType, E0, E1, E2>, Kokkos::layout_left>> const& prim_arrays,
        PerfectGas<T> const& eos)
{
    namespace b = euler_gb300_bridge;
    using ty = b::types<T>;
    auto const& s = cons_arrays.d;
    int st;
    if constexpr (std::is_same_v<T, double>) {
        st = eulr_cons_to_prim_f64(b::cons_ptrs<typename ty::ccons>(cons_arrays), b::prim_ptrs<typename ty::prim>(prim_arrays),
                                   b::extent_int(s, 0), b::extent_int(s, 1), b::extent_int(s, 2), eos.gamma(),
                                   b::stream_of(exec_space));
    } else {
        st = eulr_cons_to_prim_f32(b::cons_ptrs<typename ty::ccons>(cons_arrays), b::prim_ptrs<typename ty::prim>(prim_arrays),
                                   b::extent_int(s, 0), b::extent_int(s, 1), b::extent_int(s, 2), eos.gamma(),
                                   b::stream_of(exec_space));
    }
    b::check(st, "cons_to_prim");
}
