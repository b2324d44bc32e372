// euler_operators drop-in for GB300: godunov, the reference's
// euler_operators/godunov.hpp:15-92 -- on interior cells,
// cons -= dt/dv * sum_d ds_d (F_{d,R} - F_{d,L}) with HLLC fluxes from the
// read-only prim, cons updated in place.  Runs on the GPU through
// eulr_godunov_{f64,f32}, which solves each face once (the reference solves
// each interior face from both sides); results agree with the reference
// within 1e-12 relative L-infinity in FP64.  Defining EULR_GODUNOV_BIT_EXACT
// before including this header routes it to eulr_godunov_exact_{f64,f32}
// instead: the reference's results bit for bit, about twice as slow.
// Enqueued on the execution space's stream; returns without waiting.
#pragma once

#include <euler_arrays.hpp>
#include <euler_gb300_bridge.hpp>
#include <hllc.hpp>
#include <perfect_gas.hpp>
#include <uniform_mesh.hpp>

template <std::size_t N>
using dir_t = std::integral_constant<std::size_t, N>;

template <class T, class IndexType, std::size_t E0, std::size_t E1, std::size_t E2>
void godunov(
        Kokkos::DefaultExecutionSpace const& exec_space,
        EulerPrimArrays<Kokkos::mdspan<T const, Kokkos::extents<IndexType, E0, E1, E2>, Kokkos::layout_left>> const&
                prim_arrays,
        EulerConsArrays<Kokkos::mdspan<T, Kokkos::extents<IndexType, E0, E1, E2>, Kokkos::layout_left>> const& cons_arrays,
        PerfectGas<T> const& eos,
        UniformMesh3d<T> const& mesh,
        hllc const& /*riemann_solver*/,
        T const dt)
{
    namespace b = euler_gb300_bridge;
    using ty = b::types<T>;
    auto const& s = prim_arrays.d;
    int st;
#ifdef EULR_GODUNOV_BIT_EXACT
    auto* const f64 = &eulr_godunov_exact_f64;
    auto* const f32 = &eulr_godunov_exact_f32;
#else
    auto* const f64 = &eulr_godunov_f64;
    auto* const f32 = &eulr_godunov_f32;
#endif
    if constexpr (std::is_same_v<T, double>) {
        st = f64(b::prim_ptrs<typename ty::cprim>(prim_arrays), b::cons_ptrs<typename ty::cons>(cons_arrays),
                 b::extent_int(s, 0), b::extent_int(s, 1), b::extent_int(s, 2), eos.gamma(), mesh.dx0(), mesh.dx1(),
                 mesh.dx2(), dt, b::stream_of(exec_space));
    } else {
        st = f32(b::prim_ptrs<typename ty::cprim>(prim_arrays), b::cons_ptrs<typename ty::cons>(cons_arrays),
                 b::extent_int(s, 0), b::extent_int(s, 1), b::extent_int(s, 2), eos.gamma(), mesh.dx0(), mesh.dx1(),
                 mesh.dx2(), dt, b::stream_of(exec_space));
    }
    b::check(st, "godunov");
}
