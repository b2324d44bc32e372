// euler_operators drop-in for GB300: init_implode, the reference's
// euler_operators/init_implode.hpp:7-45 (sphere of radius 0.25 around
// (0.5,0.5,0.5), ghosts included), on the GPU through
// eulr_init_implode_{f64,f32} (bit-identical to the reference).
#pragma once

#include <euler_arrays.hpp>
#include <euler_gb300_bridge.hpp>
#include <uniform_mesh.hpp>

template <class T, class IndexType, std::size_t E0, std::size_t E1, std::size_t E2>
void init_implode(
        Kokkos::DefaultExecutionSpace const& exec_space,
        EulerPrimArrays<Kokkos::mdspan<T, Kokkos::extents<IndexType, E0, E1, E2>, Kokkos::layout_left>> const& prim_arrays,
        UniformMesh3d<T> const& mesh)
{
    namespace b = euler_gb300_bridge;
    using ty = b::types<T>;
    auto const& s = prim_arrays.d;
    int st;
    if constexpr (std::is_same_v<T, double>) {
        st = eulr_init_implode_f64(b::prim_ptrs<typename ty::prim>(prim_arrays), b::extent_int(s, 0), b::extent_int(s, 1),
                                   b::extent_int(s, 2), mesh.dx0(), mesh.dx1(), mesh.dx2(), b::stream_of(exec_space));
    } else {
        st = eulr_init_implode_f32(b::prim_ptrs<typename ty::prim>(prim_arrays), b::extent_int(s, 0), b::extent_int(s, 1),
                                   b::extent_int(s, 2), mesh.dx0(), mesh.dx1(), mesh.dx2(), b::stream_of(exec_space));
    }
    b::check(st, "init_implode");
}
