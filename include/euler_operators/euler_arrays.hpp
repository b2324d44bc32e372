// euler_operators drop-in for GB300: state types and structure-of-arrays
// bundles, with the names and semantics of the reference's
// euler_operators/euler_arrays.hpp (point states :8-36, thermodynamic
// helpers :38-75, bundles and their helpers :77-411).  The bundles hold
// five views; the operators pass their data_handle() pointers to the CUDA
// library (include/euler_gb300.h).
#pragma once

#include <cstddef>
#include <type_traits>

#include <Kokkos_Core.hpp>

template <class T>
struct EulerPrim
{
    T d;
    T p;
    T ux0;
    T ux1;
    T ux2;
};

template <class T>
struct EulerCons
{
    T d;
    T e;
    T mx0;
    T mx1;
    T mx2;
};

template <class T>
struct EulerFlux
{
    T d;
    T e;
    T mx0;
    T mx1;
    T mx2;
};

// rho |u|^2 / 2 of a primitive state
template <class T>
KOKKOS_FUNCTION T kinetic_energy(EulerPrim<T> const& q) noexcept
{
    return q.d * ((q.ux0 * q.ux0) + (q.ux1 * q.ux1) + (q.ux2 * q.ux2)) / 2;
}

// |m|^2 / rho / 2 of a conservative state
template <class T>
KOKKOS_FUNCTION T kinetic_energy(EulerCons<T> const& u) noexcept
{
    return ((u.mx0 * u.mx0) + (u.mx1 * u.mx1) + (u.mx2 * u.mx2)) / u.d / 2;
}

template <class T>
KOKKOS_FUNCTION constexpr T internal_energy(EulerCons<T> const& u) noexcept
{
    return u.e - kinetic_energy(u);
}

template <class T>
KOKKOS_FUNCTION EulerCons<T> to_cons(EulerPrim<T> const& q, T const int_e) noexcept
{
    return {q.d, kinetic_energy(q) + int_e, q.d * q.ux0, q.d * q.ux1, q.d * q.ux2};
}

template <class T>
KOKKOS_FUNCTION EulerPrim<T> to_prim(EulerCons<T> const& u, T const p) noexcept
{
    T const vol = 1 / u.d;
    return {u.d, p, u.mx0 * vol, u.mx1 * vol, u.mx2 * vol};
}

template <class View>
struct EulerPrimArrays
{
    View d;
    View p;
    View ux0;
    View ux1;
    View ux2;
};

template <class View>
struct EulerConsArrays
{
    View d;
    View e;
    View mx0;
    View mx1;
    View mx2;
};

// Re-type every view of a bundle (e.g. to its const version).
template <class MdspanOut, class E, class X, class L, class A>
EulerPrimArrays<MdspanOut> as(EulerPrimArrays<Kokkos::mdspan<E, X, L, A>> const& a) noexcept
{
    return {a.d, a.p, a.ux0, a.ux1, a.ux2};
}

template <class MdspanOut, class E, class X, class L, class A>
EulerConsArrays<MdspanOut> as(EulerConsArrays<Kokkos::mdspan<E, X, L, A>> const& a) noexcept
{
    return {a.d, a.e, a.mx0, a.mx1, a.mx2};
}

template <class T, class I, std::size_t E0, std::size_t E1, std::size_t E2, class L>
EulerPrimArrays<Kokkos::mdspan<T const, Kokkos::extents<I, E0, E1, E2>, L>> as_const(
        EulerPrimArrays<Kokkos::mdspan<T, Kokkos::extents<I, E0, E1, E2>, L>> const& a) noexcept
{
    return as<Kokkos::mdspan<T const, Kokkos::extents<I, E0, E1, E2>, L>>(a);
}

template <class T, class I, std::size_t E0, std::size_t E1, std::size_t E2, class L>
EulerConsArrays<Kokkos::mdspan<T const, Kokkos::extents<I, E0, E1, E2>, L>> as_const(
        EulerConsArrays<Kokkos::mdspan<T, Kokkos::extents<I, E0, E1, E2>, L>> const& a) noexcept
{
    return as<Kokkos::mdspan<T const, Kokkos::extents<I, E0, E1, E2>, L>>(a);
}

// The same slices of every view of a bundle (euler_arrays.hpp:106-117,
// 257-268): Kokkos::submdspan with an index, Kokkos::full_extent or a
// [first, last) pair per axis.  A slice that keeps the leading axes, all
// but the last of them whole, stays layout_left and can be passed to the
// operators; any other is layout_stride.
template <class E, class X, class L, class A, class... Slices>
auto subspan(EulerPrimArrays<Kokkos::mdspan<E, X, L, A>> const& a, Slices const&... s)
{
    using V = decltype(Kokkos::submdspan(a.d, s...));
    return EulerPrimArrays<V> {Kokkos::submdspan(a.d, s...), Kokkos::submdspan(a.p, s...),
                               Kokkos::submdspan(a.ux0, s...), Kokkos::submdspan(a.ux1, s...),
                               Kokkos::submdspan(a.ux2, s...)};
}

template <class E, class X, class L, class A, class... Slices>
auto subspan(EulerConsArrays<Kokkos::mdspan<E, X, L, A>> const& a, Slices const&... s)
{
    using V = decltype(Kokkos::submdspan(a.d, s...));
    return EulerConsArrays<V> {Kokkos::submdspan(a.d, s...), Kokkos::submdspan(a.e, s...),
                               Kokkos::submdspan(a.mx0, s...), Kokkos::submdspan(a.mx1, s...),
                               Kokkos::submdspan(a.mx2, s...)};
}

template <class E, class X, class L, class A>
EulerPrimArrays<typename A::data_handle_type> data_handle(EulerPrimArrays<Kokkos::mdspan<E, X, L, A>> const& a) noexcept
{
    return {a.d.data_handle(), a.p.data_handle(), a.ux0.data_handle(), a.ux1.data_handle(), a.ux2.data_handle()};
}

template <class E, class X, class L, class A>
EulerConsArrays<typename A::data_handle_type> data_handle(EulerConsArrays<Kokkos::mdspan<E, X, L, A>> const& a) noexcept
{
    return {a.d.data_handle(), a.e.data_handle(), a.mx0.data_handle(), a.mx1.data_handle(), a.mx2.data_handle()};
}

// Views over the owning 1D arrays of a bundle (euler_arrays.hpp:130-142).
template <class MdspanOut, class View>
EulerPrimArrays<MdspanOut> to_mdspan(EulerPrimArrays<View> const& a, typename MdspanOut::index_type nx,
                                     typename MdspanOut::index_type ny, typename MdspanOut::index_type nz) noexcept
{
    return {MdspanOut(a.d.data(), nx, ny, nz), MdspanOut(a.p.data(), nx, ny, nz), MdspanOut(a.ux0.data(), nx, ny, nz),
            MdspanOut(a.ux1.data(), nx, ny, nz), MdspanOut(a.ux2.data(), nx, ny, nz)};
}

template <class MdspanOut, class View>
EulerConsArrays<MdspanOut> to_mdspan(EulerConsArrays<View> const& a, typename MdspanOut::index_type nx,
                                     typename MdspanOut::index_type ny, typename MdspanOut::index_type nz) noexcept
{
    return {MdspanOut(a.d.data(), nx, ny, nz), MdspanOut(a.e.data(), nx, ny, nz), MdspanOut(a.mx0.data(), nx, ny, nz),
            MdspanOut(a.mx1.data(), nx, ny, nz), MdspanOut(a.mx2.data(), nx, ny, nz)};
}

// Host-side point access (the arrays are managed or host memory).
template <class E, class I, std::size_t E0, std::size_t E1, std::size_t E2, class L, class A>
EulerPrim<std::remove_const_t<E>> load(EulerPrimArrays<Kokkos::mdspan<E, Kokkos::extents<I, E0, E1, E2>, L, A>> const& a,
                                       I i, I j, I k) noexcept
{
    return {a.d(i, j, k), a.p(i, j, k), a.ux0(i, j, k), a.ux1(i, j, k), a.ux2(i, j, k)};
}

template <class E, class I, std::size_t E0, std::size_t E1, std::size_t E2, class L, class A>
EulerCons<std::remove_const_t<E>> load(EulerConsArrays<Kokkos::mdspan<E, Kokkos::extents<I, E0, E1, E2>, L, A>> const& a,
                                       I i, I j, I k) noexcept
{
    return {a.d(i, j, k), a.e(i, j, k), a.mx0(i, j, k), a.mx1(i, j, k), a.mx2(i, j, k)};
}

template <class E, class I, std::size_t E0, std::size_t E1, std::size_t E2, class L, class A>
void store(EulerPrim<E> const& q, EulerPrimArrays<Kokkos::mdspan<E, Kokkos::extents<I, E0, E1, E2>, L, A>> const& a,
           I i, I j, I k) noexcept
{
    a.d(i, j, k) = q.d;
    a.p(i, j, k) = q.p;
    a.ux0(i, j, k) = q.ux0;
    a.ux1(i, j, k) = q.ux1;
    a.ux2(i, j, k) = q.ux2;
}

template <class E, class I, std::size_t E0, std::size_t E1, std::size_t E2, class L, class A>
void store(EulerCons<E> const& u, EulerConsArrays<Kokkos::mdspan<E, Kokkos::extents<I, E0, E1, E2>, L, A>> const& a,
           I i, I j, I k) noexcept
{
    a.d(i, j, k) = u.d;
    a.e(i, j, k) = u.e;
    a.mx0(i, j, k) = u.mx0;
    a.mx1(i, j, k) = u.mx1;
    a.mx2(i, j, k) = u.mx2;
}

template <class E, class X, class L, class A>
std::size_t size(EulerPrimArrays<Kokkos::mdspan<E, X, L, A>> const& a) noexcept
{
    return a.d.size();
}

template <class E, class X, class L, class A>
std::size_t size(EulerConsArrays<Kokkos::mdspan<E, X, L, A>> const& a) noexcept
{
    return a.d.size();
}

// bytes of the five arrays of a bundle (euler_arrays.hpp:381-399)
template <class E, class X, class L, class A>
std::size_t size_bytes(EulerPrimArrays<Kokkos::mdspan<E, X, L, A>> const& a) noexcept
{
    return 5 * sizeof(E) * size(a);
}

template <class E, class X, class L, class A>
std::size_t size_bytes(EulerConsArrays<Kokkos::mdspan<E, X, L, A>> const& a) noexcept
{
    return 5 * sizeof(E) * size(a);
}

template <class T>
EulerPrimArrays<Kokkos::View<T*>> create_prim_arrays_1d(Kokkos::DefaultExecutionSpace const& exec, std::size_t n)
{
    return {Kokkos::View<T*>(Kokkos::view_alloc(exec, "density"), n),
            Kokkos::View<T*>(Kokkos::view_alloc(exec, "pressure"), n),
            Kokkos::View<T*>(Kokkos::view_alloc(exec, "ux0"), n), Kokkos::View<T*>(Kokkos::view_alloc(exec, "ux1"), n),
            Kokkos::View<T*>(Kokkos::view_alloc(exec, "ux2"), n)};
}

template <class T>
EulerConsArrays<Kokkos::View<T*>> create_cons_arrays_1d(Kokkos::DefaultExecutionSpace const& exec, std::size_t n)
{
    return {Kokkos::View<T*>(Kokkos::view_alloc(exec, "density"), n),
            Kokkos::View<T*>(Kokkos::view_alloc(exec, "energy"), n),
            Kokkos::View<T*>(Kokkos::view_alloc(exec, "mx0"), n), Kokkos::View<T*>(Kokkos::view_alloc(exec, "mx1"), n),
            Kokkos::View<T*>(Kokkos::view_alloc(exec, "mx2"), n)};
}
