// Test-only C ABI over the reference's own operators.
//
// This translation unit includes the reference headers
// (euler_operators/{euler_arrays,perfect_gas,uniform_mesh,hllc,godunov,
// time_step,prim_to_cons,cons_to_prim,init_implode}.hpp) UNMODIFIED, compiled
// against the Kokkos compatibility layer in oracle/kokkos_compat, and exposes
// them as plain C functions over host arrays.  The recipe in oracle/Makefile
// builds it into oracle/_ref/libeuler_ref.so.  It is the reference build that pins the
// C restatement (oracle/euler_oracle.c) and generates the committed golden
// fixtures; it is never part of the product.
//
// Array arguments are 5 host pointers per bundle in the reference's field
// order: prim = (d, p, ux0, ux1, ux2), cons = (d, e, mx0, mx1, mx2), each a
// layout_left (i fastest) block of n0*n1*n2 values.

#include <cons_to_prim.hpp>
#include <euler_arrays.hpp>
#include <godunov.hpp>
#include <hllc.hpp>
#include <init_implode.hpp>
#include <perfect_gas.hpp>
#include <prim_to_cons.hpp>
#include <time_step.hpp>
#include <uniform_mesh.hpp>

namespace {

using index_t = int; // benchmarks/index_type.hpp:4

template <class T>
using span3 = Kokkos::mdspan<T, Kokkos::dextents<index_t, 3>, Kokkos::layout_left>;

template <class T>
EulerPrimArrays<span3<T>> prim_view(T* const* f, int n0, int n1, int n2)
{
    return {.d = span3<T>(f[0], n0, n1, n2),
            .p = span3<T>(f[1], n0, n1, n2),
            .ux0 = span3<T>(f[2], n0, n1, n2),
            .ux1 = span3<T>(f[3], n0, n1, n2),
            .ux2 = span3<T>(f[4], n0, n1, n2)};
}

template <class T>
EulerConsArrays<span3<T>> cons_view(T* const* f, int n0, int n1, int n2)
{
    return {.d = span3<T>(f[0], n0, n1, n2),
            .e = span3<T>(f[1], n0, n1, n2),
            .mx0 = span3<T>(f[2], n0, n1, n2),
            .mx1 = span3<T>(f[3], n0, n1, n2),
            .mx2 = span3<T>(f[4], n0, n1, n2)};
}

template <class T>
void init_implode_t(T* const* prim, int n0, int n1, int n2, T dx0, T dx1, T dx2)
{
    Kokkos::DefaultExecutionSpace const exec;
    init_implode(exec, prim_view(prim, n0, n1, n2), UniformMesh3d<T>(dx0, dx1, dx2));
}

template <class T>
void prim_to_cons_t(T* const* prim, T* const* cons, int n0, int n1, int n2, T gamma)
{
    Kokkos::DefaultExecutionSpace const exec;
    prim_to_cons(
            exec,
            as_const(prim_view(prim, n0, n1, n2)),
            cons_view(cons, n0, n1, n2),
            PerfectGas<T>(gamma));
}

template <class T>
void cons_to_prim_t(T* const* cons, T* const* prim, int n0, int n1, int n2, T gamma)
{
    Kokkos::DefaultExecutionSpace const exec;
    cons_to_prim(
            exec,
            as_const(cons_view(cons, n0, n1, n2)),
            prim_view(prim, n0, n1, n2),
            PerfectGas<T>(gamma));
}

template <class T>
T time_step_t(T* const* prim, int n0, int n1, int n2, T gamma, T dx0, T dx1, T dx2)
{
    Kokkos::DefaultExecutionSpace const exec;
    return time_step(
            exec,
            as_const(prim_view(prim, n0, n1, n2)),
            PerfectGas<T>(gamma),
            UniformMesh3d<T>(dx0, dx1, dx2));
}

template <class T>
void godunov_t(
        T* const* prim,
        T* const* cons,
        int n0,
        int n1,
        int n2,
        T gamma,
        T dx0,
        T dx1,
        T dx2,
        T dt)
{
    Kokkos::DefaultExecutionSpace const exec;
    godunov(exec,
            as_const(prim_view(prim, n0, n1, n2)),
            cons_view(cons, n0, n1, n2),
            PerfectGas<T>(gamma),
            UniformMesh3d<T>(dx0, dx1, dx2),
            hllc(),
            dt);
}

// The time loop of simulations/euler_simulation.cpp:56-68 (without output).
template <class T>
void simulate_t(
        T* const* prim,
        T* const* cons,
        int n0,
        int n1,
        int n2,
        T gamma,
        T dx0,
        T dx1,
        T dx2,
        T cfl,
        int nsteps,
        double* t_out)
{
    Kokkos::DefaultExecutionSpace const exec;
    PerfectGas<T> const eos(gamma);
    UniformMesh3d<T> const mesh(dx0, dx1, dx2);
    auto const pv = prim_view(prim, n0, n1, n2);
    auto const cv = cons_view(cons, n0, n1, n2);
    double t = 0;
    for (int it = 0; it < nsteps; ++it) {
        T const dt = time_step(exec, as_const(pv), eos, mesh);
        godunov(exec, as_const(pv), cv, eos, mesh, hllc(), cfl * dt);
        cons_to_prim(exec, as_const(cv), pv, eos);
        t += static_cast<double>(cfl * dt);
    }
    if (t_out != nullptr) {
        *t_out = t;
    }
}

// One face through the reference's own hllc functor (hllc.hpp:50-105).
template <class T>
void hllc_face_t(int dir, T g, T const* qL, T const* qR, T* f)
{
    PerfectGas<T> const eos(g);
    EulerPrim<T> const a {.d = qL[0], .p = qL[1], .ux0 = qL[2], .ux1 = qL[3], .ux2 = qL[4]};
    EulerPrim<T> const b {.d = qR[0], .p = qR[1], .ux0 = qR[2], .ux1 = qR[3], .ux2 = qR[4]};
    EulerFlux<T> r {};
    if (dir == 0) {
        r = hllc()(dir_t<0>(), eos, a, b);
    } else if (dir == 1) {
        r = hllc()(dir_t<1>(), eos, a, b);
    } else {
        r = hllc()(dir_t<2>(), eos, a, b);
    }
    f[0] = r.d;
    f[1] = r.e;
    f[2] = r.mx0;
    f[3] = r.mx1;
    f[4] = r.mx2;
}

} // namespace

extern "C" {

#define EULER_REF_DEFINE(SUFFIX, T)                                                                 \
    void ref_init_implode_##SUFFIX(T* const* prim, int n0, int n1, int n2, T dx0, T dx1, T dx2)    \
    {                                                                                              \
        init_implode_t<T>(prim, n0, n1, n2, dx0, dx1, dx2);                                        \
    }                                                                                              \
    void ref_prim_to_cons_##SUFFIX(T* const* prim, T* const* cons, int n0, int n1, int n2, T g)   \
    {                                                                                              \
        prim_to_cons_t<T>(prim, cons, n0, n1, n2, g);                                              \
    }                                                                                              \
    void ref_cons_to_prim_##SUFFIX(T* const* cons, T* const* prim, int n0, int n1, int n2, T g)   \
    {                                                                                              \
        cons_to_prim_t<T>(cons, prim, n0, n1, n2, g);                                              \
    }                                                                                              \
    T ref_time_step_##SUFFIX(T* const* prim, int n0, int n1, int n2, T g, T dx0, T dx1, T dx2)    \
    {                                                                                              \
        return time_step_t<T>(prim, n0, n1, n2, g, dx0, dx1, dx2);                                 \
    }                                                                                              \
    void ref_godunov_##SUFFIX(                                                                     \
            T* const* prim, T* const* cons, int n0, int n1, int n2, T g, T dx0, T dx1, T dx2, T dt) \
    {                                                                                              \
        godunov_t<T>(prim, cons, n0, n1, n2, g, dx0, dx1, dx2, dt);                                \
    }                                                                                              \
    void ref_simulate_##SUFFIX(                                                                    \
            T* const* prim,                                                                        \
            T* const* cons,                                                                        \
            int n0,                                                                                \
            int n1,                                                                                \
            int n2,                                                                                \
            T g,                                                                                   \
            T dx0,                                                                                 \
            T dx1,                                                                                 \
            T dx2,                                                                                 \
            T cfl,                                                                                 \
            int nsteps,                                                                            \
            double* t_out)                                                                         \
    {                                                                                              \
        simulate_t<T>(prim, cons, n0, n1, n2, g, dx0, dx1, dx2, cfl, nsteps, t_out);               \
    }                                                                                              \
    void ref_hllc_face_##SUFFIX(int dir, T g, T const* qL, T const* qR, T* f)                      \
    {                                                                                              \
        hllc_face_t<T>(dir, g, qL, qR, f);                                                         \
    }

EULER_REF_DEFINE(f64, double)
EULER_REF_DEFINE(f32, float)

#undef EULER_REF_DEFINE
}
