// euler_operators drop-in for GB300: the HLLC approximate Riemann solver of
// the reference's euler_operators/hllc.hpp -- the normal-component accessors
// get(dir, state) (:11-48) and hllc::operator() (:50-105), the flux across
// one face whose normal is axis Dir, from the primitive states on its left
// and right.
//
// godunov (godunov.hpp) does not call this functor: the CUDA library's
// kernels solve each face once with their own reorganised arithmetic.  The
// functor is here for code written against the reference that calls the
// solver itself, on the host or, compiled by nvcc, in device code.
//
// Its result is the reference's bit for bit: every operation is the
// reference's, in the reference's order, and each is rounded separately.
// On the device that is enforced with the _rn intrinsics (nvcc would
// otherwise fuse products and sums into FMAs); host code must be compiled
// without floating-point contraction (-ffp-contract=off; GCC's GNU dialects
// contract by default on targets with an FMA instruction, e.g. aarch64), as
// the reference must be for its own results to be reproducible.
#pragma once

#include <cmath>
#include <cstddef>
#include <type_traits>

#include <euler_arrays.hpp>
#include <perfect_gas.hpp>

#if defined(__CUDACC__)
#define EULR_HOST_DEVICE __host__ __device__
#else
#define EULR_HOST_DEVICE
#endif

namespace euler_gb300_hllc_detail {

// IEEE operations rounded one at a time.  Generic scalars use their own
// operators; double and float on the device use the round-to-nearest
// intrinsics, which the compiler never contracts.
template <class T>
EULR_HOST_DEVICE inline T add(T a, T b) noexcept { return a + b; }
template <class T>
EULR_HOST_DEVICE inline T sub(T a, T b) noexcept { return a - b; }
template <class T>
EULR_HOST_DEVICE inline T mul(T a, T b) noexcept { return a * b; }
template <class T>
EULR_HOST_DEVICE inline T quo(T a, T b) noexcept { return a / b; }
template <class T>
EULR_HOST_DEVICE inline T root(T a) noexcept
{
    using std::sqrt;
    return sqrt(a);
}

#if defined(__CUDA_ARCH__)
template <>
__device__ inline double add<double>(double a, double b) noexcept { return __dadd_rn(a, b); }
template <>
__device__ inline double sub<double>(double a, double b) noexcept { return __dsub_rn(a, b); }
template <>
__device__ inline double mul<double>(double a, double b) noexcept { return __dmul_rn(a, b); }
template <>
__device__ inline double quo<double>(double a, double b) noexcept { return __ddiv_rn(a, b); }
template <>
__device__ inline double root<double>(double a) noexcept { return __dsqrt_rn(a); }
template <>
__device__ inline float add<float>(float a, float b) noexcept { return __fadd_rn(a, b); }
template <>
__device__ inline float sub<float>(float a, float b) noexcept { return __fsub_rn(a, b); }
template <>
__device__ inline float mul<float>(float a, float b) noexcept { return __fmul_rn(a, b); }
template <>
__device__ inline float quo<float>(float a, float b) noexcept { return __fdiv_rn(a, b); }
template <>
__device__ inline float root<float>(float a) noexcept { return __fsqrt_rn(a); }
#endif

// Kokkos::min / Kokkos::max: the second argument only when it is strictly
// smaller / larger, so ties (including +0 against -0) keep the first.
template <class T>
EULR_HOST_DEVICE inline T lesser(T a, T b) noexcept { return b < a ? b : a; }
template <class T>
EULR_HOST_DEVICE inline T greater(T a, T b) noexcept { return a < b ? b : a; }

// The perfect-gas relations of PerfectGas<U> (perfect_gas.hpp:15-23),
// evaluated in U as the reference's equation of state evaluates them.
template <class U, class T>
EULR_HOST_DEVICE inline T sound_speed(U gamma, T d, T p) noexcept
{
    return static_cast<T>(root(quo(mul(gamma, static_cast<U>(p)), static_cast<U>(d))));
}

template <class U, class T>
EULR_HOST_DEVICE inline U internal_energy(U gamma, T p) noexcept
{
    return quo(static_cast<U>(p), sub(gamma, static_cast<U>(1)));
}

// rho |u|^2 / 2 (euler_arrays.hpp:38-42)
template <class T>
EULR_HOST_DEVICE inline T kinetic_energy(EulerPrim<T> const& q) noexcept
{
    T const u2 = add(add(mul(q.ux0, q.ux0), mul(q.ux1, q.ux1)), mul(q.ux2, q.ux2));
    return quo(mul(q.d, u2), static_cast<T>(2));
}

} // namespace euler_gb300_hllc_detail

// The component of a state's velocity, momentum or momentum flux along axis
// Dir (hllc.hpp:11-48).
template <std::size_t Dir, class T>
EULR_HOST_DEVICE T get(std::integral_constant<std::size_t, Dir> /*axis*/, EulerPrim<T> const& q) noexcept
{
    static_assert(Dir < 3, "a state has three velocity components");
    T const u[3] = {q.ux0, q.ux1, q.ux2};
    return u[Dir];
}

template <std::size_t Dir, class T>
EULR_HOST_DEVICE T get(std::integral_constant<std::size_t, Dir> /*axis*/, EulerCons<T> const& c) noexcept
{
    static_assert(Dir < 3, "a state has three momentum components");
    T const m[3] = {c.mx0, c.mx1, c.mx2};
    return m[Dir];
}

template <std::size_t Dir, class T>
EULR_HOST_DEVICE T get(std::integral_constant<std::size_t, Dir> /*axis*/, EulerFlux<T> const& f) noexcept
{
    static_assert(Dir < 3, "a flux has three momentum components");
    T const m[3] = {f.mx0, f.mx1, f.mx2};
    return m[Dir];
}

struct hllc
{
    // The HLLC flux across a face normal to axis Dir with primitive states
    // q_L (low side) and q_R (high side), the reference's hllc::operator()
    // (hllc.hpp:50-105): Davis wave speeds S_L, S_R, the contact speed ustar
    // and star pressure pstar of the two-shock linearisation, the state on
    // the upwind side of the contact, and -- unless both waves move the same
    // way (S_L S_R > 0, where the flux is that side's own) -- its star state.
    template <std::size_t Dir, class T, class U>
    EULR_HOST_DEVICE EulerFlux<T> operator()(
            std::integral_constant<std::size_t, Dir> axis,
            PerfectGas<U> const& eos,
            EulerPrim<T> const& q_L,
            EulerPrim<T> const& q_R) const noexcept
    {
        static_assert(Dir < 3, "three axes");
        namespace a = euler_gb300_hllc_detail;
        using R = std::common_type_t<T, U>;
        U const gamma = eos.gamma();

        T const un_L = get(axis, q_L);
        T const un_R = get(axis, q_R);
        T const c_fast = a::greater(a::sound_speed(gamma, q_L.d, q_L.p), a::sound_speed(gamma, q_R.d, q_R.p));
        T const S_L = a::sub(a::lesser(un_L, un_R), c_fast);
        T const S_R = a::add(a::greater(un_L, un_R), c_fast);

        // mass fluxes relative to each wave
        T const rc_L = a::mul(q_L.d, a::sub(S_L, un_L));
        T const rc_R = a::mul(q_R.d, a::sub(S_R, un_R));

        T const num = a::sub(a::add(a::sub(q_R.p, q_L.p), a::mul(rc_L, un_L)), a::mul(rc_R, un_R));
        T const ustar = a::quo(num, a::sub(rc_L, rc_R));
        T const psum = a::add(a::add(a::add(q_L.p, q_R.p), a::mul(rc_L, a::sub(ustar, un_L))),
                              a::mul(rc_R, a::sub(ustar, un_R)));
        T const pstar = static_cast<T>(a::mul(static_cast<R>(static_cast<U>(0.5)), static_cast<R>(psum)));

        // the side the contact leaves behind: its wave and its state
        bool const from_left = ustar > 0;
        T const S = from_left ? S_L : S_R;
        EulerPrim<T> const& q = from_left ? q_L : q_R;
        T const un = get(axis, q);
        T const etot = static_cast<T>(
                a::add(static_cast<R>(a::internal_energy(gamma, q.p)), static_cast<R>(a::kinetic_energy(q))));

        // both waves on one side of the face: that side's own flux
        bool const one_sided = a::mul(S_L, S_R) > 0;
        T const un_o = one_sided ? un : ustar;
        T const ptot_o = one_sided ? q.p : pstar;

        T const gap = a::sub(S, un);
        T const gap_o = a::sub(S, un_o);
        T const d_o = a::mul(a::quo(gap, gap_o), q.d);
        T const work = a::quo(a::sub(a::mul(ptot_o, un_o), a::mul(q.p, un)), a::sub(S, ustar));
        T const etot_o = a::add(a::mul(a::quo(gap, gap_o), etot), work);

        T const mass = a::mul(d_o, un_o);
        EulerFlux<T> f {};
        f.d = mass;
        f.e = a::mul(a::add(etot_o, ptot_o), un_o);
        f.mx0 = a::mul(mass, q.ux0);
        f.mx1 = a::mul(mass, q.ux1);
        f.mx2 = a::mul(mass, q.ux2);
        T const normal = a::add(a::mul(mass, un_o), ptot_o);
        if constexpr (Dir == 0) {
            f.mx0 = normal;
        } else if constexpr (Dir == 1) {
            f.mx1 = normal;
        } else {
            f.mx2 = normal;
        }
        return f;
    }
};
