// Device-side building blocks shared by the Euler kernels (sm_103a).
//
// Two arithmetic styles are used:
//  * "exact" helpers (mul_rn, add_rn, ...) issue one IEEE-rounded operation
//    each and never contract into FMA.  The pointwise operators use them so
//    that their results are bit-identical to the reference operators, which
//    are written as separately rounded products and sums.
//  * plain C++ arithmetic, which nvcc contracts into FMAs.  The flux kernels
//    use it: every face is solved once instead of twice, shared reciprocals
//    replace divisions, and the results agree with the reference to a few
//    units in the last place per step.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "halve.cuh"

namespace eulr {

template <class T>
struct Bundle {
    T* f[5];
};

template <class T>
struct CBundle {
    const T* f[5];
};

// Grid extents and strides of a layout_left block (i fastest).
struct Geom {
    int n0, n1, n2;
    long long s1; // n0
    long long s2; // n0 * n1
    __host__ __device__ long long ncell() const { return s2 * n2; }
    __host__ __device__ long long at(int i, int j, int k) const { return i + s1 * j + s2 * k; }
};

inline Geom make_geom(int n0, int n1, int n2)
{
    Geom g;
    g.n0 = n0;
    g.n1 = n1;
    g.n2 = n2;
    g.s1 = n0;
    g.s2 = static_cast<long long>(n0) * n1;
    return g;
}

// ------------------------------------------------ separately rounded ops
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rcp_rn(double a) { return __drcp_rn(a); }
__device__ __forceinline__ float rcp_rn(float a) { return __frcp_rn(a); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double sqrt_rn(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float sqrt_rn(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double abs_(double a) { return fabs(a); }
// x * 0.5 with the bits of a DMUL by 0.5, on the integer pipe (halve.cuh);
// the asm move keeps the compiler from turning the bit arithmetic back into
// an FP64 multiply.
__device__ __forceinline__ double half_exact(double x)
{
    unsigned long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return __longlong_as_double(static_cast<long long>(halve_bits(b)));
}
__device__ __forceinline__ float half_exact(float x) { return __fmul_rn(x, 0.5f); }
__device__ __forceinline__ float abs_(float a) { return fabsf(a); }

// Correctly rounded x / y given r = RN(1/y): q0 = RN(x r) is within one ulp
// of x/y, the remainder x - q0 y is exact through one FMA, and
// RN(q0 + rem r) is the correctly rounded quotient (Markstein's correction
// step; P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990).  Valid away from
// overflow and underflow, which the Euler states here never approach.
template <class T>
__device__ __forceinline__ T div_by_rcp(T x, T y, T r)
{
    T const q0 = mul_rn(x, r);
    T const rem = fma_rn(-q0, y, x);
    return fma_rn(rem, r, q0);
}

// Faithful FP64 reciprocal and square root (within one ulp of the correctly
// rounded result, not always equal to it) for the fused step, whose parity
// bar is a relative tolerance.  Each refines the PTX hardware approximation
// (rcp.approx.ftz.f64, rsqrt.approx.ftz.f64; both measured at most 2^-19.9
// relative error on sm_103a) by one Newton-Raphson step carried to third
// order, from the series 1/(1-e) = 1 + e + e^2 + ... and
// 1/sqrt(1-e) = 1 + e/2 + 3e^2/8 + ...:
//   1/x:      r0 ~ 1/x,       e = 1 - x r0,       1/x     ~ r0 (1 + e + e^2)
//   sqrt(x):  y0 ~ 1/sqrt(x), t = x y0, e = 1 - t y0, sqrt(x) ~ t (1 + e/2 + 3e^2/8)
// The truncation error is O(e^3) <= 2^-59, so the result is within one ulp
// of the correctly rounded value (measured: at most 1 ulp over 4M arguments
// spanning 2^+-100); three (five) FP64 instructions in place of the
// correctly rounded sequences.  Zero, infinite and subnormal
// arguments give NaN or zero instead of the IEEE results (the approximations
// flush subnormals): physical Euler states never reach them, and a
// non-physical state is reported as non-finite either way.
__device__ __forceinline__ double rcp_faithful(double x)
{
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = __fma_rn(-x, r, 1.0);
    e = __fma_rn(e, e, e);
    return __fma_rn(r, e, r);
}
__device__ __forceinline__ float rcp_faithful(float x) { return __frcp_rn(x); }

__device__ __forceinline__ double sqrt_faithful(double x)
{
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double const t = x * y;
    double const e = __fma_rn(-t, y, 1.0);
    double const q = __fma_rn(0.375, e, 0.5);
    return __fma_rn(t, e * q, t);
}

// The hardware's FP32 approximations themselves (one MUFU instruction each,
// relative error below 2^-22): the FP32 steps' error is set by the state's
// own rounding.  Inputs are normal positive numbers there; ftz maps a
// subnormal input to zero (1/x = +inf) and a result below 2^-126 to zero,
// which no physical state reaches.
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// sqrt(x / d) for x, d > 0 without a reciprocal: x * rsqrt(x d), the PTX
// approximation of 1/sqrt refined by the third-order step of sqrt_faithful
// (y (1 + e/2 + 3e^2/8), e = 1 - z y^2).  Seven FP64 instructions and one
// seed where rcp_faithful + sqrt_faithful take ten and two; within two ulps
// of the correctly rounded sqrt(x/d) (checked against it on 4M argument
// pairs).  For the sound speed sqrt(gamma p / rho) of a state whose 1/rho
// is not needed otherwise.
__device__ __forceinline__ double sqrt_quotient_faithful(double x, double d)
{
    double const z = x * d;
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(z));
    double const e = __fma_rn(-(z * y), y, 1.0);
    double const q = __fma_rn(0.375, e, 0.5);
    return x * __fma_rn(y, e * q, y);
}

// Non-negative values ordered as their bit patterns; NaN maps to 0 so that it
// never wins a max (the reference's Kokkos::min over 1/invdt skips NaN).
__device__ __forceinline__ unsigned long long order_bits(double v)
{
    return (v >= 0.0) ? static_cast<unsigned long long>(__double_as_longlong(v)) : 0ull;
}
__device__ __forceinline__ unsigned long long order_bits(float v)
{
    return order_bits(static_cast<double>(v));
}

template <class T>
__device__ __forceinline__ T warp_max(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T const w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (w > v) ? w : v;
    }
    return v;
}

// cons_to_prim of one cell, bit-identical to cons_to_prim.hpp:20-32 with
// kinetic_energy(cons) (euler_arrays.hpp:44-48), PerfectGas::pressure
// (perfect_gas.hpp:25-28) and to_prim (euler_arrays.hpp:66-75):
//   ke = ((m.m)/d)/2, p = (gamma-1)*(e-ke), u_i = m_i * (1/d).
// Both quotients come from one reciprocal of d (div_by_rcp).
template <class T>
__device__ __forceinline__ void cons_to_prim_exact(T d, T e, T m0, T m1, T m2, T gm1, T& p, T& u0, T& u1, T& u2)
{
    T const r = rcp_rn(d);
    T const mm = add_rn(add_rn(mul_rn(m0, m0), mul_rn(m1, m1)), mul_rn(m2, m2));
    T const ke = half_exact(div_by_rcp(mm, d, r));
    p = mul_rn(gm1, sub_rn(e, ke));
    u0 = mul_rn(m0, r);
    u1 = mul_rn(m1, r);
    u2 = mul_rn(m2, r);
}

// (c + |u0|)/dx0 + (c + |u1|)/dx1 + (c + |u2|)/dx2 of one cell with
// c = sqrt((gamma p)/d), bit-identical to time_step.hpp:28-33 and
// perfect_gas.hpp:15-18 (ix_d = 1/dx_d computed by the caller in T).
template <class T>
__device__ __forceinline__ T cell_invdt_exact(T d, T p, T u0, T u1, T u2, T gamma, T ix0, T ix1, T ix2)
{
    T const cs = sqrt_rn(div_rn(mul_rn(gamma, p), d));
    T const c0 = add_rn(cs, abs_(u0));
    T const c1 = add_rn(cs, abs_(u1));
    T const c2 = add_rn(cs, abs_(u2));
    return add_rn(add_rn(mul_rn(c0, ix0), mul_rn(c1, ix1)), mul_rn(c2, ix2));
}

// ------------------------------------------- FP32 cons_to_prim with FP64 rescue
// Below this fraction of e the FP32 internal-energy subtraction
// e - |m|^2/(2 rho) has lost more than 8 of its 24 bits.
constexpr float kLowPressure = 1.0f / 256.0f;

// The FP64 internal energy of a low-pressure cell, (gamma-1) (e - |m|^2/(2 rho))
// from the FP32 words (hi, plus the low words when the state stores them).
// 1/rho is the FP32 reciprocal r refined by one Newton step in FP64
// (relative error about 2^-44): no FP64 division routine.  Out of line: the
// path is rare, and inlined its FP64 registers weigh on every cell's code.
static __device__ __noinline__ float pressure_f64_rescue(float d, float e, float m0, float m1, float m2, float r, float gm1,
                                                  const float* lo)
{
    double const dd = static_cast<double>(d) + (lo ? static_cast<double>(lo[0]) : 0.0);
    double const ed = static_cast<double>(e) + (lo ? static_cast<double>(lo[1]) : 0.0);
    double const a0 = static_cast<double>(m0) + (lo ? static_cast<double>(lo[2]) : 0.0);
    double const a1 = static_cast<double>(m1) + (lo ? static_cast<double>(lo[3]) : 0.0);
    double const a2 = static_cast<double>(m2) + (lo ? static_cast<double>(lo[4]) : 0.0);
    double rd = static_cast<double>(r);
    rd = rd * __fma_rn(-dd, rd, 2.0);
    double const ke = 0.5 * (a0 * a0 + a1 * a1 + a2 * a2) * rd;
    return static_cast<float>(static_cast<double>(gm1) * (ed - ke));
}

// Pressure of an FP32 conservative state: the subtraction runs in FP32
// unless the cell's internal energy is below kLowPressure of its total
// energy, where it is redone in FP64 (pressure_f64_rescue).
__device__ __forceinline__ float pressure_f32c(float d, float e, float m0, float m1, float m2, float r, float gm1,
                                               const float* lo)
{
    float const mm = m0 * m0 + m1 * m1 + m2 * m2;
    float const eint = e - (0.5f * r) * mm;
    if (eint > kLowPressure * e) {
        return gm1 * eint;
    }
    return pressure_f64_rescue(d, e, m0, m1, m2, r, gm1, lo);
}

// ------------------------------------------------------------------ HLLC
// One side of a face in the face's frame: normal velocity un, tangential
// velocities ut1/ut2 (in the cyclic order of the axes after the normal), sound
// speed c and, in `e`, the sum e + p of total energy density and pressure:
// the HLLC needs only that sum, which the staging forms once per cell.
template <class T>
struct Side {
    T d, p, un, ut1, ut2, c, e;
};

template <class T>
struct Flux {
    T d, e, n, t1, t2;
};

// ------------------------------------------------- integer-pipe predicates
// On GB300 an FP64 compare, min or max takes a full slot of the FP64 pipe
// (1/64 of the FP32 rate); the same decisions taken on the bit patterns run
// on the integer pipe, which the flux kernels leave almost idle.
// The bit pattern through an opaque move: tests written on the bits must stay
// on the integer pipe.  With a plain reinterpretation the compiler rewrote
// (bits << 1) != 0 into the equivalent FP64 compare x != 0, which takes an
// FP64 slot (four per HLLC face: 12.6 FP64 instructions per cell of the step).
__device__ __forceinline__ long long dbits(double x)
{
    long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return b;
}

// Signed key with the order of the doubles (-0 sorts just below +0).
__device__ __forceinline__ long long order_key(double x)
{
    long long const b = dbits(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

// x is neither +0 nor -0.
__device__ __forceinline__ bool nonzero_(double x) { return (dbits(x) << 1) != 0; }

// a*b > 0 for non-NaN a, b, decided from signs: both non-zero and of one sign.
__device__ __forceinline__ bool product_positive(double a, double b)
{
    return nonzero_(a) && nonzero_(b) && ((dbits(a) ^ dbits(b)) >= 0);
}

// a < b with IEEE semantics (false when either is NaN; -0 and +0 equal),
// decided on the integer pipe: the bit patterns mapped to ordered keys with
// both zeros at 0.  The same answer as the FP64 compare, which would take an
// FP64 slot.
__device__ __forceinline__ bool is_nan_bits(long long b) { return (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }
__device__ __forceinline__ bool less_ieee(double a, double b)
{
    long long const x = dbits(a), y = dbits(b);
    long long const kx = (x << 1) == 0 ? 0 : (x ^ ((x >> 63) & 0x7fffffffffffffffLL));
    long long const ky = (y << 1) == 0 ? 0 : (y ^ ((y >> 63) & 0x7fffffffffffffffLL));
    return !is_nan_bits(x) && !is_nan_bits(y) && kx < ky;
}
__device__ __forceinline__ bool less_ieee(float a, float b) { return a < b; }

// Finite and > 0.
__device__ __forceinline__ bool finite_positive(double x)
{
    long long const b = dbits(x);
    return b > 0 && b < 0x7ff0000000000000LL;
}

// HLLC flux of hllc::operator() (euler_operators/hllc.hpp:50-105) in the face
// frame: wave speeds (:64-68), acoustic star state (:70-76), upwind side by
// the sign of ustar (:78-79), supersonic test S_L*S_R > 0 (:84-85), star
// density and energy (:86-88) and the flux (:90-102).  Reformulated to spend
// as few FP64 instructions as possible; in exact arithmetic it is the same
// function:
//  * ustar = num/den and 1/(S - ustar) = den/(S den - num) come from ONE
//    reciprocal R = 1/(den (S den - num)): ustar = num (S den - num) R and
//    1/(S - ustar) = den^2 R.  The side (sign of ustar) is read from the signs
//    of num and den before any division.
//  * pstar: the reference averages p_L + rc_L (ustar-u_L) and
//    p_R + rc_R (ustar-u_R), which are equal by the definition of ustar; the
//    upwind one is used.
//  * the energy flux needs only e_star + pstar.  With a = S - un (already
//    formed for rc = d a), w = ustar - un and ratio = a/(S - ustar):
//    e_star + pstar = [a e + pstar ustar - p un + pstar (S - ustar)]/(S - ustar)
//                   = [a (e + p) + S (pstar - p)]/(S - ustar)
//                   = ratio (e + p) + w S d_star,
//    since pstar - p = rc w = d a w and d_star = ratio d.
//  * in the supersonic case the reference's ratio (S-un)/(S-un) is exactly 1
//    and its energy correction exactly 0: a select returns the upwind state.
//  * min/max and the sign tests run on the integer pipe (order_key etc.).
// Results agree with the reference to a few ulps per face.
__device__ __forceinline__ Flux<double> hllc_flux(Side<double> const& L, Side<double> const& R)
{
    double const cmax = (dbits(L.c) > dbits(R.c)) ? L.c : R.c; // sound speeds are >= 0
    bool const lt = order_key(L.un) < order_key(R.un);
    double const umin = lt ? L.un : R.un;
    double const umax = lt ? R.un : L.un;
    double const S_L = umin - cmax;
    double const S_R = umax + cmax;

    double const a_L = S_L - L.un; // S - un of each side, <= -cmax and >= cmax
    double const a_R = S_R - R.un;
    double const rc_L = L.d * a_L;
    double const rc_R = R.d * a_R;
    double const num = (R.p - L.p) + rc_L * L.un - rc_R * R.un;
    double const den = rc_L - rc_R;

    bool const left = product_positive(num, den); // ustar > 0
    double const S = left ? S_L : S_R;
    double const qa = left ? a_L : a_R;
    double const qd = left ? L.d : R.d;
    double const qp = left ? L.p : R.p;
    double const qun = left ? L.un : R.un;
    double const qut1 = left ? L.ut1 : R.ut1;
    double const qut2 = left ? L.ut2 : R.ut2;
    double const qh = left ? L.e : R.e; // e + p of the upwind side
    double const qrc = left ? rc_L : rc_R;

    double const M = S * den - num; // den (S - ustar)
    double const Rr = rcp_faithful(den * M);
    double const ustar = num * (M * Rr);
    double const inv = den * (den * Rr); // 1 / (S - ustar)
    double const w = ustar - qun;
    double const pstar = qp + qrc * w;

    bool const supersonic = product_positive(S_L, S_R);
    double const ratio = qa * inv;
    double const d_star = ratio * qd;
    double const h_star = ratio * qh + w * (S * d_star); // e_star + pstar

    double const un_o = supersonic ? qun : ustar;
    double const ptot_o = supersonic ? qp : pstar;
    double const d_o = supersonic ? qd : d_star;
    double const h_o = supersonic ? qh : h_star;

    Flux<double> f;
    f.d = d_o * un_o;
    f.e = h_o * un_o;
    f.n = f.d * un_o + ptot_o;
    f.t1 = f.d * qut1;
    f.t2 = f.d * qut2;
    return f;
}

// FP32 version (real_t = float operators): same algebra, FP32 min/max and
// the hardware reciprocal.
__device__ __forceinline__ Flux<float> hllc_flux(Side<float> const& L, Side<float> const& R)
{
    float const cmax = fmaxf(L.c, R.c);
    float const S_L = fminf(L.un, R.un) - cmax;
    float const S_R = fmaxf(L.un, R.un) + cmax;
    float const rc_L = L.d * (S_L - L.un);
    float const rc_R = R.d * (S_R - R.un);
    float const num = (R.p - L.p) + rc_L * L.un - rc_R * R.un;
    float const den = rc_L - rc_R;
    // rc_L <= 0 <= rc_R (S_L - un_L <= -cmax, S_R - un_R >= cmax, and rounding is
    // monotone), so den <= 0 and ustar = num/den > 0 exactly when num < 0
    bool const left = num < 0.0f;
    float const S = left ? S_L : S_R;
    float const qd = left ? L.d : R.d;
    float const qp = left ? L.p : R.p;
    float const qun = left ? L.un : R.un;
    float const qut1 = left ? L.ut1 : R.ut1;
    float const qut2 = left ? L.ut2 : R.ut2;
    float const qh = left ? L.e : R.e; // e + p of the upwind side
    float const qrc = left ? rc_L : rc_R;
    float const M = S * den - num;
    float const Rr = rcp_approx(den * M); // |den M| is far from the ends of the float range for any physical state
    // Supersonic faces take the upwind state's own flux.  ustar := un and
    // ratio := 1 give it exactly (w = 0, so pstar = p, d_star = d and
    // h_star = e + p), with two selects instead of four.
    bool const supersonic = S_L * S_R > 0.0f;
    float const ustar = supersonic ? qun : num * (M * Rr);
    float const inv = den * (den * Rr);
    float const w = ustar - qun;
    float const pstar = qp + qrc * w;
    float const ratio = supersonic ? 1.0f : (S - qun) * inv;
    float const d_star = ratio * qd;
    float const h_star = ratio * qh + w * (S * d_star); // e_star + pstar
    float const un_o = ustar;
    float const ptot_o = pstar;
    float const d_o = d_star;
    float const h_o = h_star;
    Flux<float> f;
    f.d = d_o * un_o;
    f.e = h_o * un_o;
    f.n = f.d * un_o + ptot_o;
    f.t1 = f.d * qut1;
    f.t2 = f.d * qut2;
    return f;
}

} // namespace eulr
