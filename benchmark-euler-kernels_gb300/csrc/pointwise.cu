// Pointwise Euler operators and the CFL reduction (sm_103a).
//
// Each kernel restates one reference operator with separately rounded
// operations in the reference's operand order, so the results are
// bit-identical to euler_operators/*.hpp compiled without FMA contraction.
// All of them are bound by the FP64 pipe on GB300 (1/64 of the FP32 rate),
// not by HBM, so the only optimisation that matters is issuing fewer FP64
// instructions: divisions by the loop-invariant gamma-1 use a precomputed
// reciprocal plus one Markstein correction, and cons_to_prim derives both of
// its quotients from one reciprocal of rho.
#include "euler_device.cuh"
#include "kernels.h"
#include "step_common.cuh"

#include <cfloat>

namespace eulr {

// ------------------------------------------------------------ init_implode
// init_implode.hpp:24-44.  Cell centres are computed in double (the literal 0.5
// promotes (i-1) to double) and rounded to T, as in the reference's float
// instantiation.
template <class T>
__global__ void __launch_bounds__(256) init_implode_kernel(Bundle<T> prim, Geom g, double dx0, double dx1, double dx2)
{
    long long const n = g.ncell();
    T const radius2 = static_cast<T>(0.25 * 0.25);
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        int const i = static_cast<int>(c % g.n0);
        long long const jk = c / g.n0;
        int const j = static_cast<int>(jk % g.n1);
        int const k = static_cast<int>(jk / g.n1);
        T const x0 = static_cast<T>(__dsub_rn(__dmul_rn(__dadd_rn(static_cast<double>(i - 1), 0.5), dx0), 0.5));
        T const x1 = static_cast<T>(__dsub_rn(__dmul_rn(__dadd_rn(static_cast<double>(j - 1), 0.5), dx1), 0.5));
        T const x2 = static_cast<T>(__dsub_rn(__dmul_rn(__dadd_rn(static_cast<double>(k - 1), 0.5), dx2), 0.5));
        T const r2 = add_rn(add_rn(mul_rn(x0, x0), mul_rn(x1, x1)), mul_rn(x2, x2));
        bool const inside = r2 < radius2;
        prim.f[0][c] = inside ? T(1) : T(0.125);
        prim.f[1][c] = inside ? T(1) : T(0.14);
        prim.f[2][c] = T(0);
        prim.f[3][c] = T(0);
        prim.f[4][c] = T(0);
    }
}

// ------------------------------------------------------------ prim_to_cons
// prim_to_cons.hpp:20-32 with to_cons (euler_arrays.hpp:56-64):
//   e = d*((u0*u0 + u1*u1) + u2*u2)/2 + p/(gamma-1),  m_i = d*u_i.
template <class T>
__global__ void __launch_bounds__(256) prim_to_cons_kernel(CBundle<T> prim, Bundle<T> cons, long long n, T gm1, T rgm1)
{
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        T const d = prim.f[0][c];
        T const p = prim.f[1][c];
        T const u0 = prim.f[2][c];
        T const u1 = prim.f[3][c];
        T const u2 = prim.f[4][c];
        T const int_e = div_by_rcp(p, gm1, rgm1);
        T const ke = half_exact(mul_rn(d, add_rn(add_rn(mul_rn(u0, u0), mul_rn(u1, u1)), mul_rn(u2, u2))));
        cons.f[0][c] = d;
        cons.f[1][c] = add_rn(ke, int_e);
        cons.f[2][c] = mul_rn(d, u0);
        cons.f[3][c] = mul_rn(d, u1);
        cons.f[4][c] = mul_rn(d, u2);
    }
}

// ------------------------------------------------------------ cons_to_prim
// cons_to_prim.hpp:20-32 with kinetic_energy(cons) (euler_arrays.hpp:44-48),
// PerfectGas::pressure and to_prim (euler_arrays.hpp:66-75):
//   ke = ((m.m)/d)/2, p = (gamma-1)*(e-ke), u_i = m_i * (1/d).
template <class T>
__global__ void __launch_bounds__(256) cons_to_prim_kernel(CBundle<T> cons, Bundle<T> prim, long long n, T gm1)
{
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        T const d = cons.f[0][c];
        T p, u0, u1, u2;
        cons_to_prim_exact(d, cons.f[1][c], cons.f[2][c], cons.f[3][c], cons.f[4][c], gm1, p, u0, u1, u2);
        prim.f[0][c] = d;
        prim.f[1][c] = p;
        prim.f[2][c] = u0;
        prim.f[3][c] = u1;
        prim.f[4][c] = u2;
    }
}

// --------------------------------------------------------------- time_step
// time_step.hpp:22-39.  The reference takes min over cells of 1/invdt; since
// correctly rounded division is monotonic, min_c RN(1/x_c) = RN(1/max_c x_c),
// so the kernel reduces max(invdt) (exact, order-free) and divides once.
// FP64: the max is screened (WaveScreen), so the kernel reads 40 B per cell
// and issues FP64 instructions only for the few cells evaluated exactly; the
// dt is still the reference's bit for bit.  NaN never wins (the reference's Kokkos::min
// skips it) and an all-zero grid returns the reduction identity T's max, as
// the reference's Min reducer does.
template <class T>
__global__ void __launch_bounds__(256) time_step_kernel(CBundle<T> prim, long long n, T gamma, T ix0, T ix1, T ix2,
                                                        T* partials, unsigned int* counter, T* dt_out)
{
    T local = T(0);
    if constexpr (sizeof(T) == 8) {
        WaveScreen screen(gamma, ix0, ix1, ix2);
        int const lane = threadIdx.x & 31;
        long long const stride = static_cast<long long>(gridDim.x) * blockDim.x;
        // warp-uniform trip count: every lane of a warp runs every iteration
        for (long long base = blockIdx.x * static_cast<long long>(blockDim.x) + (threadIdx.x & ~31); base < n;
             base += stride) {
            long long const c = base + lane;
            bool const valid = c < n;
            T d = T(1), p = T(1), u0 = T(0), u1 = T(0), u2 = T(0);
            if (valid) {
                d = prim.f[0][c];
                p = prim.f[1][c];
                u0 = prim.f[2][c];
                u1 = prim.f[3][c];
                u2 = prim.f[4][c];
            }
            if (screen.exact_needed(valid, d, p, u0, u1, u2)) {
                T const v = cell_invdt_exact(d, p, u0, u1, u2, gamma, ix0, ix1, ix2);
                local = (v > local) ? v : local;
            }
        }
    } else {
        for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
             c += static_cast<long long>(gridDim.x) * blockDim.x) {
            T const v = cell_invdt_exact(prim.f[0][c], prim.f[1][c], prim.f[2][c], prim.f[3][c], prim.f[4][c], gamma,
                                         ix0, ix1, ix2);
            local = (v > local) ? v : local;
        }
    }
    __shared__ T warp_best[8];
    __shared__ bool is_last;
    local = warp_max(local);
    if ((threadIdx.x & 31) == 0) {
        warp_best[threadIdx.x >> 5] = local;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        T b = warp_best[0];
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) {
            b = (warp_best[w] > b) ? warp_best[w] : b;
        }
        partials[blockIdx.x] = b;
        __threadfence();
        unsigned int const done = atomicAdd(counter, 1u);
        is_last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (is_last) {
        // Last block to finish: fold the per-block maxima and publish dt.
        __threadfence();
        T b = T(0);
        for (unsigned int w = threadIdx.x; w < gridDim.x; w += blockDim.x) {
            T const v = __ldcg(&partials[w]);
            b = (v > b) ? v : b;
        }
        b = warp_max(b);
        if ((threadIdx.x & 31) == 0) {
            warp_best[threadIdx.x >> 5] = b;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            T m = warp_best[0];
            for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) {
                m = (warp_best[w] > m) ? warp_best[w] : m;
            }
            *dt_out = (m > T(0)) ? rcp_rn(m) : (sizeof(T) == 8 ? T(DBL_MAX) : T(FLT_MAX));
            *counter = 0u;
        }
    }
}

// Max invdt over all cells of a cons-only FP32 state, with the pressure the
// fused FP32 step uses (compensated states rescue low-pressure cells in FP64).
__global__ void __launch_bounds__(256) invdt_max_cons_kernel(CBundle<float> cons, long long n, float gamma, float ix0,
                                                             float ix1, float ix2, int comp, unsigned long long* wmax)
{
    float local = 0.0f;
    float const gm1 = gamma - 1.0f;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        float const d = cons.f[0][c];
        float const e = cons.f[1][c];
        float const m0 = cons.f[2][c];
        float const m1 = cons.f[3][c];
        float const m2 = cons.f[4][c];
        float const r = 1.0f / d;
        float const pr = comp ? pressure_f32c(d, e, m0, m1, m2, r, gm1, nullptr)
                              : gm1 * (e - (0.5f * r) * (m0 * m0 + m1 * m1 + m2 * m2));
        float const v = cell_invdt_exact(d, pr, m0 * r, m1 * r, m2 * r, gamma, ix0, ix1, ix2);
        local = (v > local) ? v : local;
    }
    __shared__ float warp_best[8];
    local = warp_max(local);
    if ((threadIdx.x & 31) == 0) {
        warp_best[threadIdx.x >> 5] = local;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = warp_best[0];
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) {
            b = (warp_best[w] > b) ? warp_best[w] : b;
        }
        atomicMax(wmax, order_bits(b));
    }
}

// Loading a primitive state into an FP64 simulation or batch grid, in one
// pass:
//  * cons = prim_to_cons(prim) when cons is set, bit-identical to
//    prim_to_cons_kernel;
//  * the stored sound speed in the form the fused step stores it
//    (fast_sound_speed of (gamma/rho) p, faithful), so a loaded state and a
//    stepped one carry the same kind of value;
//  * the EXACT max wavespeed of time_step.hpp:28-33 for the first dt, with
//    the exact per-cell value evaluated only where WaveScreen says it can be
//    the max.
template <class T>
__global__ void __launch_bounds__(256) load_prim_kernel(CBundle<T> prim, Bundle<T> cons, T* cs, long long n, T gamma,
                                                        T gm1, T rgm1, T ix0, T ix1, T ix2, unsigned long long* wmax,
                                                        T* h, const T* e_in)
{
    T local = T(0);
    WaveScreen screen(gamma, ix0, ix1, ix2);
    int const lane = threadIdx.x & 31;
    long long const stride = static_cast<long long>(gridDim.x) * blockDim.x;
    // warp-uniform trip count: every lane of a warp runs every iteration
    for (long long base = blockIdx.x * static_cast<long long>(blockDim.x) + (threadIdx.x & ~31); base < n;
         base += stride) {
        long long const c = base + lane;
        bool const valid = c < n;
        T d = T(1), p = T(1), u0 = T(0), u1 = T(0), u2 = T(0);
        if (valid) {
            d = prim.f[0][c];
            p = prim.f[1][c];
            u0 = prim.f[2][c];
            u1 = prim.f[3][c];
            u2 = prim.f[4][c];
            if (cons.f[0] != nullptr) {
                T const int_e = div_by_rcp(p, gm1, rgm1);
                T const ke = half_exact(mul_rn(d, add_rn(add_rn(mul_rn(u0, u0), mul_rn(u1, u1)), mul_rn(u2, u2))));
                T const e = add_rn(ke, int_e);
                cons.f[0][c] = d;
                cons.f[1][c] = e;
                cons.f[2][c] = mul_rn(d, u0);
                cons.f[3][c] = mul_rn(d, u1);
                cons.f[4][c] = mul_rn(d, u2);
                if (h != nullptr) {
                    h[c] = add_rn(e, p);
                }
            } else if (h != nullptr) {
                h[c] = add_rn(e_in[c], p);
            }
        }
        bool cand = valid;
        if constexpr (sizeof(T) == 8) {
            if (valid) {
                cs[c] = sqrt_quotient_faithful(gamma * p, d); // 1/rho is not needed here
            }
            cand = screen.exact_needed(valid, d, p, u0, u1, u2);
        } else if (valid) {
            cs[c] = sqrt_rn(div_rn(mul_rn(gamma, p), d));
        }
        if (cand) {
            T const v = cell_invdt_exact(d, p, u0, u1, u2, gamma, ix0, ix1, ix2);
            local = (v > local) ? v : local; // NaN never wins
        }
    }
    __shared__ T warp_best[8];
    local = warp_max(local);
    if (lane == 0) {
        warp_best[threadIdx.x >> 5] = local;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        T b = warp_best[0];
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) {
            b = (warp_best[w] > b) ? warp_best[w] : b;
        }
        atomicMax(wmax, order_bits(b));
    }
}

// ----------------------------------------------------------- init_step
// Step discontinuity on x + y + z < c, the initial condition of the batched
// workload (it has no counterpart in the reference): cell centres
// ((i-1)+0.5) dx in double as in init_implode.hpp:33-36 but on [0,1]^3,
// (rho_in, p_in) below the plane, (rho_out, p_out) above it, u = 0.
template <class T>
__global__ void __launch_bounds__(256) init_step_kernel(Bundle<T> prim, Geom g, double dx0, double dx1, double dx2,
                                                        double c, double rho_in, double p_in, double rho_out,
                                                        double p_out)
{
    long long const n = g.ncell();
    for (long long idx = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; idx < n;
         idx += static_cast<long long>(gridDim.x) * blockDim.x) {
        int const i = static_cast<int>(idx % g.n0);
        long long const jk = idx / g.n0;
        int const j = static_cast<int>(jk % g.n1);
        int const k = static_cast<int>(jk / g.n1);
        double const x0 = __dmul_rn(__dadd_rn(static_cast<double>(i - 1), 0.5), dx0);
        double const x1 = __dmul_rn(__dadd_rn(static_cast<double>(j - 1), 0.5), dx1);
        double const x2 = __dmul_rn(__dadd_rn(static_cast<double>(k - 1), 0.5), dx2);
        bool const inside = __dadd_rn(__dadd_rn(x0, x1), x2) < c;
        prim.f[0][idx] = static_cast<T>(inside ? rho_in : rho_out);
        prim.f[1][idx] = static_cast<T>(inside ? p_in : p_out);
        prim.f[2][idx] = T(0);
        prim.f[3][idx] = T(0);
        prim.f[4][idx] = T(0);
    }
}

// ------------------------------------------------------------------ launch
static int grid_for(long long n, int sms)
{
    long long const blocks = (n + 255) / 256;
    long long const cap = static_cast<long long>(sms) * 8;
    return static_cast<int>(blocks < cap ? (blocks > 0 ? blocks : 1) : cap);
}

template <class T>
cudaError_t launch_init_implode(Bundle<T> prim, Geom g, double dx0, double dx1, double dx2, int sms, cudaStream_t s)
{
    init_implode_kernel<T><<<grid_for(g.ncell(), sms), 256, 0, s>>>(prim, g, dx0, dx1, dx2);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_prim_to_cons(CBundle<T> prim, Bundle<T> cons, long long n, T gm1, T rgm1, int sms, cudaStream_t s)
{
    prim_to_cons_kernel<T><<<grid_for(n, sms), 256, 0, s>>>(prim, cons, n, gm1, rgm1);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_cons_to_prim(CBundle<T> cons, Bundle<T> prim, long long n, T gm1, int sms, cudaStream_t s)
{
    cons_to_prim_kernel<T><<<grid_for(n, sms), 256, 0, s>>>(cons, prim, n, gm1);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_time_step(CBundle<T> prim, long long n, T gamma, T ix0, T ix1, T ix2, T* partials,
                             int max_partials, unsigned int* counter, T* dt_out, int sms, cudaStream_t s)
{
    int grid = grid_for(n, sms);
    if (grid > max_partials) {
        grid = max_partials;
    }
    time_step_kernel<T><<<grid, 256, 0, s>>>(prim, n, gamma, ix0, ix1, ix2, partials, counter, dt_out);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_load_prim(CBundle<T> prim, Bundle<T> cons, T* cs, long long n, T gamma, T ix0, T ix1, T ix2,
                             unsigned long long* wmax, int sms, cudaStream_t s, T* h, const T* e_in)
{
    T const gm1 = gamma - T(1);
    load_prim_kernel<T><<<grid_for(n, sms), 256, 0, s>>>(prim, cons, cs, n, gamma, gm1, T(1) / gm1, ix0, ix1, ix2,
                                                          wmax, h, e_in);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(256) add_fields_kernel(const double* a, const double* b, double* out, long long n)
{
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        out[c] = __dadd_rn(a[c], b[c]);
    }
}

cudaError_t launch_add_fields(const double* a, const double* b, double* out, long long n, int sms, cudaStream_t s)
{
    add_fields_kernel<<<grid_for(n, sms), 256, 0, s>>>(a, b, out, n);
    return cudaGetLastError();
}

cudaError_t launch_init_step(Bundle<double> prim, Geom g, double dx0, double dx1, double dx2, double c,
                             double rho_in, double p_in, double rho_out, double p_out, int sms, cudaStream_t s)
{
    init_step_kernel<double><<<grid_for(g.ncell(), sms), 256, 0, s>>>(prim, g, dx0, dx1, dx2, c, rho_in, p_in, rho_out,
                                                                       p_out);
    return cudaGetLastError();
}

cudaError_t launch_invdt_max_cons(CBundle<float> cons, long long n, float gamma, float ix0, float ix1, float ix2,
                                  int comp, unsigned long long* wmax, int sms, cudaStream_t s)
{
    invdt_max_cons_kernel<<<grid_for(n, sms), 256, 0, s>>>(cons, n, gamma, ix0, ix1, ix2, comp, wmax);
    return cudaGetLastError();
}

#define EULR_INSTANTIATE_POINTWISE(T)                                                                        \
    template cudaError_t launch_init_implode<T>(Bundle<T>, Geom, double, double, double, int, cudaStream_t); \
    template cudaError_t launch_prim_to_cons<T>(CBundle<T>, Bundle<T>, long long, T, T, int, cudaStream_t);  \
    template cudaError_t launch_cons_to_prim<T>(CBundle<T>, Bundle<T>, long long, T, int, cudaStream_t);     \
    template cudaError_t launch_time_step<T>(CBundle<T>, long long, T, T, T, T, T*, int, unsigned int*, T*,  \
                                             int, cudaStream_t);                                             \
    template cudaError_t launch_load_prim<T>(CBundle<T>, Bundle<T>, T*, long long, T, T, T, T, unsigned long long*,    \
                                             int, cudaStream_t, T*, const T*);

EULR_INSTANTIATE_POINTWISE(double)
EULR_INSTANTIATE_POINTWISE(float)

} // namespace eulr
