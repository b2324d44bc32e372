// Measurement and diagnostic kernels: the FMA-rate probe behind the roofline
// denominator, and deterministic FP64 conservation totals.
#include "euler_device.cuh"
#include "kernels.h"

namespace eulr {

namespace {

constexpr int kChains = 8;

// Every thread advances kChains independent FMA chains, so the pipe never
// waits on a dependency; the result is folded into `sink` so nothing is
// dead code.  The multiplier is slightly below one and the addend small, so
// the values stay finite and normal for any iteration count.
template <class T>
__global__ void __launch_bounds__(256) fma_probe_kernel(int iters, float* sink)
{
    T a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
        a[c] = T(threadIdx.x + c) * T(1e-3);
    }
    T const m = T(0.999999);
    T const b = T(1e-7);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) {
            a[c] = fma(a[c], m, b);
        }
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
        s += a[c];
    }
    if (s == T(-1)) { // never true; keeps the chains alive
        sink[blockIdx.x] = static_cast<float>(s);
    }
}

// Sum over interior cells of the 5 conservative fields in FP64, one partial
// per block in a fixed order, then one block folds the partials in order:
// the result does not depend on scheduling.  FP32 states add their low
// words (compensated storage) in FP64 too.
template <class T>
__global__ void __launch_bounds__(256) totals_partial_kernel(CBundle<T> cons, CBundle<T> lo, Geom g, double* partials)
{
    int const ix = g.n0 - 2, iy = g.n1 - 2, iz = g.n2 - 2;
    long long const n = (ix > 0 && iy > 0 && iz > 0) ? static_cast<long long>(ix) * iy * iz : 0;
    double acc[5] = {0, 0, 0, 0, 0};
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        int const i = 1 + static_cast<int>(c % ix);
        long long const jk = c / ix;
        int const j = 1 + static_cast<int>(jk % iy);
        int const k = 1 + static_cast<int>(jk / iy);
        long long const o = g.at(i, j, k);
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            acc[f] += static_cast<double>(cons.f[f][o]);
            if (lo.f[0] != nullptr) {
                acc[f] += static_cast<double>(lo.f[f][o]);
            }
        }
    }
    __shared__ double red[5][256];
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        red[f][threadIdx.x] = acc[f];
    }
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (static_cast<int>(threadIdx.x) < s) {
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                red[f][threadIdx.x] += red[f][threadIdx.x + s];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 5) {
        partials[blockIdx.x * 5 + threadIdx.x] = red[threadIdx.x][0];
    }
}

__global__ void totals_final_kernel(const double* partials, int nblocks, double* out5)
{
    if (threadIdx.x < 5) {
        double s = 0;
        for (int b = 0; b < nblocks; ++b) {
            s += partials[b * 5 + threadIdx.x];
        }
        out5[threadIdx.x] = s;
    }
}

} // namespace

constexpr int kTotalsBlocks = 256;

cudaError_t launch_fma_probe(int kind, int blocks, int iters, float* sink, cudaStream_t s)
{
    if (kind == 0) {
        fma_probe_kernel<double><<<blocks, 256, 0, s>>>(iters, sink);
    } else {
        fma_probe_kernel<float><<<blocks, 256, 0, s>>>(iters, sink);
    }
    return cudaGetLastError();
}

// `work` must have room for kTotalsBlocks*5 partials followed by the 5 totals.
template <class T>
cudaError_t launch_totals(CBundle<T> cons, CBundle<T> lo, Geom g, double* work, cudaStream_t s)
{
    totals_partial_kernel<T><<<kTotalsBlocks, 256, 0, s>>>(cons, lo, g, work);
    totals_final_kernel<<<1, 32, 0, s>>>(work, kTotalsBlocks, work + kTotalsBlocks * 5);
    return cudaGetLastError();
}

// FP64 state -> cons-only FP32 simulation state.  cons in FP64 (given, or
// prim_to_cons of the FP64 prim, bit-identical to the reference) is split
// into hi = RN(cons) and, when `lo` is set, lo = RN(cons - hi).  With
// `fp32_cons` (plain FP32 mode) cons is instead prim_to_cons of the prim
// rounded to FP32, computed in FP32 as the reference's real_t = float build
// does.
__global__ void __launch_bounds__(256) state_to_f32_kernel(CBundle<double> prim, CBundle<double> cons, Bundle<float> hi,
                                                           Bundle<float> lo, long long n, double gamma, int fp32_cons)
{
    double const gm1 = gamma - 1.0;
    double const rgm1 = 1.0 / gm1;
    float const gm1f = static_cast<float>(gamma) - 1.0f;
    float const rgm1f = 1.0f / gm1f;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (fp32_cons) {
            float q[5];
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                q[f] = static_cast<float>(prim.f[f][c]);
            }
            float const int_e = div_by_rcp(q[1], gm1f, rgm1f);
            float const ke =
                    mul_rn(mul_rn(q[0], add_rn(add_rn(mul_rn(q[2], q[2]), mul_rn(q[3], q[3])), mul_rn(q[4], q[4]))),
                           0.5f);
            hi.f[0][c] = q[0];
            hi.f[1][c] = add_rn(ke, int_e);
            hi.f[2][c] = mul_rn(q[0], q[2]);
            hi.f[3][c] = mul_rn(q[0], q[3]);
            hi.f[4][c] = mul_rn(q[0], q[4]);
            continue;
        }
        double u[5];
        if (cons.f[0] != nullptr) {
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                u[f] = cons.f[f][c];
            }
        } else {
            double q[5];
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                q[f] = prim.f[f][c];
            }
            double const int_e = div_by_rcp(q[1], gm1, rgm1);
            double const ke =
                    mul_rn(mul_rn(q[0], add_rn(add_rn(mul_rn(q[2], q[2]), mul_rn(q[3], q[3])), mul_rn(q[4], q[4]))),
                           0.5);
            u[0] = q[0];
            u[1] = add_rn(ke, int_e);
            u[2] = mul_rn(q[0], q[2]);
            u[3] = mul_rn(q[0], q[3]);
            u[4] = mul_rn(q[0], q[4]);
        }
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            float const h = static_cast<float>(u[f]);
            hi.f[f][c] = h;
            if (lo.f[0] != nullptr) {
                lo.f[f][c] = static_cast<float>(u[f] - static_cast<double>(h));
            }
        }
    }
}

// Cons-only FP32 simulation state -> FP64: cons = hi (+ lo) in FP64 and prim
// = cons_to_prim of it in FP64 (the reference's formula, cons_to_prim.hpp).
__global__ void __launch_bounds__(256) state_from_f32_kernel(CBundle<float> hi, CBundle<float> lo, Bundle<double> prim,
                                                             Bundle<double> cons, long long n, double gamma)
{
    double const gm1 = gamma - 1.0;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        double u[5];
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            u[f] = static_cast<double>(hi.f[f][c]);
            if (lo.f[0] != nullptr) {
                u[f] += static_cast<double>(lo.f[f][c]);
            }
            if (cons.f[0] != nullptr) {
                cons.f[f][c] = u[f];
            }
        }
        if (prim.f[0] != nullptr) {
            double pr, v0, v1, v2;
            cons_to_prim_exact(u[0], u[1], u[2], u[3], u[4], gm1, pr, v0, v1, v2);
            prim.f[0][c] = u[0];
            prim.f[1][c] = pr;
            prim.f[2][c] = v0;
            prim.f[3][c] = v1;
            prim.f[4][c] = v2;
        }
    }
}

static int grid256(long long n, int sms)
{
    long long const b = (n + 255) / 256;
    long long const cap = static_cast<long long>(sms) * 8;
    return static_cast<int>(b < 1 ? 1 : (b < cap ? b : cap));
}

cudaError_t launch_state_to_f32(CBundle<double> prim, CBundle<double> cons, Bundle<float> hi, Bundle<float> lo,
                                long long n, double gamma, int fp32_cons, int sms, cudaStream_t s)
{
    state_to_f32_kernel<<<grid256(n, sms), 256, 0, s>>>(prim, cons, hi, lo, n, gamma, fp32_cons);
    return cudaGetLastError();
}

cudaError_t launch_state_from_f32(CBundle<float> hi, CBundle<float> lo, Bundle<double> prim, Bundle<double> cons,
                                  long long n, double gamma, int sms, cudaStream_t s)
{
    state_from_f32_kernel<<<grid256(n, sms), 256, 0, s>>>(hi, lo, prim, cons, n, gamma);
    return cudaGetLastError();
}

template cudaError_t launch_totals<double>(CBundle<double>, CBundle<double>, Geom, double*, cudaStream_t);
template cudaError_t launch_totals<float>(CBundle<float>, CBundle<float>, Geom, double*, cudaStream_t);

} // namespace eulr
