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
// the result does not depend on scheduling.
__global__ void __launch_bounds__(256) totals_partial_kernel(CBundle<double> cons, Geom g, double* partials)
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
            acc[f] += cons.f[f][o];
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

// out5 must have room for kTotalsBlocks*5 partials followed by the 5 totals.
cudaError_t launch_totals(CBundle<double> cons, Geom g, double* work, int /*sms*/, cudaStream_t s)
{
    totals_partial_kernel<<<kTotalsBlocks, 256, 0, s>>>(cons, g, work);
    totals_final_kernel<<<1, 32, 0, s>>>(work, kTotalsBlocks, work + kTotalsBlocks * 5);
    return cudaGetLastError();
}

} // namespace eulr
