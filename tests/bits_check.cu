// The integer-pipe replacements of FP64 instructions in csrc/euler_device.cuh
// and csrc/step_common.cuh against the FP64 instructions they stand for, on
// the GPU: less_ieee(a, b) against the compare a < b, half_exact(x) against
// __dmul_rn(x, 0.5) bit for bit (NaN against NaN), product_positive(a, b)
// against a * b > 0 where the product neither underflows nor is NaN, and
// div_small against integer division over the face-index range.  Test
// harness, built and run by tests/test_gpu_bits.py.  Operands: seeded random
// bit patterns of every class (normal, subnormal, zero, infinite, NaN) plus
// a table of special values combined pairwise.  Prints one JSON line of
// mismatch counts.
#include "step_common.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

__global__ void bits_kernel(const double* a, const double* b, int n, unsigned long long* bad)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    double const x = a[i], y = b[i];
    if (eulr::less_ieee(x, y) != (x < y)) {
        atomicAdd(bad + 0, 1ull);
    }
    double const h = eulr::half_exact(x), r = __dmul_rn(x, 0.5);
    bool const both_nan = (h != h) && (r != r);
    if (!both_nan && __double_as_longlong(h) != __double_as_longlong(r)) {
        atomicAdd(bad + 1, 1ull);
    }
    double const p = __dmul_rn(x, y);
    bool const defined = (p == p) && (p != 0.0 || x == 0.0 || y == 0.0);
    if (defined && eulr::product_positive(x, y) != (p > 0.0)) {
        atomicAdd(bad + 2, 1ull);
    }
    if (i < 4096) {
        if (eulr::div_small<17>(i) != i / 17 || eulr::div_small<16>(i) != i / 16 || eulr::div_small<33>(i) != i / 33 ||
            eulr::div_small<9>(i) != i / 9) {
            atomicAdd(bad + 3, 1ull);
        }
    }
}

} // namespace

int main()
{
    std::vector<double> va, vb;
    unsigned long long s = 0x2545f4914f6cdd1dull;
    auto next = [&s]() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return s;
    };
    auto from_bits = [](unsigned long long u) {
        double d;
        std::memcpy(&d, &u, sizeof d);
        return d;
    };
    for (int i = 0; i < (1 << 22); ++i) {
        unsigned long long u = next(), w = next();
        switch (i & 7) {
        case 1: u &= 0x800fffffffffffffull; break;                                  // subnormal or zero
        case 2: u = (u & 0x800fffffffffffffull) | 0x0010000000000000ull; break;    // exponent field 1
        case 3: w = u ^ (next() & 0x00000000000000ffull); break;                   // near-equal pairs
        case 4: w = u ^ 0x8000000000000000ull; break;                              // opposite signs
        case 5: u = (u & 0x800fffffffffffffull) | 0x7ff0000000000000ull; break;    // inf or NaN
        default: break;
        }
        va.push_back(from_bits(u));
        vb.push_back(from_bits(w));
    }
    double const special[] = {0.0, -0.0, 1.0, -1.0, 0.5, 2.0, INFINITY, -INFINITY, NAN, -NAN,
                              from_bits(1ull), from_bits(0x8000000000000001ull), from_bits(0x000fffffffffffffull),
                              from_bits(0x0010000000000000ull), from_bits(0x0020000000000000ull), 1e-300, -1e300,
                              from_bits(0x7fefffffffffffffull)};
    for (double x : special) {
        for (double y : special) {
            va.push_back(x);
            vb.push_back(y);
        }
    }
    int const n = static_cast<int>(va.size());
    double *da = nullptr, *db = nullptr;
    unsigned long long* dbad = nullptr;
    if (cudaMalloc(&da, sizeof(double) * n) != cudaSuccess || cudaMalloc(&db, sizeof(double) * n) != cudaSuccess ||
        cudaMalloc(&dbad, 4 * sizeof(unsigned long long)) != cudaSuccess) {
        std::printf("cudaMalloc failed\n");
        return 1;
    }
    cudaMemcpy(da, va.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(db, vb.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemset(dbad, 0, 4 * sizeof(unsigned long long));
    bits_kernel<<<(n + 255) / 256, 256>>>(da, db, n, dbad);
    cudaError_t const err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        std::printf("kernel failed: %s\n", cudaGetErrorString(err));
        return 1;
    }
    unsigned long long bad[4];
    cudaMemcpy(bad, dbad, sizeof bad, cudaMemcpyDeviceToHost);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dbad);
    std::printf("{\"n\": %d, \"less_ieee\": %llu, \"half_exact\": %llu, \"product_positive\": %llu, \"div_small\": %llu}\n",
                n, bad[0], bad[1], bad[2], bad[3]);
    return 0;
}
