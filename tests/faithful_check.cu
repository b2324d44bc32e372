// Accuracy check of the library's faithful FP64 reciprocal, square root and
// square root of a quotient (rcp_faithful, sqrt_faithful,
// sqrt_quotient_faithful in csrc/euler_device.cuh) against the correctly
// rounded __drcp_rn / __dsqrt_rn / __dsqrt_rn(__ddiv_rn), and of the PTX
// approximations they refine.  Test harness, built and run by
// tests/test_gpu_faithful.py.
//
// Arguments m * 2^e with m uniform in [1, 2) and e uniform in [-100, 100]
// (4M of them, a fixed LCG stream), plus the binade edges 1, 2 - ulp, 2^e,
// and arguments near and beyond FP32's exponent range up to 2^+-400.
// Prints one line: max ulp distances and the approximations' max relative
// errors.
#include "euler_device.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

__global__ void check_kernel(const double* x, double* out, int n)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) {
        return;
    }
    double const v = x[i];
    double const w = x[(static_cast<long long>(i) * 7 + 3) % n]; // a second argument for the quotient
    out[6 * static_cast<long long>(n) + 2 * static_cast<long long>(i) + 0] = __dsqrt_rn(__ddiv_rn(v, w));
    out[6 * static_cast<long long>(n) + 2 * static_cast<long long>(i) + 1] = eulr::sqrt_quotient_faithful(v, w);
    double ra, sa;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(ra) : "d"(v));
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(sa) : "d"(v));
    out[6 * static_cast<long long>(i) + 0] = ra;
    out[6 * static_cast<long long>(i) + 1] = __drcp_rn(v);
    out[6 * static_cast<long long>(i) + 2] = eulr::rcp_faithful(v);
    out[6 * static_cast<long long>(i) + 3] = sa;
    out[6 * static_cast<long long>(i) + 4] = __dsqrt_rn(v);
    out[6 * static_cast<long long>(i) + 5] = eulr::sqrt_faithful(v);
}

long long bits(double v)
{
    long long b;
    std::memcpy(&b, &v, sizeof b);
    return b;
}

} // namespace

int main()
{
    int const n_random = 1 << 22;
    std::vector<double> h;
    h.reserve(n_random + 512);
    unsigned long long s = 0x9e3779b97f4a7c15ull;
    auto next = [&s]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return s >> 11; // 53 random bits
    };
    for (int i = 0; i < n_random; ++i) {
        double const m = 1.0 + static_cast<double>(next()) * 0x1.0p-53;
        int const e = static_cast<int>(next() % 201) - 100;
        h.push_back(std::ldexp(m, e));
    }
    for (int e = -100; e <= 100; ++e) {
        h.push_back(std::ldexp(1.0, e));
        h.push_back(std::ldexp(std::nextafter(2.0, 1.0), e));
    }
    // the seeds' FP32 range ends (2^-125, 2^126) and beyond, where they fall
    // back to the FP64 approximation
    for (int e : {-400, -300, -200, -130, -127, -126, -125, -124, 124, 125, 126, 127, 128, 130, 200, 300, 400}) {
        h.push_back(std::ldexp(1.0, e));
        h.push_back(std::ldexp(std::nextafter(2.0, 1.0), e));
        h.push_back(std::ldexp(1.5, e));
    }
    int const n = static_cast<int>(h.size());
    double* dx = nullptr;
    double* dout = nullptr;
    if (cudaMalloc(&dx, sizeof(double) * n) != cudaSuccess ||
        cudaMalloc(&dout, sizeof(double) * 8 * static_cast<size_t>(n)) != cudaSuccess) {
        std::printf("cudaMalloc failed\n");
        return 1;
    }
    cudaMemcpy(dx, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    check_kernel<<<(n + 255) / 256, 256>>>(dx, dout, n);
    cudaError_t const err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        std::printf("kernel failed: %s\n", cudaGetErrorString(err));
        return 1;
    }
    std::vector<double> o(8 * static_cast<size_t>(n));
    cudaMemcpy(o.data(), dout, sizeof(double) * o.size(), cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dout);
    double rcp_approx = 0.0, rsqrt_approx = 0.0;
    long long rcp_ulp = 0, sqrt_ulp = 0, rcp_diff = 0, sqrt_diff = 0, quot_ulp = 0;
    for (int i = 0; i < n; ++i) {
        double const* r = o.data() + 6 * static_cast<size_t>(i);
        rcp_approx = std::fmax(rcp_approx, std::fabs(r[0] * h[static_cast<size_t>(i)] - 1.0));
        rsqrt_approx = std::fmax(rsqrt_approx, std::fabs(r[3] * r[4] - 1.0)); // rsqrt(x) sqrt(x) = 1
        long long const du = std::llabs(bits(r[2]) - bits(r[1]));
        long long const ds = std::llabs(bits(r[5]) - bits(r[4]));
        rcp_ulp = du > rcp_ulp ? du : rcp_ulp;
        sqrt_ulp = ds > sqrt_ulp ? ds : sqrt_ulp;
        rcp_diff += du != 0;
        sqrt_diff += ds != 0;
        double const* qv = o.data() + 6 * static_cast<size_t>(n) + 2 * static_cast<size_t>(i);
        long long const dq = std::llabs(bits(qv[1]) - bits(qv[0]));
        quot_ulp = dq > quot_ulp ? dq : quot_ulp;
    }
    std::printf("{\"n\": %d, \"rcp_approx_rel\": %.6e, \"rsqrt_approx_rel\": %.6e, \"rcp_max_ulp\": %lld, "
                "\"sqrt_max_ulp\": %lld, \"rcp_differ\": %lld, \"sqrt_differ\": %lld, \"quot_max_ulp\": %lld}\n",
                n, rcp_approx, rsqrt_approx, rcp_ulp, sqrt_ulp, rcp_diff, sqrt_diff, quot_ulp);
    return 0;
}
