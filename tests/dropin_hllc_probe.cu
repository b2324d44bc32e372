// Test program for the drop-in HLLC solver (include/euler_operators/hllc.hpp).
//
// Reads faces from a binary file, solves each with hllc{}(dir_t<D>(), eos,
// qL, qR) and writes the fluxes.  Compiled as host C++ (g++ -x c++
// -ffp-contract=off) it runs the functor on the host; compiled by nvcc it
// runs the same functor in a CUDA kernel, one thread per face.
//
//   dropin_hllc_probe f64|f32 in.bin out.bin
//
// in.bin:  int64 N, int32 dir[N], T gamma[N], T qL[N][5], T qR[N][5]
//          (q = d, p, ux0, ux1, ux2)
// out.bin: T flux[N][5] (d, e, mx0, mx1, mx2)
#include <hllc.hpp>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

template <std::size_t N>
using axis_t = std::integral_constant<std::size_t, N>;

template <class T>
EULR_HOST_DEVICE void solve(int dir, T gamma, T const* l, T const* r, T* f)
{
    PerfectGas<T> const eos(gamma);
    EulerPrim<T> const qL {l[0], l[1], l[2], l[3], l[4]};
    EulerPrim<T> const qR {r[0], r[1], r[2], r[3], r[4]};
    EulerFlux<T> x {};
    if (dir == 0) {
        x = hllc {}(axis_t<0>(), eos, qL, qR);
    } else if (dir == 1) {
        x = hllc {}(axis_t<1>(), eos, qL, qR);
    } else {
        x = hllc {}(axis_t<2>(), eos, qL, qR);
    }
    // the normal component through get(), the rest field by field
    T const normal = dir == 0 ? get(axis_t<0>(), x) : dir == 1 ? get(axis_t<1>(), x) : get(axis_t<2>(), x);
    f[0] = x.d;
    f[1] = x.e;
    f[2] = dir == 0 ? normal : x.mx0;
    f[3] = dir == 1 ? normal : x.mx1;
    f[4] = dir == 2 ? normal : x.mx2;
}

#if defined(__CUDACC__)
template <class T>
__global__ void solve_kernel(std::int64_t n, int const* dir, T const* gamma, T const* qL, T const* qR, T* f)
{
    std::int64_t const k = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x;
    if (k < n) {
        solve(dir[k], gamma[k], qL + 5 * k, qR + 5 * k, f + 5 * k);
    }
}

#define CHECK(x)                                                                                   \
    do {                                                                                           \
        cudaError_t const e_ = (x);                                                                \
        if (e_ != cudaSuccess) {                                                                   \
            std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));                         \
            return 1;                                                                              \
        }                                                                                          \
    } while (0)

template <class T>
int run_faces(std::int64_t n, std::vector<int> const& dir, std::vector<T> const& g, std::vector<T> const& qL,
              std::vector<T> const& qR, std::vector<T>& f)
{
    int* d_dir = nullptr;
    T *d_g = nullptr, *d_l = nullptr, *d_r = nullptr, *d_f = nullptr;
    CHECK(cudaMalloc(&d_dir, n * sizeof(int)));
    CHECK(cudaMalloc(&d_g, n * sizeof(T)));
    CHECK(cudaMalloc(&d_l, 5 * n * sizeof(T)));
    CHECK(cudaMalloc(&d_r, 5 * n * sizeof(T)));
    CHECK(cudaMalloc(&d_f, 5 * n * sizeof(T)));
    CHECK(cudaMemcpy(d_dir, dir.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_g, g.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_l, qL.data(), 5 * n * sizeof(T), cudaMemcpyHostToDevice));
    CHECK(cudaMemcpy(d_r, qR.data(), 5 * n * sizeof(T), cudaMemcpyHostToDevice));
    unsigned const blocks = static_cast<unsigned>((n + 127) / 128);
    solve_kernel<T><<<blocks, 128>>>(n, d_dir, d_g, d_l, d_r, d_f);
    CHECK(cudaGetLastError());
    CHECK(cudaMemcpy(f.data(), d_f, 5 * n * sizeof(T), cudaMemcpyDeviceToHost));
    CHECK(cudaFree(d_dir));
    CHECK(cudaFree(d_g));
    CHECK(cudaFree(d_l));
    CHECK(cudaFree(d_r));
    CHECK(cudaFree(d_f));
    return 0;
}
#else
template <class T>
int run_faces(std::int64_t n, std::vector<int> const& dir, std::vector<T> const& g, std::vector<T> const& qL,
              std::vector<T> const& qR, std::vector<T>& f)
{
    for (std::int64_t k = 0; k < n; ++k) {
        solve(dir[k], g[k], &qL[5 * k], &qR[5 * k], &f[5 * k]);
    }
    return 0;
}
#endif

template <class T>
int run(char const* in, char const* out)
{
    std::FILE* fi = std::fopen(in, "rb");
    if (fi == nullptr) {
        return 2;
    }
    std::int64_t n = 0;
    bool ok = std::fread(&n, sizeof n, 1, fi) == 1 && n > 0;
    std::vector<int> dir(ok ? n : 0);
    std::vector<T> g(ok ? n : 0), qL(ok ? 5 * n : 0), qR(ok ? 5 * n : 0), f(ok ? 5 * n : 0);
    ok = ok && std::fread(dir.data(), sizeof(int), n, fi) == static_cast<std::size_t>(n)
         && std::fread(g.data(), sizeof(T), n, fi) == static_cast<std::size_t>(n)
         && std::fread(qL.data(), sizeof(T), 5 * n, fi) == static_cast<std::size_t>(5 * n)
         && std::fread(qR.data(), sizeof(T), 5 * n, fi) == static_cast<std::size_t>(5 * n);
    std::fclose(fi);
    if (!ok) {
        return 3;
    }
    for (int d : dir) {
        if (d < 0 || d > 2) {
            return 4;
        }
    }
    if (run_faces<T>(n, dir, g, qL, qR, f) != 0) {
        return 5;
    }
    std::FILE* fo = std::fopen(out, "wb");
    if (fo == nullptr) {
        return 6;
    }
    ok = std::fwrite(f.data(), sizeof(T), 5 * n, fo) == static_cast<std::size_t>(5 * n);
    std::fclose(fo);
    return ok ? 0 : 7;
}

int main(int argc, char** argv)
{
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s f64|f32 in.bin out.bin\n", argv[0]);
        return 1;
    }
    if (std::strcmp(argv[1], "f64") == 0) {
        return run<double>(argv[2], argv[3]);
    }
    if (std::strcmp(argv[1], "f32") == 0) {
        return run<float>(argv[2], argv[3]);
    }
    return 1;
}
