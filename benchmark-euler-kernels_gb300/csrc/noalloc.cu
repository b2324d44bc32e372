// time_step without any allocation: eulr_time_step_noalloc_f64.
//
// Some callers cannot call cudaMalloc: code that runs inside a memory pool
// or arena that owns every device byte (a host application that hands the
// solver pre-sized buffers and forbids hidden allocations), code on a path
// where an allocation could synchronise the device or fail late, and
// embedders that must know the library's whole device footprint before they
// start.  eulr_time_step_f64 needs scratch for its reduction (one maximum per
// block and a completion counter) and takes it from a cudaMalloc the library
// makes on first use.  This entry point uses instead a fixed array that
// lives in the library's own device image: every GPU that loads the library
// holds it until the process exits, and nothing is allocated at call time.
//
// Limits and rules:
//  * the array holds kNoallocPartials (1024) block maxima plus a counter,
//    about 8 KiB; the reduction kernel is launched with at most 1024 blocks
//    whose threads stride over the whole grid, so every grid the library
//    accepts fits; grids of 2^31 cells or more are rejected with
//    EULR_ERR_TOO_LARGE, like the other entry points;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current); make
//    that first call before any stream capture on that device;
//  * all calls on a device share the one array and each call leaves its
//    contents behind; the call clears the counter before the kernel runs, so
//    a stale value never leaks into a result, but calls whose kernels can
//    overlap on the GPU (different streams, no ordering between them) race
//    on the array and must not be issued.
#include "euler_gb300.h"
#include "kernels.h"

#include <map>
#include <mutex>

namespace eulr {
int sim_fail(int status, const char* msg);
}

namespace {

constexpr int kNoallocPartials = 1024;
constexpr int kCounterSlots = 32; // 256 bytes in front of the partials: the counter and padding

// Device-side scratch of eulr_time_step_noalloc_f64: [counter | pad][partials].
// In host code this name is only a stand-in for the device array; its device
// address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_time_step_scratch[kCounterSlots + kNoallocPartials];

struct NoallocScratch {
    unsigned int* counter = nullptr;
    double* partials = nullptr;
};

// Device address of the scratch on the current device, looked up once per
// device (cudaGetSymbolAddress allocates nothing).
int scratch_for_current_device(NoallocScratch* out)
{
    static std::mutex mu;
    static std::map<int, NoallocScratch> table;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        return eulr::sim_fail(EULR_ERR_CUDA, cudaGetErrorString(e));
    }
    std::lock_guard<std::mutex> lock(mu);
    auto it = table.find(dev);
    if (it == table.end()) {
        void* base = nullptr;
        e = cudaGetSymbolAddress(&base, g_time_step_scratch);
        if (e != cudaSuccess || base == nullptr) {
            return eulr::sim_fail(EULR_ERR_CUDA, "cudaGetSymbolAddress(time_step scratch) failed");
        }
        NoallocScratch s;
        s.counter = static_cast<unsigned int*>(base);
        s.partials = static_cast<double*>(base) + kCounterSlots;
        it = table.emplace(dev, s).first;
    }
    *out = it->second;
    return EULR_SUCCESS;
}

} // namespace

extern "C" int eulr_time_step_noalloc_f64(eulr_prim_cf64 prim, int n0, int n1, int n2, double gamma, double dx0,
                                          double dx1, double dx2, double* dt_out, eulr_stream_t stream)
{
    if (n0 < 1 || n1 < 1 || n2 < 1) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "grid extents must be >= 1");
    }
    if (static_cast<long long>(n0) * n1 * n2 > 2147483647LL) {
        return eulr::sim_fail(EULR_ERR_TOO_LARGE,
                              "eulr_time_step_noalloc_f64: grids of 2^31 cells or more are not supported");
    }
    const double* f[5] = {prim.d, prim.p, prim.ux0, prim.ux1, prim.ux2};
    for (auto const* p : f) {
        if (p == nullptr) {
            return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "prim field is NULL");
        }
        if (reinterpret_cast<uintptr_t>(p) % sizeof(double) != 0) {
            return eulr::sim_fail(EULR_ERR_MISALIGNED, "prim field is not 8-byte aligned");
        }
    }
    if (dt_out == nullptr) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "dt_out is NULL");
    }
    if (reinterpret_cast<uintptr_t>(dt_out) % sizeof(double) != 0) {
        return eulr::sim_fail(EULR_ERR_MISALIGNED, "dt_out is not 8-byte aligned");
    }
    if (!(gamma > 1.0) || !(gamma < 1.0e300)) {
        return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "gamma must be finite and > 1");
    }
    if (!(dx0 > 0.0 && dx0 < 1.0e300) || !(dx1 > 0.0 && dx1 < 1.0e300) || !(dx2 > 0.0 && dx2 < 1.0e300)) {
        return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "mesh spacings must be finite and > 0");
    }
    NoallocScratch scratch;
    int const st = scratch_for_current_device(&scratch);
    if (st != EULR_SUCCESS) {
        return st;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) {
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    // the completion counter must start at zero whatever an earlier call left
    if (e == cudaSuccess) {
        e = cudaMemsetAsync(scratch.counter, 0, sizeof(unsigned int), stream);
    }
    if (e == cudaSuccess) {
        eulr::CBundle<double> pv;
        for (int i = 0; i < 5; ++i) {
            pv.f[i] = f[i];
        }
        e = eulr::launch_time_step<double>(pv, static_cast<long long>(n0) * n1 * n2, gamma, 1.0 / dx0, 1.0 / dx1,
                                           1.0 / dx2, scratch.partials, kNoallocPartials, scratch.counter, dt_out,
                                           sms, stream);
    }
    if (e != cudaSuccess) {
        return eulr::sim_fail(EULR_ERR_CUDA, cudaGetErrorString(e));
    }
    return EULR_SUCCESS;
}
