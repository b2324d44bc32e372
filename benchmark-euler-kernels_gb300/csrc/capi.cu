// C ABI of the Euler operators (declared in include/euler_gb300.h): argument
// validation, per-device scratch, the device-resident simulation object and
// the measurement probe.  No exception crosses this boundary; every entry
// point returns an eulr_status.
#include "euler_gb300.h"
#include "kernels.h"

#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>

using namespace eulr;

namespace {

thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int cuda_fail(cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation) {
        return fail(EULR_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    }
    return fail(EULR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define EULR_CUDA_TRY(call, what)              \
    do {                                       \
        cudaError_t const _e = (call);         \
        if (_e != cudaSuccess) {               \
            return cuda_fail(_e, what);        \
        }                                      \
    } while (0)

int current_sms(int* sms)
{
    static std::mutex mu;
    static std::map<int, int> cache;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        return cuda_fail(e, "cudaGetDevice");
    }
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(dev);
    if (it == cache.end()) {
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) {
            return cuda_fail(e, "cudaDeviceGetAttribute");
        }
        it = cache.emplace(dev, n).first;
    }
    *sms = it->second;
    return EULR_SUCCESS;
}

int check_dims(int n0, int n1, int n2)
{
    if (n0 < 1 || n1 < 1 || n2 < 1) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "grid extents must be >= 1 (got %d x %d x %d)", n0, n1, n2);
    }
    long long const n = static_cast<long long>(n0) * n1 * n2;
    if (n > INT_MAX) {
        return fail(EULR_ERR_TOO_LARGE, "grid of %lld cells exceeds the int index range of the reference", n);
    }
    return EULR_SUCCESS;
}

template <class T>
int check_fields(const void* const* f, int count, const char* what)
{
    for (int i = 0; i < count; ++i) {
        if (f[i] == nullptr) {
            return fail(EULR_ERR_INVALID_ARGUMENT, "%s field %d is NULL", what, i);
        }
        if (reinterpret_cast<std::uintptr_t>(f[i]) % sizeof(T) != 0) {
            return fail(EULR_ERR_MISALIGNED, "%s field %d is not %zu-byte aligned", what, i, sizeof(T));
        }
    }
    return EULR_SUCCESS;
}

// Rejects partial or full overlap between any two of the given arrays of
// `bytes` each (pairs listed as allowed_equal may be identical).
int check_disjoint(const void* const* f, int count, size_t bytes, const char* what)
{
    for (int a = 0; a < count; ++a) {
        for (int b = a + 1; b < count; ++b) {
            auto const pa = reinterpret_cast<std::uintptr_t>(f[a]);
            auto const pb = reinterpret_cast<std::uintptr_t>(f[b]);
            if (pa < pb + bytes && pb < pa + bytes) {
                return fail(EULR_ERR_INVALID_ARGUMENT, "%s: arrays %d and %d overlap", what, a, b);
            }
        }
    }
    return EULR_SUCCESS;
}

template <class T>
bool finite_pos(T v)
{
    return std::isfinite(v) && v > T(0);
}

template <class T>
int check_gamma(T gamma)
{
    if (!std::isfinite(gamma) || !(gamma > T(1))) {
        return fail(EULR_ERR_INVALID_VALUE, "gamma must be finite and > 1 (got %g)", static_cast<double>(gamma));
    }
    return EULR_SUCCESS;
}

template <class T>
int check_dx(T dx0, T dx1, T dx2)
{
    if (!finite_pos(dx0) || !finite_pos(dx1) || !finite_pos(dx2)) {
        return fail(EULR_ERR_INVALID_VALUE, "mesh spacings must be finite and > 0 (got %g, %g, %g)",
                    static_cast<double>(dx0), static_cast<double>(dx1), static_cast<double>(dx2));
    }
    return EULR_SUCCESS;
}

#define EULR_TRY(expr)                 \
    do {                               \
        int const _s = (expr);         \
        if (_s != EULR_SUCCESS) {      \
            return _s;                 \
        }                              \
    } while (0)

template <class T, class B>
Bundle<T> to_bundle(B const& b)
{
    Bundle<T> r;
    std::memcpy(r.f, &b, sizeof(r.f));
    return r;
}

template <class T, class B>
CBundle<T> to_cbundle(B const& b)
{
    CBundle<T> r;
    std::memcpy(r.f, &b, sizeof(r.f));
    return r;
}

// ------------------------------------------------- per-device scratch
// The reduction behind time_step needs one partial per block and a
// completion counter.  The library allocates them once per device on first
// use (cudaMalloc) and keeps them until exit.
constexpr int kMaxPartials = 4096;

struct DeviceScratch {
    void* base = nullptr;
    unsigned int* counter = nullptr;
    double* partials = nullptr; // kMaxPartials doubles (floats use the same bytes)
};

int device_scratch(DeviceScratch** out)
{
    static std::mutex mu;
    static std::map<int, DeviceScratch> table;
    int dev = 0;
    EULR_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(mu);
    auto it = table.find(dev);
    if (it == table.end()) {
        DeviceScratch s;
        size_t const bytes = 256 + kMaxPartials * sizeof(double);
        EULR_CUDA_TRY(cudaMalloc(&s.base, bytes), "cudaMalloc(time_step scratch)");
        EULR_CUDA_TRY(cudaMemset(s.base, 0, bytes), "cudaMemset(time_step scratch)");
        s.counter = static_cast<unsigned int*>(s.base);
        s.partials = reinterpret_cast<double*>(static_cast<char*>(s.base) + 256);
        it = table.emplace(dev, s).first;
    }
    *out = &it->second;
    return EULR_SUCCESS;
}

// ------------------------------------------------- operator bodies
template <class T, class PB>
int init_implode_impl(PB prim, int n0, int n1, int n2, T dx0, T dx1, T dx2, cudaStream_t s)
{
    EULR_TRY(check_dims(n0, n1, n2));
    EULR_TRY(check_fields<T>(reinterpret_cast<const void* const*>(&prim), 5, "prim"));
    EULR_TRY(check_dx(dx0, dx1, dx2));
    size_t const bytes = static_cast<size_t>(n0) * n1 * n2 * sizeof(T);
    EULR_TRY(check_disjoint(reinterpret_cast<const void* const*>(&prim), 5, bytes, "init_implode"));
    int sms = 0;
    EULR_TRY(current_sms(&sms));
    EULR_CUDA_TRY(launch_init_implode<T>(to_bundle<T>(prim), make_geom(n0, n1, n2), static_cast<double>(dx0),
                                         static_cast<double>(dx1), static_cast<double>(dx2), sms, s),
                  "init_implode launch");
    return EULR_SUCCESS;
}

template <class T, class IB, class OB>
int pointwise_check(IB const& in, OB const& out, int n0, int n1, int n2, T gamma, const char* what)
{
    EULR_TRY(check_dims(n0, n1, n2));
    EULR_TRY(check_fields<T>(reinterpret_cast<const void* const*>(&in), 5, "input"));
    EULR_TRY(check_fields<T>(reinterpret_cast<const void* const*>(&out), 5, "output"));
    EULR_TRY(check_gamma(gamma));
    const void* all[10];
    std::memcpy(all, &in, 5 * sizeof(void*));
    std::memcpy(all + 5, &out, 5 * sizeof(void*));
    size_t const bytes = static_cast<size_t>(n0) * n1 * n2 * sizeof(T);
    return check_disjoint(all, 10, bytes, what);
}

template <class T, class PB, class CB>
int prim_to_cons_impl(PB prim, CB cons, int n0, int n1, int n2, T gamma, cudaStream_t s)
{
    EULR_TRY(pointwise_check<T>(prim, cons, n0, n1, n2, gamma, "prim_to_cons"));
    int sms = 0;
    EULR_TRY(current_sms(&sms));
    T const gm1 = gamma - T(1);
    T const rgm1 = T(1) / gm1;
    EULR_CUDA_TRY(launch_prim_to_cons<T>(to_cbundle<T>(prim), to_bundle<T>(cons),
                                         static_cast<long long>(n0) * n1 * n2, gm1, rgm1, sms, s),
                  "prim_to_cons launch");
    return EULR_SUCCESS;
}

template <class T, class CB, class PB>
int cons_to_prim_impl(CB cons, PB prim, int n0, int n1, int n2, T gamma, cudaStream_t s)
{
    EULR_TRY(pointwise_check<T>(cons, prim, n0, n1, n2, gamma, "cons_to_prim"));
    int sms = 0;
    EULR_TRY(current_sms(&sms));
    EULR_CUDA_TRY(launch_cons_to_prim<T>(to_cbundle<T>(cons), to_bundle<T>(prim),
                                         static_cast<long long>(n0) * n1 * n2, gamma - T(1), sms, s),
                  "cons_to_prim launch");
    return EULR_SUCCESS;
}

template <class T, class PB>
int time_step_impl(PB prim, int n0, int n1, int n2, T gamma, T dx0, T dx1, T dx2, T* dt_out, cudaStream_t s)
{
    EULR_TRY(check_dims(n0, n1, n2));
    EULR_TRY(check_fields<T>(reinterpret_cast<const void* const*>(&prim), 5, "prim"));
    EULR_TRY(check_gamma(gamma));
    EULR_TRY(check_dx(dx0, dx1, dx2));
    if (dt_out == nullptr) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "dt_out is NULL");
    }
    if (reinterpret_cast<std::uintptr_t>(dt_out) % sizeof(T) != 0) {
        return fail(EULR_ERR_MISALIGNED, "dt_out is not aligned");
    }
    int sms = 0;
    EULR_TRY(current_sms(&sms));
    DeviceScratch* scratch = nullptr;
    EULR_TRY(device_scratch(&scratch));
    EULR_CUDA_TRY(launch_time_step<T>(to_cbundle<T>(prim), static_cast<long long>(n0) * n1 * n2, gamma, T(1) / dx0,
                                      T(1) / dx1, T(1) / dx2, reinterpret_cast<T*>(scratch->partials), kMaxPartials,
                                      scratch->counter, dt_out, sms, s),
                  "time_step launch");
    return EULR_SUCCESS;
}

template <class T, class PB, class CB>
int godunov_impl(PB prim, CB cons, int n0, int n1, int n2, T gamma, T dx0, T dx1, T dx2, T dt, const T* dt_dev,
                 T cfl, cudaStream_t s, bool exact = false)
{
    EULR_TRY(check_dims(n0, n1, n2));
    EULR_TRY(check_fields<T>(reinterpret_cast<const void* const*>(&prim), 5, "prim"));
    EULR_TRY(check_fields<T>(reinterpret_cast<const void* const*>(&cons), 5, "cons"));
    EULR_TRY(check_gamma(gamma));
    EULR_TRY(check_dx(dx0, dx1, dx2));
    if (dt_dev == nullptr && !std::isfinite(dt)) {
        return fail(EULR_ERR_INVALID_VALUE, "dt must be finite");
    }
    if (dt_dev != nullptr && !std::isfinite(cfl)) {
        return fail(EULR_ERR_INVALID_VALUE, "cfl must be finite");
    }
    const void* all[10];
    std::memcpy(all, &prim, 5 * sizeof(void*));
    std::memcpy(all + 5, &cons, 5 * sizeof(void*));
    EULR_TRY(check_disjoint(all, 10, static_cast<size_t>(n0) * n1 * n2 * sizeof(T), "godunov"));
    int sms = 0;
    EULR_TRY(current_sms(&sms));
    if (exact) {
        EULR_CUDA_TRY(launch_godunov_exact<T>(to_cbundle<T>(prim), to_bundle<T>(cons), make_geom(n0, n1, n2), gamma,
                                              dx0, dx1, dx2, dt, sms, s),
                      "godunov (exact) launch");
        return EULR_SUCCESS;
    }
    FluxParams<T> p{};
    p.g = make_geom(n0, n1, n2);
    p.prim = to_cbundle<T>(prim);
    p.cons_in = to_cbundle<T>(cons);
    p.cons_out = to_bundle<T>(cons);
    p.gamma = gamma;
    p.gm1 = gamma - T(1);
    p.inv_gm1 = T(1) / (gamma - T(1));
    p.half_gm1 = T(0.5) * (gamma - T(1));
    p.ds0 = dx1 * dx2; // uniform_mesh.hpp:62-75
    p.ds1 = dx2 * dx0;
    p.ds2 = dx0 * dx1;
    p.dv = static_cast<double>(dx0 * dx1 * dx2);
    p.dtodv = dt / (dx0 * dx1 * dx2);
    if constexpr (sizeof(T) == sizeof(double)) {
        p.dt_dev = dt_dev; // the device-dt variant exists for FP64 only
    } else {
        p.dt_dev = nullptr;
    }
    p.cfl = static_cast<double>(cfl);
    EULR_CUDA_TRY(configure_flux<T>(kModeGodunov, false, kCompNone, &p.per_sm), "godunov configure");
    EULR_CUDA_TRY(launch_flux<T>(p, nullptr, kModeGodunov, kCompNone, sms, s), "godunov launch");
    return EULR_SUCCESS;
}

// Rejects overlap between any output array and any input array (inputs may
// overlap one another).
int check_out_disjoint(const void* const* out, int nout, const void* const* in, int nin, size_t bytes,
                       const char* what)
{
    for (int a = 0; a < nout; ++a) {
        for (int b = 0; b < nin; ++b) {
            auto const pa = reinterpret_cast<std::uintptr_t>(out[a]);
            auto const pb = reinterpret_cast<std::uintptr_t>(in[b]);
            if (pa < pb + bytes && pb < pa + bytes) {
                return fail(EULR_ERR_INVALID_ARGUMENT, "%s: output %d overlaps input %d", what, a, b);
            }
        }
    }
    return EULR_SUCCESS;
}

// The two pointwise transposes: kind 0 = cons_to_prim (out is cons_bar), 1 = prim_to_cons (out is prim_bar).
int pointwise_adjoint_impl(int kind, const void* const* prim, const void* const* in_bar, void* const* out_bar, int n0,
                           int n1, int n2, double gamma, int accumulate, cudaStream_t s)
{
    EULR_TRY(check_dims(n0, n1, n2));
    EULR_TRY(check_fields<double>(prim, 5, "prim"));
    EULR_TRY(check_fields<double>(in_bar, 5, "input adjoint"));
    EULR_TRY(check_fields<double>(out_bar, 5, "output adjoint"));
    EULR_TRY(check_gamma(gamma));
    long long const n = static_cast<long long>(n0) * n1 * n2;
    size_t const bytes = static_cast<size_t>(n) * sizeof(double);
    EULR_TRY(check_disjoint(out_bar, 5, bytes, "adjoint output"));
    const void* ins[10];
    std::memcpy(ins, prim, 5 * sizeof(void*));
    std::memcpy(ins + 5, in_bar, 5 * sizeof(void*));
    EULR_TRY(check_out_disjoint(out_bar, 5, ins, 10, bytes, "adjoint"));
    int sms = 0;
    EULR_TRY(current_sms(&sms));
    CBundle<double> pv, iv;
    Bundle<double> ov;
    for (int f = 0; f < 5; ++f) {
        pv.f[f] = static_cast<const double*>(prim[f]);
        iv.f[f] = static_cast<const double*>(in_bar[f]);
        ov.f[f] = static_cast<double*>(out_bar[f]);
    }
    cudaError_t const e = kind == 0 ? launch_cons_to_prim_adjoint(pv, iv, ov, accumulate, n, gamma, sms, s)
                                    : launch_prim_to_cons_adjoint(pv, iv, ov, accumulate, n, gamma, sms, s);
    EULR_CUDA_TRY(e, "adjoint launch");
    return EULR_SUCCESS;
}

} // namespace

namespace eulr {
// Error reporting for the simulation entry points (sim.cu).
int sim_fail(int status, const char* msg)
{
    g_last_error = msg;
    return status;
}
} // namespace eulr

// ================================================================ C ABI
extern "C" {

int eulr_version(void) { return 100; }

const char* eulr_status_string(int status)
{
    switch (status) {
    case EULR_SUCCESS: return "success";
    case EULR_ERR_INVALID_ARGUMENT: return "invalid argument";
    case EULR_ERR_INVALID_VALUE: return "invalid value";
    case EULR_ERR_MISALIGNED: return "misaligned pointer";
    case EULR_ERR_CUDA: return "CUDA error";
    case EULR_ERR_OUT_OF_MEMORY: return "out of device memory";
    case EULR_ERR_TOO_LARGE: return "size too large";
    case EULR_ERR_NONFINITE: return "non-finite or non-physical state";
    case EULR_ERR_NO_DEVICE: return "no CUDA device";
    case EULR_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

const char* eulr_last_error(void) { return g_last_error.c_str(); }

int eulr_init_implode_f64(eulr_prim_f64 prim, int n0, int n1, int n2, double dx0, double dx1, double dx2,
                          eulr_stream_t stream)
{
    return init_implode_impl<double>(prim, n0, n1, n2, dx0, dx1, dx2, stream);
}

int eulr_init_implode_f32(eulr_prim_f32 prim, int n0, int n1, int n2, float dx0, float dx1, float dx2,
                          eulr_stream_t stream)
{
    return init_implode_impl<float>(prim, n0, n1, n2, dx0, dx1, dx2, stream);
}

int eulr_prim_to_cons_f64(eulr_prim_cf64 prim, eulr_cons_f64 cons, int n0, int n1, int n2, double gamma,
                          eulr_stream_t stream)
{
    return prim_to_cons_impl<double>(prim, cons, n0, n1, n2, gamma, stream);
}

int eulr_prim_to_cons_f32(eulr_prim_cf32 prim, eulr_cons_f32 cons, int n0, int n1, int n2, float gamma,
                          eulr_stream_t stream)
{
    return prim_to_cons_impl<float>(prim, cons, n0, n1, n2, gamma, stream);
}

int eulr_cons_to_prim_f64(eulr_cons_cf64 cons, eulr_prim_f64 prim, int n0, int n1, int n2, double gamma,
                          eulr_stream_t stream)
{
    return cons_to_prim_impl<double>(cons, prim, n0, n1, n2, gamma, stream);
}

int eulr_cons_to_prim_f32(eulr_cons_cf32 cons, eulr_prim_f32 prim, int n0, int n1, int n2, float gamma,
                          eulr_stream_t stream)
{
    return cons_to_prim_impl<float>(cons, prim, n0, n1, n2, gamma, stream);
}

int eulr_time_step_f64(eulr_prim_cf64 prim, int n0, int n1, int n2, double gamma, double dx0, double dx1,
                       double dx2, double* dt_out, eulr_stream_t stream)
{
    return time_step_impl<double>(prim, n0, n1, n2, gamma, dx0, dx1, dx2, dt_out, stream);
}

int eulr_time_step_f32(eulr_prim_cf32 prim, int n0, int n1, int n2, float gamma, float dx0, float dx1, float dx2,
                       float* dt_out, eulr_stream_t stream)
{
    return time_step_impl<float>(prim, n0, n1, n2, gamma, dx0, dx1, dx2, dt_out, stream);
}

int eulr_godunov_f64(eulr_prim_cf64 prim, eulr_cons_f64 cons, int n0, int n1, int n2, double gamma, double dx0,
                     double dx1, double dx2, double dt, eulr_stream_t stream)
{
    return godunov_impl<double>(prim, cons, n0, n1, n2, gamma, dx0, dx1, dx2, dt, nullptr, 0.0, stream);
}

int eulr_godunov_f32(eulr_prim_cf32 prim, eulr_cons_f32 cons, int n0, int n1, int n2, float gamma, float dx0,
                     float dx1, float dx2, float dt, eulr_stream_t stream)
{
    return godunov_impl<float>(prim, cons, n0, n1, n2, gamma, dx0, dx1, dx2, dt, nullptr, 0.0f, stream);
}

int eulr_godunov_exact_f64(eulr_prim_cf64 prim, eulr_cons_f64 cons, int n0, int n1, int n2, double gamma, double dx0,
                           double dx1, double dx2, double dt, eulr_stream_t stream)
{
    return godunov_impl<double>(prim, cons, n0, n1, n2, gamma, dx0, dx1, dx2, dt, nullptr, 0.0, stream, true);
}

int eulr_godunov_exact_f32(eulr_prim_cf32 prim, eulr_cons_f32 cons, int n0, int n1, int n2, float gamma, float dx0,
                           float dx1, float dx2, float dt, eulr_stream_t stream)
{
    return godunov_impl<float>(prim, cons, n0, n1, n2, gamma, dx0, dx1, dx2, dt, nullptr, 0.0f, stream, true);
}

int eulr_godunov_devdt_f64(eulr_prim_cf64 prim, eulr_cons_f64 cons, int n0, int n1, int n2, double gamma,
                           double dx0, double dx1, double dx2, const double* dt_dev, double cfl,
                           eulr_stream_t stream)
{
    if (dt_dev == nullptr) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "dt_dev is NULL");
    }
    return godunov_impl<double>(prim, cons, n0, n1, n2, gamma, dx0, dx1, dx2, 0.0, dt_dev, cfl, stream);
}

size_t eulr_godunov_adjoint_workspace_bytes(int n0, int n1, int n2)
{
    if (n0 < 1 || n1 < 1 || n2 < 1 || static_cast<long long>(n0) * n1 * n2 > INT_MAX) {
        return 0;
    }
    return adjoint_workspace_bytes(static_cast<long long>(n0) * n1 * n2);
}

int eulr_godunov_adjoint_f64(eulr_prim_cf64 prim, eulr_cons_cf64 cons_bar, eulr_prim_f64 prim_bar, int n0, int n1,
                             int n2, double gamma, double dx0, double dx1, double dx2, double dt, void* workspace,
                             size_t workspace_bytes, eulr_stream_t stream)
{
    EULR_TRY(check_dims(n0, n1, n2));
    EULR_TRY(check_fields<double>(reinterpret_cast<const void* const*>(&prim), 5, "prim"));
    EULR_TRY(check_fields<double>(reinterpret_cast<const void* const*>(&cons_bar), 5, "cons_bar"));
    EULR_TRY(check_fields<double>(reinterpret_cast<const void* const*>(&prim_bar), 5, "prim_bar"));
    EULR_TRY(check_gamma(gamma));
    EULR_TRY(check_dx(dx0, dx1, dx2));
    if (!std::isfinite(dt)) {
        return fail(EULR_ERR_INVALID_VALUE, "dt must be finite");
    }
    long long const n = static_cast<long long>(n0) * n1 * n2;
    size_t const need = adjoint_workspace_bytes(n);
    if (workspace == nullptr || workspace_bytes < need) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "workspace of %zu bytes needed (got %zu)", need,
                    workspace == nullptr ? static_cast<size_t>(0) : workspace_bytes);
    }
    if (reinterpret_cast<std::uintptr_t>(workspace) % 256 != 0) {
        return fail(EULR_ERR_MISALIGNED, "workspace must be 256-byte aligned");
    }
    size_t const bytes = static_cast<size_t>(n) * sizeof(double);
    const void* outs[5];
    std::memcpy(outs, &prim_bar, sizeof(outs));
    EULR_TRY(check_disjoint(outs, 5, bytes, "godunov adjoint output"));
    const void* ins[10];
    std::memcpy(ins, &prim, 5 * sizeof(void*));
    std::memcpy(ins + 5, &cons_bar, 5 * sizeof(void*));
    EULR_TRY(check_out_disjoint(outs, 5, ins, 10, bytes, "godunov adjoint"));
    auto const ws = reinterpret_cast<std::uintptr_t>(workspace);
    for (int f = 0; f < 15; ++f) {
        auto const pf = reinterpret_cast<std::uintptr_t>(f < 10 ? ins[f] : outs[f - 10]);
        if (pf < ws + need && ws < pf + bytes) {
            return fail(EULR_ERR_INVALID_ARGUMENT, "godunov adjoint: the workspace overlaps argument array %d", f);
        }
    }
    int sms = 0;
    EULR_TRY(current_sms(&sms));
    AdjWork const w = adjoint_workspace(workspace, n);
    EULR_CUDA_TRY(launch_step_adjoint(to_cbundle<double>(prim), to_cbundle<double>(cons_bar),
                                      to_bundle<double>(prim_bar), kAdjGodunov, make_geom(n0, n1, n2), gamma, dx0,
                                      dx1, dx2, dt, w, sms, stream),
                  "godunov adjoint launch");
    return EULR_SUCCESS;
}

int eulr_cons_to_prim_adjoint_f64(eulr_prim_cf64 prim, eulr_prim_cf64 prim_bar, eulr_cons_f64 cons_bar, int n0,
                                  int n1, int n2, double gamma, int accumulate, eulr_stream_t stream)
{
    return pointwise_adjoint_impl(0, reinterpret_cast<const void* const*>(&prim),
                                  reinterpret_cast<const void* const*>(&prim_bar),
                                  reinterpret_cast<void* const*>(&cons_bar), n0, n1, n2, gamma, accumulate, stream);
}

int eulr_prim_to_cons_adjoint_f64(eulr_prim_cf64 prim, eulr_cons_cf64 cons_bar, eulr_prim_f64 prim_bar, int n0,
                                  int n1, int n2, double gamma, int accumulate, eulr_stream_t stream)
{
    return pointwise_adjoint_impl(1, reinterpret_cast<const void* const*>(&prim),
                                  reinterpret_cast<const void* const*>(&cons_bar),
                                  reinterpret_cast<void* const*>(&prim_bar), n0, n1, n2, gamma, accumulate, stream);
}

int eulr_probe_fma_rate(int kind, int iters, double* flops)
{
    if (flops == nullptr || iters < 1 || (kind != 0 && kind != 1)) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "eulr_probe_fma_rate: bad arguments");
    }
    int sms = 0;
    EULR_TRY(current_sms(&sms));
    int const blocks = sms * 8;
    float* sink = nullptr;
    EULR_CUDA_TRY(cudaMalloc(&sink, blocks * sizeof(float)), "cudaMalloc(probe)");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t err = launch_fma_probe(kind, blocks, iters / 10 + 1, sink, nullptr); // warm-up
    if (err == cudaSuccess) {
        cudaEventRecord(e0, nullptr);
        err = launch_fma_probe(kind, blocks, iters, sink, nullptr);
        cudaEventRecord(e1, nullptr);
    }
    if (err == cudaSuccess) {
        err = cudaEventSynchronize(e1);
    }
    float ms = 0.0f;
    if (err == cudaSuccess) {
        err = cudaEventElapsedTime(&ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess) {
        return cuda_fail(err, "FMA probe");
    }
    double const fl = 2.0 * 8.0 * static_cast<double>(iters) * 256.0 * blocks;
    *flops = fl / (static_cast<double>(ms) * 1e-3);
    return EULR_SUCCESS;
}

} // extern "C"
