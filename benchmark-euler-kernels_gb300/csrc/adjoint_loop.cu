// Checkpointed adjoint of the time loop (eulr_adjoint_*).
//
// Forward: the FP64 fused simulation (sim.cu) runs nsteps steps from prim0,
// either with CFL time steps (recorded) or with a given dt sequence, and the
// full state (prim, cons, sound speed) is copied aside every
// checkpoint_every steps.  Backward: segments are processed last to first.
// Each is recomputed from its checkpoint with the recorded dt sequence --
// bit-identical to the forward pass -- keeping prim_n of every step in the
// segment, and then the reverse steps (adjoint.cu) run from its last step
// down to its first.  A segment of k steps needs prim_n for its k steps:
// the first is the checkpoint's own prim, and the k-1 recomputed steps
// write theirs into the segment buffer from the step kernels themselves (a
// second prim output), so recording costs no copies.  The final state is
// kept from the forward pass.  Memory: ceil(nsteps/k) checkpoints of 11
// fields plus k-1 primitive states, instead of nsteps states.
//
// Device memory (one allocation, fields of n0*n1*n2 doubles padded to 256 B):
//   checkpoints   nckpt x 11
//   segment prims (k-1) x 5
//   cbar 5, prim0_bar 5, final prim_bar 5, final prim 5
//   reverse-step workspace kAdjWorkFields
#include "euler_gb300.h"
#include "kernels.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

using namespace eulr;

struct eulr_adjoint {
    int device = 0;
    int sms = 0;
    int n0 = 0, n1 = 0, n2 = 0;
    double gamma = 1.4, dx[3] = {1, 1, 1}, cfl = 0.4;
    int nsteps = 0, every = 1, nckpt = 0;
    cudaStream_t stream = nullptr;
    eulr_sim* sim = nullptr;
    long long ncell = 0;
    size_t field = 0;
    void* slab = nullptr;
    std::vector<double> dts;
    bool have_forward = false;
    double fwd_ms = 0, rec_ms = 0, rev_ms = 0;

    double* at(size_t index) const { return reinterpret_cast<double*>(static_cast<char*>(slab) + field * index); }
    double* ckpt(int c, int f) const { return at(static_cast<size_t>(c) * 11 + f); }
    // prim of the n-th step after a segment's checkpoint, n = 1 .. every-1
    double* seg(int n, int f) const
    {
        return at(static_cast<size_t>(nckpt) * 11 + static_cast<size_t>(n - 1) * 5 + f);
    }
    size_t tail() const { return static_cast<size_t>(nckpt) * 11 + static_cast<size_t>(every - 1) * 5; }
    double* cbar(int f) const { return at(tail() + f); }
    double* pbar0(int f) const { return at(tail() + 5 + f); }
    double* pbarT(int f) const { return at(tail() + 10 + f); }
    double* primN(int f) const { return at(tail() + 15 + f); }
    void* work() const { return at(tail() + 20); }
    size_t nfields() const { return tail() + 20 + kAdjWorkFields; }
};

namespace {

int fail(int status, const char* msg) { return eulr::sim_fail(status, msg); }

int cfail(cudaError_t e, const char* what)
{
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return fail(e == cudaErrorMemoryAllocation ? EULR_ERR_OUT_OF_MEMORY : EULR_ERR_CUDA, buf);
}

#define ADJ_TRY(expr)                     \
    do {                                  \
        int const _st = (expr);           \
        if (_st != EULR_SUCCESS) {        \
            return _st;                   \
        }                                 \
    } while (0)

#define ADJ_CUDA(call, what)              \
    do {                                  \
        cudaError_t const _e = (call);    \
        if (_e != cudaSuccess) {          \
            return cfail(_e, what);       \
        }                                 \
    } while (0)

int check_adj(eulr_adjoint* a)
{
    if (a == nullptr) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "adjoint handle is NULL");
    }
    int dev = 0;
    ADJ_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev != a->device) {
        ADJ_CUDA(cudaSetDevice(a->device), "cudaSetDevice");
    }
    return EULR_SUCCESS;
}

CBundle<double> cb(double* const* f)
{
    CBundle<double> b;
    for (int i = 0; i < 5; ++i) {
        b.f[i] = f[i];
    }
    return b;
}

Bundle<double> bb(double* const* f)
{
    Bundle<double> b;
    for (int i = 0; i < 5; ++i) {
        b.f[i] = f[i];
    }
    return b;
}

// Times a stretch of stream work with a pair of events.
struct Span {
    cudaEvent_t a = nullptr, b = nullptr;
    Span()
    {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    Span(Span const&) = delete;
    Span& operator=(Span const&) = delete;
    ~Span()
    {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    double ms() const
    {
        float v = 0.0f;
        return cudaEventElapsedTime(&v, a, b) == cudaSuccess ? static_cast<double>(v) : 0.0;
    }
};

int copy5(eulr_adjoint* a, double* const* dst, const double* const* src)
{
    size_t const bytes = static_cast<size_t>(a->ncell) * sizeof(double);
    for (int f = 0; f < 5; ++f) {
        if (dst[f] != nullptr && src[f] != nullptr) {
            ADJ_CUDA(cudaMemcpyAsync(dst[f], src[f], bytes, cudaMemcpyDefault, a->stream), "cudaMemcpyAsync");
        }
    }
    return EULR_SUCCESS;
}

} // namespace

extern "C" {

int eulr_adjoint_create(int n0, int n1, int n2, double gamma, double dx0, double dx1, double dx2, double cfl,
                        int nsteps, int checkpoint_every, eulr_stream_t stream, eulr_adjoint** out)
{
    if (out == nullptr) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "out is NULL");
    }
    *out = nullptr;
    if (nsteps < 0 || checkpoint_every < 1) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "nsteps must be >= 0 and checkpoint_every >= 1");
    }
    auto* a = new (std::nothrow) eulr_adjoint();
    if (a == nullptr) {
        return fail(EULR_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    eulr_sim* sim = nullptr;
    int st = eulr_sim_create(EULR_PRECISION_F64, n0, n1, n2, gamma, dx0, dx1, dx2, cfl, stream, &sim);
    if (st != EULR_SUCCESS) {
        delete a;
        return st;
    }
    a->sim = sim;
    a->n0 = n0;
    a->n1 = n1;
    a->n2 = n2;
    a->gamma = gamma;
    a->dx[0] = dx0;
    a->dx[1] = dx1;
    a->dx[2] = dx2;
    a->cfl = cfl;
    a->nsteps = nsteps;
    a->every = checkpoint_every < nsteps ? checkpoint_every : (nsteps > 0 ? nsteps : 1);
    a->nckpt = nsteps > 0 ? (nsteps + a->every - 1) / a->every : 1;
    a->stream = eulr::sim_stream(sim); // the reverse steps follow the simulation's work in stream order
    a->ncell = static_cast<long long>(n0) * n1 * n2;
    a->field = (static_cast<size_t>(a->ncell) * sizeof(double) + 255) & ~static_cast<size_t>(255);
    a->dts.assign(static_cast<size_t>(nsteps), 0.0);
    cudaError_t e = cudaGetDevice(&a->device);
    if (e == cudaSuccess) {
        e = cudaDeviceGetAttribute(&a->sms, cudaDevAttrMultiProcessorCount, a->device);
    }
    if (e == cudaSuccess) {
        e = cudaMalloc(&a->slab, a->field * a->nfields());
    }
    if (e != cudaSuccess) {
        st = cfail(e, "eulr_adjoint_create");
        eulr_adjoint_destroy(a);
        return st;
    }
    *out = a;
    return EULR_SUCCESS;
}

int eulr_adjoint_destroy(eulr_adjoint* a)
{
    if (a == nullptr) {
        return EULR_SUCCESS;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != a->device) {
        cudaSetDevice(a->device);
    }
    if (a->slab != nullptr) {
        cudaStreamSynchronize(a->stream);
        cudaFree(a->slab);
    }
    if (a->sim != nullptr) {
        eulr_sim_destroy(a->sim);
    }
    if (dev != a->device) {
        cudaSetDevice(dev);
    }
    delete a;
    return EULR_SUCCESS;
}

int eulr_adjoint_forward(eulr_adjoint* a, eulr_prim_cf64 prim0, const double* dts, eulr_prim_f64 prim_final)
{
    ADJ_TRY(check_adj(a));
    a->have_forward = false;
    bool const fixed = dts != nullptr;
    if (fixed) {
        for (int n = 0; n < a->nsteps; ++n) {
            if (!std::isfinite(dts[n]) || !(dts[n] > 0.0)) {
                return fail(EULR_ERR_INVALID_VALUE, "dt sequence entries must be finite and > 0");
            }
            a->dts[static_cast<size_t>(n)] = dts[n];
        }
        ADJ_TRY(eulr_sim_set_dt_sequence(a->sim, a->dts.data(), a->nsteps));
    } else {
        ADJ_TRY(eulr_sim_set_dt_sequence(a->sim, nullptr, 0));
    }
    ADJ_TRY(eulr_sim_set_prim_f64(a->sim, prim0));
    Span span;
    ADJ_CUDA(cudaEventRecord(span.a, a->stream), "cudaEventRecord");
    for (int c = 0; c < a->nckpt; ++c) {
        double* dst[11];
        for (int f = 0; f < 11; ++f) {
            dst[f] = a->ckpt(c, f);
        }
        ADJ_TRY(eulr::sim_snapshot(a->sim, dst, 11));
        int const s0 = c * a->every;
        int const s1 = s0 + a->every < a->nsteps ? s0 + a->every : a->nsteps;
        if (fixed) {
            ADJ_TRY(eulr_sim_advance(a->sim, s1 - s0));
        } else {
            for (int n = s0; n < s1; ++n) {
                double next = 0.0;
                ADJ_TRY(eulr_sim_time(a->sim, nullptr, &next, nullptr));
                a->dts[static_cast<size_t>(n)] = next;
                ADJ_TRY(eulr_sim_advance(a->sim, 1));
            }
        }
    }
    ADJ_CUDA(cudaEventRecord(span.b, a->stream), "cudaEventRecord");
    double* fin[5];
    for (int f = 0; f < 5; ++f) {
        fin[f] = a->primN(f);
    }
    ADJ_TRY(eulr::sim_snapshot(a->sim, fin, 5));
    ADJ_TRY(eulr_sim_status(a->sim));
    ADJ_TRY(eulr_sim_get_state_f64(a->sim, prim_final, eulr_cons_f64{nullptr, nullptr, nullptr, nullptr, nullptr}));
    a->fwd_ms = span.ms();
    if (!fixed) { // the recompute replays the recorded steps
        ADJ_TRY(eulr_sim_set_dt_sequence(a->sim, a->dts.data(), a->nsteps));
    }
    a->have_forward = true;
    return EULR_SUCCESS;
}

int eulr_adjoint_dts(eulr_adjoint* a, double* dts)
{
    ADJ_TRY(check_adj(a));
    if (dts == nullptr) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "dts is NULL");
    }
    if (!a->have_forward) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "no forward pass yet");
    }
    std::memcpy(dts, a->dts.data(), a->dts.size() * sizeof(double));
    return EULR_SUCCESS;
}

int eulr_adjoint_backward(eulr_adjoint* a, eulr_prim_cf64 prim_final_bar, eulr_prim_f64 prim0_bar)
{
    ADJ_TRY(check_adj(a));
    if (!a->have_forward) {
        return fail(EULR_ERR_INVALID_ARGUMENT, "no forward pass yet");
    }
    const double* in[5] = {prim_final_bar.d, prim_final_bar.p, prim_final_bar.ux0, prim_final_bar.ux1,
                           prim_final_bar.ux2};
    double* out[5] = {prim0_bar.d, prim0_bar.p, prim0_bar.ux0, prim0_bar.ux1, prim0_bar.ux2};
    for (int f = 0; f < 5; ++f) {
        if (in[f] == nullptr || out[f] == nullptr) {
            return fail(EULR_ERR_INVALID_ARGUMENT, "gradient field is NULL");
        }
    }
    double* pT[5];
    double* p0[5];
    double* cbar[5];
    for (int f = 0; f < 5; ++f) {
        pT[f] = a->pbarT(f);
        p0[f] = a->pbar0(f);
        cbar[f] = a->cbar(f);
    }
    ADJ_TRY(copy5(a, pT, in));
    if (a->nsteps == 0) { // the final state is the initial one
        ADJ_TRY(copy5(a, out, pT));
        ADJ_CUDA(cudaStreamSynchronize(a->stream), "cudaStreamSynchronize");
        return EULR_SUCCESS;
    }
    Geom const g = make_geom(a->n0, a->n1, a->n2);
    AdjWork const w = adjoint_workspace(a->work(), a->ncell);
    std::vector<Span> spans(static_cast<size_t>(a->nckpt) * 2);
    for (int c = a->nckpt - 1; c >= 0; --c) {
        int const s0 = c * a->every;
        int const s1 = s0 + a->every < a->nsteps ? s0 + a->every : a->nsteps;
        Span& rec = spans[static_cast<size_t>(c) * 2];
        Span& rev = spans[static_cast<size_t>(c) * 2 + 1];
        ADJ_CUDA(cudaEventRecord(rec.a, a->stream), "cudaEventRecord");
        const double* src[11];
        for (int f = 0; f < 11; ++f) {
            src[f] = a->ckpt(c, f);
        }
        ADJ_TRY(eulr::sim_restore(a->sim, src, s0));
        // prim of steps s0+1 .. s1-1, written by the recomputing step kernels
        // themselves (prim of step s0 is the checkpoint's)
        for (int n = s0 + 1; n < s1; ++n) {
            double* dst[5];
            for (int f = 0; f < 5; ++f) {
                dst[f] = a->seg(n - s0, f);
            }
            ADJ_TRY(eulr::sim_advance_recording(a->sim, dst));
        }
        ADJ_CUDA(cudaEventRecord(rec.b, a->stream), "cudaEventRecord");
        ADJ_CUDA(cudaEventRecord(rev.a, a->stream), "cudaEventRecord");
        if (c == a->nckpt - 1) { // dJ/dcons_N = cons_to_prim'(prim_N)^T dJ/dprim_N
            double* pN[5];
            for (int f = 0; f < 5; ++f) {
                pN[f] = a->primN(f);
            }
            ADJ_CUDA(launch_cons_to_prim_adjoint(cb(pN), cb(pT), bb(cbar), 0, a->ncell, a->gamma, a->sms, a->stream),
                     "cons_to_prim adjoint");
        }
        // each gather pass also prepares the next reverse step of the segment
        for (int n = s1 - 1; n >= s0; --n) {
            double* pn[5];
            double* pp[5];
            for (int f = 0; f < 5; ++f) {
                pn[f] = n == s0 ? a->ckpt(c, f) : a->seg(n - s0, f);
                pp[f] = n - 1 > s0 ? a->seg(n - 1 - s0, f) : (n - 1 == s0 ? a->ckpt(c, f) : nullptr);
            }
            int const mode = n == 0 ? kAdjInitial : kAdjStep;
            CBundle<double> const prev = cb(pp);
            bool const fuse = mode == kAdjStep && n - 1 >= s0;
            ADJ_CUDA(launch_step_adjoint(cb(pn), cb(cbar), bb(mode == kAdjStep ? cbar : p0), mode, g, a->gamma,
                                         a->dx[0], a->dx[1], a->dx[2], a->dts[static_cast<size_t>(n)], w, a->sms,
                                         a->stream, n < s1 - 1, fuse ? &prev : nullptr,
                                         fuse ? a->dts[static_cast<size_t>(n - 1)] : 0.0),
                     "reverse step");
        }
        ADJ_CUDA(cudaEventRecord(rev.b, a->stream), "cudaEventRecord");
    }
    ADJ_TRY(copy5(a, out, p0));
    ADJ_CUDA(cudaStreamSynchronize(a->stream), "cudaStreamSynchronize");
    ADJ_TRY(eulr_sim_status(a->sim));
    a->rec_ms = 0;
    a->rev_ms = 0;
    for (int c = 0; c < a->nckpt; ++c) {
        a->rec_ms += spans[static_cast<size_t>(c) * 2].ms();
        a->rev_ms += spans[static_cast<size_t>(c) * 2 + 1].ms();
    }
    return EULR_SUCCESS;
}

int eulr_adjoint_timing(eulr_adjoint* a, double* forward_ms, double* recompute_ms, double* reverse_ms)
{
    ADJ_TRY(check_adj(a));
    if (forward_ms != nullptr) {
        *forward_ms = a->fwd_ms;
    }
    if (recompute_ms != nullptr) {
        *recompute_ms = a->rec_ms;
    }
    if (reverse_ms != nullptr) {
        *reverse_ms = a->rev_ms;
    }
    return EULR_SUCCESS;
}

} // extern "C"
