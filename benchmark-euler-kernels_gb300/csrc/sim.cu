// Device-resident simulation (eulr_sim_*): the time loop of
// simulations/euler_simulation.cpp:56-68 advanced entirely on the GPU.
//
// State layout in HBM: one allocation holding two copies (ping-pong A/B) of
// the 5 prim fields, the 5 cons fields and the sound speed, each field a
// layout_left block of n0*n1*n2 values padded to 256 bytes, then the device
// scalars (SimScalars) and the totals workspace.  One step reads copy `cur`
// and writes copy `1-cur`:
//   ghost_shell  -- out ghosts: cons copied, prim = cons_to_prim(cons)
//                   (the reference runs cons_to_prim over ghosts too)
//   flux (step)  -- out interior: HLLC update + cons_to_prim + sound speed,
//                   and the max wavespeed of the new state
//   finalize_dt  -- dt of the new state, simulated time += cfl*dt
// Two steps (A->B, B->A) are captured once into a CUDA graph and replayed.
#include "euler_gb300.h"
#include "kernels.h"

#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

using namespace eulr;

namespace eulr {
// capi.cu
int sim_fail(int status, const char* msg);
}

namespace {

constexpr int kTotalsWork = 256 * 5 + 5;

size_t pad256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

int cfail(cudaError_t e, const char* what)
{
    char buf[400];
    std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return eulr::sim_fail(e == cudaErrorMemoryAllocation ? EULR_ERR_OUT_OF_MEMORY : EULR_ERR_CUDA, buf);
}

#define SIM_CUDA(call, what)            \
    do {                                \
        cudaError_t const _e = (call);  \
        if (_e != cudaSuccess) {        \
            return cfail(_e, what);     \
        }                               \
    } while (0)

#define SIM_TRY(expr)                 \
    do {                              \
        int const _s = (expr);        \
        if (_s != EULR_SUCCESS) {     \
            return _s;                \
        }                             \
    } while (0)

} // namespace

struct eulr_sim {
    int precision = EULR_PRECISION_F64;
    int device = 0;
    int sms = 0;
    Geom g{};
    double gamma = 1.4, dx[3] = {1, 1, 1}, cfl = 0.4;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void* slab = nullptr;
    double* prim[2][5] = {};
    double* cons[2][5] = {};
    double* cs[2] = {};
    SimScalars* sc = nullptr;
    double* totals = nullptr;
    int cur = 0;
    int per_sm = 1; // resident CTAs per SM of the step kernel
    bool tma = false; // stage planes by TMA (row pitch a multiple of 16 bytes)
    TmaMaps maps[2] = {}; // descriptors of copy 0 and copy 1 as step input
    bool loaded = false;
    cudaGraphExec_t graph = nullptr;
};

namespace {

int check_sim(eulr_sim* s)
{
    if (s == nullptr) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "simulation handle is NULL");
    }
    int dev = 0;
    SIM_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev != s->device) {
        SIM_CUDA(cudaSetDevice(s->device), "cudaSetDevice");
    }
    return EULR_SUCCESS;
}

long long ncell(eulr_sim const* s) { return s->g.ncell(); }

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
// (no link-time dependency on libcuda).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                    cudaSuccess &&
            q == cudaDriverEntryPointSuccess) {
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        }
    });
    return fn;
}

// 3D tensor (n0, n1, n2) of doubles, layout_left, box (TX+2, TY+2, 1).
// Requires the row pitch n0*8 to be a multiple of 16 bytes and a 16-byte
// aligned base (fields are 256-byte aligned in the simulation's allocation).
bool encode_field_map(CUtensorMap* m, double* base, Geom const& g)
{
    auto enc = tensor_map_encoder();
    if (enc == nullptr) {
        return false;
    }
    cuuint64_t dims[3] = {static_cast<cuuint64_t>(g.n0), static_cast<cuuint64_t>(g.n1),
                          static_cast<cuuint64_t>(g.n2)};
    cuuint64_t strides[2] = {static_cast<cuuint64_t>(g.s1) * sizeof(double),
                             static_cast<cuuint64_t>(g.s2) * sizeof(double)};
    cuuint32_t box[3] = {static_cast<cuuint32_t>(flux_tile_x() + 2), static_cast<cuuint32_t>(flux_tile_y() + 2), 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult const r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// TMA staging needs 16-byte row and plane pitches; the descriptors of both
// copies are built once.  On any failure the plain-load staging is used.
void setup_tma(eulr_sim* s)
{
    s->tma = false;
    if ((static_cast<size_t>(s->g.n0) * sizeof(double)) % 16 != 0) {
        return;
    }
    for (int c = 0; c < 2; ++c) {
        double* f[7] = {s->prim[c][0], s->prim[c][1], s->prim[c][2], s->prim[c][3], s->prim[c][4], s->cs[c],
                        s->cons[c][1]};
        for (int i = 0; i < 7; ++i) {
            if (!encode_field_map(&s->maps[c].m[i], f[i], s->g)) {
                return;
            }
        }
    }
    s->tma = true;
}

// One fused step from copy `in` to copy `1-in`; with `ev` (4 events) the
// launches are bracketed for per-kernel timing.
int enqueue_step(eulr_sim* s, int in, cudaEvent_t* ev = nullptr)
{
    int const out = 1 - in;
    double const ix0 = 1.0 / s->dx[0], ix1 = 1.0 / s->dx[1], ix2 = 1.0 / s->dx[2];

    GhostParams<double> gp{};
    gp.g = s->g;
    std::memcpy(gp.cons_in.f, s->cons[in], sizeof(gp.cons_in.f));
    std::memcpy(gp.cons_out.f, s->cons[out], sizeof(gp.cons_out.f));
    std::memcpy(gp.prim_out.f, s->prim[out], sizeof(gp.prim_out.f));
    gp.cs_out = s->cs[out];
    gp.gamma = s->gamma;
    gp.gm1 = s->gamma - 1.0;
    gp.invdx0 = ix0;
    gp.invdx1 = ix1;
    gp.invdx2 = ix2;
    gp.wmax = &s->sc->wmax;
    if (ev != nullptr) {
        SIM_CUDA(cudaEventRecord(ev[0], s->stream), "cudaEventRecord");
    }
    SIM_CUDA(launch_ghost_shell<double>(gp, s->sms, s->stream), "ghost shell launch");

    FluxParams<double> p{};
    p.g = s->g;
    std::memcpy(p.prim.f, s->prim[in], sizeof(p.prim.f));
    p.cs = s->cs[in];
    std::memcpy(p.cons_in.f, s->cons[in], sizeof(p.cons_in.f));
    std::memcpy(p.cons_out.f, s->cons[out], sizeof(p.cons_out.f));
    std::memcpy(p.prim_out.f, s->prim[out], sizeof(p.prim_out.f));
    p.cs_out = s->cs[out];
    p.gamma = s->gamma;
    p.gm1 = s->gamma - 1.0;
    p.inv_gm1 = 1.0 / (s->gamma - 1.0);
    p.half_gm1 = 0.5 * (s->gamma - 1.0);
    p.ds0 = s->dx[1] * s->dx[2];
    p.ds1 = s->dx[2] * s->dx[0];
    p.ds2 = s->dx[0] * s->dx[1];
    p.dv = s->dx[0] * s->dx[1] * s->dx[2];
    p.dt_dev = &s->sc->dt;
    p.cfl = s->cfl;
    p.invdx0 = ix0;
    p.invdx1 = ix1;
    p.invdx2 = ix2;
    p.wmax = &s->sc->wmax;
    p.status = &s->sc->status;
    p.per_sm = s->per_sm;
    if (ev != nullptr) {
        SIM_CUDA(cudaEventRecord(ev[1], s->stream), "cudaEventRecord");
    }
    SIM_CUDA(launch_flux<double>(p, s->tma ? &s->maps[in] : nullptr, kModeStep, s->sms, s->stream), "step launch");
    if (ev != nullptr) {
        SIM_CUDA(cudaEventRecord(ev[2], s->stream), "cudaEventRecord");
    }
    SIM_CUDA(launch_finalize_dt<double>(s->sc, s->cfl, 1, s->stream), "finalize launch");
    if (ev != nullptr) {
        SIM_CUDA(cudaEventRecord(ev[3], s->stream), "cudaEventRecord");
    }
    return EULR_SUCCESS;
}

// After a state was loaded into copy 0: sound speed, dt of the state, zeroed
// clock and status.
int prepare_loaded(eulr_sim* s)
{
    s->cur = 0;
    CBundle<double> pv;
    std::memcpy(pv.f, s->prim[0], sizeof(pv.f));
    SIM_CUDA(launch_sound_speed<double>(pv, s->cs[0], ncell(s), s->gamma, s->sms, s->stream), "sound speed launch");
    SIM_CUDA(cudaMemsetAsync(s->sc, 0, sizeof(SimScalars), s->stream), "cudaMemsetAsync");
    SIM_CUDA(launch_invdt_max<double>(pv, ncell(s), s->gamma, 1.0 / s->dx[0], 1.0 / s->dx[1], 1.0 / s->dx[2],
                                      &s->sc->wmax, s->sms, s->stream),
             "invdt launch");
    SIM_CUDA(launch_finalize_dt<double>(s->sc, s->cfl, 0, s->stream), "finalize launch");
    s->loaded = true;
    return EULR_SUCCESS;
}

template <class B>
int copy_in(eulr_sim* s, double* const* dst, B const& src)
{
    const double* f[5];
    std::memcpy(f, &src, sizeof(f));
    size_t const bytes = static_cast<size_t>(ncell(s)) * sizeof(double);
    for (int i = 0; i < 5; ++i) {
        if (f[i] == nullptr) {
            return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "state field is NULL");
        }
        SIM_CUDA(cudaMemcpyAsync(dst[i], f[i], bytes, cudaMemcpyDefault, s->stream), "cudaMemcpyAsync(in)");
    }
    return EULR_SUCCESS;
}

} // namespace

extern "C" {

int eulr_sim_create(int precision, int n0, int n1, int n2, double gamma, double dx0, double dx1, double dx2,
                    double cfl, eulr_stream_t stream, eulr_sim** out)
{
    if (out == nullptr) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "out is NULL");
    }
    *out = nullptr;
    if (precision != EULR_PRECISION_F64) {
        return eulr::sim_fail(EULR_ERR_UNSUPPORTED, "only EULR_PRECISION_F64 is available in this build");
    }
    if (n0 < 1 || n1 < 1 || n2 < 1) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "grid extents must be >= 1");
    }
    if (static_cast<long long>(n0) * n1 * n2 > 2147483647LL) {
        return eulr::sim_fail(EULR_ERR_TOO_LARGE, "grid exceeds the int index range");
    }
    if (!std::isfinite(gamma) || !(gamma > 1.0)) {
        return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "gamma must be finite and > 1");
    }
    if (!(std::isfinite(dx0) && dx0 > 0 && std::isfinite(dx1) && dx1 > 0 && std::isfinite(dx2) && dx2 > 0)) {
        return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "mesh spacings must be finite and > 0");
    }
    if (!std::isfinite(cfl) || !(cfl > 0.0)) {
        return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "cfl must be finite and > 0");
    }
    eulr_sim* s = new (std::nothrow) eulr_sim();
    if (s == nullptr) {
        return eulr::sim_fail(EULR_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    s->precision = precision;
    s->g = make_geom(n0, n1, n2);
    s->gamma = gamma;
    s->dx[0] = dx0;
    s->dx[1] = dx1;
    s->dx[2] = dx2;
    s->cfl = cfl;
    auto bail = [&](int st) {
        eulr_sim_destroy(s);
        return st;
    };
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) {
        return bail(cfail(e, "cudaGetDevice"));
    }
    e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    if (e != cudaSuccess) {
        return bail(cfail(e, "cudaDeviceGetAttribute"));
    }
    if (stream != nullptr) {
        s->stream = stream;
    } else {
        e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            return bail(cfail(e, "cudaStreamCreate"));
        }
        s->own_stream = true;
    }
    size_t const field = pad256(static_cast<size_t>(ncell(s)) * sizeof(double));
    size_t const scal = pad256(sizeof(SimScalars));
    size_t const tot = pad256(kTotalsWork * sizeof(double));
    size_t const bytes = 22 * field + scal + tot;
    e = cudaMalloc(&s->slab, bytes);
    if (e != cudaSuccess) {
        return bail(cfail(e, "cudaMalloc(simulation state)"));
    }
    char* b = static_cast<char*>(s->slab);
    for (int c = 0; c < 2; ++c) {
        for (int f = 0; f < 5; ++f) {
            s->prim[c][f] = reinterpret_cast<double*>(b);
            b += field;
        }
        for (int f = 0; f < 5; ++f) {
            s->cons[c][f] = reinterpret_cast<double*>(b);
            b += field;
        }
        s->cs[c] = reinterpret_cast<double*>(b);
        b += field;
    }
    s->sc = reinterpret_cast<SimScalars*>(b);
    b += scal;
    s->totals = reinterpret_cast<double*>(b);
    setup_tma(s);
    e = configure_flux<double>(kModeStep, s->tma, &s->per_sm);
    if (e != cudaSuccess) {
        return bail(cfail(e, "step kernel configure"));
    }
    e = cudaMemsetAsync(s->sc, 0, sizeof(SimScalars), s->stream);
    if (e != cudaSuccess) {
        return bail(cfail(e, "cudaMemsetAsync"));
    }
    *out = s;
    return EULR_SUCCESS;
}

int eulr_sim_destroy(eulr_sim* s)
{
    if (s == nullptr) {
        return EULR_SUCCESS;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != s->device) {
        cudaSetDevice(s->device);
    }
    if (s->stream != nullptr) {
        cudaStreamSynchronize(s->stream);
    }
    if (s->graph != nullptr) {
        cudaGraphExecDestroy(s->graph);
    }
    if (s->slab != nullptr) {
        cudaFree(s->slab);
    }
    if (s->own_stream && s->stream != nullptr) {
        cudaStreamDestroy(s->stream);
    }
    if (dev != s->device) {
        cudaSetDevice(dev);
    }
    delete s;
    return EULR_SUCCESS;
}

int eulr_sim_set_prim_f64(eulr_sim* s, eulr_prim_cf64 prim)
{
    SIM_TRY(check_sim(s));
    SIM_TRY(copy_in(s, s->prim[0], prim));
    CBundle<double> pv;
    Bundle<double> cv;
    std::memcpy(pv.f, s->prim[0], sizeof(pv.f));
    std::memcpy(cv.f, s->cons[0], sizeof(cv.f));
    double const gm1 = s->gamma - 1.0;
    SIM_CUDA(launch_prim_to_cons<double>(pv, cv, ncell(s), gm1, 1.0 / gm1, s->sms, s->stream), "prim_to_cons");
    return prepare_loaded(s);
}

int eulr_sim_set_state_f64(eulr_sim* s, eulr_prim_cf64 prim, eulr_cons_cf64 cons)
{
    SIM_TRY(check_sim(s));
    SIM_TRY(copy_in(s, s->prim[0], prim));
    SIM_TRY(copy_in(s, s->cons[0], cons));
    return prepare_loaded(s);
}

int eulr_sim_init_implode(eulr_sim* s)
{
    SIM_TRY(check_sim(s));
    Bundle<double> pw;
    CBundle<double> pv;
    Bundle<double> cv;
    std::memcpy(pw.f, s->prim[0], sizeof(pw.f));
    std::memcpy(pv.f, s->prim[0], sizeof(pv.f));
    std::memcpy(cv.f, s->cons[0], sizeof(cv.f));
    SIM_CUDA(launch_init_implode<double>(pw, s->g, s->dx[0], s->dx[1], s->dx[2], s->sms, s->stream), "init_implode");
    double const gm1 = s->gamma - 1.0;
    SIM_CUDA(launch_prim_to_cons<double>(pv, cv, ncell(s), gm1, 1.0 / gm1, s->sms, s->stream), "prim_to_cons");
    return prepare_loaded(s);
}

int eulr_sim_advance(eulr_sim* s, int nsteps)
{
    SIM_TRY(check_sim(s));
    if (nsteps < 0) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "nsteps must be >= 0");
    }
    if (!s->loaded) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "no state loaded");
    }
    int left = nsteps;
    if (left > 0 && s->cur == 1) {
        SIM_TRY(enqueue_step(s, 1));
        s->cur = 0;
        --left;
    }
    if (left >= 2 && s->graph == nullptr) {
        cudaGraph_t graph = nullptr;
        SIM_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        int const st0 = enqueue_step(s, 0);
        int const st1 = (st0 == EULR_SUCCESS) ? enqueue_step(s, 1) : st0;
        cudaError_t const ec = cudaStreamEndCapture(s->stream, &graph);
        if (st1 != EULR_SUCCESS) {
            if (graph != nullptr) {
                cudaGraphDestroy(graph);
            }
            return st1;
        }
        SIM_CUDA(ec, "cudaStreamEndCapture");
        cudaError_t const ei = cudaGraphInstantiate(&s->graph, graph, 0);
        cudaGraphDestroy(graph);
        SIM_CUDA(ei, "cudaGraphInstantiate");
    }
    while (left >= 2) {
        SIM_CUDA(cudaGraphLaunch(s->graph, s->stream), "cudaGraphLaunch");
        left -= 2;
    }
    if (left == 1) {
        SIM_TRY(enqueue_step(s, 0));
        s->cur = 1;
    }
    return EULR_SUCCESS;
}

int eulr_sim_get_state_f64(eulr_sim* s, eulr_prim_f64 prim, eulr_cons_f64 cons)
{
    SIM_TRY(check_sim(s));
    size_t const bytes = static_cast<size_t>(ncell(s)) * sizeof(double);
    double* pf[5];
    double* cf[5];
    std::memcpy(pf, &prim, sizeof(pf));
    std::memcpy(cf, &cons, sizeof(cf));
    for (int i = 0; i < 5; ++i) {
        if (pf[i] != nullptr) {
            SIM_CUDA(cudaMemcpyAsync(pf[i], s->prim[s->cur][i], bytes, cudaMemcpyDefault, s->stream), "copy out");
        }
        if (cf[i] != nullptr) {
            SIM_CUDA(cudaMemcpyAsync(cf[i], s->cons[s->cur][i], bytes, cudaMemcpyDefault, s->stream), "copy out");
        }
    }
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    return EULR_SUCCESS;
}

int eulr_sim_time(eulr_sim* s, double* t, double* next_dt, long long* steps)
{
    SIM_TRY(check_sim(s));
    SimScalars h{};
    SIM_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(h), cudaMemcpyDeviceToHost, s->stream), "copy scalars");
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    if (t != nullptr) {
        *t = h.t;
    }
    if (next_dt != nullptr) {
        *next_dt = s->cfl * h.dt;
    }
    if (steps != nullptr) {
        *steps = h.steps;
    }
    return EULR_SUCCESS;
}

int eulr_sim_status(eulr_sim* s)
{
    SIM_TRY(check_sim(s));
    SimScalars h{};
    SIM_CUDA(cudaMemcpyAsync(&h, s->sc, sizeof(h), cudaMemcpyDeviceToHost, s->stream), "copy scalars");
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    if (h.status != 0) {
        return eulr::sim_fail(EULR_ERR_NONFINITE, "a cell became non-finite or non-physical");
    }
    return EULR_SUCCESS;
}

int eulr_sim_launches_per_step(eulr_sim* s)
{
    (void)s;
    return 3;
}

int eulr_sim_profile_step(eulr_sim* s, float ms[3])
{
    SIM_TRY(check_sim(s));
    if (ms == nullptr) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "ms is NULL");
    }
    if (!s->loaded) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "no state loaded");
    }
    cudaEvent_t ev[4] = {};
    for (auto& e : ev) {
        SIM_CUDA(cudaEventCreate(&e), "cudaEventCreate");
    }
    int st = enqueue_step(s, s->cur, ev);
    if (st == EULR_SUCCESS) {
        s->cur = 1 - s->cur;
        cudaError_t e = cudaEventSynchronize(ev[3]);
        for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
            e = cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
        }
        if (e != cudaSuccess) {
            st = cfail(e, "event timing");
        }
    }
    for (auto& e : ev) {
        cudaEventDestroy(e);
    }
    return st;
}

int eulr_sim_totals(eulr_sim* s, double out[5])
{
    SIM_TRY(check_sim(s));
    if (out == nullptr) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "out is NULL");
    }
    CBundle<double> cv;
    std::memcpy(cv.f, s->cons[s->cur], sizeof(cv.f));
    SIM_CUDA(launch_totals(cv, s->g, s->totals, s->sms, s->stream), "totals launch");
    SIM_CUDA(cudaMemcpyAsync(out, s->totals + 256 * 5, 5 * sizeof(double), cudaMemcpyDeviceToHost, s->stream),
             "copy totals");
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    return EULR_SUCCESS;
}

} // extern "C"
