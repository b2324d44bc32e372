// Device-resident simulation (eulr_sim_*): the time loop of
// simulations/euler_simulation.cpp:56-68 advanced entirely on the GPU.
//
// State layout in HBM: one allocation holding two copies (ping-pong A/B) of
// the state, each field a layout_left block of n0*n1*n2 values padded to 256
// bytes, then the device scalars (SimScalars) and the totals workspace.  The
// FP64 state keeps prim (5 fields), cons (5) and the sound speed (1): on
// GB300 the FP64 pipe, not HBM, bounds the step, so values that cost FP64
// instructions are stored rather than recomputed.  The FP32 states keep cons
// only (plus 5 low-word fields for EULR_PRECISION_F32C_HILO): their step is
// bound by HBM, so prim and the sound speed are rebuilt on chip.  One step reads copy
// `cur` and writes copy `1-cur`, and is ONE launch of the fused step kernel:
// the HLLC update, cons_to_prim and the sound speed of the interior, the max
// wavespeed of the new state, and -- by the last CTA to finish -- the dt of
// the new state and the simulated time (+= cfl*dt, FP64).
// Ghost layers: the reference runs cons_to_prim over the ghosts every step
// (cons_to_prim.hpp:26-27) while godunov never changes their cons, so from
// the second step on every ghost prim is the round trip
// cons_to_prim(prim_to_cons(loaded prim)), the same every step.  Loading
// therefore writes copy 1's ghost layer once (cons copied, prim and sound
// speed from cons, their max wavespeed kept in ghost_wmax, which every dt
// includes); copy 0 keeps the loaded ghost prim for the first step and gets
// the round trip once, right after it.  The recording steps of the adjoint
// (a second prim output) still rebuild the output's ghost layer each step.
// Two steps (A->B, B->A) are captured once into a CUDA graph and replayed.
//
// Precisions: EULR_PRECISION_F64 (FP64 state and arithmetic),
// EULR_PRECISION_F32C (FP32 state, compensated update, FP64 only for the
// internal energy of low-pressure cells; 4-byte state words),
// EULR_PRECISION_F32C_HILO (the same with an FP32 low word per conservative
// field, a double-float state) and EULR_PRECISION_F32 (plain FP32, the
// reference's real_t = float).  The ABI stays FP64 at the boundary: FP32
// states are converted on the device when loaded and read back.
#include "euler_gb300.h"
#include "kernels.h"

#include <cudaTypedefs.h>

#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
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
    int comp = kCompNone; // FP32 update arithmetic (kComp*)
    size_t esize = 8;     // bytes per state word
    int device = 0;
    int sms = 0;
    Geom g{};
    double gamma = 1.4, dx[3] = {1, 1, 1}, cfl = 0.4;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void* slab = nullptr;
    void* prim[2][5] = {};
    void* cons[2][5] = {};
    void* lo[2][5] = {}; // compensated FP32 state with stored low words
    void* cs[2] = {};
    void* h[2] = {};     // FP64: e + p, the HLLC's energy-flux input (staged by TMA instead of e)
    SimScalars* sc = nullptr;
    double* totals = nullptr;
    int cur = 0;
    int per_sm = 1;       // resident CTAs per SM of the step kernel
    bool tma = false;     // stage planes by TMA (FP64, row pitch a multiple of 16 bytes)
    TmaMaps maps[2] = {}; // descriptors of copy 0 and copy 1 as step input
    bool loaded = false;
    cudaGraphExec_t graph = nullptr;
    double* dt_seq = nullptr;  // device copy of a fixed dt sequence (owned), or null
    long long dt_seq_len = 0;
    long long host_steps = 0;  // steps taken since the state was loaded (host-side count)
    double* rec[5] = {};       // set only inside sim_advance_recording: a second prim output
    bool ghost_fix = false;    // FP64: copy 0 still holds the loaded ghost prim; fixed after the next step
};

namespace {

bool is_f64(eulr_sim const* s) { return s->precision == EULR_PRECISION_F64; }

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

template <class T>
Bundle<T> bundle_of(void* const* f)
{
    Bundle<T> b;
    for (int i = 0; i < 5; ++i) {
        b.f[i] = static_cast<T*>(f[i]);
    }
    return b;
}

template <class T>
CBundle<T> cbundle_of(void* const* f)
{
    CBundle<T> b;
    for (int i = 0; i < 5; ++i) {
        b.f[i] = static_cast<const T*>(f[i]);
    }
    return b;
}

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
bool encode_field_map(CUtensorMap* m, void* base, Geom const& g)
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

// TMA staging (FP64 state) needs 16-byte row and plane pitches; the
// descriptors of both copies are built once.  On any failure the plain-load
// staging is used.
void setup_tma(eulr_sim* s)
{
    s->tma = false;
    if (!is_f64(s) || (static_cast<size_t>(s->g.n0) * sizeof(double)) % 16 != 0) {
        return;
    }
    for (int c = 0; c < 2; ++c) {
        void* f[7] = {s->prim[c][0], s->prim[c][1], s->prim[c][2], s->prim[c][3], s->prim[c][4], s->cs[c],
                      s->h[c]};
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
// The ghost layer of copy `in` carried to copy `out` (cons, low words, and
// for FP64 prim and sound speed), its max invdt into *wmax.
template <class T>
GhostParams<T> ghost_params(eulr_sim* s, int in, int out, unsigned long long* wmax)
{
    T const gamma = static_cast<T>(s->gamma);
    GhostParams<T> gp{};
    gp.g = s->g;
    gp.cons_in = cbundle_of<T>(s->cons[in]);
    gp.cons_out = bundle_of<T>(s->cons[out]);
    if (s->comp == kCompHiLo) {
        gp.lo_in = cbundle_of<T>(s->lo[in]);
        gp.lo_out = bundle_of<T>(s->lo[out]);
    }
    if (is_f64(s)) {
        gp.prim_out = bundle_of<T>(s->prim[out]);
        gp.cs_out = static_cast<T*>(s->cs[out]);
        gp.h_out = static_cast<T*>(s->h[out]);
        if (s->rec[0] != nullptr) {
            gp.prim_rec = bundle_of<T>(reinterpret_cast<void* const*>(s->rec));
        }
    }
    gp.comp = s->comp;
    gp.gamma = gamma;
    gp.gm1 = gamma - T(1);
    gp.invdx0 = T(1) / static_cast<T>(s->dx[0]);
    gp.invdx1 = T(1) / static_cast<T>(s->dx[1]);
    gp.invdx2 = T(1) / static_cast<T>(s->dx[2]);
    gp.wmax = wmax;
    return gp;
}

// One fused step from copy `in` to copy `1-in`: one launch of the step
// kernel, which also finalizes the step (next dt, clock).  With `ev` (4
// events) the launches are bracketed for per-kernel timing (ghost layer,
// step, finalize; the first and last are empty except when recording or on
// grids without interior cells).  Ghost layers are set at load (see the top
// of this file); recording steps rebuild the output's ghost layer, which
// writes its prim into the recording too.  A grid without interior cells
// launches no step kernel: a finalize launch takes its step.
template <class T>
int enqueue_step_t(eulr_sim* s, int in, cudaEvent_t* ev)
{
    int const out = 1 - in;
    bool const interior = s->g.n0 > 2 && s->g.n1 > 2 && s->g.n2 > 2;
    T const ix0 = T(1) / static_cast<T>(s->dx[0]);
    T const ix1 = T(1) / static_cast<T>(s->dx[1]);
    T const ix2 = T(1) / static_cast<T>(s->dx[2]);
    T const gamma = static_cast<T>(s->gamma);
    bool const has_lo = s->comp == kCompHiLo;
    if (ev != nullptr) {
        SIM_CUDA(cudaEventRecord(ev[0], s->stream), "cudaEventRecord");
    }
    if (is_f64(s) && s->rec[0] != nullptr) {
        SIM_CUDA(launch_ghost_shell<T>(ghost_params<T>(s, in, out, &s->sc->wmax), s->sms, s->stream),
                 "ghost shell launch");
    }

    FluxParams<T> p{};
    p.g = s->g;
    if (is_f64(s)) {
        p.prim = cbundle_of<T>(s->prim[in]);
        p.cs = static_cast<const T*>(s->cs[in]);
        p.prim_out = bundle_of<T>(s->prim[out]);
        p.cs_out = static_cast<T*>(s->cs[out]);
        p.h_out = static_cast<T*>(s->h[out]);
        if (s->rec[0] != nullptr) {
            p.prim_rec = bundle_of<T>(reinterpret_cast<void* const*>(s->rec));
        }
    }
    p.cons_in = cbundle_of<T>(s->cons[in]);
    p.cons_out = bundle_of<T>(s->cons[out]);
    if (has_lo) {
        p.lo_in = cbundle_of<T>(s->lo[in]);
        p.lo_out = bundle_of<T>(s->lo[out]);
    }
    p.gamma = gamma;
    p.gm1 = gamma - T(1);
    p.inv_gm1 = T(1) / (gamma - T(1));
    p.half_gm1 = T(0.5) * (gamma - T(1));
    p.ds0 = static_cast<T>(s->dx[1] * s->dx[2]);
    p.ds1 = static_cast<T>(s->dx[2] * s->dx[0]);
    p.ds2 = static_cast<T>(s->dx[0] * s->dx[1]);
    p.dv = s->dx[0] * s->dx[1] * s->dx[2];
    p.dt_dev = &s->sc->dt;
    p.cfl = s->cfl;
    p.dt_seq = s->dt_seq;
    p.step_dev = &s->sc->steps;
    p.invdx0 = ix0;
    p.invdx1 = ix1;
    p.invdx2 = ix2;
    p.wmax = &s->sc->wmax;
    p.status = &s->sc->status;
    p.per_sm = s->per_sm;
    p.fin = s->sc;
    if (ev != nullptr) {
        SIM_CUDA(cudaEventRecord(ev[1], s->stream), "cudaEventRecord");
    }
    if (interior) {
        SIM_CUDA(launch_flux<T>(p, s->tma ? &s->maps[in] : nullptr, kModeStep, s->comp, s->sms, s->stream),
                 "step launch");
    }
    if (ev != nullptr) {
        SIM_CUDA(cudaEventRecord(ev[2], s->stream), "cudaEventRecord");
    }
    if (!interior) {
        SIM_CUDA(launch_finalize_dt<T>(s->sc, static_cast<T>(s->cfl), 1, s->stream, s->dt_seq), "finalize launch");
    }
    if (ev != nullptr) {
        SIM_CUDA(cudaEventRecord(ev[3], s->stream), "cudaEventRecord");
    }
    return EULR_SUCCESS;
}

int enqueue_step(eulr_sim* s, int in, cudaEvent_t* ev = nullptr)
{
    return is_f64(s) ? enqueue_step_t<double>(s, in, ev) : enqueue_step_t<float>(s, in, ev);
}

// FP64: copy 1 gets copy 0's ghost layer with its prim and sound speed
// rebuilt from cons, and their max wavespeed goes to ghost_wmax (zero
// before).  Copy 0 keeps its ghost prim until the first step has read it.
int set_ghost_layer(eulr_sim* s)
{
    SIM_CUDA(launch_ghost_shell<double>(ghost_params<double>(s, 0, 1, &s->sc->ghost_wmax), s->sms, s->stream),
             "ghost shell launch");
    s->ghost_fix = true;
    return EULR_SUCCESS;
}

// After a step: the first step since a load has read copy 0's loaded ghost
// prim, which every later step replaces by the round trip; copy 0 takes it
// from copy 1 now (same cons, same prim, the same wavespeeds again).
int after_step(eulr_sim* s)
{
    if (s->ghost_fix) {
        int const in = s->cur;     // the copy the step wrote
        int const out = 1 - in;    // the copy it read
        GhostParams<double> q = ghost_params<double>(s, in, out, &s->sc->ghost_wmax);
        q.prim_rec = Bundle<double>{}; // a recording step has recorded its own ghost layer
        SIM_CUDA(launch_ghost_shell<double>(q, s->sms, s->stream), "ghost shell launch");
        s->ghost_fix = false;
    }
    return EULR_SUCCESS;
}

// One step launched directly (not from the graph), the copies swapped.
int step_direct(eulr_sim* s, cudaEvent_t* ev = nullptr)
{
    SIM_TRY(enqueue_step(s, s->cur, ev));
    s->cur = 1 - s->cur;
    return after_step(s);
}

// After a state was loaded into copy 0: sound speed (FP64 state), dt of the
// state, zeroed clock and status.
// Resets the clocks of copy 0 and computes its first dt.  FP64: with
// derive_cons, cons = prim_to_cons(prim) is computed in the same pass as the
// sound speed and the wavespeed (launch_load_prim); otherwise cons is taken
// as loaded.
int prepare_loaded(eulr_sim* s, bool derive_cons = false)
{
    s->cur = 0;
    s->host_steps = 0;
    SIM_CUDA(cudaMemsetAsync(s->sc, 0, sizeof(SimScalars), s->stream), "cudaMemsetAsync");
    if (is_f64(s)) {
        CBundle<double> pv = cbundle_of<double>(s->prim[0]);
        Bundle<double> cv{};
        if (derive_cons) {
            cv = bundle_of<double>(s->cons[0]);
        }
        SIM_CUDA(launch_load_prim<double>(pv, cv, static_cast<double*>(s->cs[0]), ncell(s), s->gamma, 1.0 / s->dx[0],
                                          1.0 / s->dx[1], 1.0 / s->dx[2], &s->sc->wmax, s->sms, s->stream,
                                          static_cast<double*>(s->h[0]),
                                          derive_cons ? nullptr : static_cast<const double*>(s->cons[0][1])),
                 "load launch");
        SIM_CUDA(launch_finalize_dt<double>(s->sc, s->cfl, 0, s->stream), "finalize launch");
        SIM_TRY(set_ghost_layer(s)); // after the first dt, which the loaded ghost prim sets
    } else {
        float const g = static_cast<float>(s->gamma);
        SIM_CUDA(launch_invdt_max_cons(cbundle_of<float>(s->cons[0]), ncell(s), g, 1.0f / static_cast<float>(s->dx[0]),
                                       1.0f / static_cast<float>(s->dx[1]), 1.0f / static_cast<float>(s->dx[2]),
                                       s->comp != kCompNone ? 1 : 0, &s->sc->wmax, s->sms, s->stream),
                 "invdt launch");
        SIM_CUDA(launch_finalize_dt<float>(s->sc, static_cast<float>(s->cfl), 0, s->stream), "finalize launch");
        // the ghost layer, once for every later step: copy 1 gets copy 0's ghost cons
        SIM_CUDA(launch_ghost_shell<float>(ghost_params<float>(s, 0, 1, &s->sc->ghost_wmax), s->sms, s->stream),
                 "ghost shell launch");
    }
    s->loaded = true;
    return EULR_SUCCESS;
}

// Temporary FP64 fields on the device for the FP32 states' conversions.
struct Staging {
    void* base = nullptr;
    double* f[10] = {};
    ~Staging()
    {
        if (base != nullptr) {
            cudaFree(base);
        }
    }
};

int make_staging(eulr_sim* s, Staging& st, int nfields)
{
    size_t const field = pad256(static_cast<size_t>(ncell(s)) * sizeof(double));
    SIM_CUDA(cudaMalloc(&st.base, field * nfields), "cudaMalloc(conversion staging)");
    for (int i = 0; i < nfields; ++i) {
        st.f[i] = reinterpret_cast<double*>(static_cast<char*>(st.base) + field * i);
    }
    return EULR_SUCCESS;
}

// Copy a user bundle (host or device) into device FP64 fields.
int copy_in(eulr_sim* s, void* const* dst, const double* const* src)
{
    size_t const bytes = static_cast<size_t>(ncell(s)) * sizeof(double);
    for (int i = 0; i < 5; ++i) {
        if (src[i] == nullptr) {
            return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "state field is NULL");
        }
        SIM_CUDA(cudaMemcpyAsync(dst[i], src[i], bytes, cudaMemcpyDefault, s->stream), "cudaMemcpyAsync(in)");
    }
    return EULR_SUCCESS;
}

// Load FP64 prim (and cons, or nullptr to derive it) already on the device
// into an FP32 state's copy 0.
int load_f32(eulr_sim* s, double* const* prim64, double* const* cons64)
{
    CBundle<double> pv, cv;
    for (int i = 0; i < 5; ++i) {
        pv.f[i] = prim64[i];
        cv.f[i] = cons64 != nullptr ? cons64[i] : nullptr;
    }
    Bundle<float> lo{};
    if (s->comp == kCompHiLo) {
        lo = bundle_of<float>(s->lo[0]);
    }
    SIM_CUDA(launch_state_to_f32(pv, cv, bundle_of<float>(s->cons[0]), lo, ncell(s), s->gamma,
                                 s->precision == EULR_PRECISION_F32 ? 1 : 0, s->sms, s->stream),
             "state conversion");
    return EULR_SUCCESS;
}

int set_state_impl(eulr_sim* s, const double* const* prim, const double* const* cons)
{
    if (is_f64(s)) {
        SIM_TRY(copy_in(s, s->prim[0], prim));
        if (cons != nullptr) {
            SIM_TRY(copy_in(s, s->cons[0], cons));
        }
        return prepare_loaded(s, cons == nullptr);
    }
    Staging st;
    SIM_TRY(make_staging(s, st, cons != nullptr ? 10 : 5));
    void* pd[5];
    void* cd[5];
    for (int i = 0; i < 5; ++i) {
        pd[i] = st.f[i];
        cd[i] = st.f[5 + i];
    }
    SIM_TRY(copy_in(s, pd, prim));
    if (cons != nullptr) {
        SIM_TRY(copy_in(s, cd, cons));
    }
    SIM_TRY(load_f32(s, st.f, cons != nullptr ? st.f + 5 : nullptr));
    SIM_TRY(prepare_loaded(s));
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize"); // staging is freed next
    return EULR_SUCCESS;
}

} // namespace

namespace eulr {

int sim_snapshot(eulr_sim* s, double* const* dst, int nfields)
{
    SIM_TRY(check_sim(s));
    if (!is_f64(s) || !s->loaded || nfields < 1 || nfields > 11) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "snapshot needs a loaded FP64 simulation and 1..11 fields");
    }
    size_t const bytes = static_cast<size_t>(ncell(s)) * sizeof(double);
    for (int f = 0; f < nfields; ++f) {
        void const* src = f < 5 ? s->prim[s->cur][f] : (f < 10 ? s->cons[s->cur][f - 5] : s->cs[s->cur]);
        SIM_CUDA(cudaMemcpyAsync(dst[f], src, bytes, cudaMemcpyDeviceToDevice, s->stream), "snapshot copy");
    }
    return EULR_SUCCESS;
}

cudaStream_t sim_stream(eulr_sim* s) { return s->stream; }

int sim_advance_recording(eulr_sim* s, double* const* dst)
{
    SIM_TRY(check_sim(s));
    if (!is_f64(s) || !s->loaded) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "recording needs a loaded FP64 simulation");
    }
    if (s->dt_seq != nullptr && s->host_steps + 1 > s->dt_seq_len) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "advance past the end of the fixed dt sequence");
    }
    for (int f = 0; f < 5; ++f) {
        if (dst[f] == nullptr) {
            return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "recording field is NULL");
        }
        s->rec[f] = dst[f];
    }
    int const st = step_direct(s); // launched directly: the captured graph has no second output
    for (int f = 0; f < 5; ++f) {
        s->rec[f] = nullptr;
    }
    SIM_TRY(st);
    s->host_steps += 1;
    return EULR_SUCCESS;
}

int sim_restore(eulr_sim* s, const double* const* src, long long step)
{
    SIM_TRY(check_sim(s));
    if (!is_f64(s) || step < 0) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "restore needs an FP64 simulation and a step >= 0");
    }
    size_t const bytes = static_cast<size_t>(ncell(s)) * sizeof(double);
    for (int f = 0; f < 11; ++f) {
        void* dst = f < 5 ? s->prim[0][f] : (f < 10 ? s->cons[0][f - 5] : s->cs[0]);
        SIM_CUDA(cudaMemcpyAsync(dst, src[f], bytes, cudaMemcpyDeviceToDevice, s->stream), "restore copy");
    }
    SimScalars h{};
    h.steps = step;
    SIM_CUDA(cudaMemcpyAsync(s->sc, &h, sizeof(h), cudaMemcpyHostToDevice, s->stream), "restore scalars");
    s->cur = 0;
    SIM_CUDA(launch_add_fields(static_cast<const double*>(s->cons[0][1]), static_cast<const double*>(s->prim[0][1]),
                               static_cast<double*>(s->h[0]), ncell(s), s->sms, s->stream),
             "restore e + p");
    SIM_TRY(set_ghost_layer(s));
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize"); // h is a stack value
    s->host_steps = step;
    s->loaded = true;
    return EULR_SUCCESS;
}

} // namespace eulr

extern "C" {

int eulr_sim_create(int precision, int n0, int n1, int n2, double gamma, double dx0, double dx1, double dx2,
                    double cfl, eulr_stream_t stream, eulr_sim** out)
{
    if (out == nullptr) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "out is NULL");
    }
    *out = nullptr;
    if (precision != EULR_PRECISION_F64 && precision != EULR_PRECISION_F32C && precision != EULR_PRECISION_F32 &&
        precision != EULR_PRECISION_F32C_HILO) {
        return eulr::sim_fail(EULR_ERR_UNSUPPORTED, "unknown precision");
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
    s->esize = precision == EULR_PRECISION_F64 ? sizeof(double) : sizeof(float);
    s->comp = precision == EULR_PRECISION_F32C       ? kCompSum
              : precision == EULR_PRECISION_F32C_HILO ? kCompHiLo
                                                       : kCompNone;
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
    size_t const field = pad256(static_cast<size_t>(ncell(s)) * s->esize);
    size_t const scal = pad256(sizeof(SimScalars));
    size_t const tot = pad256(kTotalsWork * sizeof(double));
    // FP64: prim + cons + sound speed + e + p per copy; FP32: cons (+ low words) only
    int const per_copy = is_f64(s) ? 12 : (s->comp == kCompHiLo ? 10 : 5);
    size_t const bytes = 2 * per_copy * field + scal + tot;
    e = cudaMalloc(&s->slab, bytes);
    if (e != cudaSuccess) {
        return bail(cfail(e, "cudaMalloc(simulation state)"));
    }
    char* b = static_cast<char*>(s->slab);
    for (int c = 0; c < 2; ++c) {
        if (is_f64(s)) {
            for (int f = 0; f < 5; ++f) {
                s->prim[c][f] = b;
                b += field;
            }
            s->cs[c] = b;
            b += field;
            s->h[c] = b;
            b += field;
        }
        for (int f = 0; f < 5; ++f) {
            s->cons[c][f] = b;
            b += field;
        }
        if (s->comp == kCompHiLo) {
            for (int f = 0; f < 5; ++f) {
                s->lo[c][f] = b;
                b += field;
            }
        }
    }
    s->sc = reinterpret_cast<SimScalars*>(b);
    b += scal;
    s->totals = reinterpret_cast<double*>(b);
    setup_tma(s);
    e = is_f64(s) ? configure_flux<double>(kModeStep, s->tma, kCompNone, &s->per_sm)
                  : configure_flux<float>(kModeStep, false, s->comp, &s->per_sm);
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
    if (s->dt_seq != nullptr) {
        cudaFree(s->dt_seq);
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
    const double* p[5] = {prim.d, prim.p, prim.ux0, prim.ux1, prim.ux2};
    return set_state_impl(s, p, nullptr);
}

int eulr_sim_set_state_f64(eulr_sim* s, eulr_prim_cf64 prim, eulr_cons_cf64 cons)
{
    SIM_TRY(check_sim(s));
    const double* p[5] = {prim.d, prim.p, prim.ux0, prim.ux1, prim.ux2};
    const double* c[5] = {cons.d, cons.e, cons.mx0, cons.mx1, cons.mx2};
    return set_state_impl(s, p, c);
}

int eulr_sim_init_implode(eulr_sim* s)
{
    SIM_TRY(check_sim(s));
    if (is_f64(s)) {
        SIM_CUDA(launch_init_implode<double>(bundle_of<double>(s->prim[0]), s->g, s->dx[0], s->dx[1], s->dx[2], s->sms,
                                             s->stream),
                 "init_implode");
        return prepare_loaded(s, true);
    }
    // FP32 states: the FP64 implosion state, converted on the device
    Staging st;
    SIM_TRY(make_staging(s, st, 5));
    Bundle<double> pw;
    for (int i = 0; i < 5; ++i) {
        pw.f[i] = st.f[i];
    }
    SIM_CUDA(launch_init_implode<double>(pw, s->g, s->dx[0], s->dx[1], s->dx[2], s->sms, s->stream), "init_implode");
    SIM_TRY(load_f32(s, st.f, nullptr));
    SIM_TRY(prepare_loaded(s));
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    return EULR_SUCCESS;
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
    if (s->dt_seq != nullptr && s->host_steps + nsteps > s->dt_seq_len) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "advance past the end of the fixed dt sequence");
    }
    s->host_steps += nsteps;
    int left = nsteps;
    if (left > 0 && s->ghost_fix) { // the first step after a load, then the ghost fix
        SIM_TRY(step_direct(s));
        --left;
    }
    if (left > 0 && s->cur == 1) {
        SIM_TRY(step_direct(s));
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
        SIM_TRY(step_direct(s));
    }
    return EULR_SUCCESS;
}

int eulr_sim_get_state_f64(eulr_sim* s, eulr_prim_f64 prim, eulr_cons_f64 cons)
{
    SIM_TRY(check_sim(s));
    size_t const bytes = static_cast<size_t>(ncell(s)) * sizeof(double);
    double* pf[5] = {prim.d, prim.p, prim.ux0, prim.ux1, prim.ux2};
    double* cf[5] = {cons.d, cons.e, cons.mx0, cons.mx1, cons.mx2};
    if (is_f64(s)) {
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
    Staging st;
    SIM_TRY(make_staging(s, st, 10));
    Bundle<double> pw, cw;
    for (int i = 0; i < 5; ++i) {
        pw.f[i] = st.f[i];
        cw.f[i] = st.f[5 + i];
    }
    CBundle<float> lo{};
    if (s->comp == kCompHiLo) {
        lo = cbundle_of<float>(s->lo[s->cur]);
    }
    SIM_CUDA(launch_state_from_f32(cbundle_of<float>(s->cons[s->cur]), lo, pw, cw, ncell(s), s->gamma, s->sms,
                                   s->stream),
             "state conversion");
    for (int i = 0; i < 5; ++i) {
        if (pf[i] != nullptr) {
            SIM_CUDA(cudaMemcpyAsync(pf[i], pw.f[i], bytes, cudaMemcpyDefault, s->stream), "copy out");
        }
        if (cf[i] != nullptr) {
            SIM_CUDA(cudaMemcpyAsync(cf[i], cw.f[i], bytes, cudaMemcpyDefault, s->stream), "copy out");
        }
    }
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize"); // staging is freed next
    return EULR_SUCCESS;
}

int eulr_sim_get_state_async_f64(eulr_sim* s, eulr_prim_f64 prim, eulr_cons_f64 cons)
{
    SIM_TRY(check_sim(s));
    if (!is_f64(s)) {
        return eulr::sim_fail(EULR_ERR_UNSUPPORTED, "asynchronous state reads need an FP64 simulation");
    }
    size_t const bytes = static_cast<size_t>(ncell(s)) * sizeof(double);
    double* pf[5] = {prim.d, prim.p, prim.ux0, prim.ux1, prim.ux2};
    double* cf[5] = {cons.d, cons.e, cons.mx0, cons.mx1, cons.mx2};
    for (int i = 0; i < 5; ++i) {
        if (pf[i] != nullptr) {
            SIM_CUDA(cudaMemcpyAsync(pf[i], s->prim[s->cur][i], bytes, cudaMemcpyDefault, s->stream), "copy out");
        }
        if (cf[i] != nullptr) {
            SIM_CUDA(cudaMemcpyAsync(cf[i], s->cons[s->cur][i], bytes, cudaMemcpyDefault, s->stream), "copy out");
        }
    }
    return EULR_SUCCESS;
}

int eulr_sim_synchronize(eulr_sim* s)
{
    SIM_TRY(check_sim(s));
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
    if (h.status & 2) {
        return eulr::sim_fail(EULR_ERR_CUDA, "a staged plane never arrived (a bounded wait ran out)");
    }
    if (h.status != 0) {
        return eulr::sim_fail(EULR_ERR_NONFINITE, "a cell became non-finite or non-physical");
    }
    return EULR_SUCCESS;
}

int eulr_sim_set_dt_sequence(eulr_sim* s, const double* dts, long long n)
{
    SIM_TRY(check_sim(s));
    if (n < 0 || (n > 0 && dts == nullptr)) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "bad dt sequence");
    }
    for (long long i = 0; i < n; ++i) {
        if (!std::isfinite(dts[i]) || !(dts[i] > 0.0)) {
            return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "dt sequence entries must be finite and > 0");
        }
    }
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    if (s->dt_seq != nullptr) {
        cudaFree(s->dt_seq);
        s->dt_seq = nullptr;
        s->dt_seq_len = 0;
    }
    if (n > 0) {
        SIM_CUDA(cudaMalloc(&s->dt_seq, sizeof(double) * n), "cudaMalloc(dt sequence)");
        SIM_CUDA(cudaMemcpy(s->dt_seq, dts, sizeof(double) * n, cudaMemcpyHostToDevice), "copy dt sequence");
        s->dt_seq_len = n;
    }
    if (s->graph != nullptr) { // the captured launches carry the old parameters
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
    return EULR_SUCCESS;
}

int eulr_sim_launches_per_step(eulr_sim* s)
{
    (void)s;
    return 1;
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
    if (s->dt_seq != nullptr && s->host_steps + 1 > s->dt_seq_len) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "advance past the end of the fixed dt sequence");
    }
    cudaEvent_t ev[4] = {};
    for (auto& e : ev) {
        SIM_CUDA(cudaEventCreate(&e), "cudaEventCreate");
    }
    int st = step_direct(s, ev);
    if (st == EULR_SUCCESS) {
        s->host_steps += 1;
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
    if (is_f64(s)) {
        SIM_CUDA(launch_totals<double>(cbundle_of<double>(s->cons[s->cur]), CBundle<double>{}, s->g, s->totals,
                                       s->stream),
                 "totals launch");
    } else {
        CBundle<float> lo{};
        if (s->comp == kCompHiLo) {
            lo = cbundle_of<float>(s->lo[s->cur]);
        }
        SIM_CUDA(launch_totals<float>(cbundle_of<float>(s->cons[s->cur]), lo, s->g, s->totals, s->stream),
                 "totals launch");
    }
    SIM_CUDA(cudaMemcpyAsync(out, s->totals + 256 * 5, 5 * sizeof(double), cudaMemcpyDeviceToHost, s->stream),
             "copy totals");
    SIM_CUDA(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    return EULR_SUCCESS;
}

int eulr_sim_state_bytes(eulr_sim* s, long long* bytes_per_step)
{
    SIM_TRY(check_sim(s));
    if (bytes_per_step == nullptr) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "bytes_per_step is NULL");
    }
    // conservative words read and written once per interior cell
    long long const words = (s->comp == kCompHiLo ? 10 : 5);
    long long const ix = s->g.n0 > 2 ? s->g.n0 - 2 : 0, iy = s->g.n1 > 2 ? s->g.n1 - 2 : 0,
                    iz = s->g.n2 > 2 ? s->g.n2 - 2 : 0;
    *bytes_per_step = 2 * words * static_cast<long long>(s->esize) * ix * iy * iz;
    return EULR_SUCCESS;
}

} // extern "C"
