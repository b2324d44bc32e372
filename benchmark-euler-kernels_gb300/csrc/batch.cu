// Multi-grid batch (eulr_batch_*): many independent grids of uneven sizes,
// each with its own gamma, mesh and dt, advanced by ONE persistent kernel
// launch per step that pulls (grid, tile, chunk) work items from a global
// queue, largest grids first.  That launch is the whole step: each grid's
// last work item computes the grid's next dt and clock, and the launch's
// last CTA rewinds the queue (and finalizes grids without interior cells).
// Ghost layers are set at load (FP64: the first copy's once more after the
// first step).  Pairs of steps are captured into a CUDA graph.  The tile shape (32x8, 16x8 or 16x16) and the chunk
// length (planes per work item) are picked by eulr_batch_autotune, which
// times every combination on the loaded state.
//
// State layout: each grid owns, inside one allocation, the same fields as a
// single simulation of its precision (FP64: prim, cons, sound speed, two
// copies; FP32 states: cons and optional low words, two copies).  The
// per-grid launch parameters of both copy directions live in device arrays
// built once at creation.
#include "euler_gb300.h"
#include "kernels.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace eulr;

namespace eulr {
int sim_fail(int status, const char* msg);
}

namespace {

size_t pad256(size_t b) { return (b + 255) & ~static_cast<size_t>(255); }

int cfail(cudaError_t e, const char* what)
{
    char buf[400];
    std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return eulr::sim_fail(e == cudaErrorMemoryAllocation ? EULR_ERR_OUT_OF_MEMORY : EULR_ERR_CUDA, buf);
}

#define B_CUDA(call, what)              \
    do {                                \
        cudaError_t const _e = (call);  \
        if (_e != cudaSuccess) {        \
            return cfail(_e, what);     \
        }                               \
    } while (0)

#define B_TRY(expr)                   \
    do {                              \
        int const _s = (expr);        \
        if (_s != EULR_SUCCESS) {     \
            return _s;                \
        }                             \
    } while (0)

struct GridState {
    Geom g{};
    double gamma = 1.4;
    double dx[3] = {1, 1, 1};
    void* prim[2][5] = {};
    void* cons[2][5] = {};
    void* lo[2][5] = {};
    void* cs[2] = {};
    bool loaded = false;
    int items = 0;          // work items of this grid in the current item list
    bool ghost_fix = false; // FP64: copy 0 still holds the loaded ghost prim; fixed after the next step
};

constexpr int kKchunks[] = {8, 16, 32, 64};

} // namespace

struct eulr_batch {
    int precision = EULR_PRECISION_F64;
    int comp = kCompNone;
    size_t esize = 8;
    int device = 0;
    int sms = 0;
    double cfl = 0.4;
    std::vector<GridState> grids;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    void* slab = nullptr;
    SimScalars* sc = nullptr;     // one per grid
    void* d_params[2] = {};       // FluxParams<T>[ngrids] per copy direction
    int4* d_items = nullptr;      // work items (capacity: the smallest tiles and chunks)
    size_t item_capacity = 0;
    int nitems = 0;
    unsigned* d_head = nullptr;
    unsigned* d_exited = nullptr; // CTAs of the running launch that found the queue empty
    int* d_idle = nullptr;        // grids without interior cells, finalized by the launch's last CTA
    int nidle = 0;
    int shape = 0;                // tile-shape variant of the batch kernel
    int kchunk = 32;
    int per_sm = 1;
    int cur = 0;
    cudaGraphExec_t graph = nullptr;
    long long interior_cells = 0;
};

namespace {

bool is_f64(eulr_batch const* b) { return b->precision == EULR_PRECISION_F64; }

int check_batch(eulr_batch* b)
{
    if (b == nullptr) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "batch handle is NULL");
    }
    int dev = 0;
    B_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev != b->device) {
        B_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    }
    return EULR_SUCCESS;
}

int check_grid(eulr_batch* b, int g)
{
    if (g < 0 || g >= static_cast<int>(b->grids.size())) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "grid index out of range");
    }
    return EULR_SUCCESS;
}

template <class T>
Bundle<T> bundle_of(void* const* f)
{
    Bundle<T> r;
    for (int i = 0; i < 5; ++i) {
        r.f[i] = static_cast<T*>(f[i]);
    }
    return r;
}

template <class T>
CBundle<T> cbundle_of(void* const* f)
{
    CBundle<T> r;
    for (int i = 0; i < 5; ++i) {
        r.f[i] = static_cast<const T*>(f[i]);
    }
    return r;
}

// Per-grid launch parameters of both copy directions, uploaded once.
template <class T>
int upload_params(eulr_batch* b)
{
    int const n = static_cast<int>(b->grids.size());
    for (int dir = 0; dir < 2; ++dir) {
        int const in = dir, out = 1 - dir;
        std::vector<FluxParams<T>> fp(n);
        for (int g = 0; g < n; ++g) {
            GridState const& G = b->grids[g];
            T const gamma = static_cast<T>(G.gamma);
            T const ix0 = T(1) / static_cast<T>(G.dx[0]);
            T const ix1 = T(1) / static_cast<T>(G.dx[1]);
            T const ix2 = T(1) / static_cast<T>(G.dx[2]);
            FluxParams<T> p{};
            p.g = G.g;
            if (is_f64(b)) {
                p.prim = cbundle_of<T>(G.prim[in]);
                p.cs = static_cast<const T*>(G.cs[in]);
                p.prim_out = bundle_of<T>(G.prim[out]);
                p.cs_out = static_cast<T*>(G.cs[out]);
            }
            p.cons_in = cbundle_of<T>(G.cons[in]);
            p.cons_out = bundle_of<T>(G.cons[out]);
            if (b->comp == kCompHiLo) {
                p.lo_in = cbundle_of<T>(G.lo[in]);
                p.lo_out = bundle_of<T>(G.lo[out]);
            }
            p.gamma = gamma;
            p.gm1 = gamma - T(1);
            p.inv_gm1 = T(1) / (gamma - T(1));
            p.half_gm1 = T(0.5) * (gamma - T(1));
            p.ds0 = static_cast<T>(G.dx[1] * G.dx[2]);
            p.ds1 = static_cast<T>(G.dx[2] * G.dx[0]);
            p.ds2 = static_cast<T>(G.dx[0] * G.dx[1]);
            p.dv = G.dx[0] * G.dx[1] * G.dx[2];
            p.dt_dev = &b->sc[g].dt;
            p.cfl = b->cfl;
            p.invdx0 = ix0;
            p.invdx1 = ix1;
            p.invdx2 = ix2;
            p.wmax = &b->sc[g].wmax;
            p.status = &b->sc[g].status;
            p.kchunk = b->kchunk;
            p.fin = &b->sc[g];
            p.grid_items = G.items;
            fp[g] = p;
        }
        B_CUDA(cudaMemcpy(b->d_params[dir], fp.data(), sizeof(FluxParams<T>) * n, cudaMemcpyHostToDevice),
               "upload batch parameters");
    }
    return EULR_SUCCESS;
}

int upload_params_any(eulr_batch* b)
{
    return is_f64(b) ? upload_params<double>(b) : upload_params<float>(b);
}

// Work items for tile shape `shape` and chunk length `kchunk`, the largest
// grids first (longest-processing-time order for the dynamic queue).
int build_items(eulr_batch* b, int shape, int kchunk)
{
    int tx = 0, ty = 0;
    batch_shape(shape, &tx, &ty);
    std::vector<int> order(b->grids.size());
    for (size_t g = 0; g < order.size(); ++g) {
        order[g] = static_cast<int>(g);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        return b->grids[a].g.ncell() > b->grids[c].g.ncell();
    });
    std::vector<int4> items;
    std::vector<int> idle;
    for (int g : order) {
        Geom const& G = b->grids[g].g;
        int const ix = G.n0 - 2, iy = G.n1 - 2, iz = G.n2 - 2;
        size_t const before = items.size();
        if (ix > 0 && iy > 0 && iz > 0) {
            int const ntx = (ix + tx - 1) / tx, nty = (iy + ty - 1) / ty, nkc = (iz + kchunk - 1) / kchunk;
            for (int kc = 0; kc < nkc; ++kc) {
                for (int y = 0; y < nty; ++y) {
                    for (int x = 0; x < ntx; ++x) {
                        items.push_back(make_int4(g, x, y, kc));
                    }
                }
            }
        }
        b->grids[g].items = static_cast<int>(items.size() - before);
        if (b->grids[g].items == 0) {
            idle.push_back(g);
        }
    }
    if (items.size() > b->item_capacity) {
        return eulr::sim_fail(EULR_ERR_TOO_LARGE, "batch work list exceeds its capacity");
    }
    b->nitems = static_cast<int>(items.size());
    if (!items.empty()) {
        B_CUDA(cudaMemcpy(b->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice),
               "upload work items");
    }
    b->nidle = static_cast<int>(idle.size());
    if (!idle.empty()) {
        B_CUDA(cudaMemcpy(b->d_idle, idle.data(), sizeof(int) * idle.size(), cudaMemcpyHostToDevice),
               "upload idle grids");
    }
    b->shape = shape;
    b->kchunk = kchunk;
    int per_sm = 1;
    B_CUDA(is_f64(b) ? launch_flux_batch<double>(shape, b->comp, nullptr, 0, &per_sm, b->stream)
                     : launch_flux_batch<float>(shape, b->comp, nullptr, 0, &per_sm, b->stream),
           "batch kernel configure");
    b->per_sm = per_sm;
    B_TRY(upload_params_any(b)); // kchunk lives in the per-grid parameters
    if (b->graph != nullptr) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return EULR_SUCCESS;
}

// One step of every grid from copy `dir` to copy `1-dir`: ONE launch of the
// persistent batch kernel.  Each grid's last work item finalizes that grid
// (its next dt and clock), the launch's last CTA finalizes the grids without
// interior cells and rewinds the queue.  Ghost layers are set at load
// (prepare_grid) and, for the FP64 state, fixed once after the first step
// (after_step).
template <class T>
int enqueue_step_t(eulr_batch* b, int dir)
{
    BatchParams<T> bp{};
    bp.grids = static_cast<FluxParams<T> const*>(b->d_params[dir]);
    bp.items = b->d_items;
    bp.nitems = b->nitems;
    bp.head = b->d_head;
    bp.exited = b->d_exited;
    bp.idle = b->d_idle;
    bp.nidle = b->nidle;
    for (auto const& gs : b->grids) {
        bp.max_cells = std::max(bp.max_cells, gs.g.ncell());
    }
    long long grid = static_cast<long long>(b->sms) * b->per_sm;
    if (grid > b->nitems) {
        grid = b->nitems > 0 ? b->nitems : 1;
    }
    B_CUDA(launch_flux_batch<T>(b->shape, b->comp, &bp, static_cast<int>(grid), nullptr, b->stream),
           "batch flux launch");
    return EULR_SUCCESS;
}

int enqueue_step(eulr_batch* b, int dir)
{
    return is_f64(b) ? enqueue_step_t<double>(b, dir) : enqueue_step_t<float>(b, dir);
}

// FP64 ghost layer of grid g from copy `in` to copy `out`: cons copied, prim
// and sound speed rebuilt from cons (the reference's cons_to_prim over the
// ghosts), their max wavespeed into the grid's ghost_wmax.
int ghost_copy(eulr_batch* b, int g, int in, int out)
{
    GridState const& G = b->grids[g];
    GhostParams<double> q{};
    q.g = G.g;
    q.cons_in = cbundle_of<double>(G.cons[in]);
    q.cons_out = bundle_of<double>(G.cons[out]);
    q.prim_out = bundle_of<double>(G.prim[out]);
    q.cs_out = static_cast<double*>(G.cs[out]);
    q.comp = kCompNone;
    q.gamma = G.gamma;
    q.gm1 = G.gamma - 1.0;
    q.invdx0 = 1.0 / G.dx[0];
    q.invdx1 = 1.0 / G.dx[1];
    q.invdx2 = 1.0 / G.dx[2];
    q.wmax = &b->sc[g].ghost_wmax;
    B_CUDA(launch_ghost_shell<double>(q, b->sms, b->stream), "ghost shell");
    return EULR_SUCCESS;
}

// After a step from copy `dir`: grids loaded since the previous step read
// their loaded ghost prim in it; every later step reads the round trip, which
// copy `dir` now takes from the copy the step wrote.
int after_step(eulr_batch* b, int dir)
{
    for (int g = 0; g < static_cast<int>(b->grids.size()); ++g) {
        if (b->grids[g].ghost_fix) {
            B_TRY(ghost_copy(b, g, 1 - dir, dir));
            b->grids[g].ghost_fix = false;
        }
    }
    return EULR_SUCCESS;
}

bool ghost_fix_pending(eulr_batch const* b)
{
    for (GridState const& G : b->grids) {
        if (G.ghost_fix) {
            return true;
        }
    }
    return false;
}

// One step launched directly (not from the graph), the copies swapped.
int step_direct(eulr_batch* b)
{
    int const dir = b->cur;
    B_TRY(enqueue_step(b, dir));
    b->cur = 1 - dir;
    return after_step(b, dir);
}

// dt of grid g's loaded state (copy 0), its clock and status zeroed.
int prepare_grid(eulr_batch* b, int g)
{
    GridState& G = b->grids[g];
    long long const n = G.g.ncell();
    B_CUDA(cudaMemsetAsync(&b->sc[g], 0, sizeof(SimScalars), b->stream), "cudaMemsetAsync");
    if (is_f64(b)) {
        // sound speed and first wavespeed as a loaded simulation computes them
        B_CUDA(launch_load_prim<double>(cbundle_of<double>(G.prim[0]), Bundle<double>{}, static_cast<double*>(G.cs[0]),
                                        n, G.gamma, 1.0 / G.dx[0], 1.0 / G.dx[1], 1.0 / G.dx[2], &b->sc[g].wmax,
                                        b->sms, b->stream),
               "load");
        B_CUDA(launch_finalize_dt<double>(&b->sc[g], b->cfl, 0, b->stream), "finalize");
        // copy 1's ghost layer once (after the first dt, which the loaded
        // ghost prim sets); copy 0's follows after the first step
        B_TRY(ghost_copy(b, g, 0, 1));
        G.ghost_fix = true;
    } else {
        float const gm = static_cast<float>(G.gamma);
        B_CUDA(launch_invdt_max_cons(cbundle_of<float>(G.cons[0]), n, gm, 1.0f / static_cast<float>(G.dx[0]),
                                     1.0f / static_cast<float>(G.dx[1]), 1.0f / static_cast<float>(G.dx[2]),
                                     b->comp != kCompNone ? 1 : 0, &b->sc[g].wmax, b->sms, b->stream),
               "invdt");
        B_CUDA(launch_finalize_dt<float>(&b->sc[g], static_cast<float>(b->cfl), 0, b->stream), "finalize");
        // the ghost layer never changes: copy 1 gets copy 0's ghost cons once, and its
        // max invdt is kept for every later step
        GhostParams<float> q{};
        q.g = G.g;
        q.cons_in = cbundle_of<float>(G.cons[0]);
        q.cons_out = bundle_of<float>(G.cons[1]);
        if (b->comp == kCompHiLo) {
            q.lo_in = cbundle_of<float>(G.lo[0]);
            q.lo_out = bundle_of<float>(G.lo[1]);
        }
        q.comp = b->comp;
        q.gamma = gm;
        q.gm1 = gm - 1.0f;
        q.invdx0 = 1.0f / static_cast<float>(G.dx[0]);
        q.invdx1 = 1.0f / static_cast<float>(G.dx[1]);
        q.invdx2 = 1.0f / static_cast<float>(G.dx[2]);
        q.wmax = &b->sc[g].ghost_wmax;
        B_CUDA(launch_ghost_shell<float>(q, b->sms, b->stream), "ghost shell");
    }
    G.loaded = true;
    return EULR_SUCCESS;
}

// Loads FP64 prim (device pointers) into grid g's copy 0.
int load_grid(eulr_batch* b, int g, double* const* prim64)
{
    GridState& G = b->grids[g];
    long long const n = G.g.ncell();
    if (is_f64(b)) {
        for (int f = 0; f < 5; ++f) {
            B_CUDA(cudaMemcpyAsync(G.prim[0][f], prim64[f], n * sizeof(double), cudaMemcpyDefault, b->stream),
                   "copy in");
        }
        double const gm1 = G.gamma - 1.0;
        B_CUDA(launch_prim_to_cons<double>(cbundle_of<double>(G.prim[0]), bundle_of<double>(G.cons[0]), n, gm1,
                                           1.0 / gm1, b->sms, b->stream),
               "prim_to_cons");
    } else {
        CBundle<double> pv, cv{};
        for (int f = 0; f < 5; ++f) {
            pv.f[f] = prim64[f];
        }
        Bundle<float> lo{};
        if (b->comp == kCompHiLo) {
            lo = bundle_of<float>(G.lo[0]);
        }
        B_CUDA(launch_state_to_f32(pv, cv, bundle_of<float>(G.cons[0]), lo, n, G.gamma,
                                   b->precision == EULR_PRECISION_F32 ? 1 : 0, b->sms, b->stream),
               "state conversion");
    }
    return prepare_grid(b, g);
}

// Temporary FP64 fields for one grid's conversions.
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

int make_staging(long long ncell, Staging& st, int nfields)
{
    size_t const field = pad256(static_cast<size_t>(ncell) * sizeof(double));
    B_CUDA(cudaMalloc(&st.base, field * nfields), "cudaMalloc(conversion staging)");
    for (int i = 0; i < nfields; ++i) {
        st.f[i] = reinterpret_cast<double*>(static_cast<char*>(st.base) + field * i);
    }
    return EULR_SUCCESS;
}

int check_loadable(eulr_batch* b)
{
    if (b->cur != 0) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT,
                              "grids can be loaded only while the batch state is in its first copy (before any "
                              "step, or after an even number of steps)");
    }
    return EULR_SUCCESS;
}

} // namespace

extern "C" {

int eulr_batch_create(int precision, int ngrids, const eulr_grid_desc* grids, double cfl, eulr_stream_t stream,
                      eulr_batch** out)
{
    if (out == nullptr || grids == nullptr || ngrids < 1) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "eulr_batch_create: bad arguments");
    }
    *out = nullptr;
    if (precision != EULR_PRECISION_F64 && precision != EULR_PRECISION_F32C && precision != EULR_PRECISION_F32 &&
        precision != EULR_PRECISION_F32C_HILO) {
        return eulr::sim_fail(EULR_ERR_UNSUPPORTED, "unknown precision");
    }
    if (!std::isfinite(cfl) || !(cfl > 0.0)) {
        return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "cfl must be finite and > 0");
    }
    for (int g = 0; g < ngrids; ++g) {
        eulr_grid_desc const& d = grids[g];
        if (d.n0 < 1 || d.n1 < 1 || d.n2 < 1 || static_cast<long long>(d.n0) * d.n1 * d.n2 > 2147483647LL) {
            return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "grid extents out of range");
        }
        if (!std::isfinite(d.gamma) || !(d.gamma > 1.0)) {
            return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "gamma must be finite and > 1");
        }
        if (!(std::isfinite(d.dx0) && d.dx0 > 0 && std::isfinite(d.dx1) && d.dx1 > 0 && std::isfinite(d.dx2) &&
              d.dx2 > 0)) {
            return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "mesh spacings must be finite and > 0");
        }
    }
    eulr_batch* b = new (std::nothrow) eulr_batch();
    if (b == nullptr) {
        return eulr::sim_fail(EULR_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    auto bail = [&](int st) {
        eulr_batch_destroy(b);
        return st;
    };
    b->precision = precision;
    b->esize = precision == EULR_PRECISION_F64 ? sizeof(double) : sizeof(float);
    b->comp = precision == EULR_PRECISION_F32C       ? kCompSum
              : precision == EULR_PRECISION_F32C_HILO ? kCompHiLo
                                                       : kCompNone;
    b->cfl = cfl;
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) {
        e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    }
    if (e != cudaSuccess) {
        return bail(cfail(e, "device query"));
    }
    if (stream != nullptr) {
        b->stream = stream;
    } else {
        e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            return bail(cfail(e, "cudaStreamCreate"));
        }
        b->own_stream = true;
    }
    b->grids.resize(ngrids);
    int const per_copy = is_f64(b) ? 11 : (b->comp == kCompHiLo ? 10 : 5);
    size_t bytes = 0;
    size_t max_items = 0;
    for (int g = 0; g < ngrids; ++g) {
        eulr_grid_desc const& d = grids[g];
        GridState& G = b->grids[g];
        G.g = make_geom(d.n0, d.n1, d.n2);
        G.gamma = d.gamma;
        G.dx[0] = d.dx0;
        G.dx[1] = d.dx1;
        G.dx[2] = d.dx2;
        bytes += 2 * per_copy * pad256(static_cast<size_t>(G.g.ncell()) * b->esize);
        long long const ix = std::max(d.n0 - 2, 0), iy = std::max(d.n1 - 2, 0), iz = std::max(d.n2 - 2, 0);
        b->interior_cells += ix * iy * iz;
        // the most items any shape/chunk choice makes (8-wide tiles bound it)
        max_items += static_cast<size_t>((ix + 15) / 16) * ((iy + 7) / 8) * ((iz + 7) / 8);
    }
    b->item_capacity = max_items;
    size_t const scal = pad256(sizeof(SimScalars) * ngrids);
    size_t const pbytes = pad256(std::max(sizeof(FluxParams<double>), sizeof(FluxParams<float>)) * ngrids);
    size_t const ibytes = pad256(sizeof(int4) * std::max<size_t>(max_items, 1));
    size_t const idle_bytes = pad256(sizeof(int) * static_cast<size_t>(ngrids));
    size_t const total = bytes + scal + 2 * pbytes + ibytes + idle_bytes + 256;
    e = cudaMalloc(&b->slab, total);
    if (e != cudaSuccess) {
        return bail(cfail(e, "cudaMalloc(batch state)"));
    }
    char* p = static_cast<char*>(b->slab);
    for (GridState& G : b->grids) {
        size_t const field = pad256(static_cast<size_t>(G.g.ncell()) * b->esize);
        for (int c = 0; c < 2; ++c) {
            if (is_f64(b)) {
                for (int f = 0; f < 5; ++f) {
                    G.prim[c][f] = p;
                    p += field;
                }
                G.cs[c] = p;
                p += field;
            }
            for (int f = 0; f < 5; ++f) {
                G.cons[c][f] = p;
                p += field;
            }
            if (b->comp == kCompHiLo) {
                for (int f = 0; f < 5; ++f) {
                    G.lo[c][f] = p;
                    p += field;
                }
            }
        }
    }
    b->sc = reinterpret_cast<SimScalars*>(p);
    p += scal;
    for (int dir = 0; dir < 2; ++dir) {
        b->d_params[dir] = p;
        p += pbytes;
    }
    b->d_items = reinterpret_cast<int4*>(p);
    p += ibytes;
    b->d_idle = reinterpret_cast<int*>(p);
    p += idle_bytes;
    b->d_head = reinterpret_cast<unsigned*>(p);
    b->d_exited = b->d_head + 1;
    e = cudaMemset(b->sc, 0, scal);
    if (e == cudaSuccess) {
        e = cudaMemset(b->d_head, 0, 2 * sizeof(unsigned));
    }
    if (e != cudaSuccess) {
        return bail(cfail(e, "cudaMemset"));
    }
    int const st = build_items(b, 0, 32);
    if (st != EULR_SUCCESS) {
        return bail(st);
    }
    *out = b;
    return EULR_SUCCESS;
}

int eulr_batch_destroy(eulr_batch* b)
{
    if (b == nullptr) {
        return EULR_SUCCESS;
    }
    if (b->stream != nullptr) {
        cudaStreamSynchronize(b->stream);
    }
    if (b->graph != nullptr) {
        cudaGraphExecDestroy(b->graph);
    }
    if (b->slab != nullptr) {
        cudaFree(b->slab);
    }
    if (b->own_stream && b->stream != nullptr) {
        cudaStreamDestroy(b->stream);
    }
    delete b;
    return EULR_SUCCESS;
}

int eulr_batch_set_prim_f64(eulr_batch* b, int grid, eulr_prim_cf64 prim)
{
    B_TRY(check_batch(b));
    B_TRY(check_grid(b, grid));
    B_TRY(check_loadable(b));
    const double* src[5] = {prim.d, prim.p, prim.ux0, prim.ux1, prim.ux2};
    for (auto const* f : src) {
        if (f == nullptr) {
            return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "prim field is NULL");
        }
    }
    long long const n = b->grids[grid].g.ncell();
    Staging st;
    B_TRY(make_staging(n, st, 5));
    for (int f = 0; f < 5; ++f) {
        B_CUDA(cudaMemcpyAsync(st.f[f], src[f], n * sizeof(double), cudaMemcpyDefault, b->stream), "copy in");
    }
    B_TRY(load_grid(b, grid, st.f));
    B_CUDA(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    return EULR_SUCCESS;
}

int eulr_batch_init_step(eulr_batch* b, int grid, double c, double rho_in, double p_in, double rho_out, double p_out)
{
    B_TRY(check_batch(b));
    B_TRY(check_grid(b, grid));
    B_TRY(check_loadable(b));
    if (!(rho_in > 0 && p_in > 0 && rho_out > 0 && p_out > 0) || !std::isfinite(c)) {
        return eulr::sim_fail(EULR_ERR_INVALID_VALUE, "densities and pressures must be > 0, c finite");
    }
    GridState& G = b->grids[grid];
    Staging st;
    B_TRY(make_staging(G.g.ncell(), st, 5));
    Bundle<double> pw;
    for (int f = 0; f < 5; ++f) {
        pw.f[f] = st.f[f];
    }
    B_CUDA(launch_init_step(pw, G.g, G.dx[0], G.dx[1], G.dx[2], c, rho_in, p_in, rho_out, p_out, b->sms, b->stream),
           "init_step");
    B_TRY(load_grid(b, grid, st.f));
    B_CUDA(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    return EULR_SUCCESS;
}

int eulr_batch_autotune(eulr_batch* b, int trial_steps, int* shape_out, int* kchunk_out, double* best_ms)
{
    B_TRY(check_batch(b));
    B_TRY(check_loadable(b));
    for (GridState const& G : b->grids) {
        if (!G.loaded) {
            return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "load every grid before autotuning");
        }
    }
    if (trial_steps < 1) {
        trial_steps = 1;
    }
    cudaEvent_t e0, e1;
    B_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
    B_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
    float best = 1e30f;
    int best_shape = 0, best_kc = 32;
    int st = EULR_SUCCESS;
    for (int shape = 0; shape < batch_shape_count() && st == EULR_SUCCESS; ++shape) {
        for (int kc : kKchunks) {
            st = build_items(b, shape, kc);
            if (st != EULR_SUCCESS) {
                break;
            }
            // every trial is the step copy 0 -> copy 1; copy 0 is never written
            st = enqueue_step(b, 0); // warm-up
            float ms_min = 1e30f;
            for (int t = 0; t < trial_steps && st == EULR_SUCCESS; ++t) {
                cudaEventRecord(e0, b->stream);
                st = enqueue_step(b, 0);
                cudaEventRecord(e1, b->stream);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                ms_min = std::min(ms_min, ms);
            }
            if (ms_min < best) {
                best = ms_min;
                best_shape = shape;
                best_kc = kc;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B_TRY(st);
    B_TRY(build_items(b, best_shape, best_kc));
    // the trials advanced the clocks and dt: restore them from copy 0
    for (int g = 0; g < static_cast<int>(b->grids.size()); ++g) {
        B_TRY(prepare_grid(b, g));
    }
    B_CUDA(cudaMemsetAsync(b->d_head, 0, 2 * sizeof(unsigned), b->stream), "cudaMemsetAsync"); // head, exited
    B_CUDA(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    if (shape_out != nullptr) {
        int tx = 0, ty = 0;
        batch_shape(best_shape, &tx, &ty);
        *shape_out = tx * 1000 + ty;
    }
    if (kchunk_out != nullptr) {
        *kchunk_out = best_kc;
    }
    if (best_ms != nullptr) {
        *best_ms = best;
    }
    return EULR_SUCCESS;
}

int eulr_batch_advance(eulr_batch* b, int nsteps)
{
    B_TRY(check_batch(b));
    if (nsteps < 0) {
        return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "nsteps must be >= 0");
    }
    for (GridState const& G : b->grids) {
        if (!G.loaded) {
            return eulr::sim_fail(EULR_ERR_INVALID_ARGUMENT, "load every grid before advancing");
        }
    }
    int left = nsteps;
    if (left > 0 && ghost_fix_pending(b)) { // the first step after a load, then the ghost fix
        B_TRY(step_direct(b));
        --left;
    }
    if (left > 0 && b->cur == 1) {
        B_TRY(step_direct(b));
        --left;
    }
    if (left >= 2 && b->graph == nullptr) {
        cudaGraph_t graph = nullptr;
        B_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        int const s0 = enqueue_step(b, 0);
        int const s1 = (s0 == EULR_SUCCESS) ? enqueue_step(b, 1) : s0;
        cudaError_t const ec = cudaStreamEndCapture(b->stream, &graph);
        if (s1 != EULR_SUCCESS) {
            if (graph != nullptr) {
                cudaGraphDestroy(graph);
            }
            return s1;
        }
        B_CUDA(ec, "cudaStreamEndCapture");
        cudaError_t const ei = cudaGraphInstantiate(&b->graph, graph, 0);
        cudaGraphDestroy(graph);
        B_CUDA(ei, "cudaGraphInstantiate");
    }
    while (left >= 2) {
        B_CUDA(cudaGraphLaunch(b->graph, b->stream), "cudaGraphLaunch");
        left -= 2;
    }
    if (left == 1) {
        B_TRY(step_direct(b));
    }
    return EULR_SUCCESS;
}

int eulr_batch_get_state_f64(eulr_batch* b, int grid, eulr_prim_f64 prim, eulr_cons_f64 cons)
{
    B_TRY(check_batch(b));
    B_TRY(check_grid(b, grid));
    GridState& G = b->grids[grid];
    long long const n = G.g.ncell();
    size_t const bytes = static_cast<size_t>(n) * sizeof(double);
    double* pf[5] = {prim.d, prim.p, prim.ux0, prim.ux1, prim.ux2};
    double* cf[5] = {cons.d, cons.e, cons.mx0, cons.mx1, cons.mx2};
    if (is_f64(b)) {
        for (int i = 0; i < 5; ++i) {
            if (pf[i] != nullptr) {
                B_CUDA(cudaMemcpyAsync(pf[i], G.prim[b->cur][i], bytes, cudaMemcpyDefault, b->stream), "copy out");
            }
            if (cf[i] != nullptr) {
                B_CUDA(cudaMemcpyAsync(cf[i], G.cons[b->cur][i], bytes, cudaMemcpyDefault, b->stream), "copy out");
            }
        }
        B_CUDA(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
        return EULR_SUCCESS;
    }
    Staging st;
    B_TRY(make_staging(n, st, 10));
    Bundle<double> pw, cw;
    for (int i = 0; i < 5; ++i) {
        pw.f[i] = st.f[i];
        cw.f[i] = st.f[5 + i];
    }
    CBundle<float> lo{};
    if (b->comp == kCompHiLo) {
        lo = cbundle_of<float>(G.lo[b->cur]);
    }
    B_CUDA(launch_state_from_f32(cbundle_of<float>(G.cons[b->cur]), lo, pw, cw, n, G.gamma, b->sms, b->stream),
           "state conversion");
    for (int i = 0; i < 5; ++i) {
        if (pf[i] != nullptr) {
            B_CUDA(cudaMemcpyAsync(pf[i], pw.f[i], bytes, cudaMemcpyDefault, b->stream), "copy out");
        }
        if (cf[i] != nullptr) {
            B_CUDA(cudaMemcpyAsync(cf[i], cw.f[i], bytes, cudaMemcpyDefault, b->stream), "copy out");
        }
    }
    B_CUDA(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    return EULR_SUCCESS;
}

int eulr_batch_time(eulr_batch* b, int grid, double* t, double* next_dt, long long* steps)
{
    B_TRY(check_batch(b));
    B_TRY(check_grid(b, grid));
    SimScalars h{};
    B_CUDA(cudaMemcpyAsync(&h, &b->sc[grid], sizeof(h), cudaMemcpyDeviceToHost, b->stream), "copy scalars");
    B_CUDA(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    if (t != nullptr) {
        *t = h.t;
    }
    if (next_dt != nullptr) {
        *next_dt = b->cfl * h.dt;
    }
    if (steps != nullptr) {
        *steps = h.steps;
    }
    return EULR_SUCCESS;
}

int eulr_batch_status(eulr_batch* b)
{
    B_TRY(check_batch(b));
    std::vector<SimScalars> h(b->grids.size());
    B_CUDA(cudaMemcpyAsync(h.data(), b->sc, sizeof(SimScalars) * h.size(), cudaMemcpyDeviceToHost, b->stream),
           "copy scalars");
    B_CUDA(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    for (size_t g = 0; g < h.size(); ++g) {
        if (h[g].status != 0) {
            char msg[128];
            std::snprintf(msg, sizeof(msg), "grid %zu became non-finite or non-physical", g);
            return eulr::sim_fail(EULR_ERR_NONFINITE, msg);
        }
    }
    return EULR_SUCCESS;
}

int eulr_batch_info(eulr_batch* b, long long* interior_cells, int* nitems, int* tile_shape, int* kchunk)
{
    B_TRY(check_batch(b));
    if (interior_cells != nullptr) {
        *interior_cells = b->interior_cells;
    }
    if (nitems != nullptr) {
        *nitems = b->nitems;
    }
    if (tile_shape != nullptr) {
        int tx = 0, ty = 0;
        batch_shape(b->shape, &tx, &ty);
        *tile_shape = tx * 1000 + ty;
    }
    if (kchunk != nullptr) {
        *kchunk = b->kchunk;
    }
    return EULR_SUCCESS;
}

} // extern "C"
