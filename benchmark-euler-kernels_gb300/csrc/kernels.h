// Host-side launch interface of the Euler kernels (internal to the library).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "euler_device.cuh"

struct eulr_sim;

namespace eulr {

constexpr int kModeGodunov = 0; // per-operator godunov: cons updated in place from prim
constexpr int kModeStep = 1;    // fused step: ping-pong buffers, next-step CFL reduction
constexpr int kModeStepCons = 2; // fused step whose state is cons only (FP32): prim rebuilt on chip

// Update arithmetic of the fused FP32 step.
constexpr int kCompNone = 0;  // plain: cons -= sum of the six face terms, FP32
constexpr int kCompSum = 1;   // compensated: one rounding at the state's scale (column engine: axis
                              // differences + TwoProduct/TwoSum; tile engine: error-free sum of six terms)
constexpr int kCompHiLo = 2;  // compensated with a stored low word: cons = hi + lo (double-float)

// Device scalars of a simulation.
struct SimScalars {
    unsigned long long wmax; // max invdt of the state being produced (ordered bits of a double)
    double dt;               // time_step() of the current state (before the CFL factor)
    double t;                // simulated time: sum of cfl*dt over the steps taken
    long long steps;         // steps taken
    int status;              // bit 0: a cell became non-finite or non-physical
    unsigned done;           // CTAs (one grid) or work items (batch) of the running step that finished;
                             // the last one finalizes the step and zeroes it
    unsigned long long ghost_wmax; // FP32 states: max invdt of the ghost layer, which never changes (set at load)
};

// TMA descriptors of the seven staged fields (d, p, u0, u1, u2, c, e) of the
// step's input copy: 3D tensors (n0, n1, n2), boxes of (TX+2) x (TY+2) x 1.
struct TmaMaps {
    CUtensorMap m[7];
};

template <class T>
struct FluxParams {
    Geom g;
    CBundle<T> prim;     // read (with halo)
    const T* cs;         // step mode: stored sound speed of prim
    CBundle<T> cons_in;  // read (centre; step mode also e with halo)
    Bundle<T> cons_out;  // written (interior); may equal cons_in in godunov mode
    Bundle<T> prim_out;  // step mode: cons_to_prim of the new state (interior)
    Bundle<T> prim_rec;  // step mode, when set: a second copy of prim_out (the adjoint's recompute)
    T* cs_out;           // step mode: sound speed of the new state (interior)
    T gamma, gm1, inv_gm1, half_gm1;
    T ds0, ds1, ds2;     // face areas dx1*dx2, dx2*dx0, dx0*dx1
    double dv;           // cell volume
    T dtodv;             // dt/dv when dt_dev is null
    const double* dt_dev; // if set: dt/dv = (cfl * *dt_dev) / dv, evaluated in double
    double cfl;
    const double* dt_seq;       // if set: step n uses dt = dt_seq[n] (a fixed sequence, CFL not applied)
    const long long* step_dev;  // the step index n (SimScalars::steps)
    CBundle<T> lo_in;    // compensated FP32 state: low words of cons (comp == 2)
    Bundle<T> lo_out;
    T invdx0, invdx1, invdx2;
    unsigned long long* wmax; // step mode: atomicMax of the next max invdt
    int* status;              // step mode: set to 1 on a non-physical cell
    int tiles_x, tiles_y, kchunk, nwork; // work decomposition (kchunk <= 0: default)
    int per_sm;                          // resident CTAs per SM (from configure_flux)
    SimScalars* fin;  // step mode, when set: the kernel finalizes the step itself (next dt, clock)
    T* h_out;         // FP64 step mode, when set: e + p of the new state (interior), the HLLC's
                      // energy-flux input, staged by TMA at the next step
    int grid_items;   // batch: work items of this grid in the current item list
};

// Launch parameters of the multi-grid batch kernel.
template <class T>
struct BatchParams {
    const FluxParams<T>* grids; // per grid, for this step's copy direction
    const int4* items;          // work items (grid, tile x, tile y, chunk), largest grids first
    int nitems;
    unsigned* head;             // work-queue head; zero before each launch
    unsigned* exited;           // CTAs that found the queue empty; the last resets head and itself
    const int* idle;            // grids without interior cells (no work item): finalized by the last CTA
    int nidle;
    long long max_cells;        // cells of the largest grid (selects 32-bit offsets where they suffice)
};

template <class T>
struct GhostParams {
    Geom g;
    CBundle<T> cons_in;
    Bundle<T> cons_out;
    CBundle<T> lo_in; // low words of cons (compensated FP32 state), copied when set
    Bundle<T> lo_out;
    int comp;         // kComp* of a cons-only FP32 state (prim_out unset)
    Bundle<T> prim_out;
    Bundle<T> prim_rec; // when set: a second copy of prim_out
    T* cs_out;
    T* h_out;           // when set (FP64 state): e + p
    T gamma, gm1;
    T invdx0, invdx1, invdx2;
    unsigned long long* wmax;
};

template <class T>
cudaError_t launch_init_implode(Bundle<T> prim, Geom g, double dx0, double dx1, double dx2, int sms, cudaStream_t s);
template <class T>
cudaError_t launch_prim_to_cons(CBundle<T> prim, Bundle<T> cons, long long n, T gm1, T rgm1, int sms, cudaStream_t s);
template <class T>
cudaError_t launch_cons_to_prim(CBundle<T> cons, Bundle<T> prim, long long n, T gm1, int sms, cudaStream_t s);
template <class T>
cudaError_t launch_time_step(CBundle<T> prim, long long n, T gamma, T ix0, T ix1, T ix2, T* partials,
                             int max_partials, unsigned int* counter, T* dt_out, int sms, cudaStream_t s);
// prim_to_cons (when cons.f[0] is set), the stored sound speed and the exact
// first max wavespeed in one pass.
template <class T>
cudaError_t launch_load_prim(CBundle<T> prim, Bundle<T> cons, T* cs, long long n, T gamma, T ix0, T ix1, T ix2,
                             unsigned long long* wmax, int sms, cudaStream_t s, T* h = nullptr,
                             const T* e_in = nullptr);
// out = a + b elementwise, rounded once (the FP64 state's e + p after a restore).
cudaError_t launch_add_fields(const double* a, const double* b, double* out, long long n, int sms, cudaStream_t s);
cudaError_t launch_init_step(Bundle<double> prim, Geom g, double dx0, double dx1, double dx2, double c,
                             double rho_in, double p_in, double rho_out, double p_out, int sms, cudaStream_t s);
// max invdt over all cells of a cons-only FP32 state (compensated: FP64
// internal energy for low-pressure cells)
cudaError_t launch_invdt_max_cons(CBundle<float> cons, long long n, float gamma, float ix0, float ix1, float ix2,
                                  int comp, unsigned long long* wmax, int sms, cudaStream_t s);

template <class T>
cudaError_t configure_flux(int mode, bool tma, int comp, int* per_sm);
// maps != nullptr selects TMA staging (step mode only); comp: kComp* (float step mode)
template <class T>
cudaError_t launch_flux(FluxParams<T> p, TmaMaps const* maps, int mode, int comp, int sms, cudaStream_t s);
// godunov bit-identical to the reference (godunov_exact.cu); cons updated in place.
template <class T>
cudaError_t launch_godunov_exact(CBundle<T> prim, Bundle<T> cons, Geom g, T gamma, T dx0, T dx1, T dx2, T dt, int sms,
                                 cudaStream_t s);
int flux_tile_x();
int flux_tile_y();

// Multi-grid batch (batch.cu): tile-shape variants of the batch kernel.
int batch_shape_count();
void batch_shape(int shape, int* tx, int* ty);
template <class T>
cudaError_t launch_flux_batch(int shape, int comp, BatchParams<T> const* b, int grid, int* per_sm, cudaStream_t s);
template <class T>
cudaError_t launch_ghost_shell(GhostParams<T> p, int sms, cudaStream_t s);
template <class T>
cudaError_t launch_finalize_dt(SimScalars* sc, T cfl, int add_time, cudaStream_t s, const double* dt_seq = nullptr);

// The FP32 step on the column engine (flux_f32.cu), comp kCompNone or kCompSum.
cudaError_t configure_step_f32col(int comp, int* per_sm);
cudaError_t launch_step_f32col(FluxParams<float> const& p, int comp, int sms, cudaStream_t s);
// b == nullptr: configure and report resident CTAs per SM; otherwise launch.
cudaError_t launch_batch_f32col(int comp, BatchParams<float> const* b, int grid, int* per_sm, cudaStream_t s);

cudaError_t launch_fma_probe(int kind, int blocks, int iters, float* sink, cudaStream_t s);
template <class T>
cudaError_t launch_totals(CBundle<T> cons, CBundle<T> lo, Geom g, double* work, cudaStream_t s);
cudaError_t launch_state_to_f32(CBundle<double> prim, CBundle<double> cons, Bundle<float> hi, Bundle<float> lo,
                                long long n, double gamma, int fp32_cons, int sms, cudaStream_t s);
cudaError_t launch_state_from_f32(CBundle<float> hi, CBundle<float> lo, Bundle<double> prim, Bundle<double> cons,
                                  long long n, double gamma, int sms, cudaStream_t s);

// Reverse mode of the time step (adjoint.cu).  Output of launch_step_adjoint
// by mode, for the state (prim, cons) a step starts from and cbar = dJ/d(cons
// the step produces):
constexpr int kAdjStep = 0;    // out = dJ/dcons: cbar + cons_to_prim'(prim)^T pbar
constexpr int kAdjInitial = 1; // out = dJ/dprim of a step that reads prim itself: pbar + prim_to_cons'(prim)^T cbar
constexpr int kAdjGodunov = 2; // out = pbar = (d godunov / d prim)^T cbar
constexpr int kAdjWorkFields = 41;

// Workspace of the reverse step: per cell and per upper face (axis a), the
// face's left half (a*5 + prim field) and its right half (15 + a*5 + prim
// field), which belongs to the neighbour c + e_a; sound speed data and
// energies; the weighted cotangent.
struct AdjWork {
    double* face[30];
    double* derived[6]; // c, dc/dp, dc/drho, total energy, kinetic energy per mass, 1/rho
    double* weight[5];  // (dt/dv) cbar on interior cells, 0 on ghosts
};

size_t adjoint_workspace_bytes(long long ncell);
AdjWork adjoint_workspace(void* base, long long ncell);
// One reverse step.  prepared: the workspace already holds this step's prep
// (a previous call's fused prep).  prev (mode kAdjStep): also prepare the
// next reverse step -- the state one step earlier, stepped with dt_prev -- in
// the gather pass.
cudaError_t launch_step_adjoint(CBundle<double> prim, CBundle<double> cbar, Bundle<double> out, int mode, Geom g,
                                double gamma, double dx0, double dx1, double dx2, double dt, AdjWork const& w, int sms,
                                cudaStream_t s, bool prepared = false, CBundle<double> const* prev = nullptr,
                                double dt_prev = 0.0);
cudaError_t launch_cons_to_prim_adjoint(CBundle<double> prim, CBundle<double> pbar, Bundle<double> cbar,
                                        int accumulate, long long n, double gamma, int sms, cudaStream_t s);
cudaError_t launch_prim_to_cons_adjoint(CBundle<double> prim, CBundle<double> cbar, Bundle<double> pbar,
                                        int accumulate, long long n, double gamma, int sms, cudaStream_t s);

// Raw state of an FP64 simulation, for the checkpointed adjoint.  The fields
// are, in order, prim (5), cons (5) and the sound speed (1) of the current
// copy.  sim_snapshot copies the first nfields of them to device memory (on
// the simulation's stream, asynchronously); sim_restore loads all 11 into the
// first copy and sets the step counter (which indexes a fixed dt sequence).
int sim_snapshot(eulr_sim* s, double* const* dst, int nfields);
// Records msg as the last error (eulr_last_error) and returns status.
int sim_fail(int status, const char* msg);
int sim_restore(eulr_sim* s, const double* const* src, long long step);
// The stream the simulation's work runs on (its own when created with NULL).
cudaStream_t sim_stream(eulr_sim* s);
// One step of a loaded FP64 simulation (as eulr_sim_advance(s, 1)) whose
// kernels also write the new prim (every cell) into dst[0..4].
int sim_advance_recording(eulr_sim* s, double* const* dst);

} // namespace eulr
