/*
 * euler_gb300 -- C ABI of the GB300 (sm_103a) first-order Godunov/HLLC step
 * for 3D compressible Euler.
 *
 * Every entry point takes plain device pointers and sizes, is asynchronous on
 * the given CUDA stream unless stated otherwise, and returns EULR_SUCCESS (0)
 * or a negative eulr_status code.  Nothing throws across this boundary.
 *
 * Data layout (the reference's, euler_operators/euler_arrays.hpp:77-85 and
 * :228-236, simulations/euler_simulation.cpp:37-48): structure of arrays, one
 * array per field, each a layout_left block (i fastest) of n0*n1*n2 cells,
 * cell (i,j,k) at offset i + n0*(j + n1*k).  Grids carry one ghost layer on
 * every face, so the interior is [1, n-1) along each axis.
 *   prim fields: d (density), p (pressure), ux0, ux1, ux2 (velocity)
 *   cons fields: d (density), e (total energy), mx0, mx1, mx2 (momentum)
 * Field arrays must be 8-byte (double) / 4-byte (float) aligned device
 * memory.  Sizes: n0, n1, n2 >= 1 and n0*n1*n2 < 2^31 (the reference indexes
 * with int, benchmarks/index_type.hpp:4).
 */
#ifndef EULER_GB300_H
#define EULER_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t; NULL is the legacy default stream. */
typedef struct CUstream_st* eulr_stream_t;

typedef enum eulr_status {
    EULR_SUCCESS = 0,
    EULR_ERR_INVALID_ARGUMENT = -1, /* null pointer, bad size or aliasing */
    EULR_ERR_INVALID_VALUE = -2,    /* gamma <= 1, dx <= 0, cfl <= 0, non-finite scalar */
    EULR_ERR_MISALIGNED = -3,       /* field pointer not aligned to its element size */
    EULR_ERR_CUDA = -4,             /* a CUDA runtime call failed (see eulr_last_error) */
    EULR_ERR_OUT_OF_MEMORY = -5,
    EULR_ERR_TOO_LARGE = -6,        /* size beyond the supported maximum */
    EULR_ERR_NONFINITE = -7,        /* the state became non-finite or non-physical */
    EULR_ERR_NO_DEVICE = -8,
    EULR_ERR_UNSUPPORTED = -9
} eulr_status;

/* Primitive-variable bundle (reference EulerPrimArrays, euler_arrays.hpp:77-85). */
typedef struct eulr_prim_f64 {
    double* d;
    double* p;
    double* ux0;
    double* ux1;
    double* ux2;
} eulr_prim_f64;

/* Conservative-variable bundle (reference EulerConsArrays, euler_arrays.hpp:228-236). */
typedef struct eulr_cons_f64 {
    double* d;
    double* e;
    double* mx0;
    double* mx1;
    double* mx2;
} eulr_cons_f64;

/* Read-only views (the reference's as_const, euler_arrays.hpp:98-104, 238-255). */
typedef struct eulr_prim_cf64 {
    const double* d;
    const double* p;
    const double* ux0;
    const double* ux1;
    const double* ux2;
} eulr_prim_cf64;

typedef struct eulr_cons_cf64 {
    const double* d;
    const double* e;
    const double* mx0;
    const double* mx1;
    const double* mx2;
} eulr_cons_cf64;

/* real_t = float bundles (benchmarks/real_type.hpp:3). */
typedef struct eulr_prim_f32 {
    float* d;
    float* p;
    float* ux0;
    float* ux1;
    float* ux2;
} eulr_prim_f32;

typedef struct eulr_cons_f32 {
    float* d;
    float* e;
    float* mx0;
    float* mx1;
    float* mx2;
} eulr_cons_f32;

typedef struct eulr_prim_cf32 {
    const float* d;
    const float* p;
    const float* ux0;
    const float* ux1;
    const float* ux2;
} eulr_prim_cf32;

typedef struct eulr_cons_cf32 {
    const float* d;
    const float* e;
    const float* mx0;
    const float* mx1;
    const float* mx2;
} eulr_cons_cf32;

/* ---------------------------------------------------------------- library */

/* Library version as major*10000 + minor*100 + patch. */
int eulr_version(void);

/* Human-readable name of a status code (static storage). */
const char* eulr_status_string(int status);

/* Message of the last error raised on the calling thread (thread-local
 * storage; empty string when none). */
const char* eulr_last_error(void);

/* ------------------------------------------------- per-operator entry points
 * Drop-in replacements of the reference operators, with the reference's
 * argument meaning.  Each launches on `stream` and returns without waiting. */

/* init_implode (euler_operators/init_implode.hpp:7-45): sphere of radius 0.25
 * centred on (0.5,0.5,0.5), cell centres ((i-1)+0.5)*dx - 0.5 (ghosts
 * included); rho=1, p=1 inside, rho=0.125, p=0.14 outside, u=0.
 * Bit-identical to the reference. */
int eulr_init_implode_f64(eulr_prim_f64 prim, int n0, int n1, int n2, double dx0, double dx1, double dx2,
                          eulr_stream_t stream);
int eulr_init_implode_f32(eulr_prim_f32 prim, int n0, int n1, int n2, float dx0, float dx1, float dx2,
                          eulr_stream_t stream);

/* prim_to_cons (euler_operators/prim_to_cons.hpp:7-33) over all cells.
 * Bit-identical to the reference. */
int eulr_prim_to_cons_f64(eulr_prim_cf64 prim, eulr_cons_f64 cons, int n0, int n1, int n2, double gamma,
                          eulr_stream_t stream);
int eulr_prim_to_cons_f32(eulr_prim_cf32 prim, eulr_cons_f32 cons, int n0, int n1, int n2, float gamma,
                          eulr_stream_t stream);

/* cons_to_prim (euler_operators/cons_to_prim.hpp:7-33) over all cells,
 * ghosts included.  Bit-identical to the reference. */
int eulr_cons_to_prim_f64(eulr_cons_cf64 cons, eulr_prim_f64 prim, int n0, int n1, int n2, double gamma,
                          eulr_stream_t stream);
int eulr_cons_to_prim_f32(eulr_cons_cf32 cons, eulr_prim_f32 prim, int n0, int n1, int n2, float gamma,
                          eulr_stream_t stream);

/* time_step (euler_operators/time_step.hpp:8-41): min over all cells of
 * 1 / sum_d (c + |u_d|) / dx_d, written to the DEVICE scalar *dt_out (the
 * CFL factor is applied by the caller, as in the reference).  The result is
 * bit-identical to the reference.  Uses a per-device scratch buffer that the
 * library allocates with cudaMalloc on the first call on each device and
 * keeps until exit; calls on the same device and different streams must not
 * overlap. */
int eulr_time_step_f64(eulr_prim_cf64 prim, int n0, int n1, int n2, double gamma, double dx0, double dx1,
                       double dx2, double* dt_out, eulr_stream_t stream);
int eulr_time_step_f32(eulr_prim_cf32 prim, int n0, int n1, int n2, float gamma, float dx0, float dx1,
                       float dx2, float* dt_out, eulr_stream_t stream);

/* eulr_time_step_f64 for callers that cannot allocate device memory -- code
 * whose device memory is owned by a pool or arena that forbids hidden
 * allocations, or that must know the library's full device footprint up
 * front.  No counterpart in the reference (its time_step allocates nothing
 * itself because Kokkos manages the reduction).  Same arguments and same
 * bit-identical result as eulr_time_step_f64; it calls no cudaMalloc/cudaFree
 * and no allocating routine.  Its scratch is a fixed ~8 KiB array inside the
 * library's device image (1024 block maxima and a counter), held by every
 * GPU that loads the library until exit; every grid below 2^31 cells fits,
 * larger ones return EULR_ERR_TOO_LARGE.  The first call on each device
 * looks up the array's address (cudaGetSymbolAddress) and should come before
 * any stream capture on that device.  All calls on a device share the array:
 * calls whose kernels can overlap on the GPU (e.g. unordered streams) race
 * and must not be issued. */
int eulr_time_step_noalloc_f64(eulr_prim_cf64 prim, int n0, int n1, int n2, double gamma, double dx0, double dx1,
                               double dx2, double* dt_out, eulr_stream_t stream);

/* godunov (euler_operators/godunov.hpp:15-92): for interior cells,
 * cons -= dt/dv * sum_d ds_d (F_{d,R} - F_{d,L}) with HLLC fluxes
 * (euler_operators/hllc.hpp:50-105) from the read-only prim; cons is updated
 * in place, ghosts untouched.  Each face is solved once.  prim and cons must
 * not overlap.  Matches the reference within 1e-12 relative L-infinity. */
int eulr_godunov_f64(eulr_prim_cf64 prim, eulr_cons_f64 cons, int n0, int n1, int n2, double gamma, double dx0,
                     double dx1, double dx2, double dt, eulr_stream_t stream);
int eulr_godunov_f32(eulr_prim_cf32 prim, eulr_cons_f32 cons, int n0, int n1, int n2, float gamma, float dx0,
                     float dx1, float dx2, float dt, eulr_stream_t stream);

/* godunov bit-identical to the reference (euler_operators/godunov.hpp:15-92,
 * hllc.hpp:50-105 compiled without FMA contraction): the same arguments and
 * result as eulr_godunov_*, computed in the reference's operation order with
 * every operation rounded separately.  Each face is solved once and shared by
 * its two cells, which gives the bits the reference gets by solving it from
 * both.  For validation against the reference; about twice as slow as
 * eulr_godunov_*. */
int eulr_godunov_exact_f64(eulr_prim_cf64 prim, eulr_cons_f64 cons, int n0, int n1, int n2, double gamma, double dx0,
                           double dx1, double dx2, double dt, eulr_stream_t stream);
int eulr_godunov_exact_f32(eulr_prim_cf32 prim, eulr_cons_f32 cons, int n0, int n1, int n2, float gamma, float dx0,
                           float dx1, float dx2, float dt, eulr_stream_t stream);

/* As eulr_godunov_f64 with the time step read on the device: the update uses
 * dt = cfl * (*dt_dev), so a time_step -> godunov loop never copies dt to the
 * host (simulations/euler_simulation.cpp:57-65). */
int eulr_godunov_devdt_f64(eulr_prim_cf64 prim, eulr_cons_f64 cons, int n0, int n1, int n2, double gamma,
                           double dx0, double dx1, double dx2, const double* dt_dev, double cfl,
                           eulr_stream_t stream);

/* ------------------------------------------------ device-resident simulation
 * A simulation owns its device state (two copies of prim, cons and sound
 * speed for ping-pong, plus a few device scalars) and advances it with one
 * fused kernel per step: the step of simulations/euler_simulation.cpp:56-68
 * (dt = time_step(prim); godunov(cfl*dt); cons_to_prim) with the CFL
 * reduction of the next step folded into the update, so dt never leaves the
 * device. */
typedef struct eulr_sim eulr_sim;

typedef enum eulr_precision {
    EULR_PRECISION_F64 = 0,      /* plain FP64 */
    EULR_PRECISION_F32C = 1,     /* FP32 state (4-byte words), FP32 fluxes, compensated update: the axis
                                    flux differences times dt/dv ds are added to the cell by TwoProduct and
                                    TwoSum with their errors folded back, one rounding at the state's
                                    scale; FP64 only for the internal energy of low-pressure cells */
    EULR_PRECISION_F32 = 2,      /* plain FP32 (the reference's real_t = float) */
    EULR_PRECISION_F32C_HILO = 3 /* EULR_PRECISION_F32C with an FP32 low word per conservative field
                                    (double-float state, 8-byte words) */
} eulr_precision;

int eulr_sim_create(int precision, int n0, int n1, int n2, double gamma, double dx0, double dx1, double dx2,
                    double cfl, eulr_stream_t stream, eulr_sim** out);
int eulr_sim_destroy(eulr_sim* sim);

/* Load the state.  Pointers may be host or device memory (copies use
 * cudaMemcpyDefault); loading is asynchronous for FP64 simulations.
 * set_prim computes cons = prim_to_cons(prim), as the reference driver does
 * after init (euler_simulation.cpp:50-51); set_state takes both bundles as
 * they are.  Host sources must stay unchanged until the stream has consumed
 * them (eulr_sim_synchronize, or the next waiting call). */
int eulr_sim_set_prim_f64(eulr_sim* sim, eulr_prim_cf64 prim);
int eulr_sim_set_state_f64(eulr_sim* sim, eulr_prim_cf64 prim, eulr_cons_cf64 cons);
/* init_implode + prim_to_cons on the device. */
int eulr_sim_init_implode(eulr_sim* sim);

/* Advance nsteps steps (asynchronous; replays a CUDA graph). */
int eulr_sim_advance(eulr_sim* sim, int nsteps);

/* Fix the time step: from the next load on, step n (counted from the
 * loaded state) uses dt = dts[n] (the step length itself; no CFL factor)
 * instead of the CFL time step; advancing past n steps is an error.  n = 0
 * returns to CFL time steps.  dts is host memory, copied.  Used to hold dt
 * at a forward sequence (adjoint checks, finite differences). */
int eulr_sim_set_dt_sequence(eulr_sim* sim, const double* dts, long long n);

/* Copy the current state out (host or device destination); waits for the
 * stream.  Either bundle pointer set may be all-NULL to skip it. */
int eulr_sim_get_state_f64(eulr_sim* sim, eulr_prim_f64 prim, eulr_cons_f64 cons);

/* As eulr_sim_get_state_f64 for an FP64 simulation, without waiting: the
 * copies are enqueued on the simulation's stream (a later set/advance on the
 * same simulation is ordered after them).  Host destinations should be
 * pinned for the copies to be asynchronous.  EULR_ERR_UNSUPPORTED for FP32
 * states. */
int eulr_sim_get_state_async_f64(eulr_sim* sim, eulr_prim_f64 prim, eulr_cons_f64 cons);
/* Waits for all work enqueued on the simulation's stream. */
int eulr_sim_synchronize(eulr_sim* sim);

/* Simulated time (sum of cfl*dt over the steps taken), the dt of the next
 * step, and the number of steps taken; waits for the stream. */
int eulr_sim_time(eulr_sim* sim, double* t, double* next_dt, long long* steps);

/* EULR_SUCCESS, or EULR_ERR_NONFINITE once any cell produced a non-finite
 * or non-positive density/pressure; waits for the stream. */
int eulr_sim_status(eulr_sim* sim);

/* Number of kernel launches one step issues (for launch accounting): 1, the
 * fused step kernel, which also turns the new state's max wavespeed into the
 * next dt (its last CTA).  Two one-off launches are not counted: the ghost
 * layer of the second state copy at load, and of the first copy after the
 * first step since a load (FP64 states). */
int eulr_sim_launches_per_step(eulr_sim* sim);

/* Runs ONE step with CUDA events around its launches on the simulation's
 * stream and returns device times in milliseconds: ms[0] ghost layer (0
 * except for the adjoint's recording steps), ms[1] the fused step kernel,
 * ms[2] dt finalize (0 except on grids without interior cells, which launch
 * no step kernel).  Synchronous; advances the state like
 * eulr_sim_advance(sim, 1). */
int eulr_sim_profile_step(eulr_sim* sim, float ms[3]);

/* Conservation totals: sum over interior cells of (d, e, mx0, mx1, mx2),
 * accumulated in FP64 on the device; waits for the stream. */
int eulr_sim_totals(eulr_sim* sim, double out[5]);

/* Algorithmic HBM bytes of one step: the conservative state read and written
 * once per interior cell (5 words, or 10 with stored low words, of the
 * state's word size). */
int eulr_sim_state_bytes(eulr_sim* sim, long long* bytes_per_step);

/* -------------------------------------------------------- multi-grid batch
 * Many independent grids of uneven sizes, each with its own gamma, mesh and
 * dt, advanced together: ONE persistent kernel launch per step pulls
 * (grid, tile, chunk) work items from a device work queue (largest grids
 * first); each grid's last item to finish computes that grid's next dt and
 * clock, and the launch's last CTA rewinds the queue.  Pairs of steps
 * replay from a CUDA graph.  The tile shape and
 * chunk length are chosen by eulr_batch_autotune.  Loading functions work on
 * the batch's first state copy: load every grid before the first step (or
 * after an even number of steps). */
typedef struct eulr_batch eulr_batch;

typedef struct eulr_grid_desc {
    int n0, n1, n2;          /* cells per axis, ghosts included */
    double gamma;            /* ratio of specific heats */
    double dx0, dx1, dx2;    /* mesh spacings */
} eulr_grid_desc;

int eulr_batch_create(int precision, int ngrids, const eulr_grid_desc* grids, double cfl, eulr_stream_t stream,
                      eulr_batch** out);
int eulr_batch_destroy(eulr_batch* batch);

/* Load grid `grid` from an FP64 prim bundle (host or device); cons is
 * prim_to_cons of it. */
int eulr_batch_set_prim_f64(eulr_batch* batch, int grid, eulr_prim_cf64 prim);

/* Step initial condition of the batched workload (no counterpart in the
 * reference): cell centres x_d = ((i_d - 1) + 0.5) dx_d on [0,1]^3,
 * (rho_in, p_in) where x0 + x1 + x2 < c, (rho_out, p_out) elsewhere, u = 0. */
int eulr_batch_init_step(eulr_batch* batch, int grid, double c, double rho_in, double p_in, double rho_out,
                         double p_out);

/* Times every tile shape (32x8, 16x8, 16x16) and chunk length (8, 16, 32,
 * 64 planes) on the loaded state over `trial_steps` steps each, keeps the
 * fastest and restores the state's clocks.  Reports the choice as
 * TX*1000+TY, the chunk length and its step time in ms (any may be NULL). */
int eulr_batch_autotune(eulr_batch* batch, int trial_steps, int* tile_shape, int* kchunk, double* step_ms);

int eulr_batch_advance(eulr_batch* batch, int nsteps);
int eulr_batch_get_state_f64(eulr_batch* batch, int grid, eulr_prim_f64 prim, eulr_cons_f64 cons);
int eulr_batch_time(eulr_batch* batch, int grid, double* t, double* next_dt, long long* steps);
/* EULR_ERR_NONFINITE when any grid produced a non-physical cell. */
int eulr_batch_status(eulr_batch* batch);
/* Interior cells of all grids, work items per step, tile shape (TX*1000+TY)
 * and chunk length in use (any may be NULL). */
int eulr_batch_info(eulr_batch* batch, long long* interior_cells, int* nitems, int* tile_shape, int* kchunk);

/* ---------------------------------------------------------------- adjoint
 * Reverse mode of the time step (no counterpart in the reference, which has
 * no derivatives).  What is differentiated is the reference's step with dt
 * held fixed: godunov (godunov.hpp:15-92, HLLC flux hllc.hpp:50-105) then
 * cons_to_prim (cons_to_prim.hpp:7-33), and prim_to_cons
 * (prim_to_cons.hpp:7-33) before the first step.  The HLLC flux is piecewise
 * smooth; at exact ties (equal arguments of its min/max, ustar == 0 in the
 * subsonic case) the derivative is the mean of the two one-sided ones, as a
 * central difference measures.  All pointers are device memory. */

/* Bytes of device workspace eulr_godunov_adjoint_f64 needs for a grid
 * (41 FP64 fields of n0*n1*n2 values, each padded to 256 bytes); 0 when the
 * extents are invalid. */
size_t eulr_godunov_adjoint_workspace_bytes(int n0, int n1, int n2);

/* Transpose of godunov with respect to prim: given cons_bar, the gradient of
 * a functional with respect to the cons that godunov(prim, cons, dt)
 * produces, writes prim_bar = (d godunov / d prim)^T cons_bar.  (With respect
 * to the incoming cons the update is the identity.)  The face solves are
 * recomputed from prim; each cell sums its six face terms without atomics.
 * workspace: device memory of eulr_godunov_adjoint_workspace_bytes bytes,
 * 256-byte aligned.  prim_bar must not overlap prim or cons_bar. */
int eulr_godunov_adjoint_f64(eulr_prim_cf64 prim, eulr_cons_cf64 cons_bar, eulr_prim_f64 prim_bar, int n0, int n1,
                             int n2, double gamma, double dx0, double dx1, double dx2, double dt, void* workspace,
                             size_t workspace_bytes, eulr_stream_t stream);

/* Transpose of cons_to_prim at the state whose primitive variables are prim:
 * cons_bar = cons_to_prim'^T prim_bar, or cons_bar += ... when accumulate is
 * nonzero.  Pointwise; cons_bar must not overlap prim or prim_bar. */
int eulr_cons_to_prim_adjoint_f64(eulr_prim_cf64 prim, eulr_prim_cf64 prim_bar, eulr_cons_f64 cons_bar, int n0,
                                  int n1, int n2, double gamma, int accumulate, eulr_stream_t stream);

/* Transpose of prim_to_cons at prim: prim_bar (+)= prim_to_cons'^T cons_bar. */
int eulr_prim_to_cons_adjoint_f64(eulr_prim_cf64 prim, eulr_cons_cf64 cons_bar, eulr_prim_f64 prim_bar, int n0,
                                  int n1, int n2, double gamma, int accumulate, eulr_stream_t stream);

/* Checkpointed time-loop adjoint.  eulr_adjoint_forward runs the FP64 fused
 * simulation from prim0 for nsteps steps, keeping the state every
 * checkpoint_every steps; eulr_adjoint_backward maps the gradient of a
 * functional with respect to the final prim to its gradient with respect to
 * prim0, recomputing each segment's states from its checkpoint and then
 * applying the reverse steps (prep, face and gather kernels per step). */
typedef struct eulr_adjoint eulr_adjoint;

int eulr_adjoint_create(int n0, int n1, int n2, double gamma, double dx0, double dx1, double dx2, double cfl,
                        int nsteps, int checkpoint_every, eulr_stream_t stream, eulr_adjoint** out);
int eulr_adjoint_destroy(eulr_adjoint* adj);

/* Forward pass from prim0 (host or device).  dts: host array of nsteps step
 * lengths to hold dt fixed at, or NULL for CFL time steps (recorded; read
 * them with eulr_adjoint_dts).  prim_final (host or device; all-NULL skips
 * it) receives the final prim.  Synchronous. */
int eulr_adjoint_forward(eulr_adjoint* adj, eulr_prim_cf64 prim0, const double* dts, eulr_prim_f64 prim_final);
/* The nsteps step lengths of the last forward pass (host array). */
int eulr_adjoint_dts(eulr_adjoint* adj, double* dts);
/* Reverse pass: prim_final_bar = dJ/d(final prim) (host or device) ->
 * prim0_bar = dJ/d prim0 (host or device).  Needs a forward pass first.
 * Synchronous. */
int eulr_adjoint_backward(eulr_adjoint* adj, eulr_prim_cf64 prim_final_bar, eulr_prim_f64 prim0_bar);
/* Device time of the last passes in ms: the forward pass, the recompute of
 * the checkpointed segments, and the reverse steps (any may be NULL). */
int eulr_adjoint_timing(eulr_adjoint* adj, double* forward_ms, double* recompute_ms, double* reverse_ms);

/* ------------------------------------------------------------ measurement */

/* Times `iters` launches of a kernel whose warps issue only dependent-free
 * FP64 FMAs (kind 0) or FP32 FMAs (kind 1) on all SMs; returns the achieved
 * rate in FLOP/s (an FMA counts 2) via *flops.  Synchronous. */
int eulr_probe_fma_rate(int kind, int iters, double* flops);

#ifdef __cplusplus
}
#endif

#endif /* EULER_GB300_H */
