// The FP32 states' fused step on the column engine, single grid and batch.
// (The FP64 step and the per-operator godunov run on the tile engine of
// flux.cu; the FP32 state with stored low words does too.)
#include "euler_device.cuh"
#include "kernels.h"
#include "step_common.cuh"

namespace eulr {

namespace {

// ------------------------------------------------- FP32 step, column engine
// The fused step of the FP32 states (cons only in HBM) with a regular
// face-per-thread mapping.  Thread (ti, tj) of a 32 x 8 CTA owns the column
// (i0 + ti, j0 + tj) and marches it up z, keeping its cell's primitive state
// of planes k and k+1 in registers.  Per plane it solves
//   x: the face on its cell's left  (the right one is lane+1's, by shuffle;
//      the tile's 8 right boundary faces are solved by the first 8 lanes of
//      one warp and read by lane 31 from shared memory: solved in lane 31 of
//      every warp, each would cost its warp a whole extra HLLC of issue),
//   y: the face below its cell      (the one above is the next row's, through
//      shared memory; row 7 also solves the tile's top boundary faces),
//   z: the face above its cell      (both sides in registers; the face below
//      is the previous plane's).
// Shared memory holds two slots of primitive tiles with their halo rings
// (for the y and boundary neighbours): plane k's, read by the faces, and
// plane k+1's, whose halo ring (threads 0..79) is staged meanwhile, so that
// no halo conversion stands between a plane's own staging and its barrier.
// The y fluxes and the right boundary fluxes go through shared memory too.
// Cons of plane k+2 (own cell) and k+2 (halo ring) are prefetched with
// cp.async a plane before they are converted.
//
// Plain (kCompNone) and compensated (kCompSum) FP32 states; the state with
// stored low words (kCompHiLo) keeps the shared-memory tile engine, whose
// register budget fits them.
//
// The compensated update rounds once at the scale of the state.  The state
// word is FP32, so its own rounding, 0.5 ulp of cons per step, is the floor
// of the error; what compensation removes is every other rounding at that
// scale.  Per field:
//   * the three flux differences F_low - F_high of the axes, each exact where
//     the two fluxes lie within a factor of two of each other (Sterbenz) and
//     otherwise rounded relative to the difference, not to the fluxes;
//   * their sum (cubic cells: k0 == k1 == k2) times k, with the product's
//     rounding error kept (TwoProduct through one FMA); other cells take
//     each axis's product k_d d_d with its error;
//   * cons + product by Knuth's TwoSum, and the rounding errors of the sum
//     and of the product added back before the one final rounding.
// The plain FP32 state instead subtracts the three axis terms from cons one
// after another: three roundings at the state's scale per step.  Summing the
// six fluxes exactly (TwoSum chains, 46 operations per field instead of 15)
// gave the same 1000-step implosion error (rho L1 1.61e-7 against 1.60e-7 at
// 256^3): the state's own rounding and the FP32 fluxes dominate it.
namespace f32col {

constexpr int TX = 32;
constexpr int TY = 8;
constexpr int NT = TX * TY;
constexpr int HX = TX + 2;
constexpr int HY = TY + 2;
constexpr int PLANE = HX * HY; // 340
constexpr int NHALO = 2 * TY + 2 * TX; // 80: left, right columns, bottom, top rows
// The warp whose first TY lanes solve the tile's right boundary x faces: one
// without halo staging (threads 0..NHALO-1) and other than the top row's warp
// (which solves the top boundary y faces), so that no warp solves more than
// one extra face per plane.
constexpr int kRightWarp = 3;
static_assert(kRightWarp * 32 >= NHALO && kRightWarp < TY - 1 && TY <= 32, "right boundary warp");

struct Prim7 {
    float d, p, u[3], c, e; // e: e + p, as the HLLC takes it
};

struct Raw5 {
    float d, e, m[3];
};

__device__ __forceinline__ Side<float> side_of(Prim7 const& q, int dir)
{
    Side<float> s;
    s.d = q.d;
    s.p = q.p;
    s.un = q.u[dir];
    s.ut1 = q.u[(dir + 1) % 3];
    s.ut2 = q.u[(dir + 2) % 3];
    s.c = q.c;
    s.e = q.e;
    return s;
}

// The flux of a face in global components (d, e, m0, m1, m2).
__device__ __forceinline__ void to_global(Flux<float> const& f, int dir, float* g)
{
    g[0] = f.d;
    g[1] = f.e;
    g[2 + dir] = f.n;
    g[2 + (dir + 1) % 3] = f.t1;
    g[2 + (dir + 2) % 3] = f.t2;
}

// Pressure (gamma-1) (e - m.u / 2) of an FP32 conservative cell from its
// velocities u = m / rho: the kinetic energy as m.u instead of |m|^2 / rho
// saves the product by 1/(2 rho).  Compensated states redo the subtraction
// in FP64 where it lost more than 8 bits (pressure_f64_rescue).
template <int COMP>
__device__ __forceinline__ float col_pressure(Raw5 const& r, float u0, float u1, float u2, float ir, float gm1)
{
    float const eint = r.e - 0.5f * (r.m[0] * u0 + r.m[1] * u1 + r.m[2] * u2);
    if (COMP == kCompNone || eint > kLowPressure * r.e) {
        return gm1 * eint;
    }
    return pressure_f64_rescue(r.d, r.e, r.m[0], r.m[1], r.m[2], ir, gm1, nullptr);
}

// Primitive state, sound speed and e + p of an FP32 conservative cell.  1/rho
// is the hardware reciprocal (one MUFU.RCP), not the correctly rounded
// sequence: the FP32 step's error budget is set by the state's own rounding,
// and the 1000-step implosion error is the same either way.
template <int COMP>
__device__ __forceinline__ Prim7 prim_of(Raw5 const& r, FluxParams<float> const& p)
{
    Prim7 q;
    float const ir = rcp_approx(r.d);
    q.d = r.d;
    q.u[0] = r.m[0] * ir;
    q.u[1] = r.m[1] * ir;
    q.u[2] = r.m[2] * ir;
    q.p = col_pressure<COMP>(r, q.u[0], q.u[1], q.u[2], ir, p.gm1);
    q.c = fast_sound_speed(p.gamma * q.p * ir);
    q.e = __fadd_rn(r.e, q.p);
    return q;
}

// A benign state for cells outside the array (no face touching one is used).
__device__ __forceinline__ Raw5 outside() { return Raw5{1.0f, 2.5f, {0.0f, 0.0f, 0.0f}}; }

// Element offset of cell (i, j, k) in the type Off: unsigned (32-bit
// arithmetic, one instruction fewer per address) when the grid has fewer
// than 2^32 cells, long long otherwise.
template <class Off>
__device__ __forceinline__ Off cell_offset(Geom const& g, int i, int j, int k)
{
    return static_cast<Off>(i) + static_cast<Off>(g.s1) * static_cast<Off>(j) +
           static_cast<Off>(g.s2) * static_cast<Off>(k);
}

template <class Off>
__device__ __forceinline__ Raw5 load_raw(FluxParams<float> const& p, int i, int j, int k)
{
    if (i >= p.g.n0 || j >= p.g.n1) {
        return outside();
    }
    Off const o = cell_offset<Off>(p.g, i, j, k);
    Raw5 r;
    r.d = __ldg(p.cons_in.f[0] + o);
    r.e = __ldg(p.cons_in.f[1] + o);
    r.m[0] = __ldg(p.cons_in.f[2] + o);
    r.m[1] = __ldg(p.cons_in.f[3] + o);
    r.m[2] = __ldg(p.cons_in.f[4] + o);
    return r;
}

// Asynchronous 4-byte global->shared copies (cp.async): the prefetched cons
// of the next planes wait in shared memory instead of registers.
__device__ __forceinline__ void cp_async4(float* dst, const float* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// All of this thread's copy groups but the last committed one have landed.
__device__ __forceinline__ void cp_async_wait_all_but_last() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Starts copying the cons of cell (i, j, k) to dst[f * stride].  A cell past
// the array's last ghost layer (a tile overhanging the grid) takes the state
// of the nearest ghost cell: physical values, read without a branch, and no
// face that touches such a cell is used.
template <class Off>
__device__ __forceinline__ void prefetch_raw(float* dst, int stride, FluxParams<float> const& p, int i, int j, int k)
{
    Off const o = cell_offset<Off>(p.g, min(i, p.g.n0 - 1), min(j, p.g.n1 - 1), k);
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        cp_async4(dst + f * stride, p.cons_in.f[f] + o);
    }
}

__device__ __forceinline__ Raw5 read_raw(float const* src, int stride)
{
    return Raw5{src[0], src[stride], {src[2 * stride], src[3 * stride], src[4 * stride]}};
}

__device__ __forceinline__ void halo_cell(int h, int& hx, int& hy)
{
    if (h < TY) {
        hx = 0;
        hy = 1 + h;
    } else if (h < 2 * TY) {
        hx = HX - 1;
        hy = 1 + h - TY;
    } else if (h < 2 * TY + TX) {
        hx = 1 + h - 2 * TY;
        hy = 0;
    } else {
        hx = 1 + h - 2 * TY - TX;
        hy = HY - 1;
    }
}

// One plane slot: a staged cell is two 16-byte words, (d, p, u0, u1) and
// (u2, c, e + p, -), written and read with two vector accesses (STS.128 and
// LDS.128) instead of seven scalar ones.  Consecutive lanes touch
// consecutive words, so the accesses are free of bank conflicts.
struct SlotPlane {
    float4 a[PLANE];
    float4 b[PLANE];
};

__device__ __forceinline__ void put(SlotPlane& q, int idx, Prim7 const& v)
{
    q.a[idx] = make_float4(v.d, v.p, v.u[0], v.u[1]);
    q.b[idx] = make_float4(v.u[2], v.c, v.e, v.e);
}

__device__ __forceinline__ Prim7 get(SlotPlane const& q, int idx)
{
    float4 const a = q.a[idx];
    float4 const b = q.b[idx];
    Prim7 v;
    v.d = a.x;
    v.p = a.y;
    v.u[0] = a.z;
    v.u[1] = a.w;
    v.u[2] = b.x;
    v.c = b.y;
    v.e = b.z;
    return v;
}

// Five flux components through shared memory as one 16-byte word and one
// 4-byte word.
__device__ __forceinline__ void put_flux(float4* a, float* b, int idx, float const* f)
{
    a[idx] = make_float4(f[0], f[1], f[2], f[3]);
    b[idx] = f[4];
}

__device__ __forceinline__ void get_flux(float4 const* a, float const* b, int idx, float* f)
{
    float4 const v = a[idx];
    f[0] = v.x;
    f[1] = v.y;
    f[2] = v.z;
    f[3] = v.w;
    f[4] = b[idx];
}

// ---- paired FP32 arithmetic: on sm_100 and later, FADD2/FMUL2/FFMA2
// carry two FP32 operations per issued instruction, each rounded once.  The
// step is bound by instruction issue, so the compensated update of fields
// (d, e) and (m0, m1) runs in pairs (the same operations, the same bits).

// a - b, rounded once (b * -1 is exact)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

// The compensated update of two fields of a cubic cell: u + k (flux balance)
// with one rounding at the state's scale, operation for operation the scalar
// form below.  nk = -k gives the product's rounding error negated,
// P - k S, which the last step subtracts.
__device__ __forceinline__ float2 comp_update2(float2 u, float2 xl, float2 xr, float2 yb, float2 yt, float2 zl, float2 zh,
                                               float2 k, float2 nk)
{
    float2 const S = __fadd2_rn(__fadd2_rn(sub2(xl, xr), sub2(yb, yt)), sub2(zl, zh));
    float2 const P = __fmul2_rn(k, S);
    float2 const nP = __ffma2_rn(nk, S, P);
    float2 const s = __fadd2_rn(u, P);
    float2 const bb = sub2(s, u);
    float2 const err = __fadd2_rn(sub2(u, sub2(s, bb)), sub2(P, bb));
    return __fadd2_rn(s, sub2(err, nP));
}

struct ColShared {
    SlotPlane slot[2];
    float4 yflux_a[NT]; // the y face below each cell
    float yflux_b[NT];
    float4 xflux_ra[TY]; // the tile's right boundary x faces
    float xflux_rb[TY];
    float raw_own[5 * NT];     // own column, two planes ahead
    float raw_halo[5 * NHALO]; // halo ring, one plane ahead
    long long warp_best[NT / 32];
    int any_bad;
};

// One work item: interior planes [kb, ke) of the 32 x 8 column tile (tx, ty),
// kb = 1 + kc * kchunk, with update coefficients k0..k2 (UNIFORM: cubic cells, k0..k2
// all equal and 1/dx_d too).  BRANCHED: the cell update sits inside the
// interior test (the batch) rather than beside it (the single grid).
// Accumulates this thread's max wavespeed and non-physical flag.
template <int COMP, bool UNIFORM, class Off, bool BRANCHED>
__device__ __forceinline__ void col_item(FluxParams<float> const& p, float k0, float k1, float k2, int tx, int ty,
                                         int kc, ColShared& sh, float& wmaxf, bool& bad)
{
    int const tid = threadIdx.x;
    int const ti = tid % TX; // == lane
    int const tj = tid / TX; // == warp
    int const own_idx = (tj + 1) * HX + ti + 1;
    int hhx = 0, hhy = 0;
    if (tid < NHALO) {
        halo_cell(tid, hhx, hhy);
    }
    int const i0 = 1 + tx * TX;
    int const j0 = 1 + ty * TY;
    int const kb = 1 + kc * p.kchunk;
    int const ke = min(kb + p.kchunk, p.g.n2 - 1);
    int const i = i0 + ti;
    int const j = j0 + tj;
    bool const own = (i < p.g.n0 - 1) && (j < p.g.n1 - 1);

    // prologue: plane kb of the halo ring staged, kb+1 on its way; planes
    // kb-1 (z face below), kb, kb+1 of the own column
    if (tid < NHALO) {
        prefetch_raw<Off>(sh.raw_halo + tid, NHALO, p, i0 - 1 + hhx, j0 - 1 + hhy, kb);
        cp_async_wait_all();
        put(sh.slot[0], hhy * HX + hhx, prim_of<COMP>(read_raw(sh.raw_halo + tid, NHALO), p));
        if (kb + 1 < ke) {
            prefetch_raw<Off>(sh.raw_halo + tid, NHALO, p, i0 - 1 + hhx, j0 - 1 + hhy, kb + 1);
        }
    }
    cp_async_commit();
    Raw5 const rb = load_raw<Off>(p, i, j, kb - 1);
    Raw5 rk = load_raw<Off>(p, i, j, kb);
    Raw5 rn = load_raw<Off>(p, i, j, kb + 1); // kb + 1 <= ke <= n2 - 1
    Prim7 q0 = prim_of<COMP>(rk, p);
    Prim7 q1 = prim_of<COMP>(rn, p);
    float zlo[5];
    to_global(hllc_flux(side_of(prim_of<COMP>(rb, p), 2), side_of(q0, 2)), 2, zlo);
    Off o = cell_offset<Off>(p.g, min(i, p.g.n0 - 1), min(j, p.g.n1 - 1), kb);

    // Unrolled twice: the plane-to-plane register rotation (q0 <- q1,
    // rk <- rn, zlo <- fzh) becomes renaming instead of moves, and the slot
    // of each copy is a constant.
#pragma unroll 2
    for (int k = kb; k < ke; ++k) {
        SlotPlane& q = sh.slot[(k - kb) & 1];
        // stage plane k: the own cell (its halo ring was staged a plane ahead)
        put(q, own_idx, q0);
        // own column plane k+2, consumed at the end of this plane
        if (k + 2 <= ke) {
            prefetch_raw<Off>(sh.raw_own + tid, NT, p, i, j, k + 2);
        }
        cp_async_commit();
        __syncthreads(); // plane k staged
        // the halo ring of plane k+1 into the other slot, off the path to the
        // barrier above (the slot's last reader finished before the previous
        // plane's second barrier)
        if (tid < NHALO && k + 1 < ke) {
            cp_async_wait_all_but_last(); // the halo copies of plane k+1 landed (own k+2 may be in flight)
            put(sh.slot[(k + 1 - kb) & 1], hhy * HX + hhx, prim_of<COMP>(read_raw(sh.raw_halo + tid, NHALO), p));
            if (k + 2 < ke) {
                prefetch_raw<Off>(sh.raw_halo + tid, NHALO, p, i0 - 1 + hhx, j0 - 1 + hhy, k + 2);
            }
        }
        cp_async_commit();

        // ---- faces
        float fxl[5], fyb[5], fzh[5], fxr[5], fyt[5];
        {
            float t[5];
            to_global(hllc_flux(side_of(get(q, own_idx - HX), 1), side_of(q0, 1)), 1, t);
            put_flux(sh.yflux_a, sh.yflux_b, tid, t); // read back after the barrier (registers are scarce here)
        }
        to_global(hllc_flux(side_of(get(q, own_idx - 1), 0), side_of(q0, 0)), 0, fxl);
        to_global(hllc_flux(side_of(q0, 2), side_of(q1, 2)), 2, fzh);
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            fxr[f] = __shfl_down_sync(0xffffffffu, fxl[f], 1);
        }
        if (tj == kRightWarp && ti < TY) { // the tile's right boundary faces, one per row
            int const c = (ti + 1) * HX + TX;
            float t[5];
            to_global(hllc_flux(side_of(get(q, c), 0), side_of(get(q, c + 1), 0)), 0, t);
            put_flux(sh.xflux_ra, sh.xflux_rb, ti, t);
        }
        if (tj == TY - 1) { // the tile's top boundary faces
            to_global(hllc_flux(side_of(q0, 1), side_of(get(q, own_idx + HX), 1)), 1, fyt);
        }
        __syncthreads(); // y fluxes and right boundary fluxes written
        get_flux(sh.yflux_a, sh.yflux_b, tid, fyb);
        if (tj < TY - 1) {
            get_flux(sh.yflux_a, sh.yflux_b, tid + TX, fyt);
        }
        {
            float xr[5];
            get_flux(sh.xflux_ra, sh.xflux_rb, tj, xr); // one broadcast read per warp
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                fxr[f] = ti == TX - 1 ? xr[f] : fxr[f];
            }
        }

        // ---- update of the own cell.  In the single-grid step every lane
        // computes it (a lane off the interior holds physical values of
        // clamped cells) and only the stores and the wavespeed are the
        // interior's, so no branch encloses the arithmetic (+1 %); the batch,
        // whose tiles overhang its small grids more often, keeps the branch
        // (measured 4 % faster there).
        if (!BRANCHED || own) {
            float u[5] = {rk.d, rk.e, rk.m[0], rk.m[1], rk.m[2]};
            constexpr bool kPaired = COMP == kCompSum && UNIFORM;
            if (kPaired) { // fields (d, e) and (m0, m1) in pairs, m2 below
                float2 const kk = make_float2(k0, k0), nk = make_float2(-k0, -k0);
#pragma unroll
                for (int f = 0; f < 4; f += 2) {
                    float2 const r = comp_update2(make_float2(u[f], u[f + 1]), make_float2(fxl[f], fxl[f + 1]),
                                                  make_float2(fxr[f], fxr[f + 1]), make_float2(fyb[f], fyb[f + 1]),
                                                  make_float2(fyt[f], fyt[f + 1]), make_float2(zlo[f], zlo[f + 1]),
                                                  make_float2(fzh[f], fzh[f + 1]), kk, nk);
                    u[f] = r.x;
                    u[f + 1] = r.y;
                }
            }
#pragma unroll
            for (int f = kPaired ? 4 : 0; f < 5; ++f) {
                if (COMP == kCompNone) {
                    u[f] = u[f] - k0 * (fxr[f] - fxl[f]) - k1 * (fyt[f] - fyb[f]) - k2 * (fzh[f] - zlo[f]);
                } else if (UNIFORM) {
                    // _rn intrinsics: no product may be fused into the sums
                    // the TwoSum and TwoProduct take apart
                    float const S = __fadd_rn(__fadd_rn(__fsub_rn(fxl[f], fxr[f]), __fsub_rn(fyb[f], fyt[f])),
                                              __fsub_rn(zlo[f], fzh[f]));
                    float const P = __fmul_rn(k0, S);
                    float const eP = fmaf(k0, S, -P);
                    float const s = __fadd_rn(u[f], P);
                    float const bb = __fsub_rn(s, u[f]);
                    float const err = __fadd_rn(__fsub_rn(u[f], __fsub_rn(s, bb)), __fsub_rn(P, bb));
                    u[f] = __fadd_rn(s, __fadd_rn(err, eP));
                } else {
                    float const d0 = __fsub_rn(fxl[f], fxr[f]);
                    float const d1 = __fsub_rn(fyb[f], fyt[f]);
                    float const d2 = __fsub_rn(zlo[f], fzh[f]);
                    float const P0 = __fmul_rn(k0, d0), P1 = __fmul_rn(k1, d1), P2 = __fmul_rn(k2, d2);
                    float const eP = __fadd_rn(__fadd_rn(fmaf(k0, d0, -P0), fmaf(k1, d1, -P1)), fmaf(k2, d2, -P2));
                    float const P = __fadd_rn(__fadd_rn(P0, P1), P2);
                    float const s = __fadd_rn(u[f], P);
                    float const bb = __fsub_rn(s, u[f]);
                    float const err = __fadd_rn(__fsub_rn(u[f], __fsub_rn(s, bb)), __fsub_rn(P, bb));
                    u[f] = __fadd_rn(s, __fadd_rn(err, eP));
                }
            }
            if (own) {
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    p.cons_out.f[f][o] = u[f];
                }
            }
            // next step's CFL wavespeed of the new state (time_step.hpp:28-33);
            // on cubic cells (3 cs + |v0| + |v1| + |v2|) / dx, one product
            Raw5 const nr{u[0], u[1], {u[2], u[3], u[4]}};
            float const r = rcp_approx(u[0]);
            float const v0 = u[2] * r, v1 = u[3] * r, v2 = u[4] * r;
            float const pr = col_pressure<COMP>(nr, v0, v1, v2, r, p.gm1);
            float const cs = fast_sound_speed((p.gamma * r) * pr);
            float const invdt = UNIFORM ? (3.0f * cs + fabsf(v0) + fabsf(v1) + fabsf(v2)) * p.invdx0
                                        : (cs + fabsf(v0)) * p.invdx0 + (cs + fabsf(v1)) * p.invdx1 +
                                                  (cs + fabsf(v2)) * p.invdx2;
            wmaxf = own ? fmaxf(wmaxf, invdt) : wmaxf; // NaN never wins
            bad |= own && !cell_ok(u[0], pr, invdt);
        }
        // march: plane k+1 becomes the current plane
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            zlo[f] = fzh[f];
        }
        rk = rn;
        q0 = q1;
        if (k + 2 <= ke) {
            cp_async_wait_all_but_last(); // the own copies of plane k+2 landed
            rn = read_raw(sh.raw_own + tid, NT);
            q1 = prim_of<COMP>(rn, p);
        }
        o += static_cast<Off>(p.g.s2);
    }
    __syncthreads(); // the slots are restaged by the next item
}

// Block max of the threads' wavespeeds into *wmax (ordered bits, one
// atomicMax per CTA) and the non-physical flag into *status; clears both.
__device__ __forceinline__ void col_flush(ColShared& sh, float& wmaxf, bool& bad, unsigned long long* wmax,
                                          int* status)
{
    int const tid = threadIdx.x;
    long long wk = wave_key(wmaxf);
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        long long const v = __shfl_xor_sync(0xffffffffu, wk, s);
        wk = v > wk ? v : wk;
    }
    __syncthreads();
    if (tid == 0) {
        sh.any_bad = 0;
    }
    __syncthreads();
    if (tid % 32 == 0) {
        sh.warp_best[tid / 32] = wk;
    }
    if (bad) {
        sh.any_bad = 1;
    }
    __syncthreads();
    if (tid == 0) {
        long long b = sh.warp_best[0];
#pragma unroll
        for (int v = 1; v < NT / 32; ++v) {
            b = sh.warp_best[v] > b ? sh.warp_best[v] : b;
        }
        atomicMax(wmax, static_cast<unsigned long long>(b));
        if (sh.any_bad) {
            atomicOr(status, 1);
        }
    }
    wmaxf = 0.0f;
    bad = false;
}

template <int COMP, bool UNIFORM, class Off>
__global__ void __launch_bounds__(NT, 3) f32_step_kernel(const __grid_constant__ FluxParams<float> p)
{
    static_assert(COMP == kCompNone || COMP == kCompSum, "low-word states use the tile engine");
    __shared__ __align__(16) ColShared sh;
    float const dtodv = dt_over_dv(p);
    float const k0 = dtodv * p.ds0, k1 = dtodv * p.ds1, k2 = dtodv * p.ds2; // UNIFORM: all equal
    float wmaxf = 0.0f;
    bool bad = false;
    int const tiles_xy = p.tiles_x * p.tiles_y;
    for (int w = blockIdx.x; w < p.nwork; w += gridDim.x) {
        col_item<COMP, UNIFORM, Off, false>(p, k0, k1, k2, w % p.tiles_x, (w / p.tiles_x) % p.tiles_y, w / tiles_xy, sh, wmaxf,
                                bad);
    }
    col_flush(sh, wmaxf, bad, p.wmax, p.status);
    step_done(p);
}

// The column engine over a batch: CTAs pop (grid, tile x, tile y, chunk)
// items from the queue, as flux_batch_kernel does; each item's wavespeed goes
// to its own grid.  Grids of cubic cells take the cubic update and wavespeed.
template <int COMP, class Off>
__global__ void __launch_bounds__(NT, 3) f32_batch_kernel(const __grid_constant__ BatchParams<float> b)
{
    static_assert(COMP == kCompNone || COMP == kCompSum, "low-word states use the tile engine");
    static_assert(sizeof(FluxParams<float>) % 4 == 0, "parameter copy in 4-byte words");
    __shared__ __align__(16) ColShared sh;
    __shared__ __align__(16) FluxParams<float> gp;
    __shared__ int s_item;
    int const tid = threadIdx.x;
    float wmaxf = 0.0f;
    bool bad = false;
    for (;;) {
        __syncthreads(); // everyone is done with the previous item's parameters
        if (tid == 0) {
            s_item = static_cast<int>(atomicAdd(b.head, 1u));
        }
        __syncthreads();
        int const item = s_item;
        if (item >= b.nitems) {
            break;
        }
        int4 const it = b.items[item];
        for (int w = tid; w < static_cast<int>(sizeof(FluxParams<float>) / 4); w += NT) {
            reinterpret_cast<int*>(&gp)[w] = reinterpret_cast<const int*>(&b.grids[it.x])[w];
        }
        __syncthreads();
        float const dtodv = dt_over_dv(gp);
        float const k0 = dtodv * gp.ds0, k1 = dtodv * gp.ds1, k2 = dtodv * gp.ds2;
        if (gp.ds0 == gp.ds1 && gp.ds1 == gp.ds2 && gp.invdx0 == gp.invdx1 && gp.invdx1 == gp.invdx2) {
            col_item<COMP, true, Off, true>(gp, k0, k1, k2, it.y, it.z, it.w, sh, wmaxf, bad);
        } else {
            col_item<COMP, false, Off, true>(gp, k0, k1, k2, it.y, it.z, it.w, sh, wmaxf, bad);
        }
        col_flush(sh, wmaxf, bad, gp.wmax, gp.status);
        item_done(gp);
    }
    batch_cta_done(b);
}

} // namespace f32col

// Grids up to this many cells index their fields with 32-bit offsets.
constexpr long long kNarrowCells = 0xffffffffLL;

template <int COMP>
cudaError_t configure_f32col(int* per_sm)
{
    int n = 0;
    cudaError_t const e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f32col::f32_step_kernel<COMP, false, long long>,
                                                                        f32col::NT, 0);
    *per_sm = n < 1 ? 1 : n;
    return e;
}

template <int COMP>
cudaError_t launch_f32col(FluxParams<float> p, int sms, cudaStream_t s)
{
    int const per_sm = p.per_sm > 0 ? p.per_sm : 1;
    int const ix = p.g.n0 - 2;
    int const iy = p.g.n1 - 2;
    int const iz = p.g.n2 - 2;
    if (ix <= 0 || iy <= 0 || iz <= 0) {
        return cudaSuccess; // no interior cell
    }
    p.tiles_x = (ix + f32col::TX - 1) / f32col::TX;
    p.tiles_y = (iy + f32col::TY - 1) / f32col::TY;
    long long const slots = static_cast<long long>(sms) * per_sm;
    if (p.kchunk <= 0) {
        p.kchunk = choose_kchunk(p.tiles_x * p.tiles_y, iz, slots);
    }
    int const kchunks = (iz + p.kchunk - 1) / p.kchunk;
    long long const nwork = static_cast<long long>(p.tiles_x) * p.tiles_y * kchunks;
    p.nwork = static_cast<int>(nwork);
    long long const grid = slots < nwork ? slots : nwork;
    // cubic cells: equal face areas give equal update coefficients dt/dv * ds_d,
    // and equal 1/dx_d the one-product wavespeed
    bool const uniform = p.ds0 == p.ds1 && p.ds1 == p.ds2 && p.invdx0 == p.invdx1 && p.invdx1 == p.invdx2;
    if (p.g.ncell() <= kNarrowCells) {
        if (uniform) {
            f32col::f32_step_kernel<COMP, true, unsigned><<<static_cast<int>(grid), f32col::NT, 0, s>>>(p);
        } else {
            f32col::f32_step_kernel<COMP, false, unsigned><<<static_cast<int>(grid), f32col::NT, 0, s>>>(p);
        }
    } else if (uniform) {
        f32col::f32_step_kernel<COMP, true, long long><<<static_cast<int>(grid), f32col::NT, 0, s>>>(p);
    } else {
        f32col::f32_step_kernel<COMP, false, long long><<<static_cast<int>(grid), f32col::NT, 0, s>>>(p);
    }
    return cudaGetLastError();
}

// The column engine as the 32 x 8 shape of the FP32 batch (states without low words).
template <int COMP>
struct ColBatchKernel {
    static cudaError_t configure(int* per_sm)
    {
        int n = 0;
        cudaError_t const e =
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f32col::f32_batch_kernel<COMP, long long>, f32col::NT, 0);
        *per_sm = n < 1 ? 1 : n;
        return e;
    }
    static cudaError_t launch(BatchParams<float> const& b, int grid, cudaStream_t s)
    {
        if (b.max_cells <= kNarrowCells) {
            f32col::f32_batch_kernel<COMP, unsigned><<<grid, f32col::NT, 0, s>>>(b);
        } else {
            f32col::f32_batch_kernel<COMP, long long><<<grid, f32col::NT, 0, s>>>(b);
        }
        return cudaGetLastError();
    }
};

} // namespace

cudaError_t configure_step_f32col(int comp, int* per_sm)
{
    return comp == kCompSum ? configure_f32col<kCompSum>(per_sm) : configure_f32col<kCompNone>(per_sm);
}

cudaError_t launch_step_f32col(FluxParams<float> const& p, int comp, int sms, cudaStream_t s)
{
    return comp == kCompSum ? launch_f32col<kCompSum>(p, sms, s) : launch_f32col<kCompNone>(p, sms, s);
}

cudaError_t launch_batch_f32col(int comp, BatchParams<float> const* b, int grid, int* per_sm, cudaStream_t s)
{
    if (comp == kCompSum) {
        return b ? ColBatchKernel<kCompSum>::launch(*b, grid, s) : ColBatchKernel<kCompSum>::configure(per_sm);
    }
    return b ? ColBatchKernel<kCompNone>::launch(*b, grid, s) : ColBatchKernel<kCompNone>::configure(per_sm);
}

} // namespace eulr
