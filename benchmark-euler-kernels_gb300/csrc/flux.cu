// Godunov/HLLC flux kernels (sm_103a): the per-operator godunov and the fused
// simulation step share one z-marching tile engine.
//
// Work decomposition: the interior [1,n0-1) x [1,n1-1) x [1,n2-1) is cut into
// TX x TY columns and each column into chunks of kchunk planes; a persistent
// grid of CTAs walks the (tile, chunk) items round-robin.  A CTA marches up
// its chunk one plane at a time through a ring of plane slots in shared
// memory, each slot holding the 7 face inputs (d, p, u0, u1, u2, c, e) of a
// (TX+2) x (TY+2) plane with its one-cell halo.  Per plane:
//   1. face phase -- every x face and y face of plane k and every z face
//      between planes k and k+1 is solved ONCE (the reference solves each
//      interior face twice, once from each side, godunov.hpp:48-82).  FP64
//      (bound by the FP64 pipe): the x, y and z faces share one index space,
//      and each face's family, cells and axis permutation are chosen by
//      selects, so a warp whose lanes straddle two families still runs the
//      HLLC once -- the 800 faces of a 16x16 tile take exactly 25
//      warp-passes.  FP32 (bound by instruction issue): each family in its
//      own warp-aligned range with compile-time axes, on a 32x8 tile.
//      Fluxes go to shared memory in global axes;
//   2. cell phase -- each thread owns one column cell and applies
//      cons -= dt/dv * sum_d ds_d (F_R - F_L) (godunov.hpp:84-90) with the
//      face-area and dt/dv factors folded into three coefficients.  The z
//      face below the cell is carried in registers from the previous plane.
// The fused step then finishes the cell on chip: cons_to_prim, sound speed
// and the next step's CFL max-wavespeed, reduced warp -> block -> one
// atomicMax per CTA, so dt never leaves the device.
//
// Staging: in the fused step the seven input fields of a plane slot are
// fetched by TMA (cp.async.bulk.tensor, one 18x18x1 FP64 box per field) into a
// ring of three slots, two planes ahead of the plane being solved, each slot
// completing on its own mbarrier.  Grids whose row pitch is not a multiple of
// 16 bytes (odd n0) and the per-operator godunov (arbitrary caller pointers)
// stage with plain cooperative loads instead.  Every mbarrier wait is bounded:
// a wait that runs out sets bit 1 of the status word, waits (bounded) for the
// copies still in flight and ends the CTA.
#include "euler_device.cuh"
#include "kernels.h"
#include "step_common.cuh"

#include <cfloat>

namespace eulr {

namespace {

constexpr int kWaitTries = 1 << 20; // mbarrier.try_wait attempts before giving up

template <class T, int TX, int TY, int NSLOT>
struct TileLayout {
    static constexpr int HX = TX + 2;
    static constexpr int HY = TY + 2;
    static constexpr int PLANE = HX * HY;
    static constexpr int PLANE_PAD = (PLANE + 15) / 16 * 16; // 128-byte aligned field tiles
    static constexpr int NFX = (TX + 1) * TY;
    static constexpr int NFY = TX * (TY + 1);
    static constexpr int NFZ = TX * TY;
    static constexpr int NFACE = NFX + NFY + NFZ;
    // FP32's index space: each face family starts on a warp boundary
    static constexpr int NFX_W = (NFX + 31) / 32 * 32;
    static constexpr int NFY_W = (NFY + 31) / 32 * 32;
    static constexpr int NFACE_W = NFX_W + NFY_W + NFZ;
    static_assert(NFACE_W >= NFACE && NFACE_W - NFACE < 64, "padding of at most one warp per family");
    static_assert(NFX < 4096 && NFY < 4096 && NFZ < 4096, "face index range of div_small");
    static constexpr int NT = TX * TY;
    // shared memory, in T elements after a 128-byte mbarrier block
    static constexpr int Q_ELEMS = NSLOT * kFields * PLANE_PAD;
    static constexpr int FX_OFF = Q_ELEMS;
    static constexpr int FY_OFF = FX_OFF + 5 * NFX;
    static constexpr int FZ_OFF = FY_OFF + 5 * NFY;
    static constexpr int ELEMS = FZ_OFF + 5 * NFZ;
    static constexpr int MBAR_BYTES = 128;
    // + 128 bytes of slack to align the dynamic region to 128 bytes at run time
    static constexpr size_t BYTES = 128 + MBAR_BYTES + sizeof(T) * static_cast<size_t>(ELEMS);
    static constexpr unsigned TX_BYTES = kFields * PLANE * sizeof(T); // bytes one slot's TMA delivers
};

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait for the phase with the given parity; false if it never came.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity)
{
    unsigned const a = smem_u32(bar);
    for (int it = 0; it < kWaitTries; ++it) {
        unsigned done;
        asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(a), "r"(parity)
                : "memory");
        if (done) {
            return true;
        }
    }
    return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar)
{
    asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
            "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
            : "memory");
}

template <class T, int TX, int TY, int NSLOT>
__device__ __forceinline__ T* slot_field(T* smem, int slot, int field)
{
    using L = TileLayout<T, TX, TY, NSLOT>;
    return smem + (slot * kFields + field) * L::PLANE_PAD;
}

// Issue the TMA loads of plane k (x origin i0-1, y origin j0-1) into `slot`.
template <class T, int TX, int TY, int NSLOT>
__device__ __forceinline__ void issue_plane(T* smem, unsigned long long* bars, int slot, TmaMaps const& maps, int i0,
                                            int j0, int k)
{
    using L = TileLayout<T, TX, TY, NSLOT>;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bars[slot], L::TX_BYTES);
#pragma unroll
    for (int f = 0; f < kFields; ++f) {
        tma_load_3d(slot_field<T, TX, TY, NSLOT>(smem, slot, f), &maps.m[f], i0 - 1, j0 - 1, k, &bars[slot]);
    }
}

// Stage plane k with plain loads.  Godunov mode derives c and e from prim;
// step mode reads the stored sound speed and the conservative energy.  Cells
// outside the array get a benign uniform state; no face touching them is
// ever used.
template <class T, int TX, int TY, int NSLOT, int MODE, int COMP>
__device__ __forceinline__ void load_plane(T* smem, int slot, FluxParams<T> const& p, int i0, int j0, int k)
{
    using L = TileLayout<T, TX, TY, NSLOT>;
    T* q = slot_field<T, TX, TY, NSLOT>(smem, slot, 0);
    for (int c = threadIdx.x; c < L::PLANE; c += L::NT) {
        int const hx = c % L::HX;
        int const hy = c / L::HX;
        int const i = i0 - 1 + hx;
        int const j = j0 - 1 + hy;
        T d = T(1), pr = T(1), u0 = T(0), u1 = T(0), u2 = T(0), cs = T(1), e = T(2.5);
        if (i < p.g.n0 && j < p.g.n1) {
            long long const o = p.g.at(i, j, k);
            if (MODE != kModeStepCons) {
                d = __ldg(p.prim.f[0] + o);
                pr = __ldg(p.prim.f[1] + o);
                u0 = __ldg(p.prim.f[2] + o);
                u1 = __ldg(p.prim.f[3] + o);
                u2 = __ldg(p.prim.f[4] + o);
            }
            if (MODE == kModeStep) {
                cs = __ldg(p.cs + o);
                e = __ldg(p.cons_in.f[1] + o);
            } else if (MODE == kModeStepCons) {
                // cons-only FP32 state: cons_to_prim on chip
                T const m0 = __ldg(p.cons_in.f[2] + o);
                T const m1 = __ldg(p.cons_in.f[3] + o);
                T const m2 = __ldg(p.cons_in.f[4] + o);
                d = __ldg(p.cons_in.f[0] + o);
                e = __ldg(p.cons_in.f[1] + o);
                T const r = rcp_rn(d); // = 1/d correctly rounded, without the division routine
                u0 = m0 * r;
                u1 = m1 * r;
                u2 = m2 * r;
                pr = cons_pressure<COMP>(d, e, m0, m1, m2, r, p.gm1, nullptr);
                cs = fast_sound_speed(p.gamma * pr * r);
            } else {
                if constexpr (sizeof(T) == 8) {
                    // sqrt(gamma p / rho) from one reciprocal square root, and
                    // e + p = p gamma/(gamma-1) + (rho/2) |u|^2 with the
                    // halving on the integer pipe: 4 FP64 instructions and a
                    // seed fewer per staged cell than 1/rho, a square root
                    // and e formed before p is added
                    cs = sqrt_quotient_faithful(p.gamma * pr, d);
                    e = pr * (p.inv_gm1 + T(1)) + half_exact(d) * (u0 * u0 + u1 * u1 + u2 * u2);
                } else {
                    cs = sqrt(p.gamma * pr * (T(1) / d));
                    e = pr * p.inv_gm1 + T(0.5) * d * (u0 * u0 + u1 * u1 + u2 * u2);
                }
            }
            if (MODE != kModeGodunov || sizeof(T) == 4) {
                e += pr; // the HLLC takes e + p (formed once per staged cell, not per face)
            }
        }
        q[0 * L::PLANE_PAD + c] = d;
        q[1 * L::PLANE_PAD + c] = pr;
        q[2 * L::PLANE_PAD + c] = u0;
        q[3 * L::PLANE_PAD + c] = u1;
        q[4 * L::PLANE_PAD + c] = u2;
        q[5 * L::PLANE_PAD + c] = cs;
        q[6 * L::PLANE_PAD + c] = e;
    }
}

template <class T, int PLANE_PAD>
__device__ __forceinline__ Side<T> load_side(T const* q, int c, int dir)
{
    int const d1 = dir == 2 ? 0 : dir + 1; // the axes after the normal, cyclically
    int const d2 = dir == 0 ? 2 : dir - 1;
    Side<T> s;
    s.d = q[0 * PLANE_PAD + c];
    s.p = q[1 * PLANE_PAD + c];
    s.un = q[(2 + dir) * PLANE_PAD + c];
    s.ut1 = q[(2 + d1) * PLANE_PAD + c];
    s.ut2 = q[(2 + d2) * PLANE_PAD + c];
    s.c = q[5 * PLANE_PAD + c];
    s.e = q[6 * PLANE_PAD + c];
    return s;
}

template <class T>
__device__ __forceinline__ void store_flux(T* out, int stride, int idx, int dir, Flux<T> const& f)
{
    int const d1 = dir == 2 ? 0 : dir + 1;
    int const d2 = dir == 0 ? 2 : dir - 1;
    out[0 * stride + idx] = f.d;
    out[1 * stride + idx] = f.e;
    out[(2 + dir) * stride + idx] = f.n;
    out[(2 + d1) * stride + idx] = f.t1;
    out[(2 + d2) * stride + idx] = f.t2;
}

// Per-CTA state of the tile engine that lives across work items.
template <class T>
struct TileCtx {
    unsigned long long* bars; // one mbarrier per slot (TMA ring)
    T* smem;                  // plane slots
    T* fx;                    // x-face fluxes (5 fields)
    T* fy;                    // y-face fluxes
    T* fz;                    // z-face fluxes
    unsigned phase;           // bit s: parity of slot s's next completion (TMA ring)
    unsigned inflight;        // bit s: a TMA into slot s has not been waited for
    bool timed_out;           // a bounded mbarrier wait ran out
    long long wkey;           // ordered bits of this thread's max wavespeed (FP64)
    unsigned wrun;            // FP64 step: the warp's running max of wavespeed estimates (WaveScreen)
    float wmaxf;              // this thread's max wavespeed (FP32 states: keyed once, at the flush)
    bool bad;                 // this thread saw a non-physical cell
};

template <class T, int NSLOT>
__device__ __forceinline__ bool wait_slot(TileCtx<T>& c, int s)
{
    bool const ok = mbar_wait(&c.bars[s], (c.phase >> s) & 1u);
    c.phase ^= 1u << s;
    c.inflight &= ~(1u << s);
    return ok;
}

// One work item: interior planes [kb, ke) of the TX x TY column whose first
// cell is (1 + tx*TX, 1 + ty*TY), with update coefficients k0..k2 (dt/dv
// times the face areas).  Returns false when a staged plane never arrived.
template <class T, int TX, int TY, int NSLOT, int MODE, bool TMA, int COMP>
__device__ __forceinline__ bool tile_item(TileCtx<T>& c, FluxParams<T> const& p, TmaMaps const& maps, T k0, T k1,
                                          T k2, int tx, int ty, int kc)
{
    using L = TileLayout<T, TX, TY, NSLOT>;
    int const tid = threadIdx.x;
    int const ti = tid % TX;
    int const tj = tid / TX;
    int const center = (tj + 1) * L::HX + ti + 1;
    bool const cubic = p.invdx0 == p.invdx1 && p.invdx1 == p.invdx2;
    T* const smem = c.smem;
    T* const fx = c.fx;
    T* const fy = c.fy;
    T* const fz = c.fz;

    int const i0 = 1 + tx * TX;
    int const j0 = 1 + ty * TY;
    int const kb = 1 + kc * p.kchunk;
    int const ke = min(kb + p.kchunk, p.g.n2 - 1);
    int const i = i0 + ti;
    int const j = j0 + tj;
    bool const own = (i < p.g.n0 - 1) && (j < p.g.n1 - 1);

    __syncthreads(); // the previous item's readers of slots and fluxes are done
    if (TMA) {
        // planes kb-1, kb, kb+1 -> slots 0, 1, 2 (kb+1 <= ke always)
        if (tid == 0) {
            issue_plane<T, TX, TY, NSLOT>(smem, c.bars, 0, maps, i0, j0, kb - 1);
            issue_plane<T, TX, TY, NSLOT>(smem, c.bars, 1, maps, i0, j0, kb);
            issue_plane<T, TX, TY, NSLOT>(smem, c.bars, 2, maps, i0, j0, kb + 1);
        }
        c.inflight |= 7u;
        c.timed_out |= !wait_slot<T, NSLOT>(c, 0);
        c.timed_out |= !wait_slot<T, NSLOT>(c, 1);
    } else {
        load_plane<T, TX, TY, NSLOT, MODE, COMP>(smem, 0, p, i0, j0, kb - 1);
        load_plane<T, TX, TY, NSLOT, MODE, COMP>(smem, 1, p, i0, j0, kb);
        __syncthreads();
    }
    // z face below the chunk's first plane, kept in registers in global
    // axes (the z face frame has n = mx2, t1 = mx0, t2 = mx1)
    T zlo[5];
    {
        Flux<T> const f0 = hllc_flux(load_side<T, L::PLANE_PAD>(slot_field<T, TX, TY, NSLOT>(smem, 0, 0), center, 2),
                                     load_side<T, L::PLANE_PAD>(slot_field<T, TX, TY, NSLOT>(smem, 1, 0), center, 2));
        zlo[0] = f0.d;
        zlo[1] = f0.e;
        zlo[2] = f0.t1;
        zlo[3] = f0.t2;
        zlo[4] = f0.n;
    }
    if (__syncthreads_or(c.timed_out)) { // slot 0 is refilled next
        return false;
    }
    if (TMA) {
        if (kb + 2 <= ke) {
            if (tid == 0) {
                issue_plane<T, TX, TY, NSLOT>(smem, c.bars, 0, maps, i0, j0, kb + 2);
            }
            c.inflight |= 1u;
        }
    }

    // FP64 step: the next step's CFL wavespeed is screened (WaveScreen); the
    // running max carries over from the CTA's previous item of the same grid
    constexpr bool kScreen = sizeof(T) == 8 && MODE == kModeStep;
    WaveScreen screen(p.gamma, p.invdx0, p.invdx1, p.invdx2);
    screen.run = c.wrun;

    for (int k = kb; k < ke; ++k) {
        int const cur = (k - kb + 1) % NSLOT;
        int const nxt = (k - kb + 2) % NSLOT;
        // this cell's conservative state, fetched while the faces are solved
        T u[5];
        T ulo[5] = {T(0), T(0), T(0), T(0), T(0)};
        long long const o = p.g.at(i, j, k);
        if (own) {
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                u[f] = p.cons_in.f[f][o];
                if (COMP == kCompHiLo) {
                    ulo[f] = p.lo_in.f[f][o];
                }
            }
        }
        if (TMA) {
            c.timed_out |= !wait_slot<T, NSLOT>(c, nxt);
        } else {
            load_plane<T, TX, TY, NSLOT, MODE, COMP>(smem, nxt, p, i0, j0, k + 1);
            __syncthreads();
        }

        // ---- face phase
        T const* qc = slot_field<T, TX, TY, NSLOT>(smem, cur, 0);
        T const* qn = slot_field<T, TX, TY, NSLOT>(smem, nxt, 0);
        if constexpr (sizeof(T) == 8) {
            // FP64 (bound by the FP64 pipe): one index space over the three
            // families; each face's family, left cell and right cell are
            // chosen by selects, so a warp that straddles two families still
            // runs the HLLC once
            for (int f = tid; f < L::NFACE; f += L::NT) {
                bool const is_x = f < L::NFX;
                bool const is_y = !is_x && f < L::NFX + L::NFY;
                int const g = is_x ? f : (is_y ? f - L::NFX : f - L::NFX - L::NFY);
                int const gj = is_x ? div_small<TX + 1>(g) : div_small<TX>(g);
                int const gi = g - gj * (is_x ? TX + 1 : TX);
                int const a = (is_y ? gj : gj + 1) * L::HX + (is_x ? gi : gi + 1);
                int const dir = is_x ? 0 : (is_y ? 1 : 2);
                T const* const qr = is_x || is_y ? qc : qn;
                int const ar = a + (is_x ? 1 : (is_y ? L::HX : 0));
                store_flux(is_x ? fx : (is_y ? fy : fz), is_x ? L::NFX : (is_y ? L::NFY : L::NFZ), g, dir,
                           hllc_flux(load_side<T, L::PLANE_PAD>(qc, a, dir), load_side<T, L::PLANE_PAD>(qr, ar, dir)));
            }
        } else {
            // FP32 (bound by instruction issue, where the selects above cost
            // more than they save): each family in its own warp-aligned
            // index range, with compile-time axes
            for (int f = tid; f < L::NFACE_W; f += L::NT) {
                if (f < L::NFX_W) {
                    if (f < L::NFX) {
                        int const fj = f / (TX + 1);
                        int const fi = f % (TX + 1);
                        int const a = (fj + 1) * L::HX + fi;
                        store_flux(fx, L::NFX, f, 0,
                                   hllc_flux(load_side<T, L::PLANE_PAD>(qc, a, 0),
                                             load_side<T, L::PLANE_PAD>(qc, a + 1, 0)));
                    }
                } else if (f < L::NFX_W + L::NFY_W) {
                    int const g = f - L::NFX_W;
                    if (g < L::NFY) {
                        int const fj = g / TX;
                        int const fi = g % TX;
                        int const a = fj * L::HX + fi + 1;
                        store_flux(fy, L::NFY, g, 1,
                                   hllc_flux(load_side<T, L::PLANE_PAD>(qc, a, 1),
                                             load_side<T, L::PLANE_PAD>(qc, a + L::HX, 1)));
                    }
                } else {
                    int const g = f - L::NFX_W - L::NFY_W; // < NFZ
                    int const fj = g / TX;
                    int const fi = g % TX;
                    int const a = (fj + 1) * L::HX + fi + 1;
                    store_flux(fz, L::NFZ, g, 2,
                               hllc_flux(load_side<T, L::PLANE_PAD>(qc, a, 2), load_side<T, L::PLANE_PAD>(qn, a, 2)));
                }
            }
        }
        if (__syncthreads_or(c.timed_out)) {
            return false;
        }
        if (TMA) {
            // plane k is no longer read: refill its slot with plane k+3
            if (k + 3 <= ke) {
                if (tid == 0) {
                    issue_plane<T, TX, TY, NSLOT>(smem, c.bars, cur, maps, i0, j0, k + 3);
                }
                c.inflight |= 1u << cur;
            }
        }

        // ---- cell phase
        T fza[5];
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            fza[f] = fz[f * L::NFZ + tid];
        }
        T wv[4] = {T(0), T(0), T(0), T(0)}; // FP64 step: the new cs, v0, v1, v2, for the screened wavespeed
        if (own) {
            int const xl = tj * (TX + 1) + ti;
            int const yb = tj * TX + ti;
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                if (COMP == kCompNone) {
                    T const ax = fx[f * L::NFX + xl + 1] - fx[f * L::NFX + xl];
                    T const ay = fy[f * L::NFY + yb + TX] - fy[f * L::NFY + yb];
                    T const az = fza[f] - zlo[f];
                    u[f] = u[f] - k0 * ax - k1 * ay - k2 * az;
                } else {
                    // cons + six signed face terms, summed without
                    // intermediate rounding error (TwoProduct + TwoSum),
                    // then rounded once
                    T sum = u[f];
                    T err = ulo[f];
                    compensated_add(sum, err, -k0, fx[f * L::NFX + xl + 1]);
                    compensated_add(sum, err, k0, fx[f * L::NFX + xl]);
                    compensated_add(sum, err, -k1, fy[f * L::NFY + yb + TX]);
                    compensated_add(sum, err, k1, fy[f * L::NFY + yb]);
                    compensated_add(sum, err, -k2, fza[f]);
                    compensated_add(sum, err, k2, zlo[f]);
                    u[f] = sum + err;
                    ulo[f] = err - (u[f] - sum);
                }
            }
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                p.cons_out.f[f][o] = u[f];
                if (COMP == kCompHiLo) {
                    p.lo_out.f[f][o] = ulo[f];
                }
            }
            if (MODE == kModeStep || MODE == kModeStepCons) {
                // cons_to_prim of the new state (cons_to_prim.hpp:26-31)
                T const r = rcp_faithful(u[0]); // FP32: correctly rounded
                T const v0 = u[2] * r;
                T const v1 = u[3] * r;
                T const v2 = u[4] * r;
                T pr;
                if (MODE == kModeStep) {
                    T const mv = u[2] * v0 + u[3] * v1 + u[4] * v2; // |m|^2 / rho
                    pr = p.gm1 * u[1] - p.half_gm1 * mv;              // (gamma-1)(e - |m|^2/(2 rho))
                } else {
                    pr = cons_pressure<COMP>(u[0], u[1], u[2], u[3], u[4], r, p.gm1, COMP == kCompHiLo ? ulo : nullptr);
                }
                T const cs = fast_sound_speed((p.gamma * r) * pr);
                if (MODE == kModeStep) {
                    if constexpr (sizeof(T) == 8) {
                        if (p.h_out != nullptr) {
                            p.h_out[o] = u[1] + pr; // staged by TMA at the next step
                        }
                    }
                    p.prim_out.f[0][o] = u[0];
                    p.prim_out.f[1][o] = pr;
                    p.prim_out.f[2][o] = v0;
                    p.prim_out.f[3][o] = v1;
                    p.prim_out.f[4][o] = v2;
                    if (p.prim_rec.f[0] != nullptr) { // a second copy, for a recording caller
                        p.prim_rec.f[0][o] = u[0];
                        p.prim_rec.f[1][o] = pr;
                        p.prim_rec.f[2][o] = v0;
                        p.prim_rec.f[3][o] = v1;
                        p.prim_rec.f[4][o] = v2;
                    }
                    p.cs_out[o] = cs;
                }
                if constexpr (kScreen) {
                    wv[0] = cs;
                    wv[1] = v0;
                    wv[2] = v1;
                    wv[3] = v2;
                    c.bad |= !(finite_positive(u[0]) && finite_positive(pr)); // the wavespeed is checked below
                } else {
                    // next step's CFL wavespeed (time_step.hpp:28-33)
                    // (cubic cells: one product instead of three)
                    T const invdt = cubic ? (T(3) * cs + abs_(v0) + abs_(v1) + abs_(v2)) * p.invdx0
                                          : (cs + abs_(v0)) * p.invdx0 + (cs + abs_(v1)) * p.invdx1 +
                                                    (cs + abs_(v2)) * p.invdx2;
                    if constexpr (sizeof(T) == 4) {
                        c.wmaxf = fmaxf(c.wmaxf, invdt); // NaN never wins (fmaxf returns the other operand)
                    } else {
                        long long const key = wave_key(invdt);
                        c.wkey = key > c.wkey ? key : c.wkey;
                    }
                    c.bad |= !cell_ok(u[0], pr, invdt);
                }
            }
        }
        if constexpr (kScreen) {
            // next step's CFL wavespeed (time_step.hpp:28-33), in FP64 only
            // for the cells that can hold the max; the same expression as
            // the unscreened step, so the max and the dt are unchanged.
            // Every lane of the warp is here (the screen is warp-collective);
            // a non-finite wavespeed always takes the FP64 branch.
            if (screen.step_exact_needed(own, wv[0], wv[1], wv[2], wv[3], cubic)) {
                T const invdt = cubic ? (T(3) * wv[0] + abs_(wv[1]) + abs_(wv[2]) + abs_(wv[3])) * p.invdx0
                                      : (wv[0] + abs_(wv[1])) * p.invdx0 + (wv[0] + abs_(wv[2])) * p.invdx1 +
                                                (wv[0] + abs_(wv[3])) * p.invdx2;
                long long const key = wave_key(invdt);
                c.wkey = key > c.wkey ? key : c.wkey;
                c.bad |= dbits(invdt) >= kInfBits;
            }
        }
        // the z face above becomes the next plane's z face below
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            zlo[f] = fza[f];
        }
        __syncthreads(); // fluxes are rewritten by the next face phase
    }
    c.wrun = screen.run;
    return !__syncthreads_or(c.timed_out);
}

// Block-wide max of the threads' wavespeed keys into *wmax, and the
// non-physical flag into *status; clears the per-thread values.
template <class T, int NT>
__device__ __forceinline__ void flush_wavespeed(TileCtx<T>& c, unsigned long long* wmax, int* status)
{
    __shared__ long long warp_best[NT / 32];
    __shared__ int any_bad;
    int const tid = threadIdx.x;
    long long w = c.wkey;
    if constexpr (sizeof(T) == 4) {
        long long const kf = wave_key(c.wmaxf);
        w = kf > w ? kf : w;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long const v = __shfl_xor_sync(0xffffffffu, w, o);
        w = v > w ? v : w;
    }
    __syncthreads();
    if (tid == 0) {
        any_bad = 0;
    }
    __syncthreads();
    if ((tid & 31) == 0) {
        warp_best[tid >> 5] = w;
    }
    if (c.bad) {
        any_bad = 1;
    }
    __syncthreads();
    if (tid == 0) {
        long long b = warp_best[0];
#pragma unroll
        for (int wv = 1; wv < NT / 32; ++wv) {
            b = warp_best[wv] > b ? warp_best[wv] : b;
        }
        atomicMax(wmax, static_cast<unsigned long long>(b));
        if (any_bad) {
            atomicOr(status, 1);
        }
    }
    c.wkey = 0;
    c.wrun = 0u; // the next item may be another grid's
    c.wmaxf = 0.0f;
    c.bad = false;
}

template <class T, int TX, int TY, int NSLOT>
__device__ __forceinline__ TileCtx<T> make_ctx(unsigned char* smem_dyn)
{
    using L = TileLayout<T, TX, TY, NSLOT>;
    // TMA destinations must sit on 128-byte boundaries of the shared window
    unsigned char* raw = smem_dyn + ((128u - (smem_u32(smem_dyn) & 127u)) & 127u);
    TileCtx<T> c;
    c.bars = reinterpret_cast<unsigned long long*>(raw);
    c.smem = reinterpret_cast<T*>(raw + L::MBAR_BYTES);
    c.fx = c.smem + L::FX_OFF;
    c.fy = c.smem + L::FY_OFF;
    c.fz = c.smem + L::FZ_OFF;
    c.phase = 0;
    c.inflight = 0;
    c.timed_out = false;
    c.wkey = 0;
    c.wrun = 0u;
    c.wmaxf = 0.0f;
    c.bad = false;
    return c;
}

template <class T, int TX, int TY, int NSLOT, int MODE, bool TMA, int COMP>
__global__ void __launch_bounds__(TX* TY) flux_tile_kernel(const __grid_constant__ FluxParams<T> p,
                                                           const __grid_constant__ TmaMaps maps)
{
    static_assert(COMP == kCompNone || (sizeof(T) == 4 && MODE == kModeStepCons), "compensation is for the FP32 step");
    static_assert(!TMA || NSLOT == 3, "the TMA ring has three slots");
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    TileCtx<T> c = make_ctx<T, TX, TY, NSLOT>(smem_dyn);
    T const dtodv = dt_over_dv(p);
    // cons -= dt/dv * sum_d ds_d (F_R - F_L), coefficients folded
    T const k0 = dtodv * p.ds0, k1 = dtodv * p.ds1, k2 = dtodv * p.ds2;

    if (TMA) {
        if (threadIdx.x == 0) {
            for (int s = 0; s < NSLOT; ++s) {
                mbar_init(&c.bars[s], 1);
            }
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
    }

    int const tiles_xy = p.tiles_x * p.tiles_y;
    for (int w = blockIdx.x; w < p.nwork; w += gridDim.x) {
        int const tx = w % p.tiles_x;
        int const ty = (w / p.tiles_x) % p.tiles_y;
        int const kc = w / tiles_xy;
        if (!tile_item<T, TX, TY, NSLOT, MODE, TMA, COMP>(c, p, maps, k0, k1, k2, tx, ty, kc)) {
            break;
        }
    }

    if (TMA && __syncthreads_or(c.timed_out)) {
        // a staged plane never arrived: report, wait (bounded) for the copies
        // still in flight so none lands after the CTA is gone, and stop
        if (threadIdx.x == 0) {
            atomicOr(p.status, 2);
        }
        for (int s = 0; s < NSLOT; ++s) {
            if (c.inflight & (1u << s)) {
                wait_slot<T, NSLOT>(c, s);
            }
        }
        step_done(p); // the launch still counts this CTA, so the next launch starts from zero
        return;
    }
    if (MODE == kModeStep || MODE == kModeStepCons) {
        flush_wavespeed<T, TX * TY>(c, p.wmax, p.status);
        step_done(p);
    }
}

// Many independent grids in one launch: a persistent grid of CTAs pops
// (grid, tile, chunk) items from a global queue (largest grids first),
// copies the item's grid parameters to shared memory and runs the same tile
// engine; each item's wavespeed goes to its own grid's accumulator, so every
// grid keeps its own dt.  Plain-load staging (grids of any shape).
template <class T, int TX, int TY, int MODE, int COMP>
__global__ void __launch_bounds__(TX* TY) flux_batch_kernel(const __grid_constant__ BatchParams<T> b)
{
    constexpr int NSLOT = 2;
    constexpr int NT = TX * TY;
    static_assert(sizeof(FluxParams<T>) % 4 == 0, "parameter copy in 4-byte words");
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    __shared__ __align__(16) FluxParams<T> gp;
    __shared__ int s_item;
    TileCtx<T> c = make_ctx<T, TX, TY, NSLOT>(smem_dyn);
    int const tid = threadIdx.x;
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
        for (int w = tid; w < static_cast<int>(sizeof(FluxParams<T>) / 4); w += NT) {
            reinterpret_cast<int*>(&gp)[w] = reinterpret_cast<const int*>(&b.grids[it.x])[w];
        }
        __syncthreads();
        T const dtodv = dt_over_dv(gp);
        T const k0 = dtodv * gp.ds0, k1 = dtodv * gp.ds1, k2 = dtodv * gp.ds2;
        tile_item<T, TX, TY, NSLOT, MODE, false, COMP>(c, gp, TmaMaps{}, k0, k1, k2, it.y, it.z, it.w);
        flush_wavespeed<T, NT>(c, gp.wmax, gp.status);
        item_done(gp);
    }
    batch_cta_done(b);
}

// Ghost shell of the step's output: cons copied, prim = cons_to_prim(cons)
// (bit-identical to the reference's cons_to_prim over ghosts,
// cons_to_prim.hpp:26-27), sound speed and CFL contribution.
template <class T>
__device__ __forceinline__ void ghost_shell_body(GhostParams<T> const& p)
{
    Geom const g = p.g;
    bool const all = (g.n0 < 3) || (g.n1 < 3) || (g.n2 < 3);
    long long const plane = g.s2;
    long long const ring = 2LL * g.n0 + 2LL * (g.n1 - 2);
    long long const total = all ? g.ncell() : 2 * plane + ring * (g.n2 - 2);
    T wmax = T(0);
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        long long o;
        if (all) {
            o = c;
        } else if (c < 2 * plane) {
            o = (c < plane) ? c : c - plane + plane * (g.n2 - 1);
        } else {
            // grids hold < 2^31 cells: the ring index fits 32-bit division
            unsigned const r0 = static_cast<unsigned>(c - 2 * plane);
            unsigned const q = r0 / static_cast<unsigned>(ring);
            int const k = 1 + static_cast<int>(q);
            int const r = static_cast<int>(r0 - q * static_cast<unsigned>(ring));
            int i, j;
            if (r < g.n0) {
                i = r;
                j = 0;
            } else if (r < 2 * g.n0) {
                i = r - g.n0;
                j = g.n1 - 1;
            } else {
                int const r2 = r - 2 * g.n0;
                j = 1 + r2 / 2;
                i = (r2 & 1) ? g.n0 - 1 : 0;
            }
            o = g.at(i, j, k);
        }
        T const d = p.cons_in.f[0][o];
        T const e = p.cons_in.f[1][o];
        T const m0 = p.cons_in.f[2][o];
        T const m1 = p.cons_in.f[3][o];
        T const m2 = p.cons_in.f[4][o];
        T pr, u0, u1, u2;
        if (p.prim_out.f[0] == nullptr) {
            // cons-only FP32 state: only the cons words and the wavespeed
            T const r = rcp_rn(d); // = 1/d correctly rounded
            u0 = m0 * r;
            u1 = m1 * r;
            u2 = m2 * r;
            pr = p.comp != kCompNone ? cons_pressure<kCompSum>(d, e, m0, m1, m2, r, p.gm1, nullptr)
                                     : cons_pressure<kCompNone>(d, e, m0, m1, m2, r, p.gm1, nullptr);
        } else {
            cons_to_prim_exact(d, e, m0, m1, m2, p.gm1, pr, u0, u1, u2);
        }
        p.cons_out.f[0][o] = d;
        p.cons_out.f[1][o] = e;
        p.cons_out.f[2][o] = m0;
        p.cons_out.f[3][o] = m1;
        p.cons_out.f[4][o] = m2;
        if (p.lo_in.f[0] != nullptr) {
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                p.lo_out.f[f][o] = p.lo_in.f[f][o];
            }
        }
        if (p.h_out != nullptr) {
            p.h_out[o] = e + pr;
        }
        if (p.prim_out.f[0] != nullptr) {
            p.prim_out.f[0][o] = d;
            p.prim_out.f[1][o] = pr;
            p.prim_out.f[2][o] = u0;
            p.prim_out.f[3][o] = u1;
            p.prim_out.f[4][o] = u2;
            if (p.prim_rec.f[0] != nullptr) {
                p.prim_rec.f[0][o] = d;
                p.prim_rec.f[1][o] = pr;
                p.prim_rec.f[2][o] = u0;
                p.prim_rec.f[3][o] = u1;
                p.prim_rec.f[4][o] = u2;
            }
            p.cs_out[o] = sqrt_rn(div_rn(mul_rn(p.gamma, pr), d));
        }
        T v;
        if (p.prim_out.f[0] == nullptr) {
            // FP32 states: the sound speed as their step kernel forms it
            T const cs = fast_sound_speed((p.gamma * rcp_rn(d)) * pr);
            v = (cs + abs_(u0)) * p.invdx0 + (cs + abs_(u1)) * p.invdx1 + (cs + abs_(u2)) * p.invdx2;
        } else {
            v = cell_invdt_exact(d, pr, u0, u1, u2, p.gamma, p.invdx0, p.invdx1, p.invdx2);
        }
        wmax = (v > wmax) ? v : wmax;
    }
    __shared__ T warp_best[8];
    wmax = warp_max(wmax);
    if ((threadIdx.x & 31) == 0) {
        warp_best[threadIdx.x >> 5] = wmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        T b = warp_best[0];
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) {
            b = (warp_best[w] > b) ? warp_best[w] : b;
        }
        atomicMax(p.wmax, order_bits(b));
    }
}

template <class T>
__global__ void __launch_bounds__(256) ghost_shell_kernel(GhostParams<T> p)
{
    ghost_shell_body(p);
}

template <class T>
__global__ void finalize_dt_kernel(SimScalars* s, T cfl, int add_time, const double* dt_seq)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        finalize_one(s, cfl, add_time, dt_seq);
    }
}

// The single-grid tile.  FP64: 16x16 columns, whose 800 faces per plane
// fill exactly 25 warp-passes (a 32x8 tile's 808 need 26) with the same 256
// threads, 18x18 TMA boxes and two resident CTAs per SM.  FP32 (the state
// with stored low words; the other FP32 states run the column engine):
// 32x8, measured faster there (26.9 against 21.9 Gcell/s at 512^3).
template <class T>
struct StepTile {
    static constexpr int X = 16, Y = 16;
};
template <>
struct StepTile<float> {
    static constexpr int X = 32, Y = 8;
};

template <class T, int MODE, bool TMA, int COMP>
struct FluxKernel {
    static constexpr int NSLOT = TMA ? 3 : 2;
    static constexpr int TX = StepTile<T>::X, TY = StepTile<T>::Y;
    using L = TileLayout<T, TX, TY, NSLOT>;
    static auto fn() { return flux_tile_kernel<T, TX, TY, NSLOT, MODE, TMA, COMP>; }
};

// Opts the kernel into its dynamic shared memory size and returns its
// resident CTAs per SM.  Called outside any stream capture (by the entry
// points before they enqueue work), and cheap to repeat.
template <class T, int MODE, bool TMA, int COMP>
cudaError_t configure_flux_impl(int* per_sm)
{
    using K = FluxKernel<T, MODE, TMA, COMP>;
    auto kern = K::fn();
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(K::L::BYTES));
    if (e != cudaSuccess) {
        return e;
    }
    int n = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, K::L::NT, K::L::BYTES);
    if (e != cudaSuccess) {
        return e;
    }
    *per_sm = n < 1 ? 1 : n;
    return cudaSuccess;
}

template <class T, int MODE, bool TMA, int COMP>
cudaError_t launch_flux_impl(FluxParams<T> p, TmaMaps const& maps, int sms, cudaStream_t s)
{
    using K = FluxKernel<T, MODE, TMA, COMP>;
    int const per_sm = p.per_sm > 0 ? p.per_sm : 1;
    int const ix = p.g.n0 - 2;
    int const iy = p.g.n1 - 2;
    int const iz = p.g.n2 - 2;
    if (ix <= 0 || iy <= 0 || iz <= 0) {
        return cudaSuccess; // no interior cell
    }
    p.tiles_x = (ix + K::TX - 1) / K::TX;
    p.tiles_y = (iy + K::TY - 1) / K::TY;
    long long const slots = static_cast<long long>(sms) * per_sm;
    if (p.kchunk <= 0) {
        p.kchunk = choose_kchunk(p.tiles_x * p.tiles_y, iz, slots);
    }
    int const kchunks = (iz + p.kchunk - 1) / p.kchunk;
    long long const nwork = static_cast<long long>(p.tiles_x) * p.tiles_y * kchunks;
    p.nwork = static_cast<int>(nwork);
    long long grid = slots;
    if (grid > nwork) {
        grid = nwork;
    }
    K::fn()<<<static_cast<int>(grid), K::L::NT, K::L::BYTES, s>>>(p, maps);
    return cudaGetLastError();
}

// Tile shapes the batch kernel is built for (the autotuner picks one).  For
// FP32 states without low words the 32 x 8 shape runs the column engine.
constexpr int kBatchShapes[][2] = {{32, 8}, {16, 8}, {16, 16}};
constexpr int kNumBatchShapes = 3;

template <class T, int TX, int TY, int MODE, int COMP>
struct BatchKernel {
    using L = TileLayout<T, TX, TY, 2>;
    static auto fn() { return flux_batch_kernel<T, TX, TY, MODE, COMP>; }
    static cudaError_t configure(int* per_sm)
    {
        auto kern = fn();
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(L::BYTES));
        if (e != cudaSuccess) {
            return e;
        }
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, L::NT, L::BYTES);
        *per_sm = n < 1 ? 1 : n;
        return e;
    }
    static cudaError_t launch(BatchParams<T> const& b, int grid, cudaStream_t s)
    {
        fn()<<<grid, L::NT, L::BYTES, s>>>(b);
        return cudaGetLastError();
    }
};

template <class T, int MODE, int COMP>
cudaError_t batch_dispatch(int shape, BatchParams<T> const* b, int grid, int* per_sm, cudaStream_t s)
{
    if constexpr (sizeof(T) == 4 && COMP != kCompHiLo) {
        if (shape == 0) { // the column engine
            return launch_batch_f32col(COMP, b, grid, per_sm, s);
        }
    }
    switch (shape) {
    case 0: return b ? BatchKernel<T, 32, 8, MODE, COMP>::launch(*b, grid, s) : BatchKernel<T, 32, 8, MODE, COMP>::configure(per_sm);
    case 1: return b ? BatchKernel<T, 16, 8, MODE, COMP>::launch(*b, grid, s) : BatchKernel<T, 16, 8, MODE, COMP>::configure(per_sm);
    default: return b ? BatchKernel<T, 16, 16, MODE, COMP>::launch(*b, grid, s) : BatchKernel<T, 16, 16, MODE, COMP>::configure(per_sm);
    }
}

} // namespace

int batch_shape_count() { return kNumBatchShapes; }
void batch_shape(int shape, int* tx, int* ty)
{
    *tx = kBatchShapes[shape][0];
    *ty = kBatchShapes[shape][1];
}

// b == nullptr: configure (dynamic shared memory opt-in) and report the
// resident CTAs per SM; otherwise launch `grid` persistent CTAs.
template <class T>
cudaError_t launch_flux_batch(int shape, int comp, BatchParams<T> const* b, int grid, int* per_sm, cudaStream_t s)
{
    if constexpr (sizeof(T) == sizeof(double)) {
        return batch_dispatch<double, kModeStep, kCompNone>(shape, b, grid, per_sm, s);
    } else {
        switch (comp) {
        case kCompSum: return batch_dispatch<float, kModeStepCons, kCompSum>(shape, b, grid, per_sm, s);
        case kCompHiLo: return batch_dispatch<float, kModeStepCons, kCompHiLo>(shape, b, grid, per_sm, s);
        default: return batch_dispatch<float, kModeStepCons, kCompNone>(shape, b, grid, per_sm, s);
        }
    }
}

template cudaError_t launch_flux_batch<double>(int, int, BatchParams<double> const*, int, int*, cudaStream_t);
template cudaError_t launch_flux_batch<float>(int, int, BatchParams<float> const*, int, int*, cudaStream_t);

template <class T>
struct FluxDispatch;

template <>
struct FluxDispatch<double> {
    static cudaError_t configure(int mode, bool tma, int /*comp*/, int* per_sm)
    {
        if (mode == kModeStep) {
            return tma ? configure_flux_impl<double, kModeStep, true, kCompNone>(per_sm)
                       : configure_flux_impl<double, kModeStep, false, kCompNone>(per_sm);
        }
        return configure_flux_impl<double, kModeGodunov, false, kCompNone>(per_sm);
    }
    static cudaError_t launch(FluxParams<double> const& p, TmaMaps const* maps, int mode, int /*comp*/, int sms,
                              cudaStream_t s)
    {
        if (mode == kModeStep) {
            if (maps != nullptr) {
                return launch_flux_impl<double, kModeStep, true, kCompNone>(p, *maps, sms, s);
            }
            return launch_flux_impl<double, kModeStep, false, kCompNone>(p, TmaMaps{}, sms, s);
        }
        return launch_flux_impl<double, kModeGodunov, false, kCompNone>(p, TmaMaps{}, sms, s);
    }
};

template <>
struct FluxDispatch<float> {
    static cudaError_t configure(int mode, bool /*tma*/, int comp, int* per_sm)
    {
        if (mode == kModeStep) {
            // the stored low words do not fit the column engine's registers: the
            // double-float state keeps the shared-memory tile engine
            switch (comp) {
            case kCompSum: return configure_step_f32col(kCompSum, per_sm);
            case kCompHiLo: return configure_flux_impl<float, kModeStepCons, false, kCompHiLo>(per_sm);
            default: return configure_step_f32col(kCompNone, per_sm);
            }
        }
        return configure_flux_impl<float, kModeGodunov, false, kCompNone>(per_sm);
    }
    static cudaError_t launch(FluxParams<float> const& p, TmaMaps const* /*maps*/, int mode, int comp, int sms,
                              cudaStream_t s)
    {
        if (mode == kModeStep) {
            switch (comp) {
            case kCompSum: return launch_step_f32col(p, kCompSum, sms, s);
            case kCompHiLo: return launch_flux_impl<float, kModeStepCons, false, kCompHiLo>(p, TmaMaps{}, sms, s);
            default: return launch_step_f32col(p, kCompNone, sms, s);
            }
        }
        return launch_flux_impl<float, kModeGodunov, false, kCompNone>(p, TmaMaps{}, sms, s);
    }
};

template <class T>
cudaError_t configure_flux(int mode, bool tma, int comp, int* per_sm)
{
    return FluxDispatch<T>::configure(mode, tma, comp, per_sm);
}

template <class T>
cudaError_t launch_flux(FluxParams<T> p, TmaMaps const* maps, int mode, int comp, int sms, cudaStream_t s)
{
    return FluxDispatch<T>::launch(p, maps, mode, comp, sms, s);
}

template <class T>
cudaError_t launch_ghost_shell(GhostParams<T> p, int sms, cudaStream_t s)
{
    Geom const& g = p.g;
    long long total;
    if (g.n0 < 3 || g.n1 < 3 || g.n2 < 3) {
        total = g.ncell();
    } else {
        total = 2 * g.s2 + (2LL * g.n0 + 2LL * (g.n1 - 2)) * (g.n2 - 2);
    }
    long long blocks = (total + 255) / 256;
    long long const cap = static_cast<long long>(sms) * 8;
    if (blocks > cap) {
        blocks = cap;
    }
    if (blocks < 1) {
        blocks = 1;
    }
    ghost_shell_kernel<T><<<static_cast<int>(blocks), 256, 0, s>>>(p);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_finalize_dt(SimScalars* sc, T cfl, int add_time, cudaStream_t s, const double* dt_seq)
{
    finalize_dt_kernel<T><<<1, 32, 0, s>>>(sc, cfl, add_time, dt_seq);
    return cudaGetLastError();
}

int flux_tile_x() { return StepTile<double>::X; } // the FP64 step's TMA boxes
int flux_tile_y() { return StepTile<double>::Y; }

template cudaError_t configure_flux<double>(int, bool, int, int*);
template cudaError_t configure_flux<float>(int, bool, int, int*);
template cudaError_t launch_flux<double>(FluxParams<double>, TmaMaps const*, int, int, int, cudaStream_t);
template cudaError_t launch_flux<float>(FluxParams<float>, TmaMaps const*, int, int, int, cudaStream_t);
template cudaError_t launch_ghost_shell<double>(GhostParams<double>, int, cudaStream_t);
template cudaError_t launch_ghost_shell<float>(GhostParams<float>, int, cudaStream_t);
template cudaError_t launch_finalize_dt<double>(SimScalars*, double, int, cudaStream_t, const double*);
template cudaError_t launch_finalize_dt<float>(SimScalars*, float, int, cudaStream_t, const double*);

} // namespace eulr
