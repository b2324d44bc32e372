// Reverse mode (adjoint) of the first-order Godunov/HLLC time step.
//
// The reference has no adjoint.  What is differentiated is its time step:
// godunov (euler_operators/godunov.hpp:15-92) with the HLLC flux
// (euler_operators/hllc.hpp:50-105), then cons_to_prim
// (euler_operators/cons_to_prim.hpp:7-33), with dt held fixed.  For step n,
// with state (prim_n, cons_n):
//   cons_{n+1} = cons_n - dt_n/dv * sum_d ds_d (F_d(c+1/2) - F_d(c-1/2))   interior cells
//   prim_{n+1} = cons_to_prim(cons_{n+1})                                  every cell
// Given cbar = dJ/dcons_{n+1}, one reverse step forms
//   pbar = (d update / d prim_n)^T cbar              the face solves below
//   dJ/dcons_n  = cbar + cons_to_prim'(prim_n)^T pbar    (n >= 1)
//   dJ/dprim_0  = pbar + prim_to_cons'(prim_0)^T cbar    (n == 0: the step reads prim_0 itself)
//
// Three kernels per reverse step, all FP64:
//   adj_prep   per cell: sound speed c and its derivatives dc/dp, dc/drho,
//              total energy, kinetic energy per mass, and the face weight
//              w = (dt/dv) cbar on interior cells (0 on ghosts, which the
//              step never updates); on cubic cells w also carries the face
//              area ds, which the face kernel then need not apply.
//   adj_face   per cell, its three upper faces: the HLLC solve recomputed
//              from prim_n (nothing of the forward solve is stored), then
//              its transpose applied to g = ds (w_R - w_L); each face's left
//              half (the cell's share) and right half (the neighbour's) are
//              stored apart.  Faces with a cotangent are queued per warp and
//              solved 32 at a time.
//   adj_gather per cell: the left halves of its three upper faces plus the
//              right halves of its three lower neighbours' -- every cell
//              reads only halves meant for it, so there are no atomics --
//              then the cons_to_prim or prim_to_cons transpose.
//
// Ties.  The HLLC flux is piecewise smooth: it takes min/max of wave-speed
// estimates and branches on the sign of ustar.  At an exact tie (equal
// min/max arguments, or ustar == 0 in the subsonic case) the derivative used
// is the mean of the two one-sided derivatives, which is what a central
// difference measures.  Ties are common: a gas at rest with uniform pressure
// and uneven density has un_L == un_R == 0 and ustar == 0 exactly at every
// face, and stays at rest step after step.  (Where ustar == 0 with both
// velocities 0, the flux does not depend on the wave speeds to first order,
// so the only one-sided difference is in the mass flux, rho_L vs rho_R times
// d ustar; its mean is linear in the perturbation.)
#include "adjoint_face.cuh"
#include "kernels.h"

namespace eulr {

namespace {

constexpr int kThreads = 256;

// Division of a cell index (below 2^31) by a grid stride d without a runtime
// division: q = floor(c m / 2^shift) with l = ceil(log2 d), shift = 31 + l and
// m = ceil(2^shift / d) < 2^32, exact for every 31-bit dividend (T. Granlund
// and P. Montgomery, "Division by invariant integers using multiplication",
// PLDI 1994, theorem 4.2).  A 64-bit division per cell was a library
// routine of several dozen instructions.
struct DivMagic {
    unsigned m;
    int shift;
};

DivMagic div_magic(long long d)
{
    int l = 0;
    while ((1ll << l) < d) {
        ++l;
    }
    unsigned long long const two = 1ull << (31 + l);
    return DivMagic{static_cast<unsigned>((two + static_cast<unsigned long long>(d) - 1) / static_cast<unsigned long long>(d)),
                    31 + l};
}

__device__ __forceinline__ int div_by(long long c, DivMagic const& dm)
{
    return static_cast<int>((static_cast<unsigned long long>(static_cast<unsigned>(c)) * dm.m) >> dm.shift);
}

struct AdjParams {
    Geom g;
    DivMagic by_s1, by_s2; // cell index -> (i, j, k)
    CBundle<double> prim;
    CBundle<double> cbar;
    Bundle<double> out;
    AdjWork w;
    double gamma, gm1, inv_gm1, half_gamma;
    double ds[3];
    bool unit;     // cubic cells: ds is folded into the weights
    double wscale; // dt / dv (times ds when unit)
    int mode;
};

__device__ __forceinline__ bool interior(Geom const& g, int i, int j, int k)
{
    return i >= 1 && i < g.n0 - 1 && j >= 1 && j < g.n1 - 1 && k >= 1 && k < g.n2 - 1;
}

// (i, j, k) of cell index c; grids hold fewer than 2^31 cells (the entry
// points reject larger ones), so 32-bit arithmetic is exact.
__device__ __forceinline__ void decode(AdjParams const& p, long long c, int& i, int& j, int& k)
{
    int const cc = static_cast<int>(c);
    k = div_by(cc, p.by_s2);
    int const r = cc - k * static_cast<int>(p.g.s2);
    j = div_by(r, p.by_s1);
    i = r - j * static_cast<int>(p.g.s1);
}

// Per-cell data of the reverse step for state `prim` at cell c (coordinates
// i, j, k): sound speed and its derivatives, energies, 1/rho, and the face
// weight wscale cbar on interior cells (wscale = dt/dv, times ds on cubic
// cells).
__device__ __forceinline__ void prep_cell(AdjParams const& p, CBundle<double> const& prim, double wscale,
                                          double const cb[5], long long c, int i, int j, int k)
{
    double const d = prim.f[0][c];
    double const pr = prim.f[1][c];
    double const u0 = prim.f[2][c];
    double const u1 = prim.f[3][c];
    double const u2 = prim.f[4][c];
    // with y = 1/sqrt(gamma p rho) (one faithful reciprocal square root):
    // c = gamma p y, dc/dp = c/(2p) = gamma y / 2, 1/rho = gamma p y^2 and
    // dc/drho = -c/(2 rho)
    double const gp = p.gamma * pr;
    double const z = gp * d;
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(z));
    double const e = __fma_rn(-(z * y), y, 1.0);
    y = __fma_rn(y, e * __fma_rn(0.375, e, 0.5), y); // third-order step, as sqrt_faithful's
    double const cs = gp * y;
    double const inv_d = cs * y;
    double const ke = adj_half(u0 * u0 + u1 * u1 + u2 * u2);
    p.w.derived[0][c] = cs;
    p.w.derived[1][c] = p.half_gamma * y;
    p.w.derived[2][c] = -adj_half(cs * inv_d);
    p.w.derived[3][c] = pr * p.inv_gm1 + d * ke;
    p.w.derived[4][c] = ke;
    p.w.derived[5][c] = inv_d;
    bool const in = interior(p.g, i, j, k);
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        p.w.weight[f][c] = in ? wscale * cb[f] : 0.0;
    }
}

__global__ void __launch_bounds__(kThreads) adj_prep_kernel(AdjParams p)
{
    long long const n = p.g.ncell();
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        int i, j, k;
        decode(p, c, i, j, k);
        double cb[5];
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            cb[f] = p.cbar.f[f][c];
        }
        prep_cell(p, p.prim, p.wscale, cb, c, i, j, k);
    }
}

__device__ __forceinline__ FaceSide load_side(AdjParams const& p, long long c, int a)
{
    FaceSide s;
    s.r = p.prim.f[0][c];
    s.p = p.prim.f[1][c];
    s.un = p.prim.f[2 + a][c];
    s.t1 = p.prim.f[2 + (a + 1) % 3][c];
    s.t2 = p.prim.f[2 + (a + 2) % 3][c];
    s.c = p.w.derived[0][c];
    s.cp = p.w.derived[1][c];
    s.cr = p.w.derived[2][c];
    s.e = p.w.derived[3][c];
    s.ke = p.w.derived[4][c];
    return s;
}

// The transposed flux of the face between cell c and c + e_a, its two halves
// stored apart: the left half (c's share) in face[a*5 + f][c], the right half
// (the neighbour's share) in face[15 + a*5 + f][c].
template <bool UNIT>
__device__ __forceinline__ void face_task(AdjParams const& p, long long c, int a)
{
    int const b = a == 2 ? 0 : a + 1, e = a == 0 ? 2 : a - 1;
    long long const cr = c + (a == 0 ? 1 : (a == 1 ? p.g.s1 : p.g.s2));
    double dw[5];
#pragma unroll
    for (int f = 0; f < 5; ++f) {
        dw[f] = p.w.weight[f][cr] - p.w.weight[f][c];
    }
    FaceSide const L = load_side(p, c, a);
    FaceSide const R = load_side(p, cr, a);
    FaceBar bL, bR;
    hllc_bar<UNIT>(L, R, dw[0], dw[1], dw[2 + a], dw[2 + b], dw[2 + e], p.ds[a], p.inv_gm1, bL, bR);
    double* const* hl = p.w.face + a * 5;
    double* const* hr = p.w.face + 15 + a * 5;
    hl[0][c] = bL.r;
    hl[1][c] = bL.p;
    hl[2 + a][c] = bL.un;
    hl[2 + b][c] = bL.t1;
    hl[2 + e][c] = bL.t2;
    hr[0][c] = bR.r;
    hr[1][c] = bR.p;
    hr[2 + a][c] = bR.un;
    hr[2 + b][c] = bR.t1;
    hr[2 + e][c] = bR.t2;
}

// Each cell's three upper faces.  The faces that carry a cotangent are not
// solved where they are found: a warp queues them in shared memory and runs
// the transposed flux 32 at a time, so no lane idles for want of a face.
// (Faces outside the cotangent's support -- the functional's region grown by
// one cell per reverse step, and wherever the two cells' weights are equal --
// are interleaved with the others at the lane level; solved in place they
// left a quarter of the FP64 lanes idle.)  Two queues keep the two paths of
// the transposed flux apart: faces of gas at rest with equal pressures on
// both sides (both normal velocities +-0, equal pressure bits: every term of
// num is a signed zero, so ustar == 0 exactly and the tie path runs) and all
// the others; mixed in one warp they cost a further 15 % of the lanes.  A
// tie found any other way still takes its own path, inside the second
// queue.  A face without work gets zero halves.  The tests run on the
// integer pipe: equal finite weights give w_R - w_L == 0 in every field.
template <bool UNIT>
__global__ void __launch_bounds__(kThreads, 2) adj_face_kernel(AdjParams p)
{
    __shared__ long long queue[kThreads / 32][2][64]; // queued faces: cell * 4 + axis
    long long const n = p.g.ncell();
    int const lane = threadIdx.x & 31;
    unsigned const below = (1u << lane) - 1u;
    long long(*const q)[64] = queue[threadIdx.x >> 5];
    int qn[2] = {0, 0}; // faces queued in this warp, per queue (the same in every lane)
    long long const stride = static_cast<long long>(gridDim.x) * blockDim.x;
    // warp-uniform trip count: every lane of a warp runs every iteration
    for (long long base = blockIdx.x * static_cast<long long>(blockDim.x) + (threadIdx.x & ~31); base < n;
         base += stride) {
        long long const c = base + lane;
        bool const valid = c < n;
        int i0 = 0, i1 = 0, i2 = 0;
        if (valid) {
            decode(p, c, i0, i1, i2);
        }
#pragma unroll 1
        for (int a = 0; a < 3; ++a) {
            // the cell's coordinate and the grid's extent along axis a and the
            // two axes after it, by selects (an array indexed by the loop
            // counter would live in local memory)
            int const ia = a == 0 ? i0 : (a == 1 ? i1 : i2);
            int const ib = a == 0 ? i1 : (a == 1 ? i2 : i0);
            int const ie = a == 0 ? i2 : (a == 1 ? i0 : i1);
            int const na = a == 0 ? p.g.n0 : (a == 1 ? p.g.n1 : p.g.n2);
            int const nb = a == 0 ? p.g.n1 : (a == 1 ? p.g.n2 : p.g.n0);
            int const ne = a == 0 ? p.g.n2 : (a == 1 ? p.g.n0 : p.g.n1);
            // the face between c and c + e_a is solved by the step when one side is interior
            bool const active =
                    valid && ia <= na - 2 && ib >= 1 && ib <= nb - 2 && ie >= 1 && ie <= ne - 2;
            bool need = false;
            bool quiet = false;
            if (active) {
                long long const cr = c + (a == 0 ? 1 : (a == 1 ? p.g.s1 : p.g.s2));
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    long long const wl = adj_bits(p.w.weight[f][c]);
                    long long const wr = adj_bits(p.w.weight[f][cr]);
                    need = need || wl != wr || (wl & 0x7ff0000000000000LL) == 0x7ff0000000000000LL;
                }
                quiet = adj_zero(p.prim.f[2 + a][c]) && adj_zero(p.prim.f[2 + a][cr]) &&
                        adj_bits(p.prim.f[1][c]) == adj_bits(p.prim.f[1][cr]);
            }
            if (valid && !need) {
#pragma unroll
                for (int f = 0; f < 5; ++f) {
                    p.w.face[a * 5 + f][c] = 0.0;
                    p.w.face[15 + a * 5 + f][c] = 0.0;
                }
            }
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                bool const mine = need && (quiet == (k == 1));
                unsigned const m = __ballot_sync(0xffffffffu, mine);
                if (mine) {
                    q[k][qn[k] + __popc(m & below)] = c * 4 + a;
                }
                qn[k] += __popc(m);
            }
            __syncwarp();
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (qn[k] >= 32) {
                    long long const t = q[k][qn[k] - 32 + lane];
                    __syncwarp(); // every lane has its task before the slots are refilled
                    qn[k] -= 32;
                    face_task<UNIT>(p, t >> 2, static_cast<int>(t & 3));
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (lane < qn[k]) {
            long long const t = q[k][lane];
            face_task<UNIT>(p, t >> 2, static_cast<int>(t & 3));
        }
    }
}

// With prev.f[0] set (mode kAdjStep), the same pass also does the prep of the
// reverse step that follows -- the state one step earlier, `prev`, with
// weight scale wscale_prev -- from the cotangent it has just formed.
__global__ void __launch_bounds__(kThreads) adj_gather_kernel(AdjParams p, CBundle<double> prev, double wscale_prev)
{
    long long const n = p.g.ncell();
    long long const stride[3] = {1, p.g.s1, p.g.s2};
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        int idx[3];
        decode(p, c, idx[0], idx[1], idx[2]);
        double pb[5];
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            // the three faces where this cell is the left side ...
            double s = p.w.face[f][c] + p.w.face[5 + f][c] + p.w.face[10 + f][c];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (idx[a] >= 1) {
                    s += p.w.face[15 + a * 5 + f][c - stride[a]]; // ... and the three where it is the right
                }
            }
            pb[f] = s;
        }
        double const d = p.prim.f[0][c];
        double const u0 = p.prim.f[2][c], u1 = p.prim.f[3][c], u2 = p.prim.f[4][c];
        double const ke = p.w.derived[4][c];
        if (p.mode == kAdjStep) {
            // cons_to_prim: p = (gamma-1)(e - |m|^2/(2d)), u = m/d
            double const inv_d = p.w.derived[5][c];
            double const gp = pb[1] * p.gm1;
            double const c0 = p.cbar.f[0][c], c1 = p.cbar.f[1][c];
            double const c2 = p.cbar.f[2][c], c3 = p.cbar.f[3][c], c4 = p.cbar.f[4][c];
            double r[5];
            r[0] = c0 + pb[0] + gp * ke - inv_d * (pb[2] * u0 + pb[3] * u1 + pb[4] * u2);
            r[1] = c1 + gp;
            r[2] = c2 + pb[2] * inv_d - gp * u0;
            r[3] = c3 + pb[3] * inv_d - gp * u1;
            r[4] = c4 + pb[4] * inv_d - gp * u2;
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                p.out.f[f][c] = r[f];
            }
            if (prev.f[0] != nullptr) { // this cell's derived data were read above
                prep_cell(p, prev, wscale_prev, r, c, idx[0], idx[1], idx[2]);
            }
        } else if (p.mode == kAdjInitial) {
            // prim_to_cons: e = p/(gamma-1) + d |u|^2 / 2, m = d u
            double const c0 = p.cbar.f[0][c], c1 = p.cbar.f[1][c];
            double const c2 = p.cbar.f[2][c], c3 = p.cbar.f[3][c], c4 = p.cbar.f[4][c];
            p.out.f[0][c] = pb[0] + c0 + c1 * ke + c2 * u0 + c3 * u1 + c4 * u2;
            p.out.f[1][c] = pb[1] + c1 * p.inv_gm1;
            p.out.f[2][c] = pb[2] + (c1 * u0 + c2) * d;
            p.out.f[3][c] = pb[3] + (c1 * u1 + c3) * d;
            p.out.f[4][c] = pb[4] + (c1 * u2 + c4) * d;
        } else {
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                p.out.f[f][c] = pb[f];
            }
        }
    }
}

// cbar (+)= cons_to_prim'(prim)^T pbar
__global__ void __launch_bounds__(kThreads) c2p_bar_kernel(CBundle<double> prim, CBundle<double> pbar,
                                                          Bundle<double> cbar, long long n, double gm1, int acc)
{
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        double const d = prim.f[0][c];
        double const u0 = prim.f[2][c], u1 = prim.f[3][c], u2 = prim.f[4][c];
        double const ke = adj_half(u0 * u0 + u1 * u1 + u2 * u2);
        double const inv_d = rcp_faithful(d);
        double const b0 = pbar.f[0][c], b2 = pbar.f[2][c], b3 = pbar.f[3][c], b4 = pbar.f[4][c];
        double const gp = pbar.f[1][c] * gm1;
        double r[5];
        r[0] = b0 + gp * ke - inv_d * (b2 * u0 + b3 * u1 + b4 * u2);
        r[1] = gp;
        r[2] = b2 * inv_d - gp * u0;
        r[3] = b3 * inv_d - gp * u1;
        r[4] = b4 * inv_d - gp * u2;
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            cbar.f[f][c] = acc ? cbar.f[f][c] + r[f] : r[f];
        }
    }
}

// pbar (+)= prim_to_cons'(prim)^T cbar
__global__ void __launch_bounds__(kThreads) p2c_bar_kernel(CBundle<double> prim, CBundle<double> cbar,
                                                          Bundle<double> pbar, long long n, double inv_gm1, int acc)
{
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        double const d = prim.f[0][c];
        double const u0 = prim.f[2][c], u1 = prim.f[3][c], u2 = prim.f[4][c];
        double const ke = adj_half(u0 * u0 + u1 * u1 + u2 * u2);
        double const c0 = cbar.f[0][c], c1 = cbar.f[1][c], c2 = cbar.f[2][c], c3 = cbar.f[3][c];
        double const c4 = cbar.f[4][c];
        double r[5];
        r[0] = c0 + c1 * ke + c2 * u0 + c3 * u1 + c4 * u2;
        r[1] = c1 * inv_gm1;
        r[2] = (c1 * u0 + c2) * d;
        r[3] = (c1 * u1 + c3) * d;
        r[4] = (c1 * u2 + c4) * d;
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            pbar.f[f][c] = acc ? pbar.f[f][c] + r[f] : r[f];
        }
    }
}

int blocks_for(long long n, int sms, int per_sm)
{
    long long const b = (n + kThreads - 1) / kThreads;
    long long const cap = static_cast<long long>(sms) * per_sm;
    return static_cast<int>(b < 1 ? 1 : (b < cap ? b : cap));
}

// Blocks of `kernel` resident on one SM (queried once per kernel): the face
// and gather kernels run one resident wave of blocks that stride over the
// grid, so that no partial last wave idles most of the GPU.
template <auto Kernel>
int resident_per_sm()
{
    static int const n = [] {
        int r = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, Kernel, kThreads, 0) != cudaSuccess || r < 1) {
            (void)cudaGetLastError();
            r = 1;
        }
        return r;
    }();
    return n;
}

size_t pad_field(long long n) { return (static_cast<size_t>(n) * sizeof(double) + 255) & ~static_cast<size_t>(255); }

} // namespace

size_t adjoint_workspace_bytes(long long ncell) { return pad_field(ncell) * kAdjWorkFields; }

AdjWork adjoint_workspace(void* base, long long ncell)
{
    AdjWork w{};
    size_t const field = pad_field(ncell);
    char* p = static_cast<char*>(base);
    for (int f = 0; f < 30; ++f, p += field) {
        w.face[f] = reinterpret_cast<double*>(p);
    }
    for (int f = 0; f < 6; ++f, p += field) {
        w.derived[f] = reinterpret_cast<double*>(p);
    }
    for (int f = 0; f < 5; ++f, p += field) {
        w.weight[f] = reinterpret_cast<double*>(p);
    }
    return w;
}

namespace {

AdjParams make_params(CBundle<double> prim, CBundle<double> cbar, Bundle<double> out, int mode, Geom g, double gamma,
                      double dx0, double dx1, double dx2, double dt, AdjWork const& w)
{
    AdjParams p;
    p.g = g;
    p.by_s1 = div_magic(g.s1);
    p.by_s2 = div_magic(g.s2);
    p.prim = prim;
    p.cbar = cbar;
    p.out = out;
    p.w = w;
    p.gamma = gamma;
    p.gm1 = gamma - 1.0;
    p.inv_gm1 = 1.0 / (gamma - 1.0);
    p.half_gamma = 0.5 * gamma;
    p.ds[0] = dx1 * dx2; // uniform_mesh.hpp:33-46
    p.ds[1] = dx2 * dx0;
    p.ds[2] = dx0 * dx1;
    p.unit = p.ds[0] == p.ds[1] && p.ds[1] == p.ds[2];
    p.wscale = dt / (dx0 * dx1 * dx2) * (p.unit ? p.ds[0] : 1.0);
    p.mode = mode;
    return p;
}

} // namespace

cudaError_t launch_step_adjoint(CBundle<double> prim, CBundle<double> cbar, Bundle<double> out, int mode, Geom g,
                                double gamma, double dx0, double dx1, double dx2, double dt, AdjWork const& w, int sms,
                                cudaStream_t s, bool prepared, CBundle<double> const* prev, double dt_prev)
{
    AdjParams const p = make_params(prim, cbar, out, mode, g, gamma, dx0, dx1, dx2, dt, w);
    long long const n = g.ncell();
    if (!prepared) {
        adj_prep_kernel<<<blocks_for(n, sms, 8), kThreads, 0, s>>>(p);
    }
    if (p.unit) {
        adj_face_kernel<true><<<blocks_for(n, sms, resident_per_sm<adj_face_kernel<true>>()), kThreads, 0, s>>>(p);
    } else {
        adj_face_kernel<false><<<blocks_for(n, sms, resident_per_sm<adj_face_kernel<false>>()), kThreads, 0, s>>>(p);
    }
    CBundle<double> pv{};
    double ws_prev = 0.0;
    if (prev != nullptr && mode == kAdjStep) {
        pv = *prev;
        ws_prev = dt_prev / (dx0 * dx1 * dx2) * (p.unit ? p.ds[0] : 1.0);
    }
    adj_gather_kernel<<<blocks_for(n, sms, resident_per_sm<adj_gather_kernel>()), kThreads, 0, s>>>(p, pv, ws_prev);
    return cudaGetLastError();
}

cudaError_t launch_cons_to_prim_adjoint(CBundle<double> prim, CBundle<double> pbar, Bundle<double> cbar,
                                        int accumulate, long long n, double gamma, int sms, cudaStream_t s)
{
    c2p_bar_kernel<<<blocks_for(n, sms, 8), kThreads, 0, s>>>(prim, pbar, cbar, n, gamma - 1.0, accumulate);
    return cudaGetLastError();
}

cudaError_t launch_prim_to_cons_adjoint(CBundle<double> prim, CBundle<double> cbar, Bundle<double> pbar,
                                        int accumulate, long long n, double gamma, int sms, cudaStream_t s)
{
    p2c_bar_kernel<<<blocks_for(n, sms, 8), kThreads, 0, s>>>(prim, cbar, pbar, n, 1.0 / (gamma - 1.0), accumulate);
    return cudaGetLastError();
}

} // namespace eulr
