// The reference's godunov, bit for bit (eulr_godunov_exact_{f64,f32}).
//
// The default godunov (flux.cu) solves each face once with a reformulated
// HLLC -- one shared reciprocal, FMA contraction, selects for the
// supersonic case -- and agrees with the reference to a few ulps per face.
// This kernel is the opt-in alternative for callers who need the
// reference's numbers exactly: it follows godunov.hpp:15-92 and
// hllc.hpp:50-105 operation by operation, every product, quotient, sum and
// square root rounded separately (__dmul_rn, __ddiv_rn, ...; no FMA) in the
// reference's evaluation order, with the reference's divisions and its
// two-sided pstar.
//
// The reference solves each interior face twice, once from each of its
// cells, and recomputes a cell's sound speed and total energy for every
// face it touches.  Both are the same function on the same arguments, so
// their bits do not depend on which cell asks: here each face is solved
// once and each cell's sound speed and total energy computed once, and the
// results are still the reference's.  A CTA owns a 16 x 8 column of cells
// and marches through a chunk of z-planes:
//   * two plane buffers in shared memory hold d, p, u0..u2, the sound speed
//     and the total energy of an 18 x 10 plane (the tile and its x/y halo);
//   * per plane, the 136 x-faces and 144 y-faces (one index space, 280
//     faces for 128 threads) are solved into shared memory, and each thread
//     solves the z-face above its cell into registers (the one below is the
//     previous plane's);
//   * each cell then sums ds_a (F_R - F_L) over a = 0, 1, 2 from zero and
//     subtracts dtodv times the sum from cons, as godunov.hpp:82-90 does.
// It is FP64-bound.
#include "euler_device.cuh"
#include "kernels.h"

namespace eulr {

namespace {

constexpr int kExTX = 16;                                     // tile cells along i
constexpr int kExTY = 8;                                      // tile cells along j
constexpr int kExNT = kExTX * kExTY;                          // threads per CTA
constexpr int kExPW = kExTX + 2;                              // plane buffer row (tile + x halo)
constexpr int kExPC = kExPW * (kExTY + 2);                    // plane buffer cells
constexpr int kExNX = (kExTX + 1) * kExTY;                    // x-faces of a tile plane
constexpr int kExNF = kExNX + kExTX * (kExTY + 1);            // x- and y-faces of a tile plane
static_assert(kExNF <= 3 * kExNT && kExPC <= 2 * kExNT, "the face and load loops take at most three and two passes");

// Fields of a plane buffer: the prim fields in the global order, then the
// sound speed and the total energy of each cell.
constexpr int kFieldC = 5;
constexpr int kFieldE = 6;

// Kokkos::min / Kokkos::max on two values (the reference's helpers): the
// first argument unless the second is strictly smaller / larger.  The
// comparisons run on the integer pipe with the FP64 compare's answer
// (less_ieee), so each saves an FP64 slot.
template <class T>
__device__ __forceinline__ T kmin(T a, T b)
{
    return less_ieee(b, a) ? b : a;
}
template <class T>
__device__ __forceinline__ T kmax(T a, T b)
{
    return less_ieee(a, b) ? b : a;
}

// hllc::operator() (hllc.hpp:50-105) across the face between cell ca of
// plane A (left) and cell cb of plane B (right), normal direction dir.
// The flux comes back as (d, e, normal momentum, tangential momenta along
// t1 < t2).  PerfectGas::speed_of_sound (perfect_gas.hpp:15-18) and the
// total energy (euler_arrays.hpp:38-42) come from the plane buffers, where
// each was computed once per cell with the reference's operations.
template <class T>
__device__ __forceinline__ void solve_face_exact(T const (*A)[kExPC], int ca, T const (*B)[kExPC], int cb, int dir,
                                                 T f[5])
{
    int const t1 = dir == 0 ? 1 : 0;
    int const t2 = dir == 2 ? 1 : 2;
    T const d_L = A[0][ca], p_L = A[1][ca], un_L = A[2 + dir][ca], c_L = A[kFieldC][ca];
    T const d_R = B[0][cb], p_R = B[1][cb], un_R = B[2 + dir][cb], c_R = B[kFieldC][cb];
    T const S_L = sub_rn(kmin(un_L, un_R), kmax(c_L, c_R));
    T const S_R = add_rn(kmax(un_L, un_R), kmax(c_L, c_R));
    T const rc_L = mul_rn(d_L, sub_rn(S_L, un_L));
    T const rc_R = mul_rn(d_R, sub_rn(S_R, un_R));
    // acoustic star state: q_R.p - q_L.p + rc_L * un_L - rc_R * un_R, left to right
    T const ustar = div_rn(sub_rn(add_rn(sub_rn(p_R, p_L), mul_rn(rc_L, un_L)), mul_rn(rc_R, un_R)), sub_rn(rc_L, rc_R));
    T const pstar = half_exact(add_rn(add_rn(add_rn(p_L, p_R), mul_rn(rc_L, sub_rn(ustar, un_L))),
                                          mul_rn(rc_R, sub_rn(ustar, un_R))));
    bool const left = less_ieee(T(0), ustar);
    T const (*Q)[kExPC] = left ? A : B;
    int const cq = left ? ca : cb;
    T const S = left ? S_L : S_R;
    T const d = left ? d_L : d_R;
    T const p = left ? p_L : p_R;
    T const un = left ? un_L : un_R;
    T const etot = Q[kFieldE][cq];
    bool const supersonic = less_ieee(T(0), mul_rn(S_L, S_R));
    T const un_o = supersonic ? un : ustar;
    T const ptot_o = supersonic ? p : pstar;
    T const ratio = div_rn(sub_rn(S, un), sub_rn(S, un_o));
    T const d_o = mul_rn(ratio, d);
    T const etot_o = add_rn(mul_rn(ratio, etot), div_rn(sub_rn(mul_rn(ptot_o, un_o), mul_rn(p, un)), sub_rn(S, ustar)));
    T const m = mul_rn(d_o, un_o);
    f[0] = m;
    f[1] = mul_rn(add_rn(etot_o, ptot_o), un_o);
    f[2] = add_rn(mul_rn(m, un_o), ptot_o);
    f[3] = mul_rn(m, Q[2 + t1][cq]);
    f[4] = mul_rn(m, Q[2 + t2][cq]);
}

// Loads plane k of the tile and its x/y halo (cells outside the array are
// skipped; no face reads them) with each cell's sound speed
// sqrt(gamma p / d) and total energy p / (gamma - 1) + d |u|^2 / 2.  The
// quotient by the constant gamma - 1 is the correctly rounded one formed
// from rgm1 = RN(1 / (gamma - 1)) (div_by_rcp), as prim_to_cons forms it.
template <class T>
__device__ __forceinline__ void load_plane_exact(T (*P)[kExPC], CBundle<T> const& prim, Geom const& g, int i0, int j0,
                                                 int k, T gamma, T gm1, T rgm1)
{
    for (int t = threadIdx.x; t < kExPC; t += kExNT) {
        int const i = i0 - 1 + t % kExPW;
        int const j = j0 - 1 + t / kExPW;
        if (i < g.n0 && j < g.n1) {
            long long const c = g.at(i, j, k);
            T const d = prim.f[0][c], p = prim.f[1][c];
            T const u0 = prim.f[2][c], u1 = prim.f[3][c], u2 = prim.f[4][c];
            P[0][t] = d;
            P[1][t] = p;
            P[2][t] = u0;
            P[3][t] = u1;
            P[4][t] = u2;
            P[kFieldC][t] = sqrt_rn(div_rn(mul_rn(gamma, p), d));
            // the reference's "/ 2" as "* 0.5": both are the correctly rounded
            // value of the same real number, so the bits are equal
            T const ke = half_exact(mul_rn(d, add_rn(add_rn(mul_rn(u0, u0), mul_rn(u1, u1)), mul_rn(u2, u2))));
            P[kFieldE][t] = add_rn(div_by_rcp(p, gm1, rgm1), ke);
        }
    }
}

// godunov.hpp:32-91 for the interior cells of one 16 x 8 tile over the
// interior planes [kb, ke); blockIdx.x = tile, blockIdx.y = plane chunk.
template <class T>
__global__ void __launch_bounds__(kExNT) godunov_exact_kernel(CBundle<T> prim, Bundle<T> cons, Geom g, T gamma, T gm1,
                                                              T rgm1, T ds0, T ds1, T ds2, T dtodv, int ntx,
                                                              int kchunk)
{
    __shared__ T planes[2][7][kExPC];
    __shared__ T faces[5][kExNF];
    int const i0 = 1 + (blockIdx.x % ntx) * kExTX;
    int const j0 = 1 + (blockIdx.x / ntx) * kExTY;
    int const kb = 1 + blockIdx.y * kchunk;
    int const ke = min(kb + kchunk, g.n2 - 1);
    int const tx = threadIdx.x % kExTX;
    int const ty = threadIdx.x / kExTX;
    bool const mine = i0 + tx <= g.n0 - 2 && j0 + ty <= g.n1 - 2; // this thread's column is interior
    int const ccell = (tx + 1) + kExPW * (ty + 1);                 // its cell in a plane buffer

    T zlo[5], zhi[5];
    load_plane_exact(planes[(kb - 1) & 1], prim, g, i0, j0, kb - 1, gamma, gm1, rgm1);
    load_plane_exact(planes[kb & 1], prim, g, i0, j0, kb, gamma, gm1, rgm1);
    __syncthreads();
    if (mine) {
        solve_face_exact(planes[(kb - 1) & 1], ccell, planes[kb & 1], ccell, 2, zlo);
    }
    __syncthreads(); // plane kb - 1 is overwritten next
    for (int k = kb; k < ke; ++k) {
        T const (*cur)[kExPC] = planes[k & 1];
        load_plane_exact(planes[(k + 1) & 1], prim, g, i0, j0, k + 1, gamma, gm1, rgm1);
        __syncthreads();
        // x-faces (i-1 | i) for i in [i0, i0 + 16], then y-faces (j-1 | j) for j in [j0, j0 + 8]
        for (int t = threadIdx.x; t < kExNF; t += kExNT) {
            bool const xf = t < kExNX;
            int const u = xf ? t : t - kExNX;
            int const a = xf ? u % (kExTX + 1) : u % kExTX;
            int const b = xf ? u / (kExTX + 1) : u / kExTX;
            bool const need = xf ? (i0 + a <= g.n0 - 1 && j0 + b <= g.n1 - 2)
                                 : (i0 + a <= g.n0 - 2 && j0 + b <= g.n1 - 1);
            if (need) {
                int const cl = xf ? a + kExPW * (b + 1) : (a + 1) + kExPW * b;
                int const cr = cl + (xf ? 1 : kExPW);
                int const dir = xf ? 0 : 1;
                T f[5];
                solve_face_exact(cur, cl, cur, cr, dir, f);
                faces[0][t] = f[0];
                faces[1][t] = f[1];
                faces[2 + dir][t] = f[2];
                faces[xf ? 3 : 2][t] = f[3];
                faces[4][t] = f[4];
            }
        }
        if (mine) {
            solve_face_exact(cur, ccell, planes[(k + 1) & 1], ccell, 2, zhi);
        }
        __syncthreads();
        if (mine) {
            int const xl = tx + (kExTX + 1) * ty;
            int const yl = kExNX + tx + kExTX * ty;
            long long const c = g.at(i0 + tx, j0 + ty, k);
            T const zl[5] = {zlo[0], zlo[1], zlo[3], zlo[4], zlo[2]}; // (d, e, m0, m1, m2)
            T const zh[5] = {zhi[0], zhi[1], zhi[3], zhi[4], zhi[2]};
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                T flux = T(0);
                flux = add_rn(flux, mul_rn(ds0, sub_rn(faces[f][xl + 1], faces[f][xl])));
                flux = add_rn(flux, mul_rn(ds1, sub_rn(faces[f][yl + kExTX], faces[f][yl])));
                flux = add_rn(flux, mul_rn(ds2, sub_rn(zh[f], zl[f])));
                cons.f[f][c] = sub_rn(cons.f[f][c], mul_rn(dtodv, flux));
            }
        }
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            zlo[f] = zhi[f];
        }
    }
}

} // namespace

template <class T>
cudaError_t launch_godunov_exact(CBundle<T> prim, Bundle<T> cons, Geom g, T gamma, T dx0, T dx1, T dx2, T dt,
                                 int sms, cudaStream_t s)
{
    if (g.n0 < 3 || g.n1 < 3 || g.n2 < 3) {
        return cudaSuccess; // no interior cell
    }
    // UniformMesh3d: ds0 = dx1 dx2, ds1 = dx2 dx0, ds2 = dx0 dx1, dv = dx0 dx1 dx2
    // (uniform_mesh.hpp:33-51), and dtodv = dt / dv (godunov.hpp:31), all in T
    T const ds0 = dx1 * dx2;
    T const ds1 = dx2 * dx0;
    T const ds2 = dx0 * dx1;
    T const dv = (dx0 * dx1) * dx2;
    T const dtodv = dt / dv;
    long long const ntx = (g.n0 - 2 + kExTX - 1) / kExTX;
    long long const tiles = ntx * ((g.n1 - 2 + kExTY - 1) / kExTY);
    int const planes = g.n2 - 2;
    if (tiles > 0x7fffffffLL) {
        return cudaErrorInvalidConfiguration;
    }
    // Split the planes into chunks of at least 8 until there are about 64
    // CTAs per SM to spread, so that the last wave is a small part.
    long long want = (64LL * sms + tiles - 1) / tiles;
    long long const most = planes / 8 > 1 ? planes / 8 : 1;
    want = want < 1 ? 1 : (want > most ? most : want);
    want = want > 65535 ? 65535 : want;
    int const kchunk = static_cast<int>((planes + want - 1) / want);
    int const nchunks = (planes + kchunk - 1) / kchunk;
    dim3 const grid(static_cast<unsigned>(tiles), static_cast<unsigned>(nchunks));
    T const gm1 = gamma - T(1);
    godunov_exact_kernel<T><<<grid, kExNT, 0, s>>>(prim, cons, g, gamma, gm1, T(1) / gm1, ds0, ds1, ds2, dtodv,
                                                   static_cast<int>(ntx), kchunk);
    return cudaGetLastError();
}

template cudaError_t launch_godunov_exact<double>(CBundle<double>, Bundle<double>, Geom, double, double, double,
                                                  double, double, int, cudaStream_t);
template cudaError_t launch_godunov_exact<float>(CBundle<float>, Bundle<float>, Geom, float, float, float, float,
                                                 float, int, cudaStream_t);

} // namespace eulr
