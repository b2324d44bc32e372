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
// two-sided pstar.  One thread per interior cell solves the cell's six
// faces as the reference loop does (each interior face is solved by both of
// its cells; both get the same bits, since they call the same function on
// the same arguments).  It is FP64-bound and about four times slower than
// the default path.
#include "euler_device.cuh"
#include "kernels.h"

namespace eulr {

namespace {

template <class T>
struct ExactPrim {
    T d, p, u[3];
};

// Kokkos::min / Kokkos::max on two values (the reference's helpers): the
// first argument unless the second is strictly smaller / larger.
template <class T>
__device__ __forceinline__ T kmin(T a, T b)
{
    return (b < a) ? b : a;
}
template <class T>
__device__ __forceinline__ T kmax(T a, T b)
{
    return (a < b) ? b : a;
}

// PerfectGas::speed_of_sound: sqrt(gamma * p / rho) (perfect_gas.hpp:15-18).
template <class T>
__device__ __forceinline__ T sound_speed_exact(T gamma, T d, T p)
{
    return sqrt_rn(div_rn(mul_rn(gamma, p), d));
}

// hllc::operator() for normal direction dir (hllc.hpp:50-105); the flux in
// the global field order (d, e, mx0, mx1, mx2).
template <class T>
__device__ __forceinline__ void hllc_exact(int dir, T gamma, T gm1, ExactPrim<T> const& L, ExactPrim<T> const& R,
                                           T f[5])
{
    T const un_L = L.u[dir];
    T const un_R = R.u[dir];
    T const c_L = sound_speed_exact(gamma, L.d, L.p);
    T const c_R = sound_speed_exact(gamma, R.d, R.p);
    T const S_L = sub_rn(kmin(un_L, un_R), kmax(c_L, c_R));
    T const S_R = add_rn(kmax(un_L, un_R), kmax(c_L, c_R));
    T const rc_L = mul_rn(L.d, sub_rn(S_L, un_L));
    T const rc_R = mul_rn(R.d, sub_rn(S_R, un_R));
    // acoustic star state: q_R.p - q_L.p + rc_L * un_L - rc_R * un_R, left to right
    T const ustar = div_rn(sub_rn(add_rn(sub_rn(R.p, L.p), mul_rn(rc_L, un_L)), mul_rn(rc_R, un_R)), sub_rn(rc_L, rc_R));
    T const pstar = mul_rn(T(0.5), add_rn(add_rn(add_rn(L.p, R.p), mul_rn(rc_L, sub_rn(ustar, un_L))),
                                          mul_rn(rc_R, sub_rn(ustar, un_R))));
    bool const left = ustar > T(0);
    T const S = left ? S_L : S_R;
    ExactPrim<T> const& q = left ? L : R;
    T const un = q.u[dir];
    // eos.internal_energy(q.d, q.p) + kinetic_energy(q) (euler_arrays.hpp:38-42)
    T const ke = div_rn(mul_rn(q.d, add_rn(add_rn(mul_rn(q.u[0], q.u[0]), mul_rn(q.u[1], q.u[1])),
                                           mul_rn(q.u[2], q.u[2]))),
                        T(2));
    T const etot = add_rn(div_rn(q.p, gm1), ke);
    bool const supersonic = mul_rn(S_L, S_R) > T(0);
    T const un_o = supersonic ? un : ustar;
    T const ptot_o = supersonic ? q.p : pstar;
    T const ratio = div_rn(sub_rn(S, un), sub_rn(S, un_o));
    T const d_o = mul_rn(ratio, q.d);
    T const etot_o = add_rn(mul_rn(ratio, etot), div_rn(sub_rn(mul_rn(ptot_o, un_o), mul_rn(q.p, un)), sub_rn(S, ustar)));
    T const m = mul_rn(d_o, un_o);
    f[0] = m;
    f[1] = mul_rn(add_rn(etot_o, ptot_o), un_o);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        f[2 + a] = a == dir ? add_rn(mul_rn(m, un_o), ptot_o) : mul_rn(m, q.u[a]);
    }
}

template <class T>
__device__ __forceinline__ ExactPrim<T> load_exact(CBundle<T> const& prim, long long c)
{
    ExactPrim<T> q;
    q.d = prim.f[0][c];
    q.p = prim.f[1][c];
    q.u[0] = prim.f[2][c];
    q.u[1] = prim.f[3][c];
    q.u[2] = prim.f[4][c];
    return q;
}

// godunov.hpp:32-91 for the interior cells [1, n-1)^3: per axis the fluxes
// of the cell's two faces, flux += ds[a] * (F_R - F_L) starting from zero,
// then cons -= dtodv * flux.
template <class T>
__global__ void __launch_bounds__(256) godunov_exact_kernel(CBundle<T> prim, Bundle<T> cons, Geom g, T gamma, T gm1,
                                                            T ds0, T ds1, T ds2, T dtodv)
{
    int const ix = g.n0 - 2, iy = g.n1 - 2;
    long long const n = static_cast<long long>(ix) * iy * (g.n2 - 2);
    T const ds[3] = {ds0, ds1, ds2};
    long long const stride[3] = {1, g.s1, g.s2};
    for (long long t = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < n;
         t += static_cast<long long>(gridDim.x) * blockDim.x) {
        int const i = 1 + static_cast<int>(t % ix);
        long long const r = t / ix;
        int const j = 1 + static_cast<int>(r % iy);
        int const k = 1 + static_cast<int>(r / iy);
        long long const c = g.at(i, j, k);
        ExactPrim<T> const qc = load_exact(prim, c);
        T flux[5] = {T(0), T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            T fL[5], fR[5];
            hllc_exact(a, gamma, gm1, load_exact(prim, c - stride[a]), qc, fL);
            hllc_exact(a, gamma, gm1, qc, load_exact(prim, c + stride[a]), fR);
#pragma unroll
            for (int f = 0; f < 5; ++f) {
                flux[f] = add_rn(flux[f], mul_rn(ds[a], sub_rn(fR[f], fL[f])));
            }
        }
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            cons.f[f][c] = sub_rn(cons.f[f][c], mul_rn(dtodv, flux[f]));
        }
    }
}

} // namespace

template <class T>
cudaError_t launch_godunov_exact(CBundle<T> prim, Bundle<T> cons, Geom g, T gamma, T dx0, T dx1, T dx2, T dt,
                                 int sms, cudaStream_t s)
{
    long long const n = static_cast<long long>(g.n0 - 2) * (g.n1 - 2) * (g.n2 - 2);
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
    long long blocks = (n + 255) / 256;
    long long const cap = static_cast<long long>(sms) * 8;
    if (blocks > cap) {
        blocks = cap;
    }
    godunov_exact_kernel<T><<<static_cast<int>(blocks), 256, 0, s>>>(prim, cons, g, gamma, gamma - T(1), ds0, ds1, ds2,
                                                                    dtodv);
    return cudaGetLastError();
}

template cudaError_t launch_godunov_exact<double>(CBundle<double>, Bundle<double>, Geom, double, double, double,
                                                  double, double, int, cudaStream_t);
template cudaError_t launch_godunov_exact<float>(CBundle<float>, Bundle<float>, Geom, float, float, float, float,
                                                 float, int, cudaStream_t);

} // namespace eulr
