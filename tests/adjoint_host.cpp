// Host build of the reverse-step face arithmetic (test harness).
//
// Compiles the product header benchmark-euler-kernels_gb300/csrc/adjoint_face.cuh
// as plain C++ and runs the reverse step of godunov the way the GPU kernels
// of adjoint.cu organise it (per-cell sound-speed data, each cell's three
// upper faces solved once, each cell summing its six face halves), so the
// CPU tests can compare the transposed flux with the host tangent-linear
// model without a GPU.  Output: prim_bar = (d godunov / d prim)^T cons_bar.
#include "adjoint_face.cuh"

#include <cmath>
#include <vector>

using namespace eulr;

extern "C" void host_godunov_adjoint(const double* const* prim, const double* const* cbar, double* const* pbar, int n0,
                                     int n1, int n2, double gamma, double dx0, double dx1, double dx2, double dt)
{
    long long const s1 = n0, s2 = static_cast<long long>(n0) * n1, n = s2 * n2;
    double const inv_gm1 = 1.0 / (gamma - 1.0);
    double const ds[3] = {dx1 * dx2, dx2 * dx0, dx0 * dx1};
    // cubic cells: the face area is folded into the weights, as the GPU kernel does
    bool const unit = ds[0] == ds[1] && ds[1] == ds[2];
    double const wscale = dt / (dx0 * dx1 * dx2) * (unit ? ds[0] : 1.0);
    std::vector<double> der(static_cast<size_t>(n) * 5), w(static_cast<size_t>(n) * 5);
    auto interior = [&](int i, int j, int k) {
        return i >= 1 && i < n0 - 1 && j >= 1 && j < n1 - 1 && k >= 1 && k < n2 - 1;
    };
    for (long long c = 0; c < n; ++c) {
        double const d = prim[0][c], p = prim[1][c];
        double const u0 = prim[2][c], u1 = prim[3][c], u2 = prim[4][c];
        double const cs = std::sqrt(gamma * p / d);
        double const ke = 0.5 * (u0 * u0 + u1 * u1 + u2 * u2);
        der[c * 5 + 0] = cs;
        der[c * 5 + 1] = 0.5 * cs / p;
        der[c * 5 + 2] = -0.5 * cs / d;
        der[c * 5 + 3] = p * inv_gm1 + d * ke;
        der[c * 5 + 4] = ke;
        int const k = static_cast<int>(c / s2), j = static_cast<int>((c % s2) / s1), i = static_cast<int>(c % s1);
        for (int f = 0; f < 5; ++f) {
            w[c * 5 + f] = interior(i, j, k) ? wscale * cbar[f][c] : 0.0;
        }
    }
    auto side = [&](long long c, int a) {
        FaceSide s;
        s.r = prim[0][c];
        s.p = prim[1][c];
        s.un = prim[2 + a][c];
        s.t1 = prim[2 + (a + 1) % 3][c];
        s.t2 = prim[2 + (a + 2) % 3][c];
        s.c = der[c * 5 + 0];
        s.cp = der[c * 5 + 1];
        s.cr = der[c * 5 + 2];
        s.e = der[c * 5 + 3];
        s.ke = der[c * 5 + 4];
        return s;
    };
    for (int f = 0; f < 5; ++f) {
        for (long long c = 0; c < n; ++c) {
            pbar[f][c] = 0.0;
        }
    }
    long long const stride[3] = {1, s1, s2};
    int const ext[3] = {n0, n1, n2};
    for (long long c = 0; c < n; ++c) {
        int idx[3] = {static_cast<int>(c % s1), static_cast<int>((c % s2) / s1), static_cast<int>(c / s2)};
        for (int a = 0; a < 3; ++a) {
            int const b = (a + 1) % 3, e = (a + 2) % 3;
            bool const active = idx[a] <= ext[a] - 2 && idx[b] >= 1 && idx[b] <= ext[b] - 2 && idx[e] >= 1 &&
                                idx[e] <= ext[e] - 2;
            if (!active) {
                continue;
            }
            long long const cr = c + stride[a];
            double dw[5];
            for (int f = 0; f < 5; ++f) {
                dw[f] = w[cr * 5 + f] - w[c * 5 + f];
            }
            FaceBar bL, bR;
            zero(bL);
            zero(bR);
            if (unit) {
                hllc_bar<true>(side(c, a), side(cr, a), dw[0], dw[1], dw[2 + a], dw[2 + b], dw[2 + e], ds[a], inv_gm1,
                               bL, bR);
            } else {
                hllc_bar<false>(side(c, a), side(cr, a), dw[0], dw[1], dw[2 + a], dw[2 + b], dw[2 + e], ds[a], inv_gm1,
                                bL, bR);
            }
            double const lv[5] = {bL.r, bL.p, bL.un, bL.t1, bL.t2};
            double const rv[5] = {bR.r, bR.p, bR.un, bR.t1, bR.t2};
            int const map[5] = {0, 1, 2 + a, 2 + b, 2 + e};
            for (int f = 0; f < 5; ++f) {
                pbar[map[f]][c] += lv[f];
                pbar[map[f]][cr] += rv[f];
            }
        }
    }
}
