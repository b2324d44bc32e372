/* Host tangent-linear model of the Euler time step (TEST INFRASTRUCTURE ONLY).
 *
 * Tests use it as the reference gradient of the adjoint (dot-product tests
 * and a full gradient on small grids); the product never calls it.  It
 * differentiates, in forward mode, the reference's operators:
 *   prim_to_cons  prim_to_cons.hpp:7-33 (to_cons, euler_arrays.hpp:56-64)
 *   cons_to_prim  cons_to_prim.hpp:7-33 (euler_arrays.hpp:44-54, 66-75)
 *   godunov       godunov.hpp:15-92 with hllc.hpp:50-105
 * with dt a constant.  Every value is computed with the operand order of
 * euler_oracle_body.h (compiled with -ffp-contract=off), so the values match
 * the oracle's bit for bit; tangents follow the chain rule of the same
 * expressions.  Tie rule: where the flux takes min/max of equal arguments,
 * or ustar == 0 in the subsonic case, the tangent is the mean of the two
 * one-sided tangents (a central difference measures that mean).
 */
#include "euler_tlm.h"

#include <math.h>
#include <stddef.h>

typedef struct {
    double d, p, u[3];
} tq; /* primitive state */

typedef struct {
    double d, e, m[3];
} tf; /* flux / conservative state */

static inline double kmin(double a, double b) { return (b < a) ? b : a; }
static inline double kmax(double a, double b) { return (a < b) ? b : a; }
static inline double dmin(double a, double b, double da, double db)
{
    return a < b ? da : (b < a ? db : 0.5 * (da + db));
}
static inline double dmax(double a, double b, double da, double db)
{
    return a < b ? db : (b < a ? da : 0.5 * (da + db));
}

static inline tq load_q(double const* const* f, size_t c)
{
    tq q;
    q.d = f[0][c];
    q.p = f[1][c];
    q.u[0] = f[2][c];
    q.u[1] = f[3][c];
    q.u[2] = f[4][c];
    return q;
}

/* kinetic_energy(EulerPrim) = d (u.u) / 2 and its tangent */
static inline double ke_prim(tq q) { return q.d * ((q.u[0] * q.u[0]) + (q.u[1] * q.u[1]) + (q.u[2] * q.u[2])) / 2.0; }
static inline double dke_prim(tq q, tq dq)
{
    double const uu = (q.u[0] * q.u[0]) + (q.u[1] * q.u[1]) + (q.u[2] * q.u[2]);
    double const udu = q.u[0] * dq.u[0] + q.u[1] * dq.u[1] + q.u[2] * dq.u[2];
    return dq.d * uu / 2.0 + q.d * udu;
}

/* star-state branch of side q (hllc.hpp:78-102, subsonic): tangent only */
static void star_tangent(int dir, double gamma, tq q, tq dq, double S, double dS, double ustar, double dustar,
                         double pstar, double dpstar, tf* dF)
{
    double const un = q.u[dir];
    double const dun = dq.u[dir];
    double const etot = q.p / (gamma - 1) + ke_prim(q);
    double const detot = dq.p / (gamma - 1) + dke_prim(q, dq);
    double const Y = S - ustar;
    double const dY = dS - dustar;
    double const ratio = (S - un) / Y;
    double const dratio = ((dS - dun) - ratio * dY) / Y;
    double const d_o = ratio * q.d;
    double const dd_o = dratio * q.d + ratio * dq.d;
    double const X = pstar * ustar - q.p * un;
    double const dX = dpstar * ustar + pstar * dustar - dq.p * un - q.p * dun;
    double const eo = ratio * etot + X / Y;
    double const deo = dratio * etot + ratio * detot + (dX - (X / Y) * dY) / Y;
    double const m = d_o * ustar;
    double const dm = dd_o * ustar + d_o * dustar;
    dF->d = dm;
    dF->e = (deo + dpstar) * ustar + (eo + pstar) * dustar;
    for (int t = 0; t < 3; ++t) {
        dF->m[t] = dm * q.u[t] + m * dq.u[t];
    }
    dF->m[dir] = dm * ustar + m * dustar + dpstar;
}

/* physical flux of side q (the S_L * S_R > 0 case): tangent only */
static void physical_tangent(int dir, double gamma, tq q, tq dq, tf* dF)
{
    double const un = q.u[dir];
    double const dun = dq.u[dir];
    double const etot = q.p / (gamma - 1) + ke_prim(q);
    double const detot = dq.p / (gamma - 1) + dke_prim(q, dq);
    double const m = q.d * un;
    double const dm = dq.d * un + q.d * dun;
    dF->d = dm;
    dF->e = (detot + dq.p) * un + (etot + q.p) * dun;
    for (int t = 0; t < 3; ++t) {
        dF->m[t] = dm * q.u[t] + m * dq.u[t];
    }
    dF->m[dir] = dm * un + m * dun + dq.p;
}

/* hllc::operator() (hllc.hpp:50-105): value F as euler_oracle_body.h
 * computes it, and its tangent dF. */
static void hllc_tlm(int dir, double gamma, tq qL, tq dqL, tq qR, tq dqR, tf* F, tf* dF)
{
    double const un_L = qL.u[dir];
    double const un_R = qR.u[dir];
    double const dun_L = dqL.u[dir];
    double const dun_R = dqR.u[dir];
    double const c_L = sqrt(gamma * qL.p / qL.d);
    double const c_R = sqrt(gamma * qR.p / qR.d);
    double const dc_L = 0.5 * c_L * (dqL.p / qL.p - dqL.d / qL.d);
    double const dc_R = 0.5 * c_R * (dqR.p / qR.p - dqR.d / qR.d);
    double const cmax = kmax(c_L, c_R);
    double const dcmax = dmax(c_L, c_R, dc_L, dc_R);
    double const S_L = kmin(un_L, un_R) - cmax;
    double const S_R = kmax(un_L, un_R) + cmax;
    double const dS_L = dmin(un_L, un_R, dun_L, dun_R) - dcmax;
    double const dS_R = dmax(un_L, un_R, dun_L, dun_R) + dcmax;
    double const rc_L = qL.d * (S_L - un_L);
    double const rc_R = qR.d * (S_R - un_R);
    double const drc_L = dqL.d * (S_L - un_L) + qL.d * (dS_L - dun_L);
    double const drc_R = dqR.d * (S_R - un_R) + qR.d * (dS_R - dun_R);
    double const ustar = (qR.p - qL.p + rc_L * un_L - rc_R * un_R) / (rc_L - rc_R);
    double const pstar = 0.5 * (qL.p + qR.p + rc_L * (ustar - un_L) + rc_R * (ustar - un_R));
    double const dnum = dqR.p - dqL.p + drc_L * un_L + rc_L * dun_L - drc_R * un_R - rc_R * dun_R;
    double const dustar = (dnum - ustar * (drc_L - drc_R)) / (rc_L - rc_R);
    double const dpstar = 0.5 * (dqL.p + dqR.p + drc_L * (ustar - un_L) + rc_L * (dustar - dun_L) +
                                 drc_R * (ustar - un_R) + rc_R * (dustar - dun_R));

    /* value: exactly the oracle's expression sequence */
    double const S = ustar > 0 ? S_L : S_R;
    tq const q = ustar > 0 ? qL : qR;
    double const un = q.u[dir];
    double const etot = q.p / (gamma - 1) + ke_prim(q);
    double const un_o = S_L * S_R > 0 ? un : ustar;
    double const ptot_o = S_L * S_R > 0 ? q.p : pstar;
    double const d_o = (S - un) / (S - un_o) * q.d;
    double const etot_o = ((S - un) / (S - un_o) * etot) + ((ptot_o * un_o - q.p * un) / (S - ustar));
    F->d = d_o * un_o;
    F->e = (etot_o + ptot_o) * un_o;
    F->m[0] = d_o * un_o * q.u[0];
    F->m[1] = d_o * un_o * q.u[1];
    F->m[2] = d_o * un_o * q.u[2];
    F->m[dir] = (d_o * un_o * un_o) + ptot_o;

    /* tangent */
    if (S_L * S_R > 0) {
        physical_tangent(dir, gamma, q, ustar > 0 ? dqL : dqR, dF);
    } else if (ustar != 0) {
        int const left = ustar > 0;
        star_tangent(dir, gamma, q, left ? dqL : dqR, S, left ? dS_L : dS_R, ustar, dustar, pstar, dpstar, dF);
    } else {
        tf a, b;
        star_tangent(dir, gamma, qL, dqL, S_L, dS_L, ustar, dustar, pstar, dpstar, &a);
        star_tangent(dir, gamma, qR, dqR, S_R, dS_R, ustar, dustar, pstar, dpstar, &b);
        dF->d = 0.5 * (a.d + b.d);
        dF->e = 0.5 * (a.e + b.e);
        for (int t = 0; t < 3; ++t) {
            dF->m[t] = 0.5 * (a.m[t] + b.m[t]);
        }
    }
}

void oracle_tlm_prim_to_cons_f64(double const* const* prim, double const* const* dprim, double* const* cons,
                                 double* const* dcons, int n0, int n1, int n2, double gamma)
{
    size_t const n = (size_t)n0 * (size_t)n1 * (size_t)n2;
#pragma omp parallel for schedule(static)
    for (size_t c = 0; c < n; ++c) {
        tq const q = load_q(prim, c);
        tq const dq = load_q(dprim, c);
        double const int_e = q.p / (gamma - 1);
        cons[0][c] = q.d;
        cons[1][c] = ke_prim(q) + int_e;
        cons[2][c] = q.d * q.u[0];
        cons[3][c] = q.d * q.u[1];
        cons[4][c] = q.d * q.u[2];
        dcons[0][c] = dq.d;
        dcons[1][c] = dke_prim(q, dq) + dq.p / (gamma - 1);
        for (int t = 0; t < 3; ++t) {
            dcons[2 + t][c] = dq.d * q.u[t] + q.d * dq.u[t];
        }
    }
}

void oracle_tlm_cons_to_prim_f64(double const* const* cons, double const* const* dcons, double* const* prim,
                                 double* const* dprim, int n0, int n1, int n2, double gamma)
{
    size_t const n = (size_t)n0 * (size_t)n1 * (size_t)n2;
#pragma omp parallel for schedule(static)
    for (size_t c = 0; c < n; ++c) {
        double const d = cons[0][c];
        double const e = cons[1][c];
        double const m0 = cons[2][c];
        double const m1 = cons[3][c];
        double const m2 = cons[4][c];
        double const dd = dcons[0][c];
        double const de = dcons[1][c];
        double const dm0 = dcons[2][c];
        double const dm1 = dcons[3][c];
        double const dm2 = dcons[4][c];
        double const ke = ((m0 * m0) + (m1 * m1) + (m2 * m2)) / d / 2.0;
        double const p = (gamma - 1) * (e - ke);
        double const vol_spe = 1 / d;
        prim[0][c] = d;
        prim[1][c] = p;
        prim[2][c] = m0 * vol_spe;
        prim[3][c] = m1 * vol_spe;
        prim[4][c] = m2 * vol_spe;
        double const dke = (m0 * dm0 + m1 * dm1 + m2 * dm2) / d - ke * dd / d;
        double const dvol = -dd / (d * d);
        dprim[0][c] = dd;
        dprim[1][c] = (gamma - 1) * (de - dke);
        dprim[2][c] = dm0 * vol_spe + m0 * dvol;
        dprim[3][c] = dm1 * vol_spe + m1 * dvol;
        dprim[4][c] = dm2 * vol_spe + m2 * dvol;
    }
}

void oracle_tlm_godunov_f64(double const* const* prim, double const* const* dprim, double* const* cons,
                            double* const* dcons, int n0, int n1, int n2, double gamma, double dx0, double dx1,
                            double dx2, double dt)
{
    double const ds[3] = {dx1 * dx2, dx2 * dx0, dx0 * dx1};
    double const dtodv = dt / (dx0 * dx1 * dx2);
    ptrdiff_t const stride[3] = {1, (ptrdiff_t)n0, (ptrdiff_t)n0 * (ptrdiff_t)n1};
#pragma omp parallel for schedule(static)
    for (int k = 1; k < n2 - 1; ++k) {
        for (int j = 1; j < n1 - 1; ++j) {
            for (int i = 1; i < n0 - 1; ++i) {
                size_t const c = (size_t)i + (size_t)n0 * ((size_t)j + (size_t)n1 * (size_t)k);
                tq const qc = load_q(prim, c);
                tq const dqc = load_q(dprim, c);
                double acc[5] = {0, 0, 0, 0, 0};
                double dacc[5] = {0, 0, 0, 0, 0};
                for (int dir = 0; dir < 3; ++dir) {
                    size_t const cl = c - (size_t)stride[dir];
                    size_t const cr = c + (size_t)stride[dir];
                    tf fL, dfL, fR, dfR;
                    hllc_tlm(dir, gamma, load_q(prim, cl), load_q(dprim, cl), qc, dqc, &fL, &dfL);
                    hllc_tlm(dir, gamma, qc, dqc, load_q(prim, cr), load_q(dprim, cr), &fR, &dfR);
                    acc[0] += ds[dir] * (fR.d - fL.d);
                    acc[1] += ds[dir] * (fR.e - fL.e);
                    acc[2] += ds[dir] * (fR.m[0] - fL.m[0]);
                    acc[3] += ds[dir] * (fR.m[1] - fL.m[1]);
                    acc[4] += ds[dir] * (fR.m[2] - fL.m[2]);
                    dacc[0] += ds[dir] * (dfR.d - dfL.d);
                    dacc[1] += ds[dir] * (dfR.e - dfL.e);
                    dacc[2] += ds[dir] * (dfR.m[0] - dfL.m[0]);
                    dacc[3] += ds[dir] * (dfR.m[1] - dfL.m[1]);
                    dacc[4] += ds[dir] * (dfR.m[2] - dfL.m[2]);
                }
                for (int f = 0; f < 5; ++f) {
                    cons[f][c] -= dtodv * acc[f];
                    dcons[f][c] -= dtodv * dacc[f];
                }
            }
        }
    }
}

void oracle_tlm_simulate_f64(double* const* prim, double* const* dprim, double* const* cons, double* const* dcons,
                             int n0, int n1, int n2, double gamma, double dx0, double dx1, double dx2,
                             double const* dts, int nsteps)
{
    oracle_tlm_prim_to_cons_f64((double const* const*)prim, (double const* const*)dprim, cons, dcons, n0, n1, n2,
                                gamma);
    for (int s = 0; s < nsteps; ++s) {
        oracle_tlm_godunov_f64((double const* const*)prim, (double const* const*)dprim, cons, dcons, n0, n1, n2,
                               gamma, dx0, dx1, dx2, dts[s]);
        oracle_tlm_cons_to_prim_f64((double const* const*)cons, (double const* const*)dcons, prim, dprim, n0, n1, n2,
                                    gamma);
    }
}
