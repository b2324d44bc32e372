/* CPU oracle: C restatement of the reference's Euler operators.
 *
 * TEST INFRASTRUCTURE ONLY.  Tests, the smoke check and the CPU-baseline leg
 * of bench.py use this code as the parity reference; the product path never calls it.
 *
 * Included twice by euler_oracle.c, once with REAL=double / SUF=f64 and once
 * with REAL=float / SUF=f32 (the reference's real_t switch,
 * benchmarks/real_type.hpp:3-4).  Every expression keeps the reference's
 * operand order and parenthesisation so that, compiled with
 * -ffp-contract=off, results are bit-identical to the reference's headers
 * (checked against oracle/_ref and the committed golden fixtures).
 *
 * Layout: 5 separate arrays per bundle, layout_left (i fastest), index
 * i + n0*(j + n1*k) (euler_arrays.hpp:77-85, 228-236;
 * simulations/euler_simulation.cpp:37-48).
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, CAT(_, SUF))
#define PRIM_T CAT(oracle_prim_, SUF)
#define FLUX_T CAT(oracle_flux_, SUF)

typedef struct {
    REAL d, p, u[3];
} PRIM_T; /* EulerPrim, euler_arrays.hpp:8-16 (ux0..ux2 as u[0..2]) */

typedef struct {
    REAL d, e, m[3];
} FLUX_T; /* EulerFlux / EulerCons, euler_arrays.hpp:18-36 */

/* Kokkos::min / Kokkos::max return b when b<a / a<b, else a. */
static inline REAL FN(kmin)(REAL a, REAL b) { return (b < a) ? b : a; }
static inline REAL FN(kmax)(REAL a, REAL b) { return (a < b) ? b : a; }

static inline PRIM_T FN(load_prim)(REAL const* const* f, size_t c)
{
    PRIM_T q;
    q.d = f[0][c];
    q.p = f[1][c];
    q.u[0] = f[2][c];
    q.u[1] = f[3][c];
    q.u[2] = f[4][c];
    return q;
}

/* PerfectGas::speed_of_sound, perfect_gas.hpp:15-18 */
static inline REAL FN(speed_of_sound)(REAL gamma, REAL d, REAL p) { return SQRT(gamma * p / d); }

/* kinetic_energy(EulerPrim), euler_arrays.hpp:38-42 */
static inline REAL FN(ke_prim)(PRIM_T q)
{
    return q.d * ((q.u[0] * q.u[0]) + (q.u[1] * q.u[1]) + (q.u[2] * q.u[2])) / (REAL)2;
}

/* hllc::operator(), hllc.hpp:50-105, for normal direction dir.  Always
 * inlined, so that with the direction loop unrolled dir is a constant at each
 * call, as the reference's dir_t<D> tag makes it (hllc.hpp:52-53). */
static inline __attribute__((always_inline)) FLUX_T FN(hllc)(int dir, REAL gamma, PRIM_T qL, PRIM_T qR)
{
    REAL const un_L = qL.u[dir];
    REAL const un_R = qR.u[dir];

    REAL const c_L = FN(speed_of_sound)(gamma, qL.d, qL.p);
    REAL const c_R = FN(speed_of_sound)(gamma, qR.d, qR.p);

    REAL const S_L = FN(kmin)(un_L, un_R) - FN(kmax)(c_L, c_R);
    REAL const S_R = FN(kmax)(un_L, un_R) + FN(kmax)(c_L, c_R);

    REAL const rc_L = qL.d * (S_L - un_L);
    REAL const rc_R = qR.d * (S_R - un_R);

    REAL const ustar = (qR.p - qL.p + rc_L * un_L - rc_R * un_R) / (rc_L - rc_R);
    REAL const pstar = (REAL)0.5 * (qL.p + qR.p + rc_L * (ustar - un_L) + rc_R * (ustar - un_R));

    REAL const S = ustar > 0 ? S_L : S_R;
    PRIM_T const q = ustar > 0 ? qL : qR;

    REAL const un = q.u[dir];
    /* eos.internal_energy(q.d, q.p) + kinetic_energy(q), hllc.hpp:82 */
    REAL const etot = q.p / (gamma - 1) + FN(ke_prim)(q);

    REAL const un_o = S_L * S_R > 0 ? un : ustar;
    REAL const ptot_o = S_L * S_R > 0 ? q.p : pstar;
    REAL const d_o = (S - un) / (S - un_o) * q.d;
    REAL const etot_o = ((S - un) / (S - un_o) * etot) + ((ptot_o * un_o - q.p * un) / (S - ustar));

    FLUX_T f;
    f.d = d_o * un_o;
    f.e = (etot_o + ptot_o) * un_o;
    f.m[0] = d_o * un_o * q.u[0];
    f.m[1] = d_o * un_o * q.u[1];
    f.m[2] = d_o * un_o * q.u[2];
    f.m[dir] = (d_o * un_o * un_o) + ptot_o;
    return f;
}

/* One HLLC face, for tests of other implementations of the solver: qL, qR
 * are (d, p, u0, u1, u2), f receives (d, e, m0, m1, m2). */
void FN(oracle_hllc_face)(int dir, REAL gamma, REAL const* qL, REAL const* qR, REAL* f)
{
    PRIM_T const a = {qL[0], qL[1], {qL[2], qL[3], qL[4]}};
    PRIM_T const b = {qR[0], qR[1], {qR[2], qR[3], qR[4]}};
    FLUX_T r;
    switch (dir) {
    case 0: r = FN(hllc)(0, gamma, a, b); break;
    case 1: r = FN(hllc)(1, gamma, a, b); break;
    default: r = FN(hllc)(2, gamma, a, b); break;
    }
    f[0] = r.d;
    f[1] = r.e;
    f[2] = r.m[0];
    f[3] = r.m[1];
    f[4] = r.m[2];
}

/* init_implode, init_implode.hpp:7-45.  Cell centres are evaluated in double
 * (the literal 0.5 promotes (i - 1) to double) and then rounded to REAL. */
void FN(oracle_init_implode)(REAL* const* prim, int n0, int n1, int n2, REAL dx0, REAL dx1, REAL dx2)
{
    REAL const density_in = (REAL)1.;
    REAL const density_out = (REAL)0.125;
    REAL const pressure_in = (REAL)1.;
    REAL const pressure_out = (REAL)0.14;
    REAL const radius2 = (REAL)(0.25 * 0.25);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n2; ++k) {
        for (int j = 0; j < n1; ++j) {
            for (int i = 0; i < n0; ++i) {
                REAL const c_x0 = (REAL)((((double)(i - 1) + 0.5) * (double)dx0) - 0.5);
                REAL const c_x1 = (REAL)((((double)(j - 1) + 0.5) * (double)dx1) - 0.5);
                REAL const c_x2 = (REAL)((((double)(k - 1) + 0.5) * (double)dx2) - 0.5);
                REAL const r2 = (c_x0 * c_x0) + (c_x1 * c_x1) + (c_x2 * c_x2);
                size_t const c = (size_t)i + (size_t)n0 * ((size_t)j + (size_t)n1 * (size_t)k);
                prim[0][c] = r2 < radius2 ? density_in : density_out;
                prim[1][c] = r2 < radius2 ? pressure_in : pressure_out;
                prim[2][c] = 0;
                prim[3][c] = 0;
                prim[4][c] = 0;
            }
        }
    }
}

/* Step initial condition of the batched workload (no reference counterpart):
 * cell centres ((i-1)+0.5) dx on [0,1]^3 in double, (rho_in, p_in) where
 * x0 + x1 + x2 < c, (rho_out, p_out) elsewhere, u = 0. */
void FN(oracle_init_step)(REAL* const* prim, int n0, int n1, int n2, double dx0, double dx1, double dx2, double c,
                          double rho_in, double p_in, double rho_out, double p_out)
{
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n2; ++k) {
        for (int j = 0; j < n1; ++j) {
            for (int i = 0; i < n0; ++i) {
                double const x0 = ((double)(i - 1) + 0.5) * dx0;
                double const x1 = ((double)(j - 1) + 0.5) * dx1;
                double const x2 = ((double)(k - 1) + 0.5) * dx2;
                int const inside = (x0 + x1) + x2 < c;
                size_t const o = (size_t)i + (size_t)n0 * ((size_t)j + (size_t)n1 * (size_t)k);
                prim[0][o] = (REAL)(inside ? rho_in : rho_out);
                prim[1][o] = (REAL)(inside ? p_in : p_out);
                prim[2][o] = 0;
                prim[3][o] = 0;
                prim[4][o] = 0;
            }
        }
    }
}

/* prim_to_cons, prim_to_cons.hpp:7-33 with to_cons (euler_arrays.hpp:56-64)
 * and PerfectGas::internal_energy (perfect_gas.hpp:20-23). */
void FN(oracle_prim_to_cons)(REAL const* const* prim, REAL* const* cons, int n0, int n1, int n2, REAL gamma)
{
    size_t const n = (size_t)n0 * (size_t)n1 * (size_t)n2;
#pragma omp parallel for schedule(static)
    for (size_t c = 0; c < n; ++c) {
        PRIM_T const q = FN(load_prim)(prim, c);
        REAL const int_e = q.p / (gamma - 1);
        cons[0][c] = q.d;
        cons[1][c] = FN(ke_prim)(q) + int_e;
        cons[2][c] = q.d * q.u[0];
        cons[3][c] = q.d * q.u[1];
        cons[4][c] = q.d * q.u[2];
    }
}

/* cons_to_prim, cons_to_prim.hpp:7-33 with internal_energy/kinetic_energy of
 * cons (euler_arrays.hpp:44-54), PerfectGas::pressure (perfect_gas.hpp:25-28)
 * and to_prim (euler_arrays.hpp:66-75). */
void FN(oracle_cons_to_prim)(REAL const* const* cons, REAL* const* prim, int n0, int n1, int n2, REAL gamma)
{
    size_t const n = (size_t)n0 * (size_t)n1 * (size_t)n2;
#pragma omp parallel for schedule(static)
    for (size_t c = 0; c < n; ++c) {
        REAL const d = cons[0][c];
        REAL const e = cons[1][c];
        REAL const m0 = cons[2][c];
        REAL const m1 = cons[3][c];
        REAL const m2 = cons[4][c];
        REAL const ke = ((m0 * m0) + (m1 * m1) + (m2 * m2)) / d / (REAL)2;
        REAL const p = (gamma - 1) * (e - ke);
        REAL const vol_spe = 1 / d;
        prim[0][c] = d;
        prim[1][c] = p;
        prim[2][c] = m0 * vol_spe;
        prim[3][c] = m1 * vol_spe;
        prim[4][c] = m2 * vol_spe;
    }
}

/* time_step, time_step.hpp:8-41: min over ALL cells (ghosts included) of
 * 1 / sum_d (c + |u_d|) / dx_d.  The CFL factor is applied by the caller. */
REAL FN(oracle_time_step)(REAL const* const* prim, int n0, int n1, int n2, REAL gamma, REAL dx0, REAL dx1, REAL dx2)
{
    REAL const invdx0 = 1 / dx0;
    REAL const invdx1 = 1 / dx1;
    REAL const invdx2 = 1 / dx2;
    size_t const n = (size_t)n0 * (size_t)n1 * (size_t)n2;
    REAL dt = REAL_MAX;
#pragma omp parallel
    {
        REAL loc = REAL_MAX;
#pragma omp for schedule(static)
        for (size_t c = 0; c < n; ++c) {
            PRIM_T const q = FN(load_prim)(prim, c);
            REAL const cs = FN(speed_of_sound)(gamma, q.d, q.p);
            REAL const cx0 = cs + FABS(q.u[0]);
            REAL const cx1 = cs + FABS(q.u[1]);
            REAL const cx2 = cs + FABS(q.u[2]);
            REAL const invdt = (cx0 * invdx0) + (cx1 * invdx1) + (cx2 * invdx2);
            loc = FN(kmin)(loc, 1 / invdt);
        }
#pragma omp critical
        {
            if (loc < dt) {
                dt = loc;
            }
        }
    }
    return dt;
}

/* godunov, godunov.hpp:15-92: interior cells [1, n-1)^3, two HLLC solves per
 * axis per cell, cons updated in place from read-only prim.  The (k, j) rows
 * are shared among the threads, as Kokkos's OpenMP MDRangePolicy tiles more
 * than one axis (godunov.hpp:34-43), so a slab a few planes deep still keeps
 * every core busy; cells are independent, so the split changes no bit. */
void FN(oracle_godunov)(
        REAL const* const* prim,
        REAL* const* cons,
        int n0,
        int n1,
        int n2,
        REAL gamma,
        REAL dx0,
        REAL dx1,
        REAL dx2,
        REAL dt)
{
    REAL const ds[3] = {dx1 * dx2, dx2 * dx0, dx0 * dx1}; /* uniform_mesh.hpp:33-46 */
    REAL const dtodv = dt / (dx0 * dx1 * dx2);          /* uniform_mesh.hpp:48-51 */
    ptrdiff_t const stride[3] = {1, (ptrdiff_t)n0, (ptrdiff_t)n0 * (ptrdiff_t)n1};
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k < n2 - 1; ++k) {
        for (int j = 1; j < n1 - 1; ++j) {
            for (int i = 1; i < n0 - 1; ++i) {
                size_t const c = (size_t)i + (size_t)n0 * ((size_t)j + (size_t)n1 * (size_t)k);
                PRIM_T const qc = FN(load_prim)(prim, c);
                REAL acc[5] = {0, 0, 0, 0, 0};
#pragma GCC unroll 3
                for (int dir = 0; dir < 3; ++dir) {
                    PRIM_T const qL = FN(load_prim)(prim, c - (size_t)stride[dir]);
                    PRIM_T const qR = FN(load_prim)(prim, c + (size_t)stride[dir]);
                    FLUX_T const fL = FN(hllc)(dir, gamma, qL, qc);
                    FLUX_T const fR = FN(hllc)(dir, gamma, qc, qR);
                    acc[0] += ds[dir] * (fR.d - fL.d);
                    acc[1] += ds[dir] * (fR.e - fL.e);
                    acc[2] += ds[dir] * (fR.m[0] - fL.m[0]);
                    acc[3] += ds[dir] * (fR.m[1] - fL.m[1]);
                    acc[4] += ds[dir] * (fR.m[2] - fL.m[2]);
                }
                for (int f = 0; f < 5; ++f) {
                    cons[f][c] -= dtodv * acc[f];
                }
            }
        }
    }
}

/* One step of the time loop, simulations/euler_simulation.cpp:57-67:
 * dt = time_step(prim); godunov(cfl*dt); cons_to_prim.  Returns cfl*dt. */
REAL FN(oracle_step)(
        REAL* const* prim,
        REAL* const* cons,
        int n0,
        int n1,
        int n2,
        REAL gamma,
        REAL dx0,
        REAL dx1,
        REAL dx2,
        REAL cfl)
{
    REAL const dt = FN(oracle_time_step)((REAL const* const*)prim, n0, n1, n2, gamma, dx0, dx1, dx2);
    REAL const dtc = cfl * dt;
    FN(oracle_godunov)((REAL const* const*)prim, cons, n0, n1, n2, gamma, dx0, dx1, dx2, dtc);
    FN(oracle_cons_to_prim)((REAL const* const*)cons, prim, n0, n1, n2, gamma);
    return dtc;
}

/* nsteps of the loop; the simulated time is accumulated in double. */
void FN(oracle_simulate)(
        REAL* const* prim,
        REAL* const* cons,
        int n0,
        int n1,
        int n2,
        REAL gamma,
        REAL dx0,
        REAL dx1,
        REAL dx2,
        REAL cfl,
        int nsteps,
        double* t_out)
{
    double t = 0;
    for (int it = 0; it < nsteps; ++it) {
        t += (double)FN(oracle_step)(prim, cons, n0, n1, n2, gamma, dx0, dx1, dx2, cfl);
    }
    if (t_out) {
        *t_out = t;
    }
}

#undef CAT2
#undef CAT
#undef FN
#undef PRIM_T
#undef FLUX_T
